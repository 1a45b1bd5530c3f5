"""Shared far fields (vct_config.far_share, the default of the texture-unit
sampler): every diffuse cone takes its first sample per pixel; the rest of
the march is done once per group of 4x2 pixels (FAR_SHARE_GROUP_W x 2) along
the cones of the group's representative, by the lanes of a warp together.

Tolerances: against the same frame with every pixel marching all its cones
(far_share 0): PSNR >= 45 dB on the small scenes (96x64 and smaller frames:
a group covers more of the scene), >= 60 dB on the 1080p bench frame;
against the FP64 oracle's per-pixel rule (from the GPU's own maps and
G-buffer): PSNR >= 40 dB, the tolerance of the texture-unit sampler; against
the oracle's restatement of the sharing rule: PSNR >= 50 dB (what remains
is the texture unit's filtering); frames repeat bit for bit (the far-field
jobs are dealt to lanes in a fixed order)."""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render(vct, scene, w, h, n, **cfg):
    r = vct.Renderer(w, h, grid_res=n, keep_float_frame=1, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r, ids


def _gb64(gb):
    return dict(tri_id=gb["tri_id"], pos=gb["pos"].astype(np.float64), nrm=gb["nrm"].astype(np.float64),
                mat=gb["mat"])


def _chains(r, nmaps):
    from oracle import oracle as O
    n, levels = r.grid()
    ch = np.zeros((nmaps, O.chain_texels(n, levels), 4), np.uint8)
    off = 0
    for lvl in range(1, levels):
        s = n >> lvl
        for m in range(nmaps):
            ch[m, off:off + s ** 3] = r.read_voxels(lvl, m).reshape(-1, 4)
        off += s ** 3
    return ch


CASES = {"aniso_ref9": dict(), "iso_six60": dict(mip_mode=1, cone_set=1), "aniso_six60": dict(cone_set=1)}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("size", [(96, 64), (83, 37)], ids=["96x64", "ragged_83x37"])
def test_shared_far_fields_small(vct, oracle, case, size):
    w, h = size
    cfg = CASES[case]
    scene = scenes.scene_small(width=w, height=h)
    a, ids = _render(vct, scene, w, h, 64, **cfg)
    b, _ = _render(vct, scene, w, h, 64, far_share=0, **cfg)
    fa, fb = a.read_frame(vct.FRAME_RGBA32F), b.read_frame(vct.FRAME_RGBA32F)
    q = psnr(np.clip(fa, 0, 1), np.clip(fb, 0, 1))
    vct.queue_scene(a, scene, ids)
    a.render()
    np.testing.assert_array_equal(a.read_frame(vct.FRAME_RGBA32F), fa)
    p = oracle.Params(grid_res=64, width=w, height=h, mip_mode=cfg.get("mip_mode", 0),
                      cone_set=cfg.get("cone_set", 0))
    l0, ch, gb = a.read_voxels(0), _chains(a, p.n_maps), _gb64(a.read_gbuffer())
    ref = oracle.trace(scene, p, l0, ch, gb)
    p.far_share = vct.FAR_SHARE_GROUP_W
    ref_sh = oracle.trace(scene, p, l0, ch, gb)  # the oracle's restatement of the sharing rule
    qo = psnr(np.clip(fa, 0, 1), np.clip(ref, 0, 1))
    qs = psnr(np.clip(fa, 0, 1), np.clip(ref_sh, 0, 1))
    qr = psnr(np.clip(ref_sh, 0, 1), np.clip(ref, 0, 1))
    print(f"{case} {w}x{h}: shared vs per-pixel {q:.1f} dB; vs oracle {qo:.1f} dB, vs the oracle's sharing rule "
          f"{qs:.1f} dB (that rule vs per-pixel: {qr:.1f} dB)")
    assert q >= 45.0
    assert qo >= 40.0
    assert qs >= 50.0


def test_shared_far_fields_bench_frame(vct):
    scene = scenes.scene_sphere(width=1920, height=1080)
    a, _ = _render(vct, scene, 1920, 1080, 256)
    b, _ = _render(vct, scene, 1920, 1080, 256, far_share=0)
    fa, fb = a.read_frame(vct.FRAME_RGBA32F), b.read_frame(vct.FRAME_RGBA32F)
    q = psnr(np.clip(fa, 0, 1), np.clip(fb, 0, 1))
    d = np.abs(fa - fb).max(axis=2)
    ta, tb = a.stage_times()["trace"], b.stage_times()["trace"]
    print(f"bench frame: shared vs per-pixel {q:.1f} dB, max|d| {d.max():.2e}, trace {ta:.3f} vs {tb:.3f} ms")
    assert q >= 60.0


def test_shared_far_fields_off_for_exact_sampler(vct):
    """The FP32 software sampler is the accuracy reference: it always marches
    every pixel's cones, whatever far_share says."""
    scene = scenes.scene_small(width=48, height=32)
    a, _ = _render(vct, scene, 48, 32, 32, sampler=vct.SAMPLER_EXACT)
    b, _ = _render(vct, scene, 48, 32, 32, sampler=vct.SAMPLER_EXACT, far_share=0)
    np.testing.assert_array_equal(a.read_frame(vct.FRAME_RGBA32F), b.read_frame(vct.FRAME_RGBA32F))


@pytest.mark.parametrize("size", [(96, 64), (83, 37)], ids=["96x64", "ragged_83x37"])
def test_tile_rows_same_frame(vct, size):
    """The tracer's CTA tile (16 x 8, 16 x 16 -- the default -- or 16 x 32
    pixels) changes which warps share an SM, not what a warp computes."""
    w, h = size
    scene = scenes.scene_small(width=w, height=h)
    frames = {}
    for rows in (0, 8, 16, 32):
        r, _ = _render(vct, scene, w, h, 64, trace_tile_rows=rows)
        frames[rows] = r.read_frame(vct.FRAME_RGBA32F).copy()
        r.close()
    for rows in (8, 16, 32):
        np.testing.assert_array_equal(frames[rows], frames[0])
