"""HDR voxel maps in half precision (RGBA16F storage, radiance clamped to
[0, 16]) against the FP64 oracle, per stage, on a reduced copy of the
2M-triangle precision scene (4 displaced spheres + 16 cuboids, 64^3 grid).

Tolerances (stated per output):
  voxel contribution counts / occupancy ....... bit-exact
  level-0 texels (half) ........................ |d| <= 1 half ulp of the
                                                 FP64 mean (round to nearest
                                                 of FP32 shading)
  mip level k+1 from the GPU's level k ......... |d| <= 1 half ulp + 1e-6
  radiance, FP32 software filtering (EXACT) .... max |d| <= 2e-3 x peak
  radiance, texture-unit filtering (HW) ........ PSNR >= 40 dB (peak = the
                                                 frame's largest channel)
"""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H, N = 96, 64, 64
RMAX = scenes.HDR_RADIANCE_MAX


@pytest.fixture(scope="module")
def hdr_scene():
    return scenes.scene_hdr(freq=10, n_spheres=4, n_cuboids=16, width=W, height=H)


def _render(vct, scene, **cfg):
    cfg.setdefault("keep_counts", 1)
    cfg.setdefault("keep_float_frame", 1)
    cfg.setdefault("storage", vct.STORAGE_RGBA16F)
    cfg.setdefault("radiance_max", RMAX)
    r = vct.Renderer(W, H, grid_res=N, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r


def _half_ulp(ref):
    return np.spacing(np.abs(ref).astype(np.float16)).astype(np.float64)


def _level(r, lvl, nmaps):
    if lvl == 0:
        return r.read_voxels(0).astype(np.float32)
    return np.stack([r.read_voxels(lvl, m).astype(np.float32) for m in range(nmaps)])


def _gpu_chains_f(r, n, levels, nmaps):
    from oracle import oracle as O
    ch = np.zeros((nmaps, O.chain_texels(n, levels), 4), np.float32)
    off = 0
    for lvl in range(1, levels):
        s = n >> lvl
        for m in range(nmaps):
            ch[m, off:off + s ** 3] = r.read_voxels(lvl, m).astype(np.float32).reshape(-1, 4)
        off += s ** 3
    return ch


def _gb64(gb):
    return dict(tri_id=gb["tri_id"], pos=gb["pos"].astype(np.float64), nrm=gb["nrm"].astype(np.float64),
                mat=gb["mat"])


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_hdr_voxelize_counts_exact_values_1ulp(vct, oracle, hdr_scene, mode):
    r = _render(vct, hdr_scene, vox_mode=mode)
    got = r.read_voxels(0).astype(np.float64)
    cnt = r.read_voxel_counts()
    ref, cnt_ref, rej = oracle.voxelize_hdr(hdr_scene, oracle.Params(grid_res=N, vox_mode=mode, radiance_max=RMAX))
    assert rej == 0
    np.testing.assert_array_equal(cnt, cnt_ref)
    d = np.abs(got - ref)
    rel = d / np.maximum(np.abs(ref), 1e-30)
    print(f"mode={mode}: level 0 max|d| {d.max():.3e}, max rel {rel[ref != 0].max():.3e}, "
          f"voxels > 1: {(ref[..., :3] > 1).sum()}, max {ref.max():.2f}")
    assert (ref[..., :3] > 1.0).sum() > 100  # the HDR range is exercised
    assert ref.max() <= RMAX
    assert (d <= _half_ulp(ref)).all()


@pytest.mark.parametrize("mip_mode", [0, 1], ids=["aniso", "iso"])
def test_hdr_mip_levels_1ulp(vct, oracle, hdr_scene, mip_mode):
    """Every level k+1 against the FP64 reduction of the GPU's own level k,
    so each comparison isolates one pass of the MipBuilder."""
    r = _render(vct, hdr_scene, mip_mode=mip_mode)
    n, levels = r.grid()
    nmaps = 1 if mip_mode == 1 else 6
    worst = 0.0
    for lvl in range(levels - 1):
        ref = oracle.mip_level_f(_level(r, lvl, nmaps), mip_mode)
        got = _level(r, lvl + 1, nmaps).reshape(ref.shape).astype(np.float64)
        d = np.abs(got - ref)
        worst = max(worst, float((d / (_half_ulp(ref) + 1e-6)).max()))
        assert (d <= _half_ulp(ref) + 1e-6).all(), f"level {lvl + 1}: max|d| {d.max():.3e}"
    print(f"mip_mode={mip_mode}: worst |d| / (1 half ulp + 1e-6) = {worst:.3f}")


@pytest.mark.parametrize("sampler", [1, 0], ids=["exact", "hw"])
def test_hdr_trace_radiance(vct, oracle, hdr_scene, sampler):
    r = _render(vct, hdr_scene, sampler=sampler)
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, width=W, height=H, radiance_max=RMAX)
    ref = oracle.trace_hdr(hdr_scene, p, _level(r, 0, 6), _gpu_chains_f(r, n, levels, 6), _gb64(r.read_gbuffer()))
    got = r.read_frame(vct.FRAME_RGBA32F)
    peak = float(ref[..., :3].max())
    d = np.abs(got - ref)[..., :3]
    q = psnr(got[..., :3], ref[..., :3], peak=peak)
    print(f"sampler={sampler}: peak {peak:.2f}, PSNR {q:.1f} dB, max|d| {d.max():.3e}")
    assert peak > 1.0  # HDR radiance reaches the frame
    if sampler == 1:
        assert d.max() <= 2e-3 * peak
    else:
        assert q >= 40.0


def test_hdr_needs_half_storage(vct):
    with pytest.raises(vct.VCTError):
        vct.Renderer(16, 16, grid_res=16, storage=vct.STORAGE_RGBA8, radiance_max=RMAX)


def test_half_storage_ldr_matches_rgba8(vct, oracle):
    """With the reference's clamp (radiance_max 1) half storage renders the
    RGBA8 image up to the RGBA8 quantisation of the maps."""
    s = scenes.scene_small(width=W, height=H)
    a = _render(vct, s, storage=vct.STORAGE_RGBA8, radiance_max=1.0).read_frame(vct.FRAME_RGBA32F)
    b = _render(vct, s, storage=vct.STORAGE_RGBA16F, radiance_max=1.0).read_frame(vct.FRAME_RGBA32F)
    q = psnr(np.clip(a, 0, 1), np.clip(b, 0, 1))
    print(f"RGBA8 vs RGBA16F frame PSNR {q:.1f} dB")
    assert q >= 40.0


def test_hdr_dense_bricks(vct, oracle):
    """Half-precision level 0 of bricks whose pairs are split across CTAs
    (72,000 triangles in a 16^3 grid): the 64-bit fixed-point sums of the
    chunks add exactly, so the tolerance stays 1 half ulp."""
    s = scenes.scene_sphere(seed=78, freq=60, width=W, height=H)
    r = vct.Renderer(W, H, grid_res=16, keep_counts=1, storage=vct.STORAGE_RGBA16F, radiance_max=RMAX)
    ids = vct.load_scene(r, s)
    vct.queue_scene(r, s, ids)
    r.render()
    assert r.stage_times()["split_bricks"] > 0
    ref, cnt_ref, _ = oracle.voxelize_hdr(s, oracle.Params(grid_res=16, radiance_max=RMAX))
    np.testing.assert_array_equal(r.read_voxel_counts(), cnt_ref)
    d = np.abs(r.read_voxels(0).astype(np.float64) - ref)
    assert (d <= _half_ulp(ref)).all()
