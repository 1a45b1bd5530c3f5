"""Parity at the benchmark's full size: 1920x1080 frame, 256^3 grid,
6-direction RGBA8 mips, the room + displaced icosphere (499,290 triangles).

The oracle runs on every host core: voxel occupancy and level 0 of the whole
grid, the whole mip chain (from the GPU's level 0) and the whole G-buffer
are compared; the cone trace is compared on every 64th pixel row.
Tolerances are those of test_gpu_parity.py (occupancy / mips / triangle ids
bit-exact, level 0 within 1 LSB, EXACT-sampler radiance PSNR >= 60 dB,
texture-unit radiance PSNR >= 40 dB).
"""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H, N, ROWS = 1920, 1080, 256, 64


@pytest.fixture(scope="module")
def bench_scene():
    return scenes.scene_sphere(width=W, height=H)


def _render(vct, scene, **cfg):
    r = vct.Renderer(W, H, grid_res=N, keep_counts=1, keep_float_frame=1, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r, ids


def _chains(r, nmaps=6):
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


@pytest.fixture(scope="module")
def frame_hw(vct, bench_scene):
    return _render(vct, bench_scene)


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_fullsize_voxelize(vct, oracle, bench_scene, frame_hw, mode):
    r = frame_hw[0] if mode == 0 else _render(vct, bench_scene, vox_mode=mode)[0]
    l0, cnt, rej = oracle.voxelize(bench_scene, oracle.Params(grid_res=N, vox_mode=mode))
    assert rej == 0
    got_cnt = r.read_voxel_counts()
    np.testing.assert_array_equal(got_cnt, cnt)
    d = np.abs(r.read_voxels(0).astype(int) - l0.astype(int))
    print(f"mode={mode}: {int((cnt > 0).sum())} occupied voxels, {int(cnt.sum())} contributions, "
          f"level 0 max|d| {d.max()} LSB, identical {100 * (d == 0).mean():.4f}%")
    assert d.max() <= 1


def test_fullsize_mip_chain_exact(oracle, frame_hw):
    r = frame_hw[0]
    ref = oracle.mipmap(oracle.Params(grid_res=N), r.read_voxels(0))
    np.testing.assert_array_equal(_chains(r), ref)


def test_fullsize_gbuffer_ids_exact(oracle, bench_scene, frame_hw):
    g = frame_hw[0].read_gbuffer()
    o = oracle.gbuffer(bench_scene, oracle.Params(grid_res=N, width=W, height=H))
    np.testing.assert_array_equal(g["tri_id"], o["tri_id"])


@pytest.mark.parametrize("sampler", [1, 0], ids=["exact", "hw"])
def test_fullsize_trace_rows(vct, oracle, bench_scene, frame_hw, sampler):
    r = frame_hw[0] if sampler == 0 else _render(vct, bench_scene, sampler=1)[0]
    g = r.read_gbuffer()
    gb = dict(tri_id=g["tri_id"], pos=g["pos"].astype(np.float64), nrm=g["nrm"].astype(np.float64), mat=g["mat"])
    p = oracle.Params(grid_res=N, width=W, height=H)
    ref = oracle.trace(bench_scene, p, r.read_voxels(0), _chains(r), gb, row_stride=ROWS)[::ROWS]
    got = r.read_frame(vct.FRAME_RGBA32F)[::ROWS]
    q = psnr(np.clip(got, 0, 1), np.clip(ref, 0, 1))
    print(f"sampler={sampler}: {ref.shape[0]} rows, PSNR {q:.1f} dB, max|d| {np.abs(got - ref).max():.3e}")
    assert q >= (60.0 if sampler == 1 else 40.0)


def test_fullsize_frames_repeat_bit_exactly(vct, bench_scene, frame_hw):
    r, ids = frame_hw
    a, l0 = r.read_frame().copy(), r.read_voxels(0).copy()
    vct.queue_scene(r, bench_scene, ids)
    r.render()
    np.testing.assert_array_equal(r.read_frame(), a)
    np.testing.assert_array_equal(r.read_voxels(0), l0)


def test_fullsize_shadow_alpha_chains_bit_exact(vct, bench_scene, frame_hw):
    """Shadow cones read packed alpha-only copies of the six chains by
    default; the frame (RGBA32F, so every bit of the radiance) equals the
    one whose shadow cones read the six maps."""
    r = frame_hw[0]
    other = _render(vct, bench_scene, shadow_from_maps=1)[0]
    np.testing.assert_array_equal(r.read_frame(vct.FRAME_RGBA32F), other.read_frame(vct.FRAME_RGBA32F))


def test_fullsize_cone_exit_bit_exact(vct, bench_scene, frame_hw):
    """The exact early exit of cones leaving the grid (default) against
    full-length marches: identical RGBA32F frames at the bench size."""
    r = frame_hw[0]
    other = _render(vct, bench_scene, full_march=1, shadow_from_maps=1)[0]
    np.testing.assert_array_equal(r.read_frame(vct.FRAME_RGBA32F), other.read_frame(vct.FRAME_RGBA32F))
