"""Deferred light injection (no reference counterpart): attribute grids
with the voxelizer's coverage and averaging, level 0 lit from them.

Tolerances: contribution counts bit-exact; GPU attribute grids and GPU
injected level 0 within 1 LSB of the FP64 oracle (the injection compared on
the GPU's own grids); injected vs direct voxelization (an approximation:
lighting at the voxel centre from mean attributes) mean |d| < 2 LSB on
occupied voxels and frame PSNR >= 45 dB (oracle: 59 / 63 dB on the two
scenes).  A light change renders without voxelizing and equals a fresh
renderer's frame with the new light, bit for bit."""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

W, H, N = 96, 64, 64


@pytest.fixture(scope="module")
def small():
    return scenes.scene_small(width=W, height=H)


def test_inject_known_answer(oracle):
    """One occupied voxel, albedo (0.5, 0.25, 1), normal +y, emission (0.1,
    0, 0), one white light straight above at distance 0.5 (grid units)."""
    n = 8
    g = {k: np.zeros((n, n, n, 4), np.uint8) for k in ("albedo", "normal", "emission")}
    z, y, x = 2, 3, 4
    g["albedo"][z, y, x] = (round(0.5 * 255), round(0.25 * 255), 255, 200)
    g["normal"][z, y, x] = (round(0.5 * 255), 255, round(0.5 * 255), 0)
    g["emission"][z, y, x] = (round(0.1 * 255), 0, 0, 255)
    centre = np.array([(x + 0.5) * 2 / n - 1, (y + 0.5) * 2 / n - 1, (z + 0.5) * 2 / n - 1])
    s = scenes.scene_small(width=8, height=8)
    s.lights = np.array([scenes.point_light(tuple(centre + (0, 0.5, 0)), intensity=2.0)], scenes.LIGHT_DTYPE)
    s.cube_size = 1.0
    out = oracle.inject(s, oracle.Params(grid_res=n), g)
    k = 1 / 255
    nrm = np.array([g["normal"][z, y, x, c] * k * 2 - 1 for c in range(3)])
    nrm /= np.linalg.norm(nrm)
    lit = 2.0 * max(nrm @ np.array([0, 1, 0]), 0) / (1 + 0.25)
    exp = np.clip(g["albedo"][z, y, x, :3] * k * lit + g["emission"][z, y, x, :3] * k, 0, 1)
    np.testing.assert_array_equal(out[z, y, x, :3], np.floor(exp * 255 + 0.5).astype(np.uint8))
    assert out[z, y, x, 3] == 200
    out[z, y, x] = 0
    assert (out == 0).all()


def test_injection_approximates_direct_voxelization(oracle, small):
    p = oracle.Params(grid_res=N, width=W, height=H)
    l0, cnt, _ = oracle.voxelize(small, p)
    g = oracle.voxelize_attr(small, p)
    np.testing.assert_array_equal(g["counts"], cnt)
    inj = oracle.inject(small, p, g)
    occ = cnt > 0
    d = np.abs(inj.astype(int) - l0.astype(int))[occ]
    assert d.mean() < 2.0
    np.testing.assert_array_equal(inj[..., 3][occ], l0[..., 3][occ])
    gb = oracle.gbuffer(small, p)
    f_inj = oracle.trace(small, p, inj, oracle.mipmap(p, inj), gb)
    f_dir = oracle.trace(small, p, l0, oracle.mipmap(p, l0), gb)
    assert psnr(np.clip(f_inj, 0, 1), np.clip(f_dir, 0, 1)) >= 45.0


def _renderer(vct, scene, inject=True, light=None, **cfg):
    r = vct.Renderer(W, H, grid_res=N, keep_counts=1, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    r.set_light_injection(inject)
    return r, ids


def _frame(vct, r, scene, ids, lights):
    for mid in ids:
        r.queue_model(mid)
    for l in lights:
        r.queue_point_light(l)
    r.render()
    return r.read_frame().copy()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_gpu_injection_grids_and_level0(vct, oracle, small, mode):
    r, ids = _renderer(vct, small, vox_mode=mode)
    _frame(vct, r, small, ids, small.lights)
    g = r.read_injection_grids()
    ref = oracle.voxelize_attr(small, oracle.Params(grid_res=N, vox_mode=mode))
    np.testing.assert_array_equal(r.read_voxel_counts(), ref["counts"])
    for k in ("albedo", "normal", "emission"):
        assert np.abs(g[k].astype(int) - ref[k].astype(int)).max() <= 1, k
    inj = oracle.inject(small, oracle.Params(grid_res=N), g)
    assert np.abs(r.read_voxels(0).astype(int) - inj.astype(int)).max() <= 1


@pytest.mark.gpu
def test_gpu_light_change_skips_voxelization(vct, small):
    r, ids = _renderer(vct, small)
    _frame(vct, r, small, ids, small.lights)
    t0 = r.stage_times()
    assert t0["voxelized"]
    moved = scenes.point_light((0.2, 0.3, -0.1), color=(1.0, 0.8, 0.6), intensity=1.5)
    f = _frame(vct, r, small, ids, [moved])
    t1 = r.stage_times()
    assert not t1["voxelized"]
    assert t1["kernel_launches"] < t0["kernel_launches"]
    fresh, fids = _renderer(vct, small)
    np.testing.assert_array_equal(f, _frame(vct, fresh, small, fids, [moved]))
    # geometry changes voxelize again
    r.set_model_transform(ids[1], scenes.trs(translate=(0.1, -0.3, 0.0), scale=(0.2, 0.2, 0.2)))
    _frame(vct, r, small, ids, [moved])
    assert r.stage_times()["voxelized"]


@pytest.mark.gpu
def test_gpu_injection_frame_close_to_direct(vct, small):
    rd, idd = _renderer(vct, small, inject=False)
    ri, idi = _renderer(vct, small, inject=True)
    fd = _frame(vct, rd, small, idd, small.lights)
    fi = _frame(vct, ri, small, idi, small.lights)
    q = psnr(fd / 255.0, fi / 255.0)
    print(f"injected vs direct frame: PSNR {q:.1f} dB")
    assert q >= 40.0


@pytest.mark.gpu
def test_gpu_injection_dense_bricks(vct, oracle):
    """Attribute grids of bricks whose pairs are split across CTAs (72,000
    triangles in a 16^3 grid)."""
    s = scenes.scene_sphere(seed=79, freq=60, width=W, height=H)
    r = vct.Renderer(W, H, grid_res=16, keep_counts=1)
    ids = vct.load_scene(r, s)
    r.set_light_injection(True)
    _frame(vct, r, s, ids, s.lights)
    assert r.stage_times()["split_bricks"] > 0
    ref = oracle.voxelize_attr(s, oracle.Params(grid_res=16))
    np.testing.assert_array_equal(r.read_voxel_counts(), ref["counts"])
    g = r.read_injection_grids()
    for k in ("albedo", "normal", "emission"):
        assert np.abs(g[k].astype(int) - ref[k].astype(int)).max() <= 1, k
