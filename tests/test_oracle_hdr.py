"""The oracle's float (HDR storage) paths agree with its RGBA8 paths where
both apply: same shading, coverage and averaging, same mip rule, same cone
tracer; only the texel format differs."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes

N, W, H = 32, 48, 32


@pytest.fixture(scope="module")
def small():
    return scenes.scene_small(width=W, height=H)


@pytest.mark.parametrize("mode", [0, 1])
def test_voxelize_hdr_rounds_to_rgba8(oracle, small, mode):
    p = oracle.Params(grid_res=N, vox_mode=mode)
    l8, c8, _ = oracle.voxelize(small, p)
    lf, cf, _ = oracle.voxelize_hdr(small, p)
    np.testing.assert_array_equal(c8, cf)
    np.testing.assert_array_equal(np.floor(lf.astype(np.float64) * 255 + 0.5).astype(np.uint8), l8)


def test_radiance_max_clamps_hdr(oracle):
    s = scenes.scene_hdr(freq=6, n_spheres=2, n_cuboids=12, width=W, height=H)
    lo, _, _ = oracle.voxelize_hdr(s, oracle.Params(grid_res=N, radiance_max=1.0))
    hi, _, _ = oracle.voxelize_hdr(s, oracle.Params(grid_res=N, radiance_max=16.0))
    assert lo.max() <= 1.0
    assert 1.0 < hi.max() <= 16.0
    # A higher clamp never lowers a colour mean; alpha keeps its [0, 1] clamp.
    assert (hi[..., :3] >= lo[..., :3] - 1e-7).all()
    np.testing.assert_allclose(hi[..., 3], lo[..., 3], rtol=0, atol=1e-7)


@pytest.mark.parametrize("mip_mode", [0, 1])
def test_mip_level_f_matches_exact_rgba8(oracle, small, mip_mode):
    p = oracle.Params(grid_res=N, mip_mode=mip_mode)
    l8, _, _ = oracle.voxelize(small, p)
    ch = oracle.mipmap(p, l8)
    lvl1 = oracle.chain_level(ch, N, 1, 0) if mip_mode == 1 else np.stack(
        [oracle.chain_level(ch, N, 1, m) for m in range(6)])
    f = oracle.mip_level_f(l8.astype(np.float32) / 255.0, mip_mode).reshape(lvl1.shape)
    # The RGBA8 rule is this value rounded to nearest (ties up, so an exact
    # tie may sit 0.5 away).
    assert np.abs(f.astype(np.float64) * 255.0 - lvl1).max() <= 0.5 + 1e-4


def test_trace_hdr_matches_rgba8_trace(oracle, small):
    p = oracle.Params(grid_res=N, width=W, height=H)
    l8, _, _ = oracle.voxelize(small, p)
    ch = oracle.mipmap(p, l8)
    gb = oracle.gbuffer(small, p)
    a = oracle.trace(small, p, l8, ch, gb)
    b = oracle.trace_hdr(small, p, l8.astype(np.float32) / 255.0, ch.astype(np.float32) / 255.0, gb)
    np.testing.assert_allclose(a, b, rtol=0, atol=2e-6)
