"""The fused isotropic + anisotropic mip mode (VCT_MIP_BOTH): one MipBuilder
pass writes the six directional chains and the isotropic chain (map 6) from
the same staged children.

Tolerances: the six directional chains and the isotropic chain bit-exact
against the oracle's anisotropic and isotropic reductions of the GPU's own
level 0 (RGBA8); every chain and the traced frame bit-identical to the
renderers that build one kind only (RGBA8 and RGBA16F); the voxel view of
map 6 equal to the isotropic renderer's view of its one map."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H = 96, 64


@pytest.fixture(scope="module")
def small():
    return scenes.scene_small(width=W, height=H)


def _render(vct, scene, n, view=7, **cfg):
    r = vct.Renderer(W, H, grid_res=n, keep_float_frame=1, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(view, 0.0 if view == 7 else 1.5)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r


def _chain(r, n, levels, m):
    return [r.read_voxels(l, m) for l in range(1, levels)]


@pytest.mark.parametrize("n", [64, 128], ids=["64", "128"])
def test_both_chains_exact_against_the_oracle(vct, oracle, small, n):
    """The TMA first pass (levels 1-4), then a tail pass of 2 (64^3) or 3
    (128^3) levels."""
    r = _render(vct, small, n, mip_mode=vct.MIP_BOTH)
    n_, levels = r.grid()
    l0 = r.read_voxels(0)
    for mode, maps in ((oracle.MIP_ANISO, range(6)), (oracle.MIP_ISO, [6])):
        p = oracle.Params(grid_res=n, mip_mode=mode)
        ref = oracle.mipmap(p, l0)
        off = 0
        for lvl in range(1, levels):
            s = n >> lvl
            for k, m in enumerate(maps):
                np.testing.assert_array_equal(r.read_voxels(lvl, m).reshape(-1, 4), ref[k, off:off + s ** 3],
                                              err_msg=f"level {lvl} map {m}")
            off += s ** 3


@pytest.mark.parametrize("storage,n", [(0, 64), (1, 64), (1, 256)], ids=["rgba8", "rgba16f", "rgba16f_256"])
def test_both_equals_the_single_modes(vct, small, storage, n):
    """(256^3 RGBA16F: the tail passes take 3 levels at a time with seven
    maps, 4 with six.)"""
    both = _render(vct, small, n, mip_mode=vct.MIP_BOTH, storage=storage)
    aniso = _render(vct, small, n, mip_mode=vct.MIP_ANISO, storage=storage)
    iso = _render(vct, small, n, mip_mode=vct.MIP_ISO, storage=storage)
    _, levels = both.grid()
    for m in range(6):
        for a, b in zip(_chain(both, n, levels, m), _chain(aniso, n, levels, m)):
            np.testing.assert_array_equal(a, b)
    for a, b in zip(_chain(both, n, levels, 6), _chain(iso, n, levels, 0)):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(both.read_frame(vct.FRAME_RGBA32F), aniso.read_frame(vct.FRAME_RGBA32F))
    with pytest.raises(vct.VCTError):
        both.read_voxels(1, 7)


def test_voxel_view_of_the_isotropic_map(vct, small):
    n = 64
    both = _render(vct, small, n, view=6, mip_mode=vct.MIP_BOTH)
    iso = _render(vct, small, n, view=0, mip_mode=vct.MIP_ISO)
    f = both.read_frame(vct.FRAME_RGBA32F)
    assert np.abs(f).max() > 0.0
    np.testing.assert_allclose(f, iso.read_frame(vct.FRAME_RGBA32F), rtol=0, atol=1e-6)
    aniso = _render(vct, small, n, view=6, mip_mode=vct.MIP_ANISO)
    assert np.abs(aniso.read_frame(vct.FRAME_RGBA32F)).max() == 0.0  # no map 6 without the isotropic chain
