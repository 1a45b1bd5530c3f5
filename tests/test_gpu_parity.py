"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances (stated per output):
  voxel contribution counts / occupancy ......... bit-exact
  level-0 texels (RGBA8) ......................... |d| <= 1 LSB (mean of FP32
                                                   shading vs FP64 shading)
  mip texels, same level 0 ....................... bit-exact
  visible triangle id per pixel .................. bit-exact
  G-buffer world position / normal ............... |d| <= 2e-5 / 2e-4
  radiance, FP32 software filtering (EXACT) ...... PSNR >= 60 dB and 99.9% of
                                                   pixels |d| <= 4e-3
  radiance, texture-unit filtering (HW, 8-bit
  fixed-point weights) ........................... PSNR >= 40 dB
"""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H, N = 96, 64, 64


def _render(vct, scene, w=W, h=H, n=N, **cfg):
    cfg.setdefault("keep_counts", 1)
    cfg.setdefault("keep_float_frame", 1)
    r = vct.Renderer(w, h, grid_res=n, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r


def _gb64(gb):
    return dict(tri_id=gb["tri_id"], pos=gb["pos"].astype(np.float64), nrm=gb["nrm"].astype(np.float64),
                mat=gb["mat"])


def _gpu_chains(r, n, levels, nmaps):
    from oracle import oracle as O
    ch = np.zeros((nmaps, O.chain_texels(n, levels), 4), np.uint8)
    off = 0
    for lvl in range(1, levels):
        s = n >> lvl
        for m in range(nmaps):
            ch[m, off:off + s ** 3] = r.read_voxels(lvl, m).reshape(-1, 4)
        off += s ** 3
    return ch


@pytest.fixture(scope="module")
def small_scene():
    return scenes.scene_small(width=W, height=H)


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_voxelize_counts_exact_and_colours_1lsb(vct, oracle, small_scene, mode):
    r = _render(vct, small_scene, vox_mode=mode)
    l0_gpu = r.read_voxels(0)
    cnt_gpu = r.read_voxel_counts()
    l0_ref, cnt_ref, rej = oracle.voxelize(small_scene, oracle.Params(grid_res=N, vox_mode=mode))
    assert rej == 0
    assert cnt_ref.sum() > 1000
    np.testing.assert_array_equal(cnt_gpu, cnt_ref)
    d = np.abs(l0_gpu.astype(int) - l0_ref.astype(int))
    assert d.max() <= 1
    assert (d == 0).mean() > 0.999


@pytest.mark.parametrize("mip_mode", [0, 1], ids=["aniso", "iso"])
def test_mipmap_exact(vct, oracle, small_scene, mip_mode):
    r = _render(vct, small_scene, mip_mode=mip_mode)
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, mip_mode=mip_mode)
    ch_ref = oracle.mipmap(p, r.read_voxels(0))
    ch_gpu = _gpu_chains(r, n, levels, p.n_maps)
    np.testing.assert_array_equal(ch_gpu, ch_ref)


def test_gbuffer_ids_exact(vct, oracle, small_scene):
    r = _render(vct, small_scene)
    g = r.read_gbuffer()
    o = oracle.gbuffer(small_scene, oracle.Params(grid_res=N, width=W, height=H))
    np.testing.assert_array_equal(g["tri_id"], o["tri_id"])
    vis = o["tri_id"] != 0xffffffff
    assert vis.mean() > 0.9
    np.testing.assert_array_equal(g["mat"][vis], o["mat"][vis])
    assert np.abs(g["pos"][vis] - o["pos"][vis]).max() <= 2e-5
    assert np.abs(g["nrm"][vis] - o["nrm"][vis]).max() <= 2e-4


@pytest.mark.parametrize("sampler", [1, 0], ids=["exact", "hw"])
@pytest.mark.parametrize("mip_mode", [0, 1], ids=["aniso", "iso"])
def test_trace_radiance(vct, oracle, small_scene, sampler, mip_mode):
    """Oracle trace (FP64) from the GPU's own voxel maps and G-buffer vs the
    GPU's radiance, so the comparison isolates the ConeTracer."""
    r = _render(vct, small_scene, sampler=sampler, mip_mode=mip_mode)
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, width=W, height=H, mip_mode=mip_mode)
    l0 = r.read_voxels(0)
    ch = _gpu_chains(r, n, levels, p.n_maps)
    ref = oracle.trace(small_scene, p, l0, ch, _gb64(r.read_gbuffer()))
    got = r.read_frame(vct.FRAME_RGBA32F)
    d = np.abs(got - ref).max(axis=2)
    q = psnr(np.clip(got, 0, 1), np.clip(ref, 0, 1))
    print(f"sampler={sampler} mip={mip_mode}: PSNR {q:.1f} dB, max|d| {d.max():.3e}, "
          f"p99.9 {np.quantile(d, 0.999):.3e}")
    if sampler == 1:
        assert q >= 60.0
        assert np.quantile(d, 0.999) <= 4e-3
    else:
        assert q >= 40.0


PHASES = {"direct": (1, 0, 0, 1), "diffuse": (0, 1, 0, 1), "specular": (0, 0, 1, 1), "final": (1, 1, 1, 1)}


@pytest.mark.parametrize("sampler", [1, 0], ids=["exact", "hw"])
@pytest.mark.parametrize("phase", list(PHASES))
def test_trace_radiance_per_output(vct, oracle, small_scene, sampler, phase):
    """Each output of voxel_cone_tracing.frag:265-272 on its own (switched by
    set_rendering_phases, renderer.cpp:368-371): the oracle's FP64 trace of
    the same phase from the GPU's maps and G-buffer vs the GPU's radiance."""
    direct, diffuse, specular, shadow = PHASES[phase]
    r = vct.Renderer(W, H, grid_res=N, keep_float_frame=1, sampler=sampler)
    ids = vct.load_scene(r, small_scene)
    r.set_voxel_view_dir(7, 0.0)
    r.set_rendering_phases(direct, diffuse, specular, shadow)
    vct.queue_scene(r, small_scene, ids)
    r.render()
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, width=W, height=H, enable_direct=bool(direct), enable_diffuse=bool(diffuse),
                      enable_specular=bool(specular), enable_shadow=bool(shadow))
    ref = oracle.trace(small_scene, p, r.read_voxels(0), _gpu_chains(r, n, levels, 6), _gb64(r.read_gbuffer()))
    got = r.read_frame(vct.FRAME_RGBA32F)
    d = np.abs(got - ref)[..., :3]
    q = psnr(np.clip(got[..., :3], 0, 1), np.clip(ref[..., :3], 0, 1))
    print(f"{phase:8s} sampler={sampler}: max|d| {d.max():.3e}, mean|d| {d.mean():.3e}, PSNR {q:.1f} dB, "
          f"peak {ref[..., :3].max():.3f}")
    assert ref[..., :3].max() > 0.05  # the phase contributes
    if sampler == 1:
        assert q >= 60.0
    else:
        assert q >= 40.0


def test_frame_end_to_end_vs_oracle(vct, oracle, small_scene):
    r = _render(vct, small_scene, sampler=1)
    ref = oracle.render(small_scene, oracle.Params(grid_res=N, width=W, height=H))
    got = r.read_frame(vct.FRAME_RGBA32F)
    q = psnr(np.clip(got, 0, 1), np.clip(ref["frame"], 0, 1))
    print(f"end-to-end PSNR {q:.1f} dB")
    assert q >= 50.0
    rgba8 = r.read_frame()
    np.testing.assert_array_equal(rgba8, np.floor(np.clip(got, 0, 1) * 255 + 0.5).astype(np.uint8))


def test_render_is_deterministic(vct, small_scene):
    r = _render(vct, small_scene)
    a = r.read_frame().copy()
    l0 = r.read_voxels(0).copy()
    ids = list(range(len(small_scene.meshes)))
    vct.queue_scene(r, small_scene, ids)
    r.render()
    np.testing.assert_array_equal(r.read_frame(), a)
    np.testing.assert_array_equal(r.read_voxels(0), l0)


def test_empty_queue_gives_clear_colour(vct):
    r = vct.Renderer(16, 8, grid_res=16)
    r.set_voxel_view_dir(7, 0.0)
    r.render()
    f = r.read_frame()
    assert (f == (38, 64, 64, 255)).all()
    assert (r.read_voxels(0) == 0).all()


def test_voxel_debug_view(vct, oracle, small_scene):
    """view_voxel_dir < 7 shows textureLod(map, pos, lod) (voxel_cone_tracing
    .frag:253-257); the reference's constructor default is map 0, lod 0."""
    r = _render(vct, small_scene, sampler=1)
    r.set_voxel_view_dir(3, 1.5)
    ids = list(range(len(small_scene.meshes)))
    vct.queue_scene(r, small_scene, ids)
    r.render()
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, width=W, height=H, view_voxel_dir=3, view_voxel_lod=1.5)
    ref = oracle.trace(small_scene, p, r.read_voxels(0), _gpu_chains(r, n, levels, 6), _gb64(r.read_gbuffer()))
    got = r.read_frame(vct.FRAME_RGBA32F)
    assert np.abs(got - ref).max() < 1e-4


def test_error_paths(vct, small_scene):
    r = vct.Renderer(16, 16, grid_res=16)
    with pytest.raises(vct.VCTError):
        r.set_grid_resolution(100)
    assert r.load_model("/nonexistent/file.obj") == vct.INVALID_ID
    r.queue_model(12345)  # ignored, like the reference
    with pytest.raises(vct.VCTError):
        r.set_model_material(0, 99)
    with pytest.raises(vct.VCTError):
        r.upload_material_data(scenes.default_material(), 99)
    r.set_grid_resolution(32)
    assert r.grid() == (32, 6)


@pytest.mark.parametrize("cfg", [dict(), dict(vox_mode=1), dict(cone_set=1)], ids=["default", "sat", "six_cones"])
def test_shadow_alpha_chains_bit_exact(vct, small_scene, cfg):
    """Packed alpha-only chains for shadow cones (default) against shadow
    cones over the six maps: identical radiance, bit for bit; with the six
    maps' chains also identical (the alpha copies only add textures)."""
    a = _render(vct, small_scene, **cfg)
    b = _render(vct, small_scene, shadow_from_maps=1, **cfg)
    np.testing.assert_array_equal(a.read_frame(vct.FRAME_RGBA32F), b.read_frame(vct.FRAME_RGBA32F))
    n, levels = a.grid()
    for lvl in range(1, levels):
        for m in range(6):
            np.testing.assert_array_equal(a.read_voxels(lvl, m), b.read_voxels(lvl, m))


@pytest.mark.parametrize("cfg", [dict(), dict(sampler=1), dict(mip_mode=1), dict(cone_set=1)],
                         ids=["hw", "exact", "iso", "six_cones"])
def test_cone_exit_outside_grid_bit_exact(vct, small_scene, cfg):
    """Cones stop once every further sample can only read border texels
    (default) or march their full length as the reference's loop does
    (full_march=1): identical radiance, bit for bit."""
    a = _render(vct, small_scene, **cfg)
    b = _render(vct, small_scene, full_march=1, **cfg)
    np.testing.assert_array_equal(a.read_frame(vct.FRAME_RGBA32F), b.read_frame(vct.FRAME_RGBA32F))
