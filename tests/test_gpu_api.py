"""The Texture3D helpers (src/texture_3d.h:6-10) and the Renderer settings
that change what a frame computes, through the C ABI."""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu


def _box_mip(a):
    """glGenerateMipmap-style 2x2x2 mean, children clamped to the extent for
    odd sizes, round to nearest (ties up)."""
    d, h, w, _ = a.shape
    nd, nh, nw = max(d // 2, 1), max(h // 2, 1), max(w // 2, 1)
    s = np.zeros((nd, nh, nw, 4), np.uint32)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                z = np.minimum(2 * np.arange(nd) + dz, d - 1)
                y = np.minimum(2 * np.arange(nh) + dy, h - 1)
                x = np.minimum(2 * np.arange(nw) + dx, w - 1)
                s += a[z][:, y][:, :, x]
    return ((s + 4) >> 3).astype(np.uint8)


def test_tex3d_clear_upload_mip_download(vct):
    w, h, d, levels = 16, 12, 10, 4
    t = vct.create_tex_3d(w, h, d, levels)
    try:
        vct.activate_tex_3d(0, t, 0)
        vct.clear_tex_3d(t, (0.25, 0.5, 0.75, 1.0))
        np.testing.assert_array_equal(vct.tex3d_download(t, 0, (d, h, w)),
                                      np.broadcast_to(np.array([64, 128, 191, 255], np.uint8), (d, h, w, 4)))
        rng = np.random.default_rng(7)
        a = rng.integers(0, 256, (d, h, w, 4), dtype=np.uint8)
        vct.tex3d_upload(t, 0, a)
        np.testing.assert_array_equal(vct.tex3d_download(t, 0, (d, h, w)), a)
        vct.mip_tex_3d(t)
        ref = a
        for lvl in range(1, levels):
            ref = _box_mip(ref)
            got = vct.tex3d_download(t, lvl, ref.shape[:3])
            np.testing.assert_array_equal(got, ref)
    finally:
        vct.destroy_tex_3d(t)
    with pytest.raises(vct.VCTError):
        vct.clear_tex_3d(t, (0, 0, 0, 0))  # destroyed name
    with pytest.raises(vct.VCTError):
        vct.create_tex_3d(0, 4, 4, 1)


@pytest.fixture(scope="module")
def scene():
    return scenes.scene_small(width=64, height=48)


def _frame(vct, scene, setup=None, **cfg):
    r = vct.Renderer(64, 48, grid_res=32, keep_float_frame=1, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    if setup:
        setup(r)
    vct.queue_scene(r, scene, ids)
    r.render()
    return r, r.read_frame(vct.FRAME_RGBA32F).copy()


def test_rendering_phases_are_additive(vct, oracle, scene):
    """final = specular + diffuse + direct (voxel_cone_tracing.frag:265-272,
    no transparent materials here), each phase switched by
    set_rendering_phases (renderer.cpp:368-371)."""
    parts = {}
    for name, ph in {"all": (1, 1, 1, 1), "direct": (1, 0, 0, 1), "diffuse": (0, 1, 0, 1),
                     "specular": (0, 0, 1, 1)}.items():
        r, f = _frame(vct, scene, lambda r, ph=ph: r.set_rendering_phases(*ph), sampler=1)
        parts[name] = f
    hit = r.read_gbuffer()["tri_id"] != 0xffffffff
    assert hit.mean() > 0.9
    lit = parts["direct"] + parts["diffuse"] + parts["specular"]
    np.testing.assert_allclose(parts["all"][hit][:, :3], lit[hit][:, :3], atol=2e-5)
    # shadows off changes the direct term only
    _, ns = _frame(vct, scene, lambda r: r.set_rendering_phases(1, 0, 0, 0), sampler=1)
    assert (ns[..., :3] >= parts["direct"][..., :3] - 1e-6).all()
    assert (ns != parts["direct"]).any()


def test_material_upload_changes_the_frame(vct, scene):
    r, a = _frame(vct, scene)
    m = r.get_material(1)
    assert m.tobytes() == scene.materials[1].tobytes()
    m2 = m.copy()
    m2["diffuse"][:3] = (1.0, 0.0, 0.0)
    r.upload_material_data(m2, 1)
    assert r.get_material(1)["diffuse"][0] == 1.0
    ids = list(range(len(scene.meshes)))
    vct.queue_scene(r, scene, ids)
    r.render()
    b = r.read_frame(vct.FRAME_RGBA32F)
    assert psnr(np.clip(a, 0, 1), np.clip(b, 0, 1)) < 40.0


def test_queue_is_cleared_after_render(vct, scene):
    """Per-frame queues are cleared at the end of render()
    (renderer.cpp:403-404): a second render without queueing shows the
    clear colour and an empty grid."""
    r, a = _frame(vct, scene)
    assert (r.read_voxels(0) != 0).any()
    r.render()
    f = r.read_frame()
    assert (f == (38, 64, 64, 255)).all()
    assert (r.read_voxels(0) == 0).all()


def test_grid_resolution_and_stage_times(vct, scene):
    r, _ = _frame(vct, scene)
    assert r.grid() == (32, 6)
    r.set_grid_resolution(64)
    assert r.grid() == (64, 7)
    ids = list(range(len(scene.meshes)))
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    assert r.read_voxels(0).shape == (64, 64, 64, 4)
    t = r.stage_times()
    for k in ("voxelize", "mipmap", "gbuffer", "trace", "total"):
        assert t[k] > 0.0
    assert t["total"] >= t["trace"]
    assert t["kernel_launches"] > 5


def test_caller_stream(vct, scene):
    """vct_set_stream puts the renderer's work on the caller's stream; the
    frame is the same as on the renderer's own stream."""
    import torch
    _, a = _frame(vct, scene)
    s = torch.cuda.Stream()
    _, b = _frame(vct, scene, lambda r: r.set_stream(s.cuda_stream))
    np.testing.assert_array_equal(a, b)


def test_overlap_raster_same_frame(vct, scene):
    """Every stage on one stream (default) and the G-buffer raster beside
    voxelize and mipmap (overlap_raster = 1) give the same frame, also on a
    caller's stream."""
    import torch
    _, a = _frame(vct, scene)
    _, b = _frame(vct, scene, overlap_raster=1)
    s = torch.cuda.Stream()
    r, c = _frame(vct, scene, lambda r: r.set_stream(s.cuda_stream), overlap_raster=1)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    t = r.stage_times()
    assert t["gbuffer"] > 0.0 and t["total"] >= t["trace"]
