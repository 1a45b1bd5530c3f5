"""Batched rendering (vct_batch_*): every scene of a batch of uneven grid,
mesh and frame sizes renders exactly what a Renderer renders on the same
scene (frames, level 0 and the directional mips bit-exact), eagerly and as
a replayed CUDA graph, before and after autotuning, and when a work list
overflows and is grown."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes

CONES = {9: 0, 6: 1}


def _items():
    out = []
    for k, (seed, w, h, grid, cones) in enumerate([(11, 64, 48, 16, 9), (12, 96, 64, 32, 6), (13, 40, 40, 64, 9),
                                                    (14, 80, 30, 32, 9)]):
        out.append((scenes.scene_small(seed=seed, width=w, height=h), w, h, grid, CONES[cones]))
    out.append((scenes.scene_sphere(seed=21, freq=8, width=128, height=96), 128, 96, 64, CONES[9]))
    empty = scenes.scene_small(seed=15, width=24, height=16)
    empty.meshes, empty.models = [], []
    out.append((empty, 24, 16, 32, CONES[6]))
    return out


def _single(vct, scene, w, h, grid, cones, vox_mode=0, view=None, far_share=1):
    r = vct.Renderer(w, h, grid_res=grid, cone_set=cones, vox_mode=vox_mode, far_share=far_share)
    ids = vct.load_scene(r, scene)
    if view is not None:
        r.set_camera_transform(view, scene.proj)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    return r


def _check_scene(vct, b, i, item, vox_mode=0, view=None, far_share=1):
    scene, w, h, grid, cones = item
    r = _single(vct, scene, w, h, grid, cones, vox_mode, view, far_share)
    np.testing.assert_array_equal(b.read_frame(i), r.read_frame(), err_msg=f"scene {i} frame")
    np.testing.assert_array_equal(b.read_voxels(i, 0), r.read_voxels(0), err_msg=f"scene {i} level 0")
    n, levels = r.grid()
    for lvl in (1, levels - 1):
        for m in range(6):
            np.testing.assert_array_equal(b.read_voxels(i, lvl, m), r.read_voxels(lvl, m),
                                          err_msg=f"scene {i} level {lvl} map {m}")


def test_batch_rejects_bad_scenes(vct):
    s = scenes.scene_small(width=16, height=16)
    with pytest.raises(vct.VCTError):
        vct.Batch([(s, 16, 16, 100, 0)])   # grid not a power of two
    with pytest.raises(vct.VCTError):
        vct.Batch([(s, 16, 16, 512, 0)])   # above the batch limit
    with pytest.raises(vct.VCTError):
        vct.Batch([(s, 16, 16, 32, 7)])    # no such cone set
    with pytest.raises(vct.VCTError):
        vct.Batch([])


@pytest.mark.gpu
@pytest.mark.parametrize("far_share", [1, 0], ids=["shared_far", "per_pixel"])
@pytest.mark.parametrize("form", ["persistent", "tiles", "per_scene", "per_scene_16_rows"])
@pytest.mark.parametrize("use_graph", [False, True], ids=["eager", "graph"])
def test_batch_matches_renderer(vct, use_graph, form, far_share):
    """Every trace form (one persistent launch; one launch with one CTA per
    tile; one launch per scene with 16x8 or 16x16 tiles) renders each scene
    exactly as a Renderer with the same far_share does."""
    items = _items()
    b = vct.Batch(items, use_graph=use_graph, far_share=far_share)
    b.shape = dict(b.shape, trace_per_scene=int(form.startswith("per_scene")),
                   trace_tile_rows=16 if form == "per_scene_16_rows" else 8,
                   trace_ctas_per_sm=0 if form == "tiles" else 2)
    b.render()
    b.render()  # a second frame (a graph replay) gives the same result
    t = b.stage_times()
    assert t["kernel_launches"] > 0 and t["total"] > 0
    for i, item in enumerate(items):
        _check_scene(vct, b, i, item, far_share=far_share)


@pytest.mark.gpu
def test_batch_conservative_voxelizer(vct):
    items = _items()[:3]
    b = vct.Batch(items, vox_mode=1)
    b.render()
    for i, item in enumerate(items):
        _check_scene(vct, b, i, item, vox_mode=1)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["persistent", "tiles", "per_scene"])
def test_batch_camera_update_under_graph(vct, form):
    items = _items()[:4]
    b = vct.Batch(items, use_graph=True)
    b.shape = dict(b.shape, trace_per_scene=int(form == "per_scene"), trace_ctas_per_sm=0 if form == "tiles" else 2)
    b.render()
    scene = items[2][0]
    view = scenes.look_at((0.1, 0.05, 0.45), (0.0, -0.1, -0.5))
    b.set_camera(2, view, scene.proj)
    b.render()
    _check_scene(vct, b, 2, items[2], view=view)
    _check_scene(vct, b, 1, items[1])


@pytest.mark.gpu
def test_batch_autotune_keeps_results(vct):
    items = _items()
    b = vct.Batch(items, use_graph=True)
    b.render()
    before = [b.read_frame(i).copy() for i in range(len(items))]
    rep = b.autotune(frames=1)
    assert rep["shape"] == b.shape
    assert rep["ms_after"] <= rep["ms_before"] + 1e-6
    assert rep["shape"]["trace_ctas_per_sm"] in (0, 2, 3) and rep["shape"]["trace_dynamic"] in (0, 1)
    assert rep["shape"]["trace_per_scene"] in (0, 1) and rep["shape"]["trace_tile_rows"] in (8, 16, 32)
    b.render()
    for i in range(len(items)):
        np.testing.assert_array_equal(b.read_frame(i), before[i])


@pytest.mark.gpu
def test_batch_work_lists_grow(vct):
    """64 large random triangles in a 256^3 grid need more (triangle, brick)
    pairs than the initial list holds: the batch grows it and renders the
    frame again, like a Renderer."""
    rng = np.random.default_rng(5)
    tris = rng.uniform(-0.9, 0.9, (64, 3, 3)).astype(np.float32)
    from tests.helpers import tri_scene
    s = tri_scene(tris, lights=[((0.0, 0.5, 0.0),)], cube_size=1.0,
                  view=scenes.look_at((0.0, 0.0, 0.95), (0.0, 0.0, 0.0)),
                  proj=scenes.perspective(1.0, 1.0, 0.01, 10.0))
    items = [(s, 48, 48, 256, 0), _items()[0]]
    b = vct.Batch(items, use_graph=True)
    b.render()
    for i, item in enumerate(items):
        _check_scene(vct, b, i, item)


@pytest.mark.gpu
@pytest.mark.parametrize("vox_mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_batch_dense_bricks(vct, vox_mode):
    """Dense spheres in coarse grids (the batch's brick pairs split across
    CTAs) render what a Renderer renders."""
    items = [(scenes.scene_sphere(seed=31, freq=60, width=64, height=48), 64, 48, 16, CONES[9]),
             (scenes.scene_sphere(seed=32, freq=40, width=48, height=48), 48, 48, 32, CONES[6]),
             _items()[0]]
    b = vct.Batch(items, vox_mode=vox_mode)
    b.render()
    assert b.stage_times()["split_bricks"] > 0
    for i, item in enumerate(items):
        _check_scene(vct, b, i, item, vox_mode=vox_mode)


@pytest.mark.gpu
def test_batch_scenes_against_oracle(vct, oracle):
    """Batch scenes checked against the FP64 oracle directly, not only
    against a Renderer: the 16^3 room and the 64^3 sphere of the small batch,
    and scenes 0, 1 and 6 of the benchmark's 64-scene batch (640x480 at 64^3
    with 6 cones, 960x540 at 256^3 with 6 cones, 386,430 triangles at 64^3
    with 9 cones).  Level 0 within 1 LSB of the oracle's with the same
    occupancy, every directional mip level bit-exact from the GPU's level 0,
    and the RGBA8 frame against the oracle's own voxelize -> mip -> G-buffer
    -> trace (its restatement of the shared far fields, the batch's default)
    at PSNR >= 40 dB (texture-unit sampler, end to end)."""
    bench_items = scenes.batch_scenes(n=7)
    items = [_items()[0], _items()[4], bench_items[0], bench_items[1], bench_items[6]]
    b = vct.Batch(items, use_graph=True)
    b.render()
    for i, (scene, w, h, grid, cones) in enumerate(items):
        p = oracle.Params(grid_res=grid, width=w, height=h, cone_set=cones, far_share=vct.FAR_SHARE_GROUP_W)
        ref = oracle.render(scene, p)
        l0 = b.read_voxels(i, 0)
        d = np.abs(l0.astype(int) - ref["level0"].astype(int))
        assert d.max() <= 1, f"scene {i}: level 0 max |d| {d.max()}"
        np.testing.assert_array_equal(l0[..., 3] > 0, ref["counts"] > 0, err_msg=f"scene {i} occupancy")
        ch = oracle.mipmap(p, l0)
        for lvl in range(1, p.levels):
            for m in range(6):
                np.testing.assert_array_equal(b.read_voxels(i, lvl, m), oracle.chain_level(ch, grid, lvl, m),
                                              err_msg=f"scene {i} level {lvl} map {m}")
        got = b.read_frame(i).astype(np.float64) / 255.0
        q = 10 * np.log10(1.0 / max(np.mean((got - np.clip(ref["frame"], 0, 1)) ** 2), 1e-30))
        print(f"batch scene {i} ({scene.n_tris} triangles, {w}x{h}, {grid}^3): level 0 identical "
              f"{100 * (d == 0).mean():.4f}%, frame PSNR {q:.1f} dB")
        assert q >= 40.0, f"scene {i}"
