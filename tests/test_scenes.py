"""Seeded synthetic scenes: sizes, layouts, determinism; and the per-pixel
texture work of the benchmark frame that bench.py's roofline uses."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes


def test_layout_sizes():
    assert scenes.MATERIAL_DTYPE.itemsize == 128   # material_data_t, renderer.h:94-120
    assert scenes.LIGHT_DTYPE.itemsize == 28       # point_light_t, renderer.h:87-92
    assert scenes.DRAWOBJ_DTYPE.itemsize == 12


def test_small_scene_counts():
    s = scenes.scene_small()
    assert s.n_tris == 10 + 2 * 12
    assert s.meshes[0].n_tris == 10                 # closed box room, 5 walls
    assert s.materials.shape[0] == 1 + 5 + 12       # default + per-face albedo
    alb = s.materials["diffuse"][1:, :3]
    assert (alb >= 0.2).all() and (alb <= 0.9).all()


def test_geodesic_sphere_is_closed_and_sized():
    m = scenes.geodesic_sphere(158, seed=1)
    assert m.n_tris == 20 * 158 * 158 == 499280
    assert m.verts.shape[0] == 10 * 158 * 158 + 2
    # every edge shared by exactly two triangles (watertight)
    e = np.sort(np.concatenate([m.indices[:, [0, 1]], m.indices[:, [1, 2]], m.indices[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    assert (cnt == 2).all()
    r = np.linalg.norm(m.verts[:, :3], axis=1)
    assert r.min() >= 0.95 - 1e-6 and r.max() <= 1.05 + 1e-6
    # outward, unit normals
    n = m.verts[:, 3:6]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    assert ((n * m.verts[:, :3]).sum(1) > 0).mean() > 0.99


def test_bench_scene_is_seeded():
    a = scenes.scene_sphere(freq=20)
    b = scenes.scene_sphere(freq=20)
    for ma, mb in zip(a.meshes, b.meshes):
        np.testing.assert_array_equal(ma.verts, mb.verts)
        np.testing.assert_array_equal(ma.indices, mb.indices)
    assert a.materials.tobytes() == b.materials.tobytes()


def test_draw_objects_cover_mesh():
    s = scenes.scene_sphere(freq=16)
    for m in s.meshes:
        tm = m.tri_material()
        assert tm.shape[0] == m.n_tris and (tm >= 1).all() and (tm < s.materials.shape[0]).all()


def test_bench_frame_work(oracle):
    """Instrumented oracle on the benchmark frame (every 32nd row): the
    per-pixel texture fetch counts bench.py reports."""
    import bench
    s = scenes.scene_sphere(seed=bench.SCENE_SEED, width=bench.WIDTH, height=bench.HEIGHT)
    p = oracle.Params(grid_res=bench.GRID, width=bench.WIDTH, height=bench.HEIGHT)
    l0, _, _ = oracle.voxelize(s, p)
    ch = oracle.mipmap(p, l0)
    gb = oracle.gbuffer(s, p)
    st = oracle.trace_stats(s, p, l0, ch, gb, row_stride=32)
    px = len(range(0, bench.HEIGHT, 32)) * bench.WIDTH
    bands = st.pop("lod_bands")
    steps = sum(v["steps"] for v in st.values()) / px
    lt1 = sum(v["lod_lt1"] for v in st.values()) / px
    assert sum(bands) == sum(v["steps"] for v in st.values())
    assert st["diffuse"]["cones"] == 9 * px
    assert 3 * steps + lt1 == pytest.approx(bench.TRACE_FETCHES_PER_PIXEL_REF, rel=0.02)
    assert st["shadow"]["beyond"] == 0  # shadow cones end at the light, inside the grid
    quad = sum(v["fetch_quad"] for v in st.values()) / px
    tri = sum(v["fetch_tri"] for v in st.values()) / px
    assert quad == pytest.approx(bench.TRACE_FETCH_QUAD_PER_PIXEL_NOSHARE, rel=0.02)
    assert tri == pytest.approx(bench.TRACE_FETCH_TRI_PER_PIXEL_NOSHARE, rel=0.02)
    # shared far fields (the default): pairs of rows, i.e. whole 2x2 quads
    from voxel_cone_tracing_gb300 import renderer
    ps = oracle.Params(grid_res=bench.GRID, width=bench.WIDTH, height=bench.HEIGHT,
                       far_share=renderer.FAR_SHARE_GROUP_W)
    sh = oracle.trace_stats(s, ps, l0, ch, gb, row_stride=-32)
    sh.pop("lod_bands")
    assert sum(v["fetch_quad"] for v in sh.values()) / (2 * px) == pytest.approx(bench.TRACE_FETCH_QUAD_PER_PIXEL,
                                                                                rel=0.02)
    assert sum(v["fetch_tri"] for v in sh.values()) / (2 * px) == pytest.approx(bench.TRACE_FETCH_TRI_PER_PIXEL,
                                                                               rel=0.02)
    for k in ("shadow", "specular"):  # only the diffuse cones share
        assert sh[k]["fetch_quad"] / (2 * px) == pytest.approx(st[k]["fetch_quad"] / px, rel=0.02)
    # at most 3 fetches per RGBA step and 2 per shadow step, +1 below lod 1
    upper = sum((2 if k == "shadow" else 3) * (v["steps"] - v["beyond"] - v["empty"]) + v["lod_lt1"] - v["empty_lt1"]
                for k, v in st.items()) / px
    assert quad + tri <= upper
