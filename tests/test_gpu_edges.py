"""Edge cases of the path, GPU against the FP64 oracle on the same inputs.

Every case checks, with the tolerances of test_gpu_parity.py: voxel
contribution counts bit-exact, level 0 within 1 LSB, the whole mip chain
bit-exact (from the GPU's level 0), visible triangle ids bit-exact, and the
frame with FP32 software filtering (EXACT sampler) against the oracle's
trace of the GPU's own maps and G-buffer at PSNR >= 60 dB.
"""
import math

import numpy as np
import pytest

from tests.helpers import psnr, quad_z, tri_scene
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu


def _parity(vct, oracle, scene, w, h, n, mode=0, mip_mode=0, cone_set=0):
    r = vct.Renderer(w, h, grid_res=n, keep_counts=1, keep_float_frame=1, vox_mode=mode, mip_mode=mip_mode,
                     sampler=1, cone_set=cone_set)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    p = oracle.Params(grid_res=n, width=w, height=h, vox_mode=mode, mip_mode=mip_mode, cone_set=cone_set)
    l0, cnt, _ = oracle.voxelize(scene, p)
    np.testing.assert_array_equal(r.read_voxel_counts(), cnt)
    assert np.abs(r.read_voxels(0).astype(int) - l0.astype(int)).max(initial=0) <= 1
    gl0 = r.read_voxels(0)
    ch = oracle.mipmap(p, gl0)
    nmaps = 1 if mip_mode == 1 else 6
    off = 0
    for lvl in range(1, r.grid()[1]):
        s = n >> lvl
        for m in range(nmaps):
            np.testing.assert_array_equal(r.read_voxels(lvl, m).reshape(-1, 4), ch[m, off:off + s ** 3])
        off += s ** 3
    g = r.read_gbuffer()
    og = oracle.gbuffer(scene, p)
    np.testing.assert_array_equal(g["tri_id"], og["tri_id"])
    gb = dict(tri_id=g["tri_id"], pos=g["pos"].astype(np.float64), nrm=g["nrm"].astype(np.float64), mat=g["mat"])
    ref = oracle.trace(scene, p, gl0, ch, gb)
    got = r.read_frame(vct.FRAME_RGBA32F)
    q = psnr(np.clip(got, 0, 1), np.clip(ref, 0, 1))
    assert q >= 60.0, q
    return r, cnt


def _camera(w, h, eye=(0.0, 0.0, 0.9), at=(0.0, 0.0, 0.0)):
    return scenes.look_at(eye, at), scenes.perspective(math.radians(60.0), w / h, 0.01, 10.0)


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_pathological_triangles(vct, oracle, mode):
    """Degenerate (collinear, a point), non-finite, far outside the grid,
    spanning the whole grid, on voxel boundaries, on the grid faces, and
    smaller than 1e-6 voxel^2."""
    n = 32
    v = 2.0 / n  # one voxel in grid units (cube_size 1)
    nan = float("nan")
    tris = [
        [(0.1, 0.1, 0.1), (0.2, 0.2, 0.2), (0.3, 0.3, 0.3)],            # collinear
        [(0.05, -0.1, 0.2)] * 3,                                         # a point
        [(nan, 0.0, 0.0), (0.1, 0.1, 0.0), (0.0, 0.1, 0.1)],             # NaN vertex
        [(float("inf"), 0.2, 0.0), (0.1, 0.2, 0.1), (0.0, 0.3, 0.1)],    # infinite vertex
        [(5.0, 5.0, 5.0), (5.5, 5.0, 5.0), (5.0, 5.5, 5.2)],             # outside the grid
        [(-3.0, -3.0, 0.31), (3.0, -3.0, 0.27), (0.0, 3.0, 0.29)],       # spans the whole grid
        [(2 * v, 4 * v, 6 * v), (10 * v, 4 * v, 6 * v), (2 * v, 12 * v, 6 * v)],  # on voxel boundaries
        [(-1.0, -0.5, -0.5), (-1.0, 0.5, -0.5), (-1.0, -0.5, 0.5)],      # on the low x face of the grid
        [(1.0, -0.5, -0.5), (1.0, 0.5, -0.5), (1.0, -0.5, 0.5)],         # on the high x face
        [(0.3, 0.3, 0.3), (0.3 + 1e-4 * v, 0.3, 0.3), (0.3, 0.3 + 1e-4 * v, 0.3)],  # area 5e-9 voxel^2
    ]
    w, h = 48, 32
    view, proj = _camera(w, h)
    mat = scenes.make_material((0.8, 0.5, 0.3), roughness=0.5)
    s = tri_scene(tris, material=mat, lights=[((0.2, 0.6, 0.4),)], cube_size=1.0, view=view, proj=proj)
    _, cnt = _parity(vct, oracle, s, w, h, n, mode=mode)
    assert cnt.sum() > 500


def test_light_limit_and_materials(vct, oracle):
    """11 queued lights (the shader reads 10, voxelize.frag:40,128), transparent
    (illum 4: refraction cone, dissolve), emissive and very glossy
    materials, instanced models, the six-cone set and isotropic mips."""
    base = scenes.scene_small(seed=31, width=72, height=48)
    mats = list(base.materials)
    mats.append(scenes.make_material((0.2, 0.6, 0.9), roughness=0.05, illum=4, dissolve=0.3, ior=1.4,
                                     transmittance=(0.9, 0.8, 0.7)))
    mats.append(scenes.make_material((0.1, 0.1, 0.1), emission=(0.9, 0.4, 0.1)))
    mats.append(scenes.make_material((0.9, 0.9, 0.9), roughness=0.0, specular=1.0))
    k = len(mats)
    meshes, models = list(base.meshes), list(base.models)
    for j, (t, sc) in enumerate([((-0.2, -0.3, -0.1), 0.12), ((0.15, -0.25, -0.2), 0.1), ((0.0, -0.1, -0.3), 0.08)]):
        meshes.append(scenes.cuboid([k - 3 + j] * 6))
        models.append(scenes.trs(translate=t, scale=(sc, sc, sc)))
    meshes.append(meshes[-1])  # the same model queued twice with another transform
    models.append(scenes.trs(translate=(0.25, -0.35, 0.05), scale=(0.07, 0.07, 0.07)))
    lights = [scenes.point_light((0.3 * math.cos(a), 0.3, 0.3 * math.sin(a)), intensity=0.15) for a in
              np.linspace(0, 2 * math.pi, 11, endpoint=False)]
    s = scenes.Scene(meshes, models, np.array(mats, scenes.MATERIAL_DTYPE), np.array(lights, scenes.LIGHT_DTYPE),
                     base.view, base.proj, base.cube_size, name="edge-materials")
    _parity(vct, oracle, s, 72, 48, 64)
    _parity(vct, oracle, s, 72, 48, 32, mip_mode=1, cone_set=1)


@pytest.mark.parametrize("w, h, n", [(1, 1, 16), (17, 5, 8), (33, 47, 16)])
def test_ragged_frames_and_small_grids(vct, oracle, w, h, n):
    s = scenes.scene_small(seed=41, width=w, height=h)
    _parity(vct, oracle, s, w, h, n)


def test_camera_outside_the_grid(vct, oracle):
    """within_cube (voxel_cone_tracing.frag:61-64, 250) tests the texture-space
    position u = 0.5 p + 0.5 against |u| < 1, i.e. grid-space p in (-3, 1):
    fragments with some p >= 1 or p <= -3 keep the clear colour, fragments
    with p in (-3, -1] are shaded although they lie outside the voxel grid."""
    w, h = 40, 30
    view, proj = _camera(w, h, eye=(0.0, 0.0, 3.0))
    s = tri_scene(quad_z(-0.2, -2.5, 2.5) + quad_z(0.1, -0.3, 0.3), material=scenes.make_material((0.6, 0.6, 0.6)),
                  lights=[((0.0, 0.5, 0.8),)], cube_size=1.0, view=view, proj=proj)
    r, _ = _parity(vct, oracle, s, w, h, 32)
    f = r.read_frame()
    g = r.read_gbuffer()
    u = 0.5 * g["pos"] + 0.5  # cube_size 1
    hit = g["tri_id"] != 0xffffffff
    outside = hit & (np.abs(u).max(axis=-1) >= 1.0)
    shaded_beyond = hit & (np.abs(u).max(axis=-1) < 1.0) & (g["pos"].min(axis=-1) <= -1.0)
    assert outside.any() and shaded_beyond.any()
    assert (f[outside] == (38, 64, 64, 255)).all()
    assert (f[shaded_beyond] != (38, 64, 64, 255)).any(axis=-1).all()


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_dense_bricks_split_across_ctas(vct, oracle, mode):
    """72,000 triangles in a 16^3 grid: the bricks around the sphere hold
    thousands of (triangle, brick) pairs each, so their pairs are spread over
    several CTAs (chunks of 1024 pairs) and summed in global memory."""
    s = scenes.scene_sphere(seed=77, freq=60, width=48, height=32)
    r, _ = _parity(vct, oracle, s, 48, 32, 16, mode=mode)
    assert r.stage_times()["split_bricks"] > 0


def test_dense_brick_plan_overflow(vct, oracle):
    """4,000 planes at random depths in the two lowest brick layers of a
    128^3 grid, each over 9 x 16 bricks: 288 dense bricks of ~2,000 pairs,
    more than the 256 accumulator slots of a new renderer.  The bricks that
    did not get a slot run whole on one CTA (still exact), the slots grow,
    and the next frame splits every dense brick."""
    rng = np.random.default_rng(9)
    z = rng.uniform(-0.995, -0.755, 4000)
    # x in [-1.2, 0.12] (brick columns 0..8), y over the whole grid
    tris = [[(-1.2, -1.2, zi), (0.12, -1.2, zi), (-1.2, 60.0, zi)] for zi in z]
    s = tri_scene(tris)
    n = 128
    p = oracle.Params(grid_res=n, width=8, height=8)
    l0, cnt, _ = oracle.voxelize(s, p)
    r = vct.Renderer(8, 8, grid_res=n, keep_counts=1)
    ids = vct.load_scene(r, s)
    for _ in range(2):
        vct.queue_scene(r, s, ids)
        r.render()
        np.testing.assert_array_equal(r.read_voxel_counts(), cnt)
        assert np.abs(r.read_voxels(0).astype(int) - l0.astype(int)).max(initial=0) <= 1
        assert r.stage_times()["split_bricks"] == 288
