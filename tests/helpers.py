"""Small scene builders shared by the tests."""
from __future__ import annotations

import numpy as np

from voxel_cone_tracing_gb300 import scenes


def emissive_material(emission=(0.2, 0.4, 0.6), diffuse=(0.0, 0.0, 0.0)):
    m = scenes.make_material(diffuse, roughness=1.0, specular=0.0, emission=emission, illum=2)
    return m


def tri_scene(tris, normals=None, material=None, lights=(), cube_size=1.0, view=None, proj=None,
              name="tris") -> scenes.Scene:
    """One mesh of independent triangles (tris: (T, 3, 3) object-space
    positions), one material (id 1), identity model matrix."""
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    t = tris.shape[0]
    pos = tris.reshape(-1, 3)
    if normals is None:
        e1 = tris[:, 1] - tris[:, 0]
        e2 = tris[:, 2] - tris[:, 0]
        fn = np.cross(e1, e2)
        fn = fn / np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
        nrm = np.repeat(fn, 3, axis=0)
    else:
        nrm = np.broadcast_to(np.asarray(normals, np.float32), pos.shape)
    verts = np.zeros((3 * t, 8), np.float32)
    verts[:, 0:3] = pos
    verts[:, 3:6] = nrm
    idx = np.arange(3 * t, dtype=np.uint32).reshape(-1, 3)
    objs = np.array([(0, 3 * t, 1)], scenes.DRAWOBJ_DTYPE)
    mats = np.array([scenes.default_material(), material if material is not None else emissive_material()],
                    scenes.MATERIAL_DTYPE)
    lights = np.array([scenes.point_light(*l) if not isinstance(l, np.ndarray) else l for l in lights],
                      scenes.LIGHT_DTYPE)
    if view is None:
        view = scenes.mat_identity()
    if proj is None:
        proj = scenes.mat_identity()
    return scenes.Scene([scenes.Mesh(verts, idx, objs)], [scenes.mat_identity()], mats, lights,
                        np.asarray(view, np.float32), np.asarray(proj, np.float32), float(cube_size), name=name)


def quad_z(z, lo=-1.0, hi=1.0):
    """Two triangles covering [lo,hi]^2 at depth z, normal +z."""
    a, b, c, d = (lo, lo, z), (hi, lo, z), (hi, hi, z), (lo, hi, z)
    return [[a, b, c], [a, c, d]]


def psnr(a, b, peak=1.0):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
