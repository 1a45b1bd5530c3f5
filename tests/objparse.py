"""An independent Wavefront OBJ/MTL reader for the loader tests (test
infrastructure): what Renderer::load_model (src/renderer.cpp:407-603) makes
of a file through tinyobjloader, written from the file format and those
lines without the engine's code.

* Polygons are triangulated as fans (v0, vk, vk+1) (LoadObj(..., true),
  renderer.cpp:417).
* A `g` or `o` line after faces starts a new shape (tinyobjloader).
* Per shape, consecutive faces with the same material form one draw object
  (renderer.cpp:519-556) whose material is the renderer's count of materials
  before the file (the file's materials are appended, :423-430) plus the
  file's index; a face with no material uses the file's first material
  (DEFAULT_MATERIAL_INDEX 0, :527-528) -- and the renderer's default
  material 0 when the file has none.
* Vertex deduplication (:510-515) changes no triangle, so the triangles keep
  their corners as read.
* MTL fields follow create_material (:49-81) with tinyobjloader's defaults
  (dissolve 1, ior 1, shininess 1); `Tr t` sets dissolve 1 - t unless the
  material has a `d` line, which wins in either order.
* Dimensions are max - min over every corner with the reference's
  arithmetic (max starts at 0, z is compared against min.y, :457-486).
"""
from __future__ import annotations

import os

import numpy as np

from voxel_cone_tracing_gb300 import scenes


def _floats(tokens, n):
    out = []
    for t in tokens[:n]:
        if t.startswith("#"):
            break
        out.append(float(t))
    return out + [0.0] * (n - len(out))


def parse_mtl(path):
    """-> (list of names, MATERIAL_DTYPE array)."""
    names, mats = [], []
    cur = None
    with open(path, "r", newline=None) as f:
        for raw in f:
            tok = raw.split()
            if not tok or tok[0].startswith("#"):
                continue
            key, args = tok[0], tok[1:]
            if key == "newmtl":
                has_d = False
                cur = np.zeros((), scenes.MATERIAL_DTYPE)
                cur["dissolve"], cur["ior"], cur["shininess"] = 1.0, 1.0, 1.0
                names.append(args[0] if args else "")
                mats.append(cur)
                continue
            if cur is None:
                continue
            vec3 = {"Ka": "ambient", "Kd": "diffuse", "Ks": "specular", "Kt": "transmittance",
                    "Tf": "transmittance", "Ke": "emission"}
            scal = {"Ns": "shininess", "Ni": "ior", "d": "dissolve", "Pr": "roughness", "Pm": "metallic",
                    "Ps": "sheen", "Pc": "clearcoat_thickness", "Pcr": "clearcoat_roughness", "aniso": "anisotropy",
                    "anisor": "anisotropy_rotation"}
            if key in vec3:
                cur[vec3[key]][:3] = _floats(args, 3)
            elif key in scal:
                cur[scal[key]] = _floats(args, 1)[0]
                has_d = has_d or key == "d"
            elif key == "Tr":
                if not has_d:
                    cur["dissolve"] = 1.0 - _floats(args, 1)[0]
            elif key == "illum":
                cur["illum"] = int(args[0])
    return names, (np.array(mats, scenes.MATERIAL_DTYPE) if mats else np.zeros(0, scenes.MATERIAL_DTYPE))


def _index(s, n):
    i = int(s)
    return i - 1 if i > 0 else n + i


class ObjModel:
    """verts (3T, 8) float32 [pos, normal, uv] per triangle corner, indices
    (T, 3), draw objects (DRAWOBJ_DTYPE), the file's materials, dimensions."""

    def __init__(self, verts, indices, draw_objs, materials, names, dims, shapes):
        self.verts, self.indices, self.draw_objs = verts, indices, draw_objs
        self.materials, self.material_names, self.dimensions, self.shapes = materials, names, dims, shapes

    def mesh(self) -> scenes.Mesh:
        return scenes.Mesh(self.verts, self.indices, self.draw_objs)


def parse_obj(path, material_base: int) -> ObjModel:
    pos, nrm, tex = [], [], []
    names, mats = [], np.zeros(0, scenes.MATERIAL_DTYPE)
    shapes = [[]]          # per shape: list of (corners, material index in file or -1)
    cur_mat = -1
    base = os.path.dirname(path)
    with open(path, "r", newline=None) as f:
        for raw in f:
            tok = raw.split()
            if not tok or tok[0].startswith("#"):
                continue
            key, args = tok[0], tok[1:]
            if key == "v":
                pos.append(_floats(args, 3))
            elif key == "vn":
                nrm.append(_floats(args, 3))
            elif key == "vt":
                tex.append(_floats(args, 2))
            elif key in ("g", "o"):
                if shapes[-1]:
                    shapes.append([])
            elif key == "mtllib":
                for lib in args:
                    n2, m2 = parse_mtl(os.path.join(base, lib))
                    names += n2
                    mats = np.concatenate([mats, m2])
            elif key == "usemtl":
                cur_mat = names.index(args[0]) if args and args[0] in names else -1
            elif key == "f":
                corners = []
                for c in args:
                    parts = c.split("/")
                    v = _index(parts[0], len(pos))
                    t = _index(parts[1], len(tex)) if len(parts) > 1 and parts[1] else -1
                    n = _index(parts[2], len(nrm)) if len(parts) > 2 and parts[2] else -1
                    corners.append((v, t, n))
                for k in range(1, len(corners) - 1):
                    shapes[-1].append(((corners[0], corners[k], corners[k + 1]), cur_mat))
    rows, objs = [], []
    mn, mx = [np.float32(np.finfo(np.float32).max)] * 3, [np.float32(0.0)] * 3
    tri = 0
    for shape in shapes:
        for corners, m in shape:
            for v, t, n in corners:
                p = [np.float32(x) for x in pos[v]]
                # renderer.cpp:464-486, including its comparison of z with min.y
                if p[0] > mx[0]:
                    mx[0] = p[0]
                if p[0] < mn[0]:
                    mn[0] = p[0]
                if p[1] > mx[1]:
                    mx[1] = p[1]
                if p[1] < mn[1]:
                    mn[1] = p[1]
                if p[2] > mx[2]:
                    mx[2] = p[2]
                if p[2] < mn[1]:
                    mn[2] = p[2]
                rows.append(p + (list(nrm[n]) if n >= 0 else [0.0] * 3) + (list(tex[t]) if t >= 0 else [0.0] * 2))
            fm = m if m >= 0 else 0
            mat = material_base + fm if len(mats) else 0
            if objs and objs[-1][2] == mat and objs[-1][3] == id(shape):
                objs[-1][1] += 3
            else:
                objs.append([3 * tri, 3, mat, id(shape)])
            tri += 1
    verts = np.array(rows, np.float32).reshape(-1, 8)
    idx = np.arange(verts.shape[0], dtype=np.uint32).reshape(-1, 3)
    draw = np.array([(a, b, c) for a, b, c, _ in objs], scenes.DRAWOBJ_DTYPE)
    dims = np.array([mx[k] - mn[k] for k in range(3)], np.float32)
    return ObjModel(verts, idx, draw, mats, names, dims, sum(1 for s in shapes if s))
