"""Seeded synthetic scenes for the voxelize -> mipmap -> cone-trace path.

The reference renders the Cornell box and Suzanne from OBJ files
(src/main.cpp:85-121).  The workloads here are seeded synthetic scenes of the
sizes the benchmark configurations name; every array uses the reference's
own layouts:

* vertices: ``vert_data_t`` (src/renderer.cpp:23-35) -- pos3, norm3, uv2 as
  float32, 32 bytes per vertex;
* indices: uint32 triangle lists (src/renderer.cpp:565);
* draw objects: runs ``(first_index, index_count, material_id)`` as the
  reference's ``draw_obj_t`` ranges (src/renderer.cpp:519-556);
* materials: ``material_data_t`` (src/renderer.h:94-120, 128 bytes packed);
* point lights: ``point_light_t`` (src/renderer.h:87-92, 28 bytes);
* matrices: column-major float32[16] (glm / GL convention).

Material 0 is the renderer's default material (src/renderer.cpp:85-98,
115-128); scene materials start at id 1, as ``add_material`` returns them.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

MATERIAL_DTYPE = np.dtype([
    ("ambient", "<f4", (4,)), ("diffuse", "<f4", (4,)), ("specular", "<f4", (4,)),
    ("transmittance", "<f4", (4,)), ("emission", "<f4", (3,)), ("shininess", "<f4"),
    ("ior", "<f4"), ("dissolve", "<f4"), ("illum", "<i4"), ("roughness", "<f4"),
    ("metallic", "<f4"), ("sheen", "<f4"), ("clearcoat_thickness", "<f4"),
    ("clearcoat_roughness", "<f4"), ("anisotropy", "<f4"), ("anisotropy_rotation", "<f4"),
    ("pad", "<f4", (2,)),
])
assert MATERIAL_DTYPE.itemsize == 128

LIGHT_DTYPE = np.dtype([("position", "<f4", (3,)), ("color", "<f4", (3,)), ("intensity", "<f4")])
assert LIGHT_DTYPE.itemsize == 28

DRAWOBJ_DTYPE = np.dtype([("first", "<u4"), ("count", "<u4"), ("material", "<u4")])


def default_material() -> np.ndarray:
    """fill_default_mat_data (src/renderer.cpp:85-98); unset fields are 0."""
    m = np.zeros((), MATERIAL_DTYPE)
    m["ambient"][:3] = (1, 0, 1)
    m["diffuse"][:3] = (1, 0, 1)
    m["shininess"] = 1
    m["ior"] = 1
    m["dissolve"] = 1
    m["illum"] = 0
    return m


def make_material(albedo, roughness=1.0, specular=None, emission=(0, 0, 0), illum=2,
                  dissolve=1.0, ior=1.5, transmittance=(1, 1, 1)) -> np.ndarray:
    """A material_data_t.  roughness r maps to the reference's shininess by
    inverting voxel_cone_tracing.frag:220 (r = sqrt(2 / (shininess + 2)))."""
    m = np.zeros((), MATERIAL_DTYPE)
    r = float(np.clip(roughness, 0.05, 1.0))
    m["ambient"][:3] = albedo
    m["diffuse"][:3] = albedo
    spec = (1.0 - r) * 0.5 if specular is None else specular
    m["specular"][:3] = spec
    m["transmittance"][:3] = transmittance
    m["emission"] = emission
    m["shininess"] = 2.0 / (r * r) - 2.0
    m["ior"] = ior
    m["dissolve"] = dissolve
    m["illum"] = illum
    m["roughness"] = r
    return m


@dataclasses.dataclass
class Mesh:
    """One loaded model: what ``Renderer::load_model`` builds from an OBJ."""
    verts: np.ndarray        # (n, 8) float32
    indices: np.ndarray      # (m, 3) uint32
    draw_objs: np.ndarray    # (k,) DRAWOBJ_DTYPE, ``first``/``count`` in indices

    @property
    def n_tris(self) -> int:
        return int(self.indices.shape[0])

    def tri_material(self) -> np.ndarray:
        """Per-triangle material id from the draw-object runs."""
        tm = np.zeros(self.n_tris, np.uint32)
        for d in self.draw_objs:
            t0, tn = int(d["first"]) // 3, int(d["count"]) // 3
            tm[t0:t0 + tn] = d["material"]
        return tm


@dataclasses.dataclass
class Scene:
    meshes: list             # [Mesh]
    models: list             # model matrix per mesh, (16,) float32 column-major
    materials: np.ndarray    # MATERIAL_DTYPE, index 0 = default material
    lights: np.ndarray       # LIGHT_DTYPE
    view: np.ndarray         # (16,) float32
    proj: np.ndarray         # (16,) float32
    cube_size: float
    name: str = ""

    @property
    def n_tris(self) -> int:
        return sum(m.n_tris for m in self.meshes)


# ----------------------------------------------------------- matrix helpers --
def mat_identity() -> np.ndarray:
    return np.eye(4, dtype=np.float32).reshape(-1, order="F").copy()


def mat_from_rows(m4: np.ndarray) -> np.ndarray:
    """Row-major 4x4 (maths order) -> column-major float32[16]."""
    return np.asarray(m4, np.float64).astype(np.float32).reshape(-1, order="F").copy()


def look_at(eye, center, up=(0, 1, 0)) -> np.ndarray:
    """glm::lookAt (right-handed), column-major."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return mat_from_rows(m)


def perspective(fovy_rad, aspect, near, far) -> np.ndarray:
    """glm::perspective (GL clip space, z in [-1, 1]), column-major."""
    t = math.tan(fovy_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2.0 * far * near / (far - near)
    m[3, 2] = -1.0
    return mat_from_rows(m)


def trs(translate=(0, 0, 0), rot=None, scale=(1, 1, 1)) -> np.ndarray:
    m = np.eye(4)
    r = np.eye(3) if rot is None else np.asarray(rot, np.float64)
    m[:3, :3] = r @ np.diag(np.asarray(scale, np.float64))
    m[:3, 3] = translate
    return mat_from_rows(m)


def random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


# ------------------------------------------------------------ geometry ------
def _pack_verts(pos, nrm, uv=None) -> np.ndarray:
    n = pos.shape[0]
    v = np.zeros((n, 8), np.float32)
    v[:, 0:3] = pos
    v[:, 3:6] = nrm
    if uv is not None:
        v[:, 6:8] = uv
    return v


def _quads_mesh(quads, normals, materials) -> Mesh:
    """Flat-shaded quads (4 corners, counter-clockwise seen from the normal
    side), two triangles each, one draw object per quad."""
    pos, nrm, idx, runs = [], [], [], []
    for q, (corners, n, mat) in enumerate(zip(quads, normals, materials)):
        base = 4 * q
        pos.extend(corners)
        nrm.extend([n] * 4)
        idx.append([base, base + 1, base + 2])
        idx.append([base, base + 2, base + 3])
        runs.append((6 * q, 6, mat))
    verts = _pack_verts(np.array(pos, np.float32), np.array(nrm, np.float32))
    return Mesh(verts, np.array(idx, np.uint32), np.array(runs, DRAWOBJ_DTYPE))


def box_room(material_ids) -> Mesh:
    """Closed box room: the unit cube [-0.5, 0.5]^3 minus its +z face (the
    camera side), 5 walls = 10 axis-aligned triangles, normals inward."""
    h = 0.5
    walls = [
        ([(-h, -h, h), (h, -h, h), (h, -h, -h), (-h, -h, -h)], (0, 1, 0)),     # floor
        ([(-h, h, -h), (h, h, -h), (h, h, h), (-h, h, h)], (0, -1, 0)),        # ceiling
        ([(-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h)], (0, 0, 1)),     # back
        ([(-h, -h, h), (-h, -h, -h), (-h, h, -h), (-h, h, h)], (1, 0, 0)),     # left
        ([(h, -h, -h), (h, -h, h), (h, h, h), (h, h, -h)], (-1, 0, 0)),        # right
    ]
    return _quads_mesh([w[0] for w in walls], [w[1] for w in walls], material_ids)


def cuboid(material_ids) -> Mesh:
    """Unit cube [-0.5, 0.5]^3 with outward normals, 12 triangles."""
    h = 0.5
    faces = [
        ([(h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h)], (1, 0, 0)),
        ([(-h, -h, h), (-h, h, h), (-h, h, -h), (-h, -h, -h)], (-1, 0, 0)),
        ([(-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h)], (0, 1, 0)),
        ([(-h, -h, h), (-h, -h, -h), (h, -h, -h), (h, -h, h)], (0, -1, 0)),
        ([(-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)], (0, 0, 1)),
        ([(h, -h, -h), (-h, -h, -h), (-h, h, -h), (h, h, -h)], (0, 0, -1)),
    ]
    return _quads_mesh([f[0] for f in faces], [f[1] for f in faces], material_ids)


_ICO_T = (1.0 + 5 ** 0.5) / 2.0
_ICO_V = np.array([(-1, _ICO_T, 0), (1, _ICO_T, 0), (-1, -_ICO_T, 0), (1, -_ICO_T, 0),
                   (0, -1, _ICO_T), (0, 1, _ICO_T), (0, -1, -_ICO_T), (0, 1, -_ICO_T),
                   (_ICO_T, 0, -1), (_ICO_T, 0, 1), (-_ICO_T, 0, -1), (-_ICO_T, 0, 1)], np.float64)
_ICO_F = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
                   (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
                   (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)


def geodesic_sphere(freq: int, seed: int, amplitude: float = 0.05, material_base: int = 1) -> Mesh:
    """Frequency-``freq`` geodesic icosphere (20*freq^2 triangles; 158 gives
    499,280), radius 1, radially displaced by ``amplitude`` x a seeded sum of
    8 random plane waves normalised to [-1, 1].  Smooth (area-weighted)
    normals.  One draw object / material per icosahedron face."""
    rng = np.random.default_rng(seed)
    v0 = _ICO_V / np.linalg.norm(_ICO_V, axis=1, keepdims=True)
    ii, jj = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = ii + jj <= freq
    ii, jj = ii[keep], jj[keep]
    lut = -np.ones((freq + 1, freq + 1), np.int64)
    lut[ii, jj] = np.arange(ii.size)
    a_i, a_j = np.meshgrid(np.arange(freq), np.arange(freq), indexing="ij")
    up = a_i + a_j < freq
    ui, uj = a_i[up], a_j[up]
    dn = a_i + a_j < freq - 1
    di, dj = a_i[dn], a_j[dn]
    local_tris = np.concatenate([
        np.stack([lut[ui, uj], lut[ui + 1, uj], lut[ui, uj + 1]], 1),
        np.stack([lut[di + 1, dj], lut[di + 1, dj + 1], lut[di, dj + 1]], 1)])
    pts, tris = [], []
    for f, (a, b, c) in enumerate(_ICO_F):
        A, B, C = v0[a], v0[b], v0[c]
        p = A[None] + (B - A)[None] * (ii[:, None] / freq) + (C - A)[None] * (jj[:, None] / freq)
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        tris.append(local_tris + f * ii.size)
        pts.append(p)
    pts = np.concatenate(pts)
    tris = np.concatenate(tris)
    key = np.round(pts * 1e9).astype(np.int64)
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    upos = np.zeros((uniq.shape[0], 3))
    upos[inv] = pts
    tris = inv[tris]
    # displacement
    dirs = rng.normal(size=(8, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    freqs = rng.uniform(2.0, 9.0, 8)
    phase = rng.uniform(0, 2 * np.pi, 8)
    amps = rng.uniform(0.5, 1.0, 8)
    noise = (amps[None] * np.sin(freqs[None] * (upos @ dirs.T) + phase[None])).sum(1) / amps.sum()
    upos = upos * (1.0 + amplitude * noise)[:, None]
    # smooth normals
    e1 = upos[tris[:, 1]] - upos[tris[:, 0]]
    e2 = upos[tris[:, 2]] - upos[tris[:, 0]]
    fn = np.cross(e1, e2)
    vn = np.zeros_like(upos)
    for k in range(3):
        np.add.at(vn, tris[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    verts = _pack_verts(upos.astype(np.float32), vn.astype(np.float32))
    per_face = freq * freq
    runs = np.array([(3 * per_face * f, 3 * per_face, material_base + f) for f in range(20)], DRAWOBJ_DTYPE)
    return Mesh(verts, tris.astype(np.uint32), runs)


def point_light(position, color=(1, 1, 1), intensity=1.0) -> np.ndarray:
    l = np.zeros((), LIGHT_DTYPE)
    l["position"], l["color"], l["intensity"] = position, color, intensity
    return l


# ------------------------------------------------------------- configs ------
ROOM_CUBE_SIZE = 0.52   # grid covers [-0.52, 0.52]^3, walls at +-0.5


def _camera(width, height):
    view = look_at((0.0, 0.02, 0.49), (0.0, -0.08, -0.5))
    proj = perspective(math.radians(60.0), width / height, 0.01, 10.0)
    return view, proj


def scene_small(seed: int = 1000, width: int = 256, height: int = 256) -> Scene:
    """Closed box room (10 wall triangles) + 2 randomly rotated/scaled cuboids
    (24 triangles), per-face diffuse albedo U[0.2, 0.9], one point light."""
    rng = np.random.default_rng(seed)
    mats = [default_material()]

    def new_mat():
        mats.append(make_material(rng.uniform(0.2, 0.9, 3), roughness=rng.uniform(0.3, 1.0)))
        return len(mats) - 1

    meshes, models = [box_room([new_mat() for _ in range(5)])], [mat_identity()]
    for _ in range(2):
        meshes.append(cuboid([new_mat() for _ in range(6)]))
        models.append(trs(translate=rng.uniform([-0.25, -0.35, -0.3], [0.25, -0.1, 0.1]),
                          rot=random_rotation(rng), scale=rng.uniform(0.12, 0.3, 3)))
    view, proj = _camera(width, height)
    return Scene(meshes, models, np.array(mats, MATERIAL_DTYPE),
                 np.array([point_light((0.0, 0.4, 0.0))], LIGHT_DTYPE), view, proj, ROOM_CUBE_SIZE,
                 name="room+2cuboids")


def scene_sphere(seed: int = 2000, freq: int = 158, width: int = 1920, height: int = 1080) -> Scene:
    """The same room plus a noise-displaced geodesic icosphere (20*freq^2
    triangles, displacement 5% of the radius); wall albedo U[0.2, 0.9],
    sphere-patch albedo and roughness U[0, 1]."""
    rng = np.random.default_rng(seed)
    mats = [default_material()]
    for _ in range(5):
        mats.append(make_material(rng.uniform(0.2, 0.9, 3), roughness=rng.uniform(0.3, 1.0)))
    room = box_room(list(range(1, 6)))
    sphere_base = len(mats)
    for _ in range(20):
        mats.append(make_material(rng.uniform(0.0, 1.0, 3), roughness=rng.uniform(0.0, 1.0)))
    sphere = geodesic_sphere(freq, seed + 1, 0.05, material_base=sphere_base)
    model = trs(translate=(0.05, -0.22, -0.12), scale=(0.25, 0.25, 0.25))
    view, proj = _camera(width, height)
    return Scene([room, sphere], [mat_identity(), model], np.array(mats, MATERIAL_DTYPE),
                 np.array([point_light((0.0, 0.4, 0.05))], LIGHT_DTYPE), view, proj, ROOM_CUBE_SIZE,
                 name=f"room+icosphere{freq}")


HDR_RADIANCE_MAX = 16.0


def scene_hdr(seed: int = 3000, freq: int = 158, n_spheres: int = 4, n_cuboids: int = 32, width: int = 1920,
              height: int = 1080) -> Scene:
    """HDR precision scene: the room, ``n_spheres`` noise-displaced geodesic
    spheres (20*freq^2 triangles each; 4 x 158 gives 1,997,120) and
    ``n_cuboids`` randomly rotated cuboids, a bright point light (intensity
    12) and emissive cuboids (emission up to 20), so that voxel radiance
    covers [0, 16] before the clamp."""
    rng = np.random.default_rng(seed)
    mats = [default_material()]
    for _ in range(5):
        mats.append(make_material(rng.uniform(0.2, 0.9, 3), roughness=rng.uniform(0.3, 1.0)))
    meshes, models = [box_room(list(range(1, 6)))], [mat_identity()]
    for k in range(n_spheres):
        base = len(mats)
        for _ in range(20):
            mats.append(make_material(rng.uniform(0.0, 1.0, 3), roughness=rng.uniform(0.0, 1.0)))
        meshes.append(geodesic_sphere(freq, seed + 1 + k, 0.05, material_base=base))
        models.append(trs(translate=rng.uniform([-0.3, -0.35, -0.35], [0.3, 0.0, 0.0]),
                          scale=np.full(3, rng.uniform(0.08, 0.16))))
    for _ in range(n_cuboids):
        ids = []
        for _ in range(6):
            emit = rng.uniform(0.0, 20.0, 3) if rng.uniform() < 0.3 else (0.0, 0.0, 0.0)
            mats.append(make_material(rng.uniform(0.1, 0.9, 3), roughness=rng.uniform(0.2, 1.0), emission=emit))
            ids.append(len(mats) - 1)
        meshes.append(cuboid(ids))
        models.append(trs(translate=rng.uniform([-0.42, -0.45, -0.45], [0.42, 0.35, 0.1]),
                          rot=random_rotation(rng), scale=rng.uniform(0.02, 0.1, 3)))
    view, proj = _camera(width, height)
    return Scene(meshes, models, np.array(mats, MATERIAL_DTYPE),
                 np.array([point_light((0.0, 0.38, 0.05), intensity=12.0)], LIGHT_DTYPE), view, proj,
                 ROOM_CUBE_SIZE, name=f"room+{n_spheres}icospheres{freq}+{n_cuboids}cuboids")


BATCH_FRAMES = [(256, 256), (512, 384), (640, 480), (960, 540), (1280, 720), (1920, 1080)]
BATCH_GRIDS = [32, 64, 128, 256]


def batch_scenes(seed: int = 5000, n: int = 64, max_tris: int = 1_000_000, min_tris: int = 1_000) -> list:
    """Seeded batch of `n` independent scenes of uneven size: triangle counts
    log-uniform in [min_tris, max_tris] (the room plus one displaced geodesic
    sphere of frequency round(sqrt((T - 10) / 20))), frames from 256^2 to
    1920x1080, grids 32^3 to 256^3, 9 or 6 diffuse cones.  Scene i uses seed
    `seed + i`.  Returns (scene, width, height, grid_res, cone_set) tuples,
    cone_set 0 = the reference's 9 cones, 1 = 6 cones."""
    out = []
    sphere_cache = {}
    for i in range(n):
        rng = np.random.default_rng(seed + i)
        target = math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))
        freq = max(2, int(round(math.sqrt(max(target - 10.0, 40.0) / 20.0))))
        w, h = BATCH_FRAMES[int(rng.integers(len(BATCH_FRAMES)))]
        grid = BATCH_GRIDS[int(rng.integers(len(BATCH_GRIDS)))]
        cones = int(rng.integers(2))
        mats = [default_material()]
        for _ in range(5):
            mats.append(make_material(rng.uniform(0.2, 0.9, 3), roughness=rng.uniform(0.3, 1.0)))
        room = box_room(list(range(1, 6)))
        base = len(mats)
        for _ in range(20):
            mats.append(make_material(rng.uniform(0.0, 1.0, 3), roughness=rng.uniform(0.0, 1.0)))
        if freq not in sphere_cache:
            sphere_cache[freq] = geodesic_sphere(freq, seed + 100000 + freq, 0.05, material_base=base)
        sphere = sphere_cache[freq]
        model = trs(translate=rng.uniform([-0.2, -0.3, -0.25], [0.2, -0.1, 0.0]),
                    scale=np.full(3, rng.uniform(0.12, 0.28)))
        view, proj = _camera(w, h)
        light = point_light(tuple(rng.uniform([-0.3, 0.3, -0.2], [0.3, 0.45, 0.2])))
        s = Scene([room, sphere], [mat_identity(), model], np.array(mats, MATERIAL_DTYPE),
                  np.array([light], LIGHT_DTYPE), view, proj, ROOM_CUBE_SIZE, name=f"batch{i}")
        out.append((s, w, h, grid, cones))
    return out
