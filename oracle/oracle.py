"""ctypes binding of the CPU oracle (oracle/vct_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, as the checker or the timed CPU
restatement -- never by the product.  Parity unpinned (the reference has no
golden vectors and cannot run here); see vct_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle_vct.so")
SRC = os.path.join(_HERE, "vct_oracle.cpp")
SRCS = [SRC, os.path.join(_HERE, "vct_oracle_mlp.cpp")]

VOX_REF_RASTER2X, VOX_CONSERVATIVE = 0, 1
MIP_ANISO, MIP_ISO = 0, 1
CONES_REF9, CONES_SIX60 = 0, 1


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no -march flags, no FMA contraction, so
    x86-64 and aarch64 give identical coverage decisions)."""
    deps = SRCS + [os.path.join(_HERE, "vct_oracle.h")]
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(map(os.path.getmtime, deps)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread",
                           "-ffp-contract=off", "-fno-fast-math", "-o", tmp, *SRCS])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_float * 3), ("intensity", C.c_float)]


class _Instance(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("indices", C.c_void_p), ("tri_material", C.c_void_p),
                ("n_verts", C.c_uint32), ("n_tris", C.c_uint32), ("model", C.c_float * 16)]


class _Scene(C.Structure):
    _fields_ = [("instances", C.c_void_p), ("materials", C.c_void_p), ("lights", C.c_void_p),
                ("n_instances", C.c_uint32), ("n_materials", C.c_uint32), ("n_lights", C.c_uint32),
                ("cube_size", C.c_float), ("view", C.c_float * 16), ("proj", C.c_float * 16)]


class _Params(C.Structure):
    _fields_ = [("grid_res", C.c_int32), ("levels", C.c_int32), ("vox_mode", C.c_int32),
                ("mip_mode", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("enable_direct", C.c_int32), ("enable_diffuse", C.c_int32),
                ("enable_specular", C.c_int32), ("enable_shadow", C.c_int32),
                ("view_voxel_dir", C.c_int32), ("view_voxel_lod", C.c_float),
                ("cone_set", C.c_int32), ("threads", C.c_int32), ("radiance_max", C.c_float),
                ("far_share", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_chain_texels.restype = C.c_uint64
        L.orc_chain_texels.argtypes = [C.c_int32, C.c_int32]
        for f in ("orc_voxelize", "orc_voxelize_f32"):
            getattr(L, f).restype = C.c_int64
            getattr(L, f).argtypes = [P, P, P, P]
        L.orc_mipmap.argtypes = [P, P, P]
        L.orc_voxelize_cas.restype = C.c_int64
        L.orc_voxelize_cas.argtypes = [P, P, C.c_int32, C.c_uint64, P]
        L.orc_cas_avg.restype = C.c_uint32
        L.orc_cas_avg.argtypes = [P, C.c_int32]
        L.orc_voxelize_attr.restype = C.c_int64
        L.orc_voxelize_attr.argtypes = [P, P, P, P, P, P]
        L.orc_inject.argtypes = [P, P, P, P, P, P]
        L.orc_voxelize_hdr.restype = C.c_int64
        L.orc_voxelize_hdr.argtypes = [P, P, P, P]
        L.orc_mip_level_f.argtypes = [C.c_int32, C.c_int32, P, C.c_int32, P]
        L.orc_trace_hdr.argtypes = [P, P, P, P, P, P, P, P, C.c_int32, P]
        L.orc_gbuffer.argtypes = [P, P, P, P, P, P]
        for f in ("orc_trace", "orc_trace_f32"):
            getattr(L, f).argtypes = [P, P, P, P, P, P, P, P, C.c_int32, P]
        L.orc_trace_stats.argtypes = [P, P, P, P, P, P, P, P, C.c_int32, P, P]
        L.orc_texture_lod.argtypes = [P, P, P, C.c_int32, P, C.c_double, P]
        L.orc_trace_cone.argtypes = [P, P, P, P, P, C.c_double, C.c_double, P, P]
        L.orc_time_frame.argtypes = [P, P, C.c_int32, P]
        L.orc_mlp_level_res.restype = C.c_int32
        L.orc_mlp_level_res.argtypes = [P, C.c_int32]
        L.orc_mlp_forward.argtypes = [P, P, P, C.c_int32, P, P, P, P]
        L.orc_mlp_grad.restype = C.c_double
        L.orc_mlp_grad.argtypes = [P, P, P, C.c_int32, P, P, P, P, P, P]
        _lib = L
    return _lib


def levels_for(n: int) -> int:
    return min(7, int(np.log2(n)) + 1)


def chain_texels(n: int, levels: int) -> int:
    return int(lib().orc_chain_texels(n, levels))


class Params:
    """Oracle parameters; field names follow the renderer's settings."""

    def __init__(self, grid_res=64, width=64, height=64, vox_mode=VOX_REF_RASTER2X, mip_mode=MIP_ANISO,
                 enable_direct=True, enable_diffuse=True, enable_specular=True, enable_shadow=True,
                 view_voxel_dir=7, view_voxel_lod=0.0, cone_set=CONES_REF9, threads=None, levels=None,
                 radiance_max=1.0, far_share=0):
        self.grid_res, self.width, self.height = grid_res, width, height
        self.levels = levels if levels is not None else levels_for(grid_res)
        self.vox_mode, self.mip_mode = vox_mode, mip_mode
        self.enable_direct, self.enable_diffuse = enable_direct, enable_diffuse
        self.enable_specular, self.enable_shadow = enable_specular, enable_shadow
        self.view_voxel_dir, self.view_voxel_lod = view_voxel_dir, view_voxel_lod
        self.cone_set = cone_set
        self.threads = threads if threads else (os.cpu_count() or 1)
        self.radiance_max = radiance_max
        self.far_share = far_share

    def c(self) -> _Params:
        p = _Params()
        for name, _ in _Params._fields_:
            setattr(p, name, type(getattr(p, name))(getattr(self, name)))
        return p

    @property
    def n_maps(self) -> int:
        return 1 if self.mip_mode == MIP_ISO else 6


class _SceneHold:
    """Keeps the numpy buffers of a ctypes scene alive."""

    def __init__(self, scene):
        self.keep = []
        n = len(scene.meshes)
        insts = (_Instance * max(n, 1))()
        for k, (mesh, model) in enumerate(zip(scene.meshes, scene.models)):
            v = np.ascontiguousarray(mesh.verts, np.float32)
            ix = np.ascontiguousarray(mesh.indices, np.uint32)
            tm = np.ascontiguousarray(mesh.tri_material(), np.uint32)
            self.keep += [v, ix, tm]
            insts[k].verts, insts[k].indices, insts[k].tri_material = v.ctypes.data, ix.ctypes.data, tm.ctypes.data
            insts[k].n_verts, insts[k].n_tris = v.shape[0], ix.shape[0]
            insts[k].model[:] = [float(x) for x in np.asarray(model, np.float32)]
        mats = np.ascontiguousarray(scene.materials)
        lights = np.ascontiguousarray(scene.lights)
        self.keep += [insts, mats, lights]
        s = _Scene()
        s.instances = C.addressof(insts)
        s.materials, s.lights = mats.ctypes.data, lights.ctypes.data
        s.n_instances, s.n_materials, s.n_lights = n, mats.shape[0], lights.shape[0]
        s.cube_size = float(scene.cube_size)
        s.view[:] = [float(x) for x in scene.view]
        s.proj[:] = [float(x) for x in scene.proj]
        self.s = s

    @property
    def ptr(self):
        return C.addressof(self.s)


def _ptr(a):
    return a.ctypes.data if a is not None else None


def voxelize(scene, params: Params, fp32: bool = False):
    """-> (level0 uint8 (N,N,N,4) indexed [z,y,x], counts uint32 (N,N,N), rejected)."""
    n = params.grid_res
    l0 = np.zeros((n, n, n, 4), np.uint8)
    cnt = np.zeros((n, n, n), np.uint32)
    sh, pc = _SceneHold(scene), params.c()
    f = lib().orc_voxelize_f32 if fp32 else lib().orc_voxelize
    rej = f(sh.ptr, C.addressof(pc), _ptr(l0), _ptr(cnt))
    return l0, cnt, int(rej)


ORDER_DRAW, ORDER_REVERSE, ORDER_SHUFFLED = 0, 1, 2


def voxelize_cas(scene, params: Params, order: int = ORDER_DRAW, seed: int = 0):
    """Informational: level 0 as the reference's running average
    (imageAtomicRGBA8Avg, voxelize.frag:62-119) leaves it for one arrival
    order of the contributions -> uint8 (N,N,N,4) [z,y,x], low bits = count."""
    n = params.grid_res
    l0 = np.zeros((n, n, n, 4), np.uint8)
    sh, pc = _SceneHold(scene), params.c()
    lib().orc_voxelize_cas(sh.ptr, C.addressof(pc), int(order), int(seed), _ptr(l0))
    return l0


def cas_avg(rgba) -> int:
    """The running average of a sequence of RGBA contributions arriving at a
    cleared voxel; returns the stored 32-bit word (R in the low byte)."""
    a = np.ascontiguousarray(np.asarray(rgba, np.float32).reshape(-1, 4))
    return int(lib().orc_cas_avg(a.ctypes.data, a.shape[0]))


def voxelize_hdr(scene, params: Params):
    """FP64 voxelize keeping the unrounded mean (HDR storage):
    -> (level0 float32 (N,N,N,4) [z,y,x], counts, rejected)."""
    n = params.grid_res
    l0 = np.zeros((n, n, n, 4), np.float32)
    cnt = np.zeros((n, n, n), np.uint32)
    sh, pc = _SceneHold(scene), params.c()
    rej = lib().orc_voxelize_hdr(sh.ptr, C.addressof(pc), _ptr(l0), _ptr(cnt))
    return l0, cnt, int(rej)


def voxelize_attr(scene, params: Params):
    """Light-injection attribute grids: -> dict(albedo, normal, emission:
    uint8 (N,N,N,4) [z,y,x], counts, rejected)."""
    n = params.grid_res
    g = {k: np.zeros((n, n, n, 4), np.uint8) for k in ("albedo", "normal", "emission")}
    cnt = np.zeros((n, n, n), np.uint32)
    sh, pc = _SceneHold(scene), params.c()
    rej = lib().orc_voxelize_attr(sh.ptr, C.addressof(pc), _ptr(g["albedo"]), _ptr(g["normal"]), _ptr(g["emission"]),
                                  _ptr(cnt))
    return dict(g, counts=cnt, rejected=int(rej))


def inject(scene, params: Params, grids: dict) -> np.ndarray:
    """Level 0 (N,N,N,4) uint8 lit from the attribute grids and the scene's lights."""
    n = params.grid_res
    out = np.zeros((n, n, n, 4), np.uint8)
    sh, pc = _SceneHold(scene), params.c()
    a, nm, e = (np.ascontiguousarray(grids[k], np.uint8) for k in ("albedo", "normal", "emission"))
    lib().orc_inject(sh.ptr, C.addressof(pc), _ptr(a), _ptr(nm), _ptr(e), _ptr(out))
    return out


def mip_level_f(src: np.ndarray, mip_mode: int) -> np.ndarray:
    """One FP64 mip level from float texels.  src: (s,s,s,4) (the shared
    level 0) or (6,s,s,s,4); -> (n_maps, s/2, s/2, s/2, 4) float32."""
    src = np.ascontiguousarray(src, np.float32)
    maps = 1 if src.ndim == 4 else src.shape[0]
    n = src.shape[-2]
    out = np.zeros((1 if mip_mode == MIP_ISO else 6, n // 2, n // 2, n // 2, 4), np.float32)
    lib().orc_mip_level_f(n, maps, _ptr(src), int(mip_mode), _ptr(out))
    return out


def trace_hdr(scene, params: Params, level0, chains, gb: dict, row_stride: int = 1):
    """FP64 trace over float maps: level0 (N,N,N,4), chains (n_maps,
    chain_texels, 4) float32.  -> float32 frame (H, W, 4)."""
    w, h = params.width, params.height
    out = np.zeros((h, w, 4), np.float32)
    sh, pc = _SceneHold(scene), params.c()
    l0 = np.ascontiguousarray(level0, np.float32)
    ch = np.ascontiguousarray(chains, np.float32)
    tid = np.ascontiguousarray(gb["tri_id"], np.uint32)
    pos = np.ascontiguousarray(gb["pos"], np.float64)
    nrm = np.ascontiguousarray(gb["nrm"], np.float64)
    mat = np.ascontiguousarray(gb["mat"], np.uint32)
    lib().orc_trace_hdr(sh.ptr, C.addressof(pc), _ptr(l0), _ptr(ch), _ptr(tid), _ptr(pos), _ptr(nrm), _ptr(mat),
                        int(row_stride), _ptr(out))
    return out


def mipmap(params: Params, level0: np.ndarray) -> np.ndarray:
    """-> chains uint8 (n_maps, chain_texels, 4)."""
    l0 = np.ascontiguousarray(level0, np.uint8)
    ch = np.zeros((params.n_maps, chain_texels(params.grid_res, params.levels), 4), np.uint8)
    pc = params.c()
    lib().orc_mipmap(C.addressof(pc), _ptr(l0), _ptr(ch))
    return ch


def chain_level(chains: np.ndarray, n: int, level: int, map_index: int = 0) -> np.ndarray:
    """View of one level (>= 1) of one map as (s, s, s, 4) indexed [z,y,x]."""
    off = 0
    for k in range(1, level):
        off += (n >> k) ** 3
    s = n >> level
    return chains[map_index, off:off + s ** 3].reshape(s, s, s, 4)


def gbuffer(scene, params: Params) -> dict:
    w, h = params.width, params.height
    out = dict(tri_id=np.zeros((h, w), np.uint32), pos=np.zeros((h, w, 3)), nrm=np.zeros((h, w, 3)),
               mat=np.zeros((h, w), np.uint32))
    sh, pc = _SceneHold(scene), params.c()
    lib().orc_gbuffer(sh.ptr, C.addressof(pc), _ptr(out["tri_id"]), _ptr(out["pos"]), _ptr(out["nrm"]),
                      _ptr(out["mat"]))
    return out


def trace(scene, params: Params, level0, chains, gb: dict, row_stride: int = 1, fp32: bool = False):
    """-> float32 frame (H, W, 4), row 0 = bottom.  Untraced rows stay 0."""
    w, h = params.width, params.height
    out = np.zeros((h, w, 4), np.float32)
    sh, pc = _SceneHold(scene), params.c()
    l0 = np.ascontiguousarray(level0, np.uint8)
    ch = np.ascontiguousarray(chains, np.uint8)
    tid = np.ascontiguousarray(gb["tri_id"], np.uint32)
    pos = np.ascontiguousarray(gb["pos"], np.float64)
    nrm = np.ascontiguousarray(gb["nrm"], np.float64)
    mat = np.ascontiguousarray(gb["mat"], np.uint32)
    f = lib().orc_trace_f32 if fp32 else lib().orc_trace
    f(sh.ptr, C.addressof(pc), _ptr(l0), _ptr(ch), _ptr(tid), _ptr(pos), _ptr(nrm), _ptr(mat),
      int(row_stride), _ptr(out))
    return out


def trace_stats(scene, params: Params, level0, chains, gb: dict, row_stride: int = 1) -> dict:
    """Instrumented FP64 trace: cones, march steps, lod<1 steps, steps
    beyond the grid (taken by the reference's loop, skipped by the engine's
    exact early exit) and the other steps the engine's occupancy rule finds
    empty (no fetch; `empty_lt1` of them with lod < 1) per cone class over
    the traced rows, and the single-level / two-level texture fetches the
    engine's texture-unit path issues for the remaining steps (`fetch_tri`,
    `fetch_quad`: the algorithmic texture work of the trace).  A negative
    row_stride samples pairs of rows (whole W x 2 groups, for far_share)."""
    w, h = params.width, params.height
    out = np.zeros((h, w, 4), np.float32)
    st = np.zeros(40, np.uint64)
    sh, pc = _SceneHold(scene), params.c()
    args = [np.ascontiguousarray(level0, np.uint8), np.ascontiguousarray(chains, np.uint8),
            np.ascontiguousarray(gb["tri_id"], np.uint32), np.ascontiguousarray(gb["pos"], np.float64),
            np.ascontiguousarray(gb["nrm"], np.float64), np.ascontiguousarray(gb["mat"], np.uint32)]
    lib().orc_trace_stats(sh.ptr, C.addressof(pc), *[_ptr(a) for a in args], int(row_stride), _ptr(out), _ptr(st))
    names = ["diffuse", "specular", "shadow", "refraction"]
    res = {n: dict(cones=int(st[i]), steps=int(st[4 + i]), lod_lt1=int(st[8 + i]), beyond=int(st[20 + i]),
                   empty=int(st[24 + i]), empty_lt1=int(st[28 + i]), fetch_tri=int(st[32 + i]),
                   fetch_quad=int(st[36 + i])) for i, n in enumerate(names)}
    res["lod_bands"] = [int(v) for v in st[12:20]]  # all classes: lod in [k, k+1), last = lod >= 7
    return res


def render(scene, params: Params):
    """Whole frame through the oracle: returns dict with every stage."""
    l0, cnt, rej = voxelize(scene, params)
    ch = mipmap(params, l0)
    gb = gbuffer(scene, params)
    frame = trace(scene, params, l0, ch, gb)
    return dict(level0=l0, counts=cnt, rejected=rej, chains=ch, gbuffer=gb, frame=frame)


def texture_lod(params: Params, level0, chains, map_index: int, u, lod: float) -> np.ndarray:
    out = np.zeros(4)
    uu = np.asarray(u, np.float64)
    pc = params.c()
    lib().orc_texture_lod(C.addressof(pc), _ptr(np.ascontiguousarray(level0, np.uint8)),
                          _ptr(np.ascontiguousarray(chains, np.uint8)), map_index, _ptr(uu), float(lod),
                          _ptr(out))
    return out


def trace_cone(params: Params, level0, chains, origin, direction, aperture, max_dist):
    out = np.zeros(4)
    steps = C.c_int32(0)
    o = np.asarray(origin, np.float64)
    d = np.asarray(direction, np.float64)
    pc = params.c()
    lib().orc_trace_cone(C.addressof(pc), _ptr(np.ascontiguousarray(level0, np.uint8)),
                         _ptr(np.ascontiguousarray(chains, np.uint8)), _ptr(o), _ptr(d), float(aperture),
                         float(max_dist), _ptr(out), C.addressof(steps))
    return out, steps.value


def time_frame(scene, params: Params, row_stride: int) -> np.ndarray:
    """Timed FP32 CPU restatement: ms for voxelize, mip, gbuffer, trace (the
    trace over rows y % row_stride == 0 only)."""
    ms = np.zeros(4)
    sh, pc = _SceneHold(scene), params.c()
    lib().orc_time_frame(sh.ptr, C.addressof(pc), int(row_stride), _ptr(ms))
    return ms


# ------------------------------------------------------------ learned term --
class MLPConfig(C.Structure):
    _fields_ = [("levels", C.c_int32), ("log2_table", C.c_int32), ("n_min", C.c_int32), ("n_max", C.c_int32)]


def mlp_config(levels=16, log2_table=19, n_min=16, n_max=512) -> MLPConfig:
    return MLPConfig(levels, log2_table, n_min, n_max)


def mlp_level_res(cfg: MLPConfig, level: int) -> int:
    return int(lib().orc_mlp_level_res(C.byref(cfg), int(level)))


def mlp_forward(cfg: MLPConfig, table, weights, pos, nrm, alb) -> np.ndarray:
    pos, nrm, alb = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (pos, nrm, alb))
    t = np.ascontiguousarray(table, np.float32)
    w = np.ascontiguousarray(weights, np.float32)
    out = np.zeros((pos.shape[0], 3), np.float32)
    lib().orc_mlp_forward(C.byref(cfg), _ptr(t), _ptr(w), pos.shape[0], _ptr(pos), _ptr(nrm), _ptr(alb), _ptr(out))
    return out


def mlp_grad(cfg: MLPConfig, table, weights, pos, nrm, alb, target, want_table=True):
    """-> (loss, dW (5,64,64) float64, dtable (levels, T, 2) float64 or None)."""
    pos, nrm, alb, tg = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (pos, nrm, alb, target))
    t = np.ascontiguousarray(table, np.float32)
    w = np.ascontiguousarray(weights, np.float32)
    dW = np.zeros((5, 64, 64))
    dt = np.zeros((cfg.levels, 1 << cfg.log2_table, 2)) if want_table else None
    loss = lib().orc_mlp_grad(C.byref(cfg), _ptr(t), _ptr(w), pos.shape[0], _ptr(pos), _ptr(nrm), _ptr(alb),
                              _ptr(tg), _ptr(dW), _ptr(dt) if dt is not None else None)
    return float(loss), dW, dt
