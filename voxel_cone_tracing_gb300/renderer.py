"""Python mirror of the reference's ``Renderer`` / Texture3D interface over the
C ABI of include/vct.h (libvct.so, built by ``build.py``).

Method names, argument meaning and error behaviour follow src/renderer.h
:122-196 and src/texture_3d.h:6-10: ``load_model`` returns ``INVALID_ID`` on
failure, ``queue_model`` ignores unknown ids; every other failure of the C
ABI raises :class:`VCTError` with the library's message.  There is no CPU
fallback: without the CUDA library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import scenes

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvct.so")

INVALID_ID = (1 << 64) - 1
VOX_REF_RASTER2X, VOX_CONSERVATIVE = 0, 1
MIP_ANISO, MIP_ISO, MIP_BOTH = 0, 1, 2
STORAGE_RGBA8, STORAGE_RGBA16F = 0, 1
SAMPLER_HW, SAMPLER_EXACT = 0, 1
CONES_REF9, CONES_SIX60 = 0, 1
FRAME_RGBA8, FRAME_RGBA32F = 0, 1

# Every entry point include/vct.h declares (the export test checks them).
EXPORTS = [
    "vct_last_error", "vct_status_string", "vct_config_default", "vct_renderer_create", "vct_renderer_destroy",
    "vct_load_mesh", "vct_load_model", "vct_load_shader", "vct_add_material", "vct_upload_material_data",
    "vct_set_model_material", "vct_get_model_dimensions", "vct_get_material", "vct_set_grid_resolution",
    "vct_set_grid_size", "vct_set_camera_transform", "vct_set_model_transform", "vct_set_rendering_phases",
    "vct_set_voxel_view_dir", "vct_queue_model", "vct_queue_point_light", "vct_render", "vct_set_stream",
    "vct_synchronize", "vct_get_stage_times", "vct_read_frame", "vct_frame_device_ptr", "vct_read_voxels",
    "vct_read_voxel_counts", "vct_read_gbuffer", "vct_get_grid", "vct_create_tex_3d", "vct_destroy_tex_3d",
    "vct_activate_tex_3d", "vct_clear_tex_3d", "vct_mip_tex_3d", "vct_tex3d_upload", "vct_tex3d_download",
    "vct_mlp_desc_default", "vct_mlp_init", "vct_mlp_train", "vct_set_diffuse_mode", "vct_mlp_save",
    "vct_mlp_load", "vct_mlp_get_params", "vct_mlp_set_params", "vct_mlp_eval", "vct_mlp_gradients",
    "vct_mlp_train_samples", "vct_voxelize_noalloc", "vct_batch_create", "vct_batch_destroy",
    "vct_batch_set_camera", "vct_batch_render", "vct_batch_synchronize", "vct_batch_set_stream",
    "vct_batch_read_frame", "vct_batch_read_voxels", "vct_batch_stage_times", "vct_batch_get_shape",
    "vct_batch_set_shape", "vct_batch_autotune", "vct_set_light_injection", "vct_read_injection_grids",
    "vct_mlp_set_tensor_kernels", "vct_measure_texture_rate", "vct_mlp_set_judge", "vct_mlp_get_judge",
    "vct_batch_config_default",
]
DIFFUSE_CONES, DIFFUSE_MLP = 0, 1
# vct_config.far_share = 1 shares the diffuse cones' far fields within groups
# of FAR_SHARE_GROUP_W x 2 pixels (k_trace.cu kShareW).
FAR_SHARE_GROUP_W = 4
MLP_WEIGHTS = 5 * 64 * 64


class MLPDesc(C.Structure):
    _fields_ = [("levels", C.c_int32), ("log2_table", C.c_int32), ("n_min", C.c_int32), ("n_max", C.c_int32),
                ("n_samples", C.c_uint32), ("batch", C.c_uint32), ("steps", C.c_uint32), ("lr", C.c_float),
                ("seed", C.c_uint64), ("reserved", C.c_uint32 * 8)]


class MLPReport(C.Structure):
    _fields_ = [("loss_first", C.c_float), ("loss_last", C.c_float), ("ms_samples", C.c_float),
                ("ms_train", C.c_float), ("steps", C.c_uint32), ("n_samples", C.c_uint32)]


class JudgeReport(C.Structure):
    _fields_ = [("last_psnr_db", C.c_float), ("judged_pixels", C.c_uint32), ("fallbacks", C.c_uint32),
                ("diffuse_mode", C.c_int32), ("stride", C.c_int32), ("min_psnr_db", C.c_float),
                ("reserved", C.c_uint32 * 4)]


def mlp_desc(**kw) -> MLPDesc:
    d = MLPDesc()
    lib().vct_mlp_desc_default(C.byref(d))
    for k, v in kw.items():
        setattr(d, k, type(getattr(d, k))(v))
    return d


class VCTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"vct status {status}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("grid_res", C.c_int32), ("vox_mode", C.c_int32), ("mip_mode", C.c_int32),
                ("storage", C.c_int32), ("sampler", C.c_int32), ("cone_set", C.c_int32),
                ("keep_counts", C.c_int32), ("keep_float_frame", C.c_int32), ("radiance_max", C.c_float),
                ("shadow_from_maps", C.c_int32), ("full_march", C.c_int32),
                ("overlap_raster", C.c_int32), ("far_share", C.c_int32), ("trace_tile_rows", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class StageTimes(C.Structure):
    _fields_ = [("voxelize", C.c_float), ("mipmap", C.c_float), ("gbuffer", C.c_float), ("trace", C.c_float),
                ("total", C.c_float), ("kernel_launches", C.c_uint32), ("voxelized", C.c_uint32),
                ("split_bricks", C.c_uint32), ("infer", C.c_float)]


class DrawObj(C.Structure):
    _fields_ = [("first_index", C.c_uint32), ("index_count", C.c_uint32), ("material_id", C.c_uint32)]


_lib = None


def lib() -> C.CDLL:
    """Load libvct.so (raises if it was not built: no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run voxel_cone_tracing_gb300/build.py "
                              "(the engine has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        P, U32, I32, U64, F = C.c_void_p, C.c_uint32, C.c_int32, C.c_uint64, C.c_float
        sig = {
            "vct_last_error": (C.c_char_p, []), "vct_status_string": (C.c_char_p, [I32]),
            "vct_config_default": (None, [P]), "vct_renderer_create": (I32, [I32, I32, P, P]),
            "vct_renderer_destroy": (None, [P]),
            "vct_load_mesh": (I32, [P, P, U32, P, U32, P, U32, P]), "vct_load_model": (U64, [P, C.c_char_p]),
            "vct_load_shader": (U64, [P, C.c_char_p, C.c_char_p, C.c_char_p]), "vct_add_material": (U64, [P, P]),
            "vct_upload_material_data": (I32, [P, P, U64]), "vct_set_model_material": (I32, [P, U64, U64]),
            "vct_get_model_dimensions": (I32, [P, U64, P]), "vct_get_material": (I32, [P, U64, P]),
            "vct_set_grid_resolution": (I32, [P, U32]), "vct_set_grid_size": (I32, [P, F]),
            "vct_set_camera_transform": (I32, [P, P, P]), "vct_set_model_transform": (I32, [P, U64, P]),
            "vct_set_rendering_phases": (I32, [P, I32, I32, I32, I32]),
            "vct_set_voxel_view_dir": (I32, [P, I32, F]), "vct_queue_model": (I32, [P, U64]),
            "vct_queue_point_light": (I32, [P, P]), "vct_render": (I32, [P]), "vct_set_stream": (I32, [P, P]),
            "vct_synchronize": (I32, [P]), "vct_get_stage_times": (I32, [P, P]),
            "vct_read_frame": (I32, [P, P, I32]), "vct_frame_device_ptr": (I32, [P, P]),
            "vct_read_voxels": (I32, [P, I32, I32, P]), "vct_read_voxel_counts": (I32, [P, P]),
            "vct_read_gbuffer": (I32, [P, P, P, P, P]), "vct_get_grid": (I32, [P, P, P]),
            "vct_create_tex_3d": (U32, [I32, I32, I32, I32]), "vct_destroy_tex_3d": (None, [U32]),
            "vct_activate_tex_3d": (I32, [U32, U32, U32]), "vct_clear_tex_3d": (I32, [U32, P]),
            "vct_mip_tex_3d": (I32, [U32]), "vct_tex3d_upload": (I32, [U32, I32, P]),
            "vct_tex3d_download": (I32, [U32, I32, P]),
            "vct_mlp_desc_default": (None, [P]), "vct_mlp_init": (I32, [P, P]), "vct_mlp_train": (I32, [P, P, P]),
            "vct_set_diffuse_mode": (I32, [P, I32]), "vct_mlp_save": (I32, [P, C.c_char_p]),
            "vct_mlp_load": (I32, [P, C.c_char_p]), "vct_mlp_get_params": (I32, [P, P, P]),
            "vct_mlp_set_params": (I32, [P, P, P]), "vct_mlp_eval": (I32, [P, P, U32, P]),
            "vct_mlp_gradients": (I32, [P, P, U32, P, P, P]), "vct_mlp_train_samples": (I32, [P, P, U32, P, P]),
            "vct_voxelize_noalloc": (I32, [P, U32, P, U32, P, U32, F, I32, I32, P, P]),
            "vct_batch_create": (I32, [P, U32, P, P]), "vct_batch_destroy": (None, [P]),
            "vct_batch_set_camera": (I32, [P, U32, P, P]), "vct_batch_render": (I32, [P]),
            "vct_batch_synchronize": (I32, [P]), "vct_batch_set_stream": (I32, [P, P]),
            "vct_batch_read_frame": (I32, [P, U32, P]), "vct_batch_read_voxels": (I32, [P, U32, I32, I32, P]),
            "vct_batch_stage_times": (I32, [P, P]), "vct_batch_get_shape": (I32, [P, P]),
            "vct_batch_set_shape": (I32, [P, P]), "vct_batch_autotune": (I32, [P, I32, P, P, P]),
            "vct_set_light_injection": (I32, [P, I32]), "vct_read_injection_grids": (I32, [P, P, P, P]),
            "vct_mlp_set_tensor_kernels": (I32, [P, I32]), "vct_measure_texture_rate": (I32, [I32, U32, P, P]),
            "vct_mlp_set_judge": (I32, [P, I32, F]), "vct_mlp_get_judge": (I32, [P, P]),
            "vct_batch_config_default": (None, [P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().vct_last_error().decode()


def _check(status: int) -> None:
    if status != 0:
        raise VCTError(status, last_error())


def _f16(m) -> C.Array:
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    return (C.c_float * 16)(*a.tolist())


def default_config(**kw) -> Config:
    c = Config()
    lib().vct_config_default(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, float(v) if k == "radiance_max" else int(v))
    return c


class Renderer:
    """``struct Renderer`` (src/renderer.h:122-196) on the GB300 engine."""

    def __init__(self, width: int, height: int, config: Config | None = None, **kw):
        self._r = C.c_void_p()
        cfg = config if config is not None else default_config(**kw)
        _check(lib().vct_renderer_create(int(width), int(height), C.byref(cfg), C.byref(self._r)))
        self.width, self.height, self.config = int(width), int(height), cfg

    def close(self) -> None:
        if self._r:
            lib().vct_renderer_destroy(self._r)
            self._r = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- resources -------------------------------------------------------
    def load_model(self, filename: str) -> int:
        return int(lib().vct_load_model(self._r, filename.encode()))

    def load_mesh(self, verts: np.ndarray, indices: np.ndarray, draw_objs) -> int:
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 8)
        ix = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        objs = np.ascontiguousarray(draw_objs, scenes.DRAWOBJ_DTYPE)
        out = C.c_uint64(INVALID_ID)
        _check(lib().vct_load_mesh(self._r, v.ctypes.data, v.shape[0], ix.ctypes.data, ix.size,
                                   objs.ctypes.data, objs.shape[0], C.byref(out)))
        return int(out.value)

    def load_shader(self, vertex_shader_name, fragment_shader_name, geometry_shader_name=None) -> int:
        enc = lambda s: s.encode() if s else None  # noqa: E731
        return int(lib().vct_load_shader(self._r, enc(vertex_shader_name), enc(fragment_shader_name),
                                         enc(geometry_shader_name)))

    def add_material(self, material_data: np.ndarray) -> int:
        m = np.ascontiguousarray(np.asarray(material_data, scenes.MATERIAL_DTYPE).reshape(()))
        mid = int(lib().vct_add_material(self._r, m.ctypes.data))
        if mid == INVALID_ID:
            raise VCTError(1, last_error())
        return mid

    def upload_material_data(self, material_data: np.ndarray, material_id: int) -> None:
        m = np.ascontiguousarray(np.asarray(material_data, scenes.MATERIAL_DTYPE).reshape(()))
        _check(lib().vct_upload_material_data(self._r, m.ctypes.data, int(material_id)))

    def set_model_material(self, material_id: int, model_id: int) -> None:
        _check(lib().vct_set_model_material(self._r, int(material_id), int(model_id)))

    def get_model_dimensions(self, model: int) -> np.ndarray:
        out = np.zeros(3, np.float32)
        _check(lib().vct_get_model_dimensions(self._r, int(model), out.ctypes.data))
        return out

    def get_material(self, material_id: int) -> np.ndarray:
        out = np.zeros((), scenes.MATERIAL_DTYPE)
        _check(lib().vct_get_material(self._r, int(material_id), out.ctypes.data))
        return out

    # ---- settings --------------------------------------------------------
    def set_grid_resolution(self, res: int) -> None:
        _check(lib().vct_set_grid_resolution(self._r, int(res)))

    def set_grid_size(self, size: float) -> None:
        _check(lib().vct_set_grid_size(self._r, float(size)))

    def set_camera_transform(self, lookat, projection) -> None:
        _check(lib().vct_set_camera_transform(self._r, _f16(lookat), _f16(projection)))

    def set_model_transform(self, model_id: int, model_matrix) -> None:
        _check(lib().vct_set_model_transform(self._r, int(model_id), _f16(model_matrix)))

    def set_rendering_phases(self, direct: bool, diffuse: bool, specular: bool, shadow: bool) -> None:
        _check(lib().vct_set_rendering_phases(self._r, int(direct), int(diffuse), int(specular), int(shadow)))

    def set_voxel_view_dir(self, direction: int, lod: float) -> None:
        _check(lib().vct_set_voxel_view_dir(self._r, int(direction), float(lod)))

    # ---- frame -----------------------------------------------------------
    def queue_model(self, model_id: int) -> None:
        _check(lib().vct_queue_model(self._r, int(model_id)))

    def queue_point_light(self, point_light: np.ndarray) -> None:
        l = np.ascontiguousarray(np.asarray(point_light, scenes.LIGHT_DTYPE).reshape(()))
        _check(lib().vct_queue_point_light(self._r, l.ctypes.data))

    def render(self) -> None:
        _check(lib().vct_render(self._r))

    # ---- streams, timing, read-back -------------------------------------
    def set_stream(self, stream_handle: int | None) -> None:
        _check(lib().vct_set_stream(self._r, C.c_void_p(stream_handle or 0)))

    def synchronize(self) -> None:
        _check(lib().vct_synchronize(self._r))

    def stage_times(self) -> dict:
        t = StageTimes()
        _check(lib().vct_get_stage_times(self._r, C.byref(t)))
        d = {k: float(getattr(t, k)) for k, _ in StageTimes._fields_}
        d["kernel_launches"] = int(t.kernel_launches)
        d["voxelized"] = bool(t.voxelized)
        d["split_bricks"] = int(t.split_bricks)
        return d

    def read_frame(self, fmt: int = FRAME_RGBA8, out: np.ndarray | None = None) -> np.ndarray:
        """(H, W, 4) uint8 or float32, row 0 = bottom."""
        dt = np.uint8 if fmt == FRAME_RGBA8 else np.float32
        if out is None:
            out = np.empty((self.height, self.width, 4), dt)
        _check(lib().vct_read_frame(self._r, out.ctypes.data, int(fmt)))
        return out

    def frame_device_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().vct_frame_device_ptr(self._r, C.byref(p)))
        return int(p.value or 0)

    def grid(self):
        n, l = C.c_int32(), C.c_int32()
        _check(lib().vct_get_grid(self._r, C.byref(n), C.byref(l)))
        return n.value, l.value

    def read_voxels(self, level: int, map_index: int = 0) -> np.ndarray:
        """(s, s, s, 4) indexed [z, y, x]: uint8 (RGBA8) or float16 (RGBA16F)."""
        n, _ = self.grid()
        s = n >> level
        dt = np.float16 if self.config.storage == STORAGE_RGBA16F else np.uint8
        out = np.empty((s, s, s, 4), dt)
        _check(lib().vct_read_voxels(self._r, int(level), int(map_index), out.ctypes.data))
        return out

    def read_voxel_counts(self) -> np.ndarray:
        n, _ = self.grid()
        out = np.empty((n, n, n), np.uint32)
        _check(lib().vct_read_voxel_counts(self._r, out.ctypes.data))
        return out

    # ---- learned diffuse term (engine extension) -------------------------
    def mlp_init(self, desc: MLPDesc | None = None) -> None:
        _check(lib().vct_mlp_init(self._r, C.byref(desc) if desc is not None else None))

    def mlp_train(self, desc: MLPDesc | None = None) -> dict:
        rep = MLPReport()
        _check(lib().vct_mlp_train(self._r, C.byref(desc) if desc is not None else None, C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in MLPReport._fields_}

    def mlp_train_samples(self, samples: np.ndarray, desc: MLPDesc | None = None) -> dict:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 12)
        rep = MLPReport()
        _check(lib().vct_mlp_train_samples(self._r, s.ctypes.data, s.shape[0],
                                           C.byref(desc) if desc is not None else None, C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in MLPReport._fields_}

    def set_diffuse_mode(self, mode: int) -> None:
        _check(lib().vct_set_diffuse_mode(self._r, int(mode)))

    def mlp_save(self, path: str) -> None:
        _check(lib().vct_mlp_save(self._r, path.encode()))

    def mlp_load(self, path: str) -> None:
        _check(lib().vct_mlp_load(self._r, path.encode()))

    def mlp_get_params(self, levels=16, log2_table=19):
        t = np.empty((levels, 1 << log2_table, 2), np.float32)
        w = np.empty((5, 64, 64), np.float32)
        _check(lib().vct_mlp_get_params(self._r, t.ctypes.data, w.ctypes.data))
        return t, w

    def mlp_set_params(self, table: np.ndarray, weights: np.ndarray) -> None:
        t = np.ascontiguousarray(table, np.float32)
        w = np.ascontiguousarray(weights, np.float32)
        _check(lib().vct_mlp_set_params(self._r, t.ctypes.data, w.ctypes.data))

    def mlp_eval(self, samples: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 12)
        out = np.empty((s.shape[0], 3), np.float32)
        _check(lib().vct_mlp_eval(self._r, s.ctypes.data, s.shape[0], out.ctypes.data))
        return out

    def mlp_gradients(self, samples: np.ndarray, levels=16, log2_table=19):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 12)
        loss = np.zeros(1, np.float32)
        dw = np.empty((5, 64, 64), np.float32)
        dt = np.empty((levels, 1 << log2_table, 2), np.float32)
        _check(lib().vct_mlp_gradients(self._r, s.ctypes.data, s.shape[0], loss.ctypes.data, dw.ctypes.data,
                                       dt.ctypes.data))
        return float(loss[0]), dw, dt

    def set_mlp_judge(self, stride: int, min_psnr_db: float = 40.0) -> None:
        """vct_mlp_set_judge: cone-traced check of the learned term at one
        pixel per stride x stride tile (0 = off)."""
        _check(lib().vct_mlp_set_judge(self._r, int(stride), float(min_psnr_db)))

    def mlp_judge(self) -> dict:
        rep = JudgeReport()
        _check(lib().vct_mlp_get_judge(self._r, C.addressof(rep)))
        return {k: getattr(rep, k) for k, _ in JudgeReport._fields_ if k != "reserved"}

    def mlp_set_tensor_kernels(self, use_tcgen05: bool) -> None:
        _check(lib().vct_mlp_set_tensor_kernels(self._r, int(bool(use_tcgen05))))

    def set_light_injection(self, enable: bool) -> None:
        _check(lib().vct_set_light_injection(self._r, int(bool(enable))))

    def read_injection_grids(self) -> dict:
        """albedo / normal / emission grids, (N, N, N, 4) uint8 indexed [z, y, x]."""
        n, _ = self.grid()
        g = {k: np.empty((n, n, n, 4), np.uint8) for k in ("albedo", "normal", "emission")}
        _check(lib().vct_read_injection_grids(self._r, g["albedo"].ctypes.data, g["normal"].ctypes.data,
                                              g["emission"].ctypes.data))
        return g

    def read_gbuffer(self) -> dict:
        h, w = self.height, self.width
        g = dict(tri_id=np.empty((h, w), np.uint32), pos=np.empty((h, w, 3), np.float32),
                 nrm=np.empty((h, w, 3), np.float32), mat=np.empty((h, w), np.uint32))
        _check(lib().vct_read_gbuffer(self._r, g["tri_id"].ctypes.data, g["pos"].ctypes.data,
                                      g["nrm"].ctypes.data, g["mat"].ctypes.data))
        return g


# ------------------------------------------------ allocation-free voxelizer --
class DeviceMesh(C.Structure):
    """vct_device_mesh: device pointers of one mesh + its host model matrix."""
    _fields_ = [("verts", C.c_void_p), ("indices", C.c_void_p), ("tri_material", C.c_void_p),
                ("n_verts", C.c_uint32), ("n_tris", C.c_uint32), ("model", C.c_float * 16)]


def voxelize_noalloc(meshes, materials_ptr: int, n_materials: int, lights: np.ndarray, cube_size: float,
                     grid_res: int, vox_mode: int, out_ptr: int, stream: int = 0) -> None:
    """vct_voxelize_noalloc for callers that own all device memory: meshes is
    a list of DeviceMesh, materials_ptr / out_ptr are device addresses (the
    output holds grid_res^3 RGBA8 texels, x fastest)."""
    arr = (DeviceMesh * max(len(meshes), 1))(*meshes)
    l = np.ascontiguousarray(np.asarray(lights, scenes.LIGHT_DTYPE).reshape(-1))
    _check(lib().vct_voxelize_noalloc(C.addressof(arr), len(meshes), C.c_void_p(materials_ptr), int(n_materials),
                                      l.ctypes.data if l.size else None, l.size, float(cube_size), int(grid_res),
                                      int(vox_mode), C.c_void_p(out_ptr), C.c_void_p(stream or 0)))


def measure_texture_rate(kind: int, iters: int = 2048) -> dict:
    """vct_measure_texture_rate: 3D RGBA8 texture fetches per second of the
    current device (kind 0: two-level, 1: level-0 trilinear, 2: one level of
    a mipmapped texture)."""
    rate, ms = C.c_double(), C.c_double()
    _check(lib().vct_measure_texture_rate(int(kind), int(iters), C.addressof(rate), C.addressof(ms)))
    return {"fetches_per_s": rate.value, "ms": ms.value}


# --------------------------------------------------------------- Texture3D --
def create_tex_3d(width: int, height: int, depth: int, levels: int) -> int:
    t = int(lib().vct_create_tex_3d(int(width), int(height), int(depth), int(levels)))
    if t == 0:
        raise VCTError(1, last_error())
    return t


def destroy_tex_3d(tex: int) -> None:
    lib().vct_destroy_tex_3d(int(tex))


def activate_tex_3d(program: int, tex: int, unit: int) -> None:
    _check(lib().vct_activate_tex_3d(int(program), int(tex), int(unit)))


def clear_tex_3d(tex: int, clear_color) -> None:
    c = (C.c_float * 4)(*[float(x) for x in clear_color])
    _check(lib().vct_clear_tex_3d(int(tex), c))


def mip_tex_3d(tex: int) -> None:
    _check(lib().vct_mip_tex_3d(int(tex)))


def tex3d_upload(tex: int, level: int, data: np.ndarray) -> None:
    d = np.ascontiguousarray(data, np.uint8)
    _check(lib().vct_tex3d_upload(int(tex), int(level), d.ctypes.data))


def tex3d_download(tex: int, level: int, shape) -> np.ndarray:
    out = np.empty(tuple(shape) + (4,), np.uint8)
    _check(lib().vct_tex3d_download(int(tex), int(level), out.ctypes.data))
    return out


# ------------------------------------------------------------ scene loading --
def load_scene(r: Renderer, scene: "scenes.Scene") -> list:
    """Load a synthetic scene: materials 1.. as add_material ids, meshes with
    their draw objects, model transforms, camera and grid size.  Returns the
    model ids (queue them with :func:`queue_scene` each frame)."""
    for k in range(1, scene.materials.shape[0]):
        mid = r.add_material(scene.materials[k])
        assert mid == k, (mid, k)
    ids = []
    for mesh, model in zip(scene.meshes, scene.models):
        mid = r.load_mesh(mesh.verts, mesh.indices, mesh.draw_objs)
        r.set_model_transform(mid, model)
        ids.append(mid)
    r.set_camera_transform(scene.view, scene.proj)
    r.set_grid_size(scene.cube_size)
    return ids


def queue_scene(r: Renderer, scene: "scenes.Scene", ids) -> None:
    for mid in ids:
        r.queue_model(mid)
    for l in scene.lights:
        r.queue_point_light(l)


# ---------------------------------------------------------------- batches --
class BatchMesh(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("n_verts", C.c_uint32), ("indices", C.c_void_p), ("n_tris", C.c_uint32),
                ("tri_material", C.c_void_p), ("model", C.c_float * 16)]


class BatchScene(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("grid_res", C.c_int32), ("cone_set", C.c_int32),
                ("cube_size", C.c_float), ("meshes", C.c_void_p), ("n_meshes", C.c_uint32),
                ("materials", C.c_void_p), ("n_materials", C.c_uint32), ("lights", C.c_void_p),
                ("n_lights", C.c_uint32), ("view", C.c_float * 16), ("proj", C.c_float * 16)]


class BatchConfig(C.Structure):
    _fields_ = [("vox_mode", C.c_int32), ("use_graph", C.c_int32), ("far_share", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class BatchShape(C.Structure):
    _fields_ = [("bin_ctas_per_sm", C.c_int32), ("bricks_ctas_per_sm", C.c_int32),
                ("trace_ctas_per_sm", C.c_int32), ("trace_dynamic", C.c_int32), ("trace_per_scene", C.c_int32),
                ("trace_tile_rows", C.c_int32)]


class Batch:
    """Many independent scenes rendered per frame (vct_batch_*): each entry
    of ``items`` is (scene, width, height, grid_res, cone_set); geometry,
    materials, lights, camera and cube size come from the scene."""

    def __init__(self, items, vox_mode: int = VOX_REF_RASTER2X, use_graph: bool = False, far_share: int = 1):
        keep = []
        descs = (BatchScene * len(items))()
        self.sizes = []
        for d, (scene, w, h, grid, cones) in zip(descs, items):
            meshes = (BatchMesh * max(len(scene.meshes), 1))()
            for m, (mesh, model) in zip(meshes, zip(scene.meshes, scene.models)):
                v = np.ascontiguousarray(mesh.verts, np.float32)
                ix = np.ascontiguousarray(mesh.indices, np.uint32)
                tm = np.ascontiguousarray(mesh.tri_material(), np.uint32)
                keep += [v, ix, tm]
                m.verts, m.n_verts = v.ctypes.data, v.shape[0]
                m.indices, m.n_tris, m.tri_material = ix.ctypes.data, ix.shape[0], tm.ctypes.data
                m.model[:] = [float(x) for x in np.asarray(model, np.float32).reshape(-1)]
            mats = np.ascontiguousarray(scene.materials)
            lights = np.ascontiguousarray(scene.lights)
            keep += [meshes, mats, lights]
            d.width, d.height, d.grid_res, d.cone_set = int(w), int(h), int(grid), int(cones)
            d.cube_size = float(scene.cube_size)
            d.meshes, d.n_meshes = C.addressof(meshes), len(scene.meshes)
            d.materials, d.n_materials = mats.ctypes.data, mats.shape[0]
            d.lights, d.n_lights = (lights.ctypes.data if lights.shape[0] else None), lights.shape[0]
            d.view[:] = [float(x) for x in np.asarray(scene.view, np.float32).reshape(-1)]
            d.proj[:] = [float(x) for x in np.asarray(scene.proj, np.float32).reshape(-1)]
            self.sizes.append((int(w), int(h), int(grid)))
        cfg = BatchConfig()
        lib().vct_batch_config_default(C.byref(cfg))
        cfg.vox_mode, cfg.use_graph, cfg.far_share = int(vox_mode), int(bool(use_graph)), int(far_share)
        self._b = C.c_void_p()
        _check(lib().vct_batch_create(descs, len(items), C.byref(cfg), C.byref(self._b)))

    def close(self) -> None:
        if getattr(self, "_b", None):
            lib().vct_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self) -> None:
        _check(lib().vct_batch_render(self._b))

    def synchronize(self) -> None:
        _check(lib().vct_batch_synchronize(self._b))

    def set_stream(self, stream_handle) -> None:
        _check(lib().vct_batch_set_stream(self._b, C.c_void_p(stream_handle or 0)))

    def set_camera(self, scene: int, view, proj) -> None:
        v, p = _f16(view), _f16(proj)
        _check(lib().vct_batch_set_camera(self._b, int(scene), v, p))

    def read_frame(self, scene: int) -> np.ndarray:
        w, h, _ = self.sizes[scene]
        out = np.empty((h, w, 4), np.uint8)
        _check(lib().vct_batch_read_frame(self._b, int(scene), out.ctypes.data))
        return out

    def read_voxels(self, scene: int, level: int, map_index: int = 0) -> np.ndarray:
        s = self.sizes[scene][2] >> level
        out = np.empty((s, s, s, 4), np.uint8)
        _check(lib().vct_batch_read_voxels(self._b, int(scene), int(level), int(map_index), out.ctypes.data))
        return out

    def stage_times(self) -> dict:
        t = StageTimes()
        _check(lib().vct_batch_stage_times(self._b, C.byref(t)))
        d = {k: float(getattr(t, k)) for k, _ in StageTimes._fields_}
        d["kernel_launches"] = int(t.kernel_launches)
        d["voxelized"] = bool(t.voxelized)
        d["split_bricks"] = int(t.split_bricks)
        return d

    @property
    def shape(self) -> dict:
        s = BatchShape()
        _check(lib().vct_batch_get_shape(self._b, C.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in BatchShape._fields_}

    @shape.setter
    def shape(self, d: dict) -> None:
        s = BatchShape()
        for k, _ in BatchShape._fields_:
            setattr(s, k, int(d[k]))
        _check(lib().vct_batch_set_shape(self._b, C.byref(s)))

    def autotune(self, frames: int = 3) -> dict:
        s, before, after = BatchShape(), C.c_float(), C.c_float()
        _check(lib().vct_batch_autotune(self._b, int(frames), C.byref(s), C.byref(before), C.byref(after)))
        return {"shape": {k: int(getattr(s, k)) for k, _ in BatchShape._fields_},
                "ms_before": float(before.value), "ms_after": float(after.value)}
