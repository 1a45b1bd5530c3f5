// api_renderer.cu -- the C ABI of include/vct.h: a GB300 `Renderer` with the
// resources, settings and frame queue of src/renderer.{h,cpp}, whose frame
// runs the Voxelizer, MipBuilder, G-buffer raster and ConeTracer kernels on
// one CUDA stream.
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "renderer_state.h"

using namespace vct;

// ------------------------------------------------------------- errors -----
namespace vct {
static thread_local std::string g_error;

vct_status set_error(vct_status s, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return s;
}
void clear_error() { g_error.clear(); }
vct_status cuda_status(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear the sticky-free error state of the runtime
  vct_status s = e == cudaErrorMemoryAllocation ? VCT_ERR_OUT_OF_MEMORY
                 : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? VCT_ERR_NO_DEVICE
                                                                                 : VCT_ERR_CUDA;
  return set_error(s, "%s: %s", what, cudaGetErrorString(e));
}
vct_status ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return set_error(VCT_ERR_NO_DEVICE, "no CUDA device available (%s)",
                     e != cudaSuccess ? cudaGetErrorString(e) : "device count 0");
  }
  return VCT_OK;
}
}  // namespace vct

extern "C" const char* vct_last_error(void) { return g_error.c_str(); }

extern "C" const char* vct_status_string(vct_status s) {
  switch (s) {
    case VCT_OK: return "ok";
    case VCT_ERR_INVALID_VALUE: return "invalid value";
    case VCT_ERR_INVALID_ID: return "invalid id";
    case VCT_ERR_CUDA: return "CUDA error";
    case VCT_ERR_OUT_OF_MEMORY: return "out of memory";
    case VCT_ERR_IO: return "I/O error";
    case VCT_ERR_UNSUPPORTED: return "unsupported";
    case VCT_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}


namespace vct {
uint32_t material_count(const vct_renderer* r) { return (uint32_t)r->materials.size(); }
}  // namespace vct

// ----------------------------------------------------------- lifetime -----
extern "C" void vct_config_default(vct_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->grid_res = 128;  // set_grid_resolution(128), renderer.cpp:146
  cfg->vox_mode = VCT_VOX_REF_RASTER2X;
  cfg->mip_mode = VCT_MIP_ANISO;
  cfg->storage = VCT_STORAGE_RGBA8;
  cfg->sampler = VCT_SAMPLER_HW;
  cfg->cone_set = VCT_CONES_REF9;
  cfg->radiance_max = 1.0f;
  cfg->far_share = 1;
}

static vct_status check_config(const vct_config& c) {
  if (!is_pow2((uint32_t)c.grid_res) || c.grid_res < 8 || c.grid_res > 1024)
    return set_error(VCT_ERR_INVALID_VALUE, "grid_res %d: need a power of two in [8, 1024]", c.grid_res);
  if (!(c.radiance_max >= 0.0f && c.radiance_max <= 65504.0f))
    return set_error(VCT_ERR_INVALID_VALUE, "radiance_max %g: need 0 <= radiance_max <= 65504", c.radiance_max);
  if (c.radiance_max > 1.0f && c.storage != VCT_STORAGE_RGBA16F)
    return set_error(VCT_ERR_INVALID_VALUE, "radiance_max %g > 1 needs RGBA16F storage", c.radiance_max);
  if (c.vox_mode < 0 || c.vox_mode > 1 || c.mip_mode < 0 || c.mip_mode > 2 || c.storage < 0 || c.storage > 1 ||
      c.sampler < 0 || c.sampler > 1 || c.cone_set < 0 || c.cone_set > 1 || c.shadow_from_maps < 0 ||
      c.shadow_from_maps > 1 || c.full_march < 0 || c.full_march > 1 || c.overlap_raster < 0 || c.overlap_raster > 1 ||
      c.far_share < 0 || c.far_share > 1 ||
      (c.trace_tile_rows != 0 && c.trace_tile_rows != 8 && c.trace_tile_rows != 16 && c.trace_tile_rows != 32))
    return set_error(VCT_ERR_INVALID_VALUE, "config field out of range");
  return VCT_OK;
}

extern "C" vct_status vct_renderer_create(int32_t width, int32_t height, const vct_config* cfg, vct_renderer** out) {
  clear_error();
  if (!out) return set_error(VCT_ERR_INVALID_VALUE, "out is NULL");
  *out = nullptr;
  if (width <= 0 || height <= 0 || (int64_t)width * height > (1 << 28))
    return set_error(VCT_ERR_INVALID_VALUE, "bad viewport %dx%d", width, height);
  vct_config c;
  if (cfg) c = *cfg; else vct_config_default(&c);
  VCT_CHECK(check_config(c));
  VCT_CHECK(ensure_device());
  std::unique_ptr<vct_renderer> r(new vct_renderer());
  VCT_CHECK(r->init(width, height, &c));
  *out = r.release();
  return VCT_OK;
}

extern "C" void vct_renderer_destroy(vct_renderer* r) { delete r; }

// ---------------------------------------------------------- resources -----
extern "C" vct_status vct_load_mesh(vct_renderer* r, const vct_vert_data* verts, uint32_t n_verts,
                                    const uint32_t* indices, uint32_t n_indices, const vct_draw_obj* objs,
                                    uint32_t n_objs, vct_model_id* out) {
  clear_error();
  if (out) *out = VCT_INVALID_ID;
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer or out");
  if ((n_verts && !verts) || (n_indices && !indices) || (n_objs && !objs))
    return set_error(VCT_ERR_INVALID_VALUE, "NULL array");
  if (n_indices % 3) return set_error(VCT_ERR_INVALID_VALUE, "index count %u is not a multiple of 3", n_indices);
  for (uint32_t i = 0; i < n_indices; ++i)
    if (indices[i] >= n_verts) return set_error(VCT_ERR_INVALID_VALUE, "index %u = %u >= %u vertices", i, indices[i], n_verts);
  const uint32_t n_tris = n_indices / 3;
  std::vector<uint32_t> tri_obj(std::max<uint32_t>(n_tris, 1), 0);
  std::vector<uint8_t> covered(n_tris, 0);
  const uint32_t obj_base = (uint32_t)r->objs.size();
  for (uint32_t o = 0; o < n_objs; ++o) {
    const vct_draw_obj& d = objs[o];
    if (d.first_index % 3 || d.index_count % 3 || (uint64_t)d.first_index + d.index_count > n_indices)
      return set_error(VCT_ERR_INVALID_VALUE, "draw object %u: bad index range", o);
    for (uint32_t t = d.first_index / 3; t < (d.first_index + d.index_count) / 3; ++t) {
      tri_obj[t] = obj_base + o;
      covered[t] = 1;
    }
  }
  for (uint32_t t = 0; t < n_tris; ++t)
    if (!covered[t]) return set_error(VCT_ERR_INVALID_VALUE, "triangle %u belongs to no draw object", t);
  std::unique_ptr<Model> m(new Model());
  m->n_verts = n_verts;
  m->n_tris = n_tris;
  std::memcpy(m->matrix, kIdentity, sizeof(m->matrix));
  VCT_CHECK(m->verts.ensure(std::max<uint32_t>(n_verts, 1)));
  VCT_CHECK(m->indices.ensure(std::max<uint32_t>(n_indices, 1)));
  VCT_CHECK(m->tri_obj.ensure(tri_obj.size()));
  if (n_verts) VCT_CUDA(cudaMemcpy(m->verts.p, verts, n_verts * sizeof(vct_vert_data), cudaMemcpyHostToDevice));
  if (n_indices) VCT_CUDA(cudaMemcpy(m->indices.p, indices, n_indices * sizeof(uint32_t), cudaMemcpyHostToDevice));
  VCT_CUDA(cudaMemcpy(m->tri_obj.p, tri_obj.data(), tri_obj.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  // Model dimensions exactly as renderer.cpp:457-486,517 computes them
  // (max starts at 0 and z is compared against min.y).
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {0, 0, 0};
  for (uint32_t i = 0; i < n_indices; ++i) {
    const float* p = verts[indices[i]].pos;
    if (p[0] > mx[0]) mx[0] = p[0];
    if (p[0] < mn[0]) mn[0] = p[0];
    if (p[1] > mx[1]) mx[1] = p[1];
    if (p[1] < mn[1]) mn[1] = p[1];
    if (p[2] > mx[2]) mx[2] = p[2];
    if (p[2] < mn[1]) mn[2] = p[2];
  }
  for (int k = 0; k < 3; ++k) m->dims[k] = mx[k] - mn[k];
  m->obj_start = obj_base;
  m->obj_count = n_objs;
  for (uint32_t o = 0; o < n_objs; ++o) r->objs.push_back(objs[o]);
  r->objs_dirty = true;
  ++r->scene_version;
  r->models.push_back(std::move(m));
  *out = r->models.size() - 1;
  return VCT_OK;
}

extern "C" vct_shader_id vct_load_shader(vct_renderer* r, const char*, const char*, const char*) {
  clear_error();
  if (!r) return VCT_INVALID_ID;
  return r->next_shader++;
}

extern "C" vct_material_id vct_add_material(vct_renderer* r, const vct_material_data* md) {
  clear_error();
  if (!r || !md) {
    set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
    return VCT_INVALID_ID;
  }
  r->materials.push_back(*md);
  r->materials_dirty = true;
  ++r->scene_version;
  return r->materials.size() - 1;
}

extern "C" vct_status vct_upload_material_data(vct_renderer* r, const vct_material_data* md, vct_material_id id) {
  clear_error();
  if (!r || !md) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (id >= r->materials.size()) return set_error(VCT_ERR_INVALID_ID, "material %llu", (unsigned long long)id);
  r->materials[id] = *md;
  r->materials_dirty = true;
  ++r->scene_version;
  return VCT_OK;
}

extern "C" vct_status vct_set_model_material(vct_renderer* r, vct_material_id mat, vct_model_id model) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (model >= r->models.size()) return set_error(VCT_ERR_INVALID_ID, "model %llu", (unsigned long long)model);
  if (mat >= r->materials.size()) return set_error(VCT_ERR_INVALID_ID, "material %llu", (unsigned long long)mat);
  const Model& m = *r->models[model];
  for (uint32_t o = 0; o < m.obj_count; ++o) r->objs[m.obj_start + o].material_id = (uint32_t)mat;
  r->objs_dirty = true;
  ++r->scene_version;
  return VCT_OK;
}

extern "C" vct_status vct_get_model_dimensions(vct_renderer* r, vct_model_id model, float out[3]) {
  clear_error();
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (model >= r->models.size()) return set_error(VCT_ERR_INVALID_ID, "model %llu", (unsigned long long)model);
  std::memcpy(out, r->models[model]->dims, 3 * sizeof(float));
  return VCT_OK;
}

extern "C" vct_status vct_get_material(vct_renderer* r, vct_material_id id, vct_material_data* out) {
  clear_error();
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (id >= r->materials.size()) return set_error(VCT_ERR_INVALID_ID, "material %llu", (unsigned long long)id);
  *out = r->materials[id];
  return VCT_OK;
}

// ----------------------------------------------------------- settings -----
extern "C" vct_status vct_set_grid_resolution(vct_renderer* r, uint32_t res) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (!is_pow2(res) || res < 8 || res > 1024)
    return set_error(VCT_ERR_INVALID_VALUE, "grid resolution %u: need a power of two in [8, 1024]", res);
  if (res == r->res && r->maps.l0_arr) return VCT_OK;
  VCT_CHECK(r->finish());
  r->cfg.grid_res = (int32_t)res;
  return r->alloc_maps(res);
}

extern "C" vct_status vct_set_grid_size(vct_renderer* r, float size) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (!(size > 0.0f) || !std::isfinite(size)) return set_error(VCT_ERR_INVALID_VALUE, "grid size %g", (double)size);
  r->cube_size = size;
  return VCT_OK;
}

extern "C" vct_status vct_set_camera_transform(vct_renderer* r, const float lookat[16], const float projection[16]) {
  clear_error();
  if (!r || !lookat || !projection) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  std::memcpy(r->view, lookat, sizeof(r->view));
  std::memcpy(r->proj, projection, sizeof(r->proj));
  return VCT_OK;
}

extern "C" vct_status vct_set_model_transform(vct_renderer* r, vct_model_id model, const float m[16]) {
  clear_error();
  if (!r || !m) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (model >= r->models.size()) return set_error(VCT_ERR_INVALID_ID, "model %llu", (unsigned long long)model);
  std::memcpy(r->models[model]->matrix, m, 16 * sizeof(float));
  return VCT_OK;
}

extern "C" vct_status vct_set_rendering_phases(vct_renderer* r, int32_t direct, int32_t diffuse, int32_t specular,
                                               int32_t shadow) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  r->en_direct = direct != 0;
  r->en_diffuse = diffuse != 0;
  r->en_specular = specular != 0;
  r->en_shadow = shadow != 0;
  return VCT_OK;
}

extern "C" vct_status vct_set_voxel_view_dir(vct_renderer* r, int32_t dir, float lod) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  r->view_dir = dir;
  r->view_lod = lod;
  return VCT_OK;
}

// -------------------------------------------------------------- frame -----
extern "C" vct_status vct_queue_model(vct_renderer* r, vct_model_id model) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (model >= r->models.size()) return VCT_OK;  // ignored, renderer.cpp:211-212
  Queued q;
  q.model = model;
  std::memcpy(q.M, r->models[model]->matrix, sizeof(q.M));
  r->queue.push_back(q);
  return VCT_OK;
}

extern "C" vct_status vct_queue_point_light(vct_renderer* r, const vct_point_light* l) {
  clear_error();
  if (!r || !l) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  r->lights.push_back(*l);
  return VCT_OK;
}

extern "C" vct_status vct_render(vct_renderer* r) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (r->frame_pending && cudaEventQuery(r->ev_done) == cudaSuccess) {
    // The previous frame (and its status copy) is complete: grow any work
    // list it needed more room in before encoding the next frame.
    r->frame_pending = false;
    const FrameStatus s = *r->h_status.p;
    if (s.pair_total > r->pair_list.n) VCT_CHECK(r->pair_list.ensure((size_t)s.pair_total + s.pair_total / 4 + 4096));
    if (s.big_total > r->big_cap) VCT_CHECK(r->grow_big(s.big_total + s.big_total / 4 + 1024));
    if (s.bigtri_total > r->bin_big_cap) VCT_CHECK(r->grow_bin_big(s.bigtri_total + s.bigtri_total / 4 + 256));
  }
  FrameInputs fi;
  fi.queue.swap(r->queue);
  fi.lights.swap(r->lights);
  std::memcpy(fi.view, r->view, sizeof(fi.view));
  std::memcpy(fi.proj, r->proj, sizeof(fi.proj));
  fi.cube_size = r->cube_size;
  fi.tp = r->trace_params();
  r->last = std::move(fi);
  r->have_last = true;
  vct_status s = r->encode(r->last);
  r->queue.clear();  // renderer.cpp:403-404
  r->lights.clear();
  return s;
}

// ---------------------------------------------- streams, timing, read-back --
extern "C" vct_status vct_set_stream(vct_renderer* r, void* stream) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  VCT_CHECK(r->finish());
  r->stream = stream ? (cudaStream_t)stream : r->own_stream;
  return VCT_OK;
}

extern "C" vct_status vct_synchronize(vct_renderer* r) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  return r->finish();
}

extern "C" vct_status vct_get_stage_times(vct_renderer* r, vct_stage_times* out) {
  clear_error();
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(r->finish());
  if (!r->have_frame) return set_error(VCT_ERR_INVALID_VALUE, "no frame rendered yet");
  // ev: voxelize start, voxelize end, mipmap end, trace start, trace end;
  // evg (raster stream): raster start, raster end, learned term end.
  float t[2], g[2], tr;
  for (int i = 0; i < 2; ++i) VCT_CUDA(cudaEventElapsedTime(&t[i], r->ev[i], r->ev[i + 1]));
  for (int i = 0; i < 2; ++i) VCT_CUDA(cudaEventElapsedTime(&g[i], r->evg[i], r->evg[i + 1]));
  VCT_CUDA(cudaEventElapsedTime(&tr, r->ev[3], r->ev[4]));
  out->voxelize = t[0];
  out->mipmap = t[1];
  out->gbuffer = g[0];
  out->trace = tr + (r->infer_ran ? g[1] : 0.0f);  // (+ the learned term's inference)
  VCT_CUDA(cudaEventElapsedTime(&out->total, r->ev_start, r->ev[4]));
  out->kernel_launches = (uint32_t)r->launches;
  out->voxelized = r->last_revoxelized ? 1u : 0u;
  out->split_bricks = r->h_status.p->heavy_total;
  out->infer = r->infer_ran ? g[1] : 0.0f;
  return VCT_OK;
}

extern "C" vct_status vct_read_frame(vct_renderer* r, void* dst, int32_t format) {
  clear_error();
  if (!r || !dst) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(r->finish());
  if (!r->have_frame) return set_error(VCT_ERR_INVALID_VALUE, "no frame rendered yet");
  const size_t px = (size_t)r->W * r->H;
  if (format == VCT_FRAME_RGBA8) {
    VCT_CUDA(cudaMemcpyAsync(dst, r->frame.p, px * 4, cudaMemcpyDeviceToHost, r->stream));
  } else if (format == VCT_FRAME_RGBA32F) {
    if (!r->cfg.keep_float_frame) return set_error(VCT_ERR_UNSUPPORTED, "keep_float_frame is off");
    VCT_CUDA(cudaMemcpyAsync(dst, r->frame_f32.p, px * 16, cudaMemcpyDeviceToHost, r->stream));
  } else {
    return set_error(VCT_ERR_INVALID_VALUE, "frame format %d", format);
  }
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}

extern "C" vct_status vct_frame_device_ptr(vct_renderer* r, void** out) {
  clear_error();
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  *out = r->frame.p;
  return VCT_OK;
}

extern "C" vct_status vct_set_light_injection(vct_renderer* r, int32_t enable) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (enable && r->cfg.storage != VCT_STORAGE_RGBA8)
    return set_error(VCT_ERR_UNSUPPORTED, "light injection needs RGBA8 storage");
  VCT_CHECK(r->finish());
  r->inject = enable != 0;
  r->inj_valid = false;
  return VCT_OK;
}

extern "C" vct_status vct_read_injection_grids(vct_renderer* r, void* albedo, void* normal, void* emission) {
  clear_error();
  if (!r || !albedo || !normal || !emission) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(r->finish());
  if (!r->inj_arr[0]) return set_error(VCT_ERR_UNSUPPORTED, "no injection grids (injection off or no frame yet)");
  void* dst[3] = {albedo, normal, emission};
  for (int k = 0; k < 3; ++k) {
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    p.srcArray = r->inj_arr[k];
    p.dstPtr = make_cudaPitchedPtr(dst[k], (size_t)r->res * 4, r->res, r->res);
    p.extent = make_cudaExtent(r->res, r->res, r->res);
    p.kind = cudaMemcpyDeviceToHost;
    VCT_CUDA(cudaMemcpy3DAsync(&p, r->stream));
  }
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}

extern "C" vct_status vct_read_voxels(vct_renderer* r, int32_t level, int32_t map, void* dst) {
  clear_error();
  if (!r || !dst) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (level < 0 || level >= r->levels) return set_error(VCT_ERR_INVALID_VALUE, "level %d of %d", level, r->levels);
  if (map < 0 || map >= r->ms.nmaps) return set_error(VCT_ERR_INVALID_VALUE, "map %d of %d", map, r->ms.nmaps);
  VCT_CHECK(r->finish());
  cudaArray_t a = r->maps.l0_arr;
  if (level > 0) VCT_CUDA(cudaGetMipmappedArrayLevel(&a, r->maps.dir_arr[map], level - 1));
  const size_t s = r->res >> level;
  const size_t bpt = r->cfg.storage == VCT_STORAGE_RGBA16F ? 8 : 4;
  cudaMemcpy3DParms p;
  std::memset(&p, 0, sizeof(p));
  p.srcArray = a;
  p.dstPtr = make_cudaPitchedPtr(dst, s * bpt, s, s);
  p.extent = make_cudaExtent(s, s, s);
  p.kind = cudaMemcpyDeviceToHost;
  VCT_CUDA(cudaMemcpy3DAsync(&p, r->stream));
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}

extern "C" vct_status vct_read_voxel_counts(vct_renderer* r, uint32_t* dst) {
  clear_error();
  if (!r || !dst) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (!r->cfg.keep_counts) return set_error(VCT_ERR_UNSUPPORTED, "keep_counts is off");
  VCT_CHECK(r->finish());
  VCT_CUDA(cudaMemcpyAsync(dst, r->counts.p, (size_t)r->res * r->res * r->res * 4, cudaMemcpyDeviceToHost, r->stream));
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}

extern "C" vct_status vct_read_gbuffer(vct_renderer* r, uint32_t* tri_id, float* pos, float* nrm, uint32_t* mat) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  VCT_CHECK(r->finish());
  const size_t px = (size_t)r->W * r->H;
  std::vector<float4> a(px), b(px);
  VCT_CUDA(cudaMemcpyAsync(a.data(), r->gb_pos.p, px * sizeof(float4), cudaMemcpyDeviceToHost, r->stream));
  VCT_CUDA(cudaMemcpyAsync(b.data(), r->gb_nrm.p, px * sizeof(float4), cudaMemcpyDeviceToHost, r->stream));
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  for (size_t i = 0; i < px; ++i) {
    uint32_t t, m;
    std::memcpy(&t, &b[i].w, 4);
    std::memcpy(&m, &a[i].w, 4);
    if (tri_id) tri_id[i] = t;
    if (mat) mat[i] = m;
    if (pos) { pos[3 * i] = a[i].x; pos[3 * i + 1] = a[i].y; pos[3 * i + 2] = a[i].z; }
    if (nrm) { nrm[3 * i] = b[i].x; nrm[3 * i + 1] = b[i].y; nrm[3 * i + 2] = b[i].z; }
  }
  return VCT_OK;
}

extern "C" vct_status vct_get_grid(vct_renderer* r, int32_t* res, int32_t* levels) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (res) *res = (int32_t)r->res;
  if (levels) *levels = r->levels;
  return VCT_OK;
}
