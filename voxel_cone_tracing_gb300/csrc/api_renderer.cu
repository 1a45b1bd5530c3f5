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

#include "api_common.h"
#include "vct_internal.h"

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

// --------------------------------------------------------- host maths -----
namespace {

// P * V in FP32, fixed summation order (the CPU oracle does the same).
void matmul_f32(const float* P, const float* V, float* o) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      float t = P[0 * 4 + r] * V[c * 4 + 0];
      t = t + P[1 * 4 + r] * V[c * 4 + 1];
      t = t + P[2 * 4 + r] * V[c * 4 + 2];
      o[c * 4 + r] = t + P[3 * 4 + r] * V[c * 4 + 3];
    }
}

// mat3(transpose(inverse(M))) (voxelize.vert:28), row-major float[9].
void normal_matrix(const float* mf, float* nm) {
  double m[16], inv[16];
  for (int i = 0; i < 16; ++i) m[i] = mf[i];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  const double id = det != 0.0 ? 1.0 / det : 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) nm[r * 3 + c] = (float)(inv[r * 4 + c] * id);
}

bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }
int ilog2(uint32_t v) {
  int l = 0;
  while ((1u << (l + 1)) <= v) ++l;
  return l;
}

struct Model {
  DevBuf<vct_vert_data> verts;
  DevBuf<uint32_t> indices;
  DevBuf<uint32_t> tri_obj;
  uint32_t n_verts = 0, n_tris = 0;
  uint32_t obj_start = 0, obj_count = 0;
  float dims[3] = {0, 0, 0};
  float matrix[16];
};

struct Queued {
  uint64_t model;
  float M[16];
};

// Everything a frame reads, captured by vct_render so that a frame can be
// re-encoded after its work buffers were grown.
struct FrameInputs {
  std::vector<Queued> queue;
  std::vector<vct_point_light> lights;
  float view[16], proj[16];
  float cube_size;
  TraceParams tp;
};

const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

}  // namespace

struct vct_renderer {
  int W = 0, H = 0;
  vct_config cfg;
  // resources (renderer.h:168-171)
  std::vector<vct_material_data> materials;
  std::vector<vct_draw_obj> objs;
  std::vector<std::unique_ptr<Model>> models;
  uint64_t next_shader = 0;
  bool materials_dirty = true, objs_dirty = true;
  // settings (renderer.h:173-186)
  float view[16], proj[16];
  float cube_size = 1.0f;
  uint32_t res = 0;
  int levels = 0;
  bool en_shadow = true, en_direct = true, en_diffuse = true, en_specular = true;
  int view_dir = 0;  // Renderer::Renderer sets m_view_voxel_dir(0), renderer.cpp:107
  float view_lod = 0.0f;
  // per frame (renderer.h:190-191)
  std::vector<Queued> queue;
  std::vector<vct_point_light> lights;
  FrameInputs last;
  bool have_last = false;
  // GPU state
  cudaStream_t own_stream = nullptr, stream = nullptr;
  cudaEvent_t ev[5] = {};
  cudaEvent_t ev_staged = nullptr;
  cudaEvent_t ev_done = nullptr;   // after the frame's status copy
  cudaArray_t l0_arr = nullptr;
  cudaMipmappedArray_t dir_arr[kMaxMaps] = {};
  MapSet ms = {};
  DevBuf<vct_material_data> d_materials;
  DevBuf<uint32_t> d_obj_material;
  DevBuf<DevInstance> d_inst;
  HostBuf<DevInstance> h_inst;
  DevBuf<uint32_t> brick_count, brick_offset, brick_cursor, pair_list, scan_tmp, counts;
  DevBuf<FrameStatus> d_status;
  HostBuf<FrameStatus> h_status;
  DevBuf<unsigned long long> vis;
  DevBuf<unsigned char> big;
  DevBuf<uint32_t> big_count, big_offset;
  uint32_t big_cap = 0;
  DevBuf<float4> gb_pos, gb_nrm;
  DevBuf<uchar4> frame;
  DevBuf<float4> frame_f32;
  bool frame_pending = false;
  bool have_frame = false;
  int launches = 0;  // engine kernels of the last encoded frame

  ~vct_renderer() {
    if (stream) cudaStreamSynchronize(stream);
    free_maps();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (ev_staged) cudaEventDestroy(ev_staged);
    if (ev_done) cudaEventDestroy(ev_done);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  void free_maps() {
    if (ms.l0_tex) cudaDestroyTextureObject(ms.l0_tex);
    if (ms.l0_surf) cudaDestroySurfaceObject(ms.l0_surf);
    for (int d = 0; d < kMaxMaps; ++d) {
      if (ms.tex[d]) cudaDestroyTextureObject(ms.tex[d]);
      for (int l = 0; l < kMaxLevels; ++l)
        if (ms.surf[d][l]) cudaDestroySurfaceObject(ms.surf[d][l]);
      if (dir_arr[d]) cudaFreeMipmappedArray(dir_arr[d]);
      dir_arr[d] = nullptr;
    }
    if (l0_arr) cudaFreeArray(l0_arr);
    l0_arr = nullptr;
    std::memset(&ms, 0, sizeof(ms));
  }

  cudaChannelFormatDesc texel_desc() const {
    return cfg.storage == VCT_STORAGE_RGBA16F ? cudaCreateChannelDesc(16, 16, 16, 16, cudaChannelFormatKindFloat)
                                              : cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
  }

  // set_grid_resolution (renderer.cpp:178-188): six 3D textures of `levels`
  // mip levels.  Here: level 0 once + one chain (levels 1..L-1) per map.
  vct_status alloc_maps(uint32_t r) {
    if (stream) VCT_CUDA(cudaStreamSynchronize(stream));
    free_maps();
    const int L = std::min(kMaxLevels, ilog2(r) + 1);
    const int nmaps = cfg.mip_mode == VCT_MIP_ISO ? 1 : 6;
    const cudaChannelFormatDesc desc = texel_desc();
    VCT_CUDA(cudaMalloc3DArray(&l0_arr, &desc, make_cudaExtent(r, r, r), cudaArraySurfaceLoadStore));
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = l0_arr;
    VCT_CUDA(cudaCreateSurfaceObject(&ms.l0_surf, &rd));
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cfg.storage == VCT_STORAGE_RGBA16F ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
    td.normalizedCoords = 1;
    td.mipmapFilterMode = cudaFilterModeLinear;
    VCT_CUDA(cudaCreateTextureObject(&ms.l0_tex, &rd, &td, nullptr));
    for (int d = 0; d < nmaps && L > 1; ++d) {
      VCT_CUDA(cudaMallocMipmappedArray(&dir_arr[d], &desc, make_cudaExtent(r / 2, r / 2, r / 2), L - 1,
                                        cudaArraySurfaceLoadStore));
      for (int l = 1; l < L; ++l) {
        cudaArray_t la;
        VCT_CUDA(cudaGetMipmappedArrayLevel(&la, dir_arr[d], l - 1));
        cudaResourceDesc lr;
        std::memset(&lr, 0, sizeof(lr));
        lr.resType = cudaResourceTypeArray;
        lr.res.array.array = la;
        VCT_CUDA(cudaCreateSurfaceObject(&ms.surf[d][l], &lr));
      }
      cudaResourceDesc mr;
      std::memset(&mr, 0, sizeof(mr));
      mr.resType = cudaResourceTypeMipmappedArray;
      mr.res.mipmap.mipmap = dir_arr[d];
      cudaTextureDesc mt = td;
      mt.minMipmapLevelClamp = 0.0f;
      mt.maxMipmapLevelClamp = (float)(L - 2);
      VCT_CUDA(cudaCreateTextureObject(&ms.tex[d], &mr, &mt, nullptr));
    }
    ms.N = (int)r;
    ms.L = L;
    ms.nmaps = nmaps;
    ms.storage = cfg.storage;
    res = r;
    levels = L;
    const size_t nb = (size_t)(r / kBrick) * (r / kBrick) * (r / kBrick);
    VCT_CHECK(brick_count.ensure(nb));
    VCT_CHECK(brick_offset.ensure(nb + 1));
    VCT_CHECK(brick_cursor.ensure(nb));
    VCT_CHECK(scan_tmp.ensure(scan_tmp_words(nb)));
    if (cfg.keep_counts) VCT_CHECK(counts.ensure((size_t)r * r * r));
    have_frame = false;
    return VCT_OK;
  }

  vct_status init(int w, int h, const vct_config* c) {
    W = w;
    H = h;
    if (c) cfg = *c; else vct_config_default(&cfg);
    std::memcpy(view, kIdentity, sizeof(view));
    std::memcpy(proj, kIdentity, sizeof(proj));
    VCT_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
    for (auto& e : ev) VCT_CUDA(cudaEventCreate(&e));
    VCT_CUDA(cudaEventCreateWithFlags(&ev_staged, cudaEventDisableTiming));
    VCT_CUDA(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
    // Default material (renderer.cpp:115-128, fill_default_mat_data :85-98).
    vct_material_data m;
    std::memset(&m, 0, sizeof(m));
    m.ambient[0] = 1; m.ambient[2] = 1;
    m.diffuse[0] = 1; m.diffuse[2] = 1;
    m.shininess = 1; m.ior = 1; m.dissolve = 1; m.illum = 0;
    materials.push_back(m);
    const size_t px = (size_t)W * H;
    VCT_CHECK(vis.ensure(px));
    VCT_CHECK(gb_pos.ensure(px));
    VCT_CHECK(gb_nrm.ensure(px));
    VCT_CHECK(frame.ensure(px));
    if (cfg.keep_float_frame) VCT_CHECK(frame_f32.ensure(px));
    VCT_CHECK(d_status.ensure(1));
    VCT_CHECK(h_status.ensure(1));
    std::memset(h_status.p, 0, sizeof(FrameStatus));
    VCT_CHECK(big_count.ensure(2));
    VCT_CHECK(grow_big(1 << 16));
    return alloc_maps((uint32_t)cfg.grid_res);
  }

  vct_status grow_big(uint32_t cap) {
    VCT_CHECK(big.ensure((size_t)cap * big_record_bytes()));
    VCT_CHECK(big_offset.ensure((size_t)cap + 1));
    big_cap = cap;
    return VCT_OK;
  }

  vct_status upload_tables() {
    if (materials_dirty) {
      VCT_CHECK(d_materials.ensure(materials.size()));
      VCT_CUDA(cudaMemcpyAsync(d_materials.p, materials.data(), materials.size() * sizeof(vct_material_data),
                               cudaMemcpyHostToDevice, stream));
      VCT_CUDA(cudaStreamSynchronize(stream));
      materials_dirty = false;
    }
    if (objs_dirty) {
      std::vector<uint32_t> om(std::max<size_t>(objs.size(), 1), 0);
      for (size_t i = 0; i < objs.size(); ++i) om[i] = objs[i].material_id;
      VCT_CHECK(d_obj_material.ensure(om.size()));
      VCT_CUDA(cudaMemcpyAsync(d_obj_material.p, om.data(), om.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               stream));
      VCT_CUDA(cudaStreamSynchronize(stream));
      objs_dirty = false;
    }
    return VCT_OK;
  }

  vct_status encode(const FrameInputs& fi) {
    // Material ids of every queued draw object must exist (the reference
    // indexes m_materials unchecked, renderer.cpp:252).
    uint64_t total = 0;
    for (const Queued& q : fi.queue) {
      const Model& m = *models[q.model];
      for (uint32_t o = 0; o < m.obj_count; ++o)
        if (objs[m.obj_start + o].material_id >= materials.size())
          return set_error(VCT_ERR_INVALID_ID, "draw object %u of model %llu uses material %u (only %zu exist)", o,
                           (unsigned long long)q.model, objs[m.obj_start + o].material_id, materials.size());
      total += m.n_tris;
    }
    if (total >= 0xffffffffull) return set_error(VCT_ERR_INVALID_VALUE, "too many queued triangles");
    VCT_CHECK(upload_tables());
    const size_t ni = std::max<size_t>(fi.queue.size(), 1);
    VCT_CHECK(d_inst.ensure(ni));
    VCT_CUDA(cudaEventSynchronize(ev_staged));  // previous upload has left the staging buffer
    VCT_CHECK(h_inst.ensure(ni));
    uint32_t base = 0;
    for (size_t i = 0; i < fi.queue.size(); ++i) {
      const Model& m = *models[fi.queue[i].model];
      DevInstance& d = h_inst.p[i];
      std::memcpy(d.M, fi.queue[i].M, sizeof(d.M));
      normal_matrix(fi.queue[i].M, d.NM);
      d.tri_base = base;
      d.n_tris = m.n_tris;
      d.verts = m.verts.p;
      d.indices = m.indices.p;
      d.tri_obj = m.tri_obj.p;
      d.n_verts = m.n_verts;
      d.pad = 0;
      base += m.n_tris;
    }
    if (!fi.queue.empty())
      VCT_CUDA(cudaMemcpyAsync(d_inst.p, h_inst.p, fi.queue.size() * sizeof(DevInstance), cudaMemcpyHostToDevice,
                               stream));
    VCT_CUDA(cudaEventRecord(ev_staged, stream));

    SceneParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.inst = d_inst.p;
    sp.materials = d_materials.p;
    sp.obj_material = d_obj_material.p;
    sp.n_instances = (uint32_t)fi.queue.size();
    sp.total_tris = (uint32_t)total;
    sp.n_materials = (uint32_t)materials.size();
    sp.n_lights = (int32_t)std::min<size_t>(fi.lights.size(), kMaxLights);
    sp.cube_size = fi.cube_size;
    for (int i = 0; i < sp.n_lights; ++i) sp.lights[i] = fi.lights[i];

    CameraParams cp;
    matmul_f32(fi.proj, fi.view, cp.PV);
    cp.cam_pos[0] = fi.view[12];  // glm::column(view, 3), renderer.cpp:279
    cp.cam_pos[1] = fi.view[13];
    cp.cam_pos[2] = fi.view[14];
    cp.W = W;
    cp.H = H;

    const uint32_t pairs_needed = (uint32_t)std::min<uint64_t>(0xffffff00ull, 4ull * total + 65536ull);
    if (pair_list.n < pairs_needed) VCT_CHECK(pair_list.ensure(pairs_needed));

    VoxBuffers vb;
    vb.brick_count = brick_count.p;
    vb.brick_offset = brick_offset.p;
    vb.brick_cursor = brick_cursor.p;
    vb.pair_list = pair_list.p;
    vb.pair_cap = (uint32_t)pair_list.n;
    vb.scan_tmp = scan_tmp.p;
    vb.counts = cfg.keep_counts ? counts.p : nullptr;
    vb.status = d_status.p;

    RasterBuffers rb;
    rb.vis = vis.p;
    rb.big = big.p;
    rb.big_cap = big_cap;
    rb.big_count = big_count.p;
    rb.big_offset = big_offset.p;
    rb.scan_tmp = nullptr;
    rb.gb_pos = gb_pos.p;
    rb.gb_nrm = gb_nrm.p;
    rb.status = d_status.p;

    VCT_CUDA(cudaMemsetAsync(d_status.p, 0, sizeof(FrameStatus), stream));
    launches = 0;
    VCT_CUDA(cudaEventRecord(ev[0], stream));
    VCT_CUDA(launch_voxelize(sp, (int)res, cfg.vox_mode, cfg.storage, vb, ms.l0_surf, stream, &launches));
    VCT_CUDA(cudaEventRecord(ev[1], stream));
    VCT_CUDA(launch_mipmap(ms, cfg.mip_mode, stream, &launches));
    VCT_CUDA(cudaEventRecord(ev[2], stream));
    VCT_CUDA(launch_gbuffer(sp, cp, rb, stream, &launches));
    VCT_CUDA(cudaEventRecord(ev[3], stream));
    VCT_CUDA(launch_trace(sp, cp, ms, fi.tp, gb_pos.p, gb_nrm.p, frame.p, cfg.keep_float_frame ? frame_f32.p : nullptr,
                          stream, &launches));
    VCT_CUDA(cudaEventRecord(ev[4], stream));
    VCT_CUDA(cudaMemcpyAsync(h_status.p, d_status.p, sizeof(FrameStatus), cudaMemcpyDeviceToHost, stream));
    VCT_CUDA(cudaEventRecord(ev_done, stream));
    frame_pending = true;
    have_frame = true;
    return VCT_OK;
  }

  // Wait for the last frame; if a work list overflowed, grow it and encode
  // the same frame again (results are exact once this returns).
  vct_status finish() {
    if (!frame_pending) return VCT_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
      VCT_CUDA(cudaStreamSynchronize(stream));
      frame_pending = false;
      const FrameStatus s = *h_status.p;
      bool redo = false;
      if (s.pair_total > pair_list.n) {
        VCT_CHECK(pair_list.ensure((size_t)s.pair_total + s.pair_total / 4 + 4096));
        redo = true;
      }
      if (s.big_total > big_cap) {
        VCT_CHECK(grow_big(s.big_total + s.big_total / 4 + 1024));
        redo = true;
      }
      if (!redo) return VCT_OK;
      if (!have_last) return VCT_OK;
      VCT_CHECK(encode(last));
    }
    return set_error(VCT_ERR_CUDA, "frame work lists kept overflowing");
  }

  TraceParams trace_params() const {
    TraceParams tp;
    tp.enable_direct = en_direct;
    tp.enable_diffuse = en_diffuse;
    tp.enable_specular = en_specular;
    tp.enable_shadow = en_shadow;
    tp.view_voxel_dir = view_dir;
    tp.view_voxel_lod = view_lod;
    tp.cone_set = cfg.cone_set;
    tp.sampler = cfg.sampler;
    tp.mip_mode = cfg.mip_mode;
    return tp;
  }
};

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
}

static vct_status check_config(const vct_config& c) {
  if (!is_pow2((uint32_t)c.grid_res) || c.grid_res < 8 || c.grid_res > 1024)
    return set_error(VCT_ERR_INVALID_VALUE, "grid_res %d: need a power of two in [8, 1024]", c.grid_res);
  if (c.vox_mode < 0 || c.vox_mode > 1 || c.mip_mode < 0 || c.mip_mode > 1 || c.storage < 0 || c.storage > 1 ||
      c.sampler < 0 || c.sampler > 1 || c.cone_set < 0 || c.cone_set > 1)
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
  return r->materials.size() - 1;
}

extern "C" vct_status vct_upload_material_data(vct_renderer* r, const vct_material_data* md, vct_material_id id) {
  clear_error();
  if (!r || !md) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (id >= r->materials.size()) return set_error(VCT_ERR_INVALID_ID, "material %llu", (unsigned long long)id);
  r->materials[id] = *md;
  r->materials_dirty = true;
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
  if (res == r->res && r->l0_arr) return VCT_OK;
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
  float t[4];
  for (int i = 0; i < 4; ++i) VCT_CUDA(cudaEventElapsedTime(&t[i], r->ev[i], r->ev[i + 1]));
  out->voxelize = t[0];
  out->mipmap = t[1];
  out->gbuffer = t[2];
  out->trace = t[3];
  VCT_CUDA(cudaEventElapsedTime(&out->total, r->ev[0], r->ev[4]));
  out->kernel_launches = (uint32_t)r->launches;
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

extern "C" vct_status vct_read_voxels(vct_renderer* r, int32_t level, int32_t map, void* dst) {
  clear_error();
  if (!r || !dst) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (level < 0 || level >= r->levels) return set_error(VCT_ERR_INVALID_VALUE, "level %d of %d", level, r->levels);
  if (map < 0 || map >= r->ms.nmaps) return set_error(VCT_ERR_INVALID_VALUE, "map %d of %d", map, r->ms.nmaps);
  VCT_CHECK(r->finish());
  cudaArray_t a = r->l0_arr;
  if (level > 0) VCT_CUDA(cudaGetMipmappedArrayLevel(&a, r->dir_arr[map], level - 1));
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
