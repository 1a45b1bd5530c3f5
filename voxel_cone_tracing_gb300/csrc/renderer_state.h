// renderer_state.h -- the state behind a vct_renderer handle (shared by the
// translation units of the C ABI; not a public header).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include "api_common.h"
#include "vct_internal.h"

using namespace vct;

// --------------------------------------------------------- host maths -----
namespace vct {
namespace detail {

// P * V in FP32, fixed summation order (the CPU oracle does the same).
inline void matmul_f32(const float* P, const float* V, float* o) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      float t = P[0 * 4 + r] * V[c * 4 + 0];
      t = t + P[1 * 4 + r] * V[c * 4 + 1];
      t = t + P[2 * 4 + r] * V[c * 4 + 2];
      o[c * 4 + r] = t + P[3 * 4 + r] * V[c * 4 + 3];
    }
}

// mat3(transpose(inverse(M))) (voxelize.vert:28), row-major float[9].
inline void normal_matrix(const float* mf, float* nm) {
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

inline bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }
inline int ilog2(uint32_t v) {
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

// A 3D tensor map (TMA descriptor) over a dense N^3 array of `elem_bytes`
// texels, boxes of 16^3, for the MipBuilder's bulk-tensor copies.  The
// driver's encoder is reached through the runtime's entry-point query, so
// the library does not link libcuda.
inline vct_status encode_box_map(CUtensorMap* map, void* base, uint32_t N, uint32_t elem_bytes) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    VCT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn)
      return set_error(VCT_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[3] = {N, N, N};
  const cuuint64_t strides[2] = {(cuuint64_t)N * elem_bytes, (cuuint64_t)N * N * elem_bytes};  // bytes, dims 1..2
  const cuuint32_t box[3] = {16, 16, 16};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(map, elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_INT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 3,
                            base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(VCT_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return VCT_OK;
}

// Everything a frame reads, captured by vct_render so that a frame can be
// re-encoded after its work buffers were grown.
struct FrameInputs {
  std::vector<Queued> queue;
  std::vector<vct_point_light> lights;
  float view[16], proj[16];
  float cube_size;
  TraceParams tp;
};

constexpr float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

}  // namespace detail
}  // namespace vct

using namespace vct::detail;

// Parameters, gradients and Adam state of the learned diffuse term.
struct MlpState {
  bool ready = false;  // parameters allocated and initialised
  bool trained = false;
  bool tc = true;      // forward on tcgen05 / TMEM, warp-specialised (else mma.sync warp tiles)
  int32_t levels = 16, log2_table = 19, n_min = 16, n_max = 512;
  int adam_t = 0;
  DevBuf<float> table, table_grad, table_m, table_v;  // levels * T * 2
  DevBuf<__nv_bfloat16> table_bf;
  DevBuf<float> w, w_grad, w_m, w_v;  // kMlpWeights
  DevBuf<__nv_bfloat16> w_bf;
  DevBuf<float> samples;  // rows of 12 floats
  uint32_t n_samples = 0;
  DevBuf<float> loss;     // one slot per optimiser step

  size_t table_floats() const { return (size_t)levels * ((size_t)1 << log2_table) * 2; }

  MlpParams params() const {
    MlpParams p;
    std::memset(&p, 0, sizeof(p));
    p.table_bf = table_bf.p;
    p.table_grad = reinterpret_cast<float2*>(table_grad.p);
    p.w_bf = w_bf.p;
    p.w_grad = w_grad.p;
    p.log2_table = log2_table;
    const double b = std::exp((std::log((double)n_max) - std::log((double)n_min)) / (levels - 1));
    for (int l = 0; l < levels && l < kMlpLevels; ++l) {
      p.res[l] = (int)std::floor((double)n_min * std::pow(b, l) + 1e-6);
      const uint64_t r1 = (uint64_t)p.res[l] + 1;
      if (r1 * r1 * r1 <= ((uint64_t)1 << log2_table)) p.dense_mask |= 1 << l;
    }
    return p;
  }
};

// Buffers of the dense-brick split (HeavyBricks): a slot index per brick,
// accumulator slots sized for the largest accumulator type, and the extra
// chunk items.  A frame whose plan overflowed them is still exact (the
// bricks that did not fit ran whole); grow() enlarges them for the next.
struct HeavyStore {
  DevBuf<int32_t> slot;
  DevBuf<uint32_t> brick, done, counters;
  DevBuf<unsigned char> acc;
  DevBuf<uint2> items;
  uint32_t slot_cap = 0, item_cap = 0;

  static size_t slot_bytes() {
    return std::max({heavy_slot_bytes(VCT_STORAGE_RGBA8), heavy_slot_bytes(VCT_STORAGE_RGBA16F),
                     heavy_slot_bytes(kStorageAttr)});
  }
  // Called between frames (no kernel of the owner in flight); `st` is the
  // owner's stream, so the zeroing is ordered before its next frame.
  vct_status reserve(size_t n_bricks, uint32_t slots, uint32_t n_items, cudaStream_t st) {
    VCT_CHECK(slot.ensure(n_bricks));
    VCT_CHECK(counters.ensure(3));
    if (slots > slot_cap) {
      // the slots and their counters start at zero and every frame leaves them so
      VCT_CHECK(brick.ensure(slots));
      VCT_CHECK(done.ensure(slots));
      VCT_CHECK(acc.ensure((size_t)slots * slot_bytes()));
      VCT_CUDA(cudaMemsetAsync(done.p, 0, (size_t)slots * sizeof(uint32_t), st));
      VCT_CUDA(cudaMemsetAsync(acc.p, 0, (size_t)slots * slot_bytes(), st));
      slot_cap = slots;
    }
    if (n_items > item_cap) {
      VCT_CHECK(items.ensure(n_items));
      item_cap = n_items;
    }
    return VCT_OK;
  }
  // After a frame: room for its split with a margin.
  vct_status grow(const FrameStatus& s, size_t n_bricks, cudaStream_t st) {
    if (s.heavy_total <= slot_cap && s.extra_total <= item_cap) return VCT_OK;
    return reserve(n_bricks, std::max(slot_cap, s.heavy_total + s.heavy_total / 4 + 64),
                   std::max(item_cap, s.extra_total + s.extra_total / 4 + 1024), st);
  }
  HeavyBricks view() const {
    HeavyBricks h;
    h.slot = slot.p;
    h.brick = brick.p;
    h.done = done.p;
    h.acc = acc.p;
    h.items = items.p;
    h.counters = counters.p;
    h.slot_cap = slot_cap;
    h.item_cap = item_cap;
    return h;
  }
};

// The voxel maps of one grid: level 0 once (surface + texture) and one
// mipmapped chain of levels 1..L-1 per map (surfaces per level + one
// texture), as set_grid_resolution allocates them (renderer.cpp:178-188).
struct MapStore {
  cudaArray_t l0_arr = nullptr;
  cudaMipmappedArray_t dir_arr[kMaxMaps] = {};
  cudaMipmappedArray_t alpha_arr[2] = {};
  void* occ_mem = nullptr;  // occupancy grids of empty-space skipping
  MapSet ms = {};

  MapStore() = default;
  MapStore(const MapStore&) = delete;
  MapStore& operator=(const MapStore&) = delete;
  ~MapStore() { release(); }

  void release() {
    if (ms.l0_tex) cudaDestroyTextureObject(ms.l0_tex);
    if (ms.l0_surf) cudaDestroySurfaceObject(ms.l0_surf);
    for (int d = 0; d < kMaxMaps; ++d) {
      if (ms.tex[d]) cudaDestroyTextureObject(ms.tex[d]);
      for (int l = 0; l < kMaxLevels; ++l)
        if (ms.surf[d][l]) cudaDestroySurfaceObject(ms.surf[d][l]);
      if (dir_arr[d]) cudaFreeMipmappedArray(dir_arr[d]);
      dir_arr[d] = nullptr;
    }
    for (int k = 0; k < 2; ++k) {
      if (ms.alpha_tex[k]) cudaDestroyTextureObject(ms.alpha_tex[k]);
      for (int l = 0; l < kMaxLevels; ++l)
        if (ms.alpha_surf[k][l]) cudaDestroySurfaceObject(ms.alpha_surf[k][l]);
      if (alpha_arr[k]) cudaFreeMipmappedArray(alpha_arr[k]);
      alpha_arr[k] = nullptr;
    }
    if (l0_arr) cudaFreeArray(l0_arr);
    l0_arr = nullptr;
    if (occ_mem) cudaFree(occ_mem);
    occ_mem = nullptr;
    std::memset(&ms, 0, sizeof(ms));
  }

  // A mipmapped array of levels 1..L-1 (base r/2) with a surface per level
  // and one filtered texture over all of them.
  static vct_status chain(uint32_t r, int L, const cudaChannelFormatDesc& desc, const cudaTextureDesc& td,
                          cudaMipmappedArray_t* arr, cudaSurfaceObject_t* surf, cudaTextureObject_t* tex) {
    VCT_CUDA(cudaMallocMipmappedArray(arr, &desc, make_cudaExtent(r / 2, r / 2, r / 2), L - 1,
                                      cudaArraySurfaceLoadStore));
    for (int l = 1; l < L; ++l) {
      cudaArray_t la;
      VCT_CUDA(cudaGetMipmappedArrayLevel(&la, *arr, l - 1));
      cudaResourceDesc lr;
      std::memset(&lr, 0, sizeof(lr));
      lr.resType = cudaResourceTypeArray;
      lr.res.array.array = la;
      VCT_CUDA(cudaCreateSurfaceObject(&surf[l], &lr));
    }
    cudaResourceDesc mr;
    std::memset(&mr, 0, sizeof(mr));
    mr.resType = cudaResourceTypeMipmappedArray;
    mr.res.mipmap.mipmap = *arr;
    cudaTextureDesc mt = td;
    mt.minMipmapLevelClamp = 0.0f;
    mt.maxMipmapLevelClamp = (float)(L - 2);
    VCT_CUDA(cudaCreateTextureObject(tex, &mr, &mt, nullptr));
    return VCT_OK;
  }

  vct_status alloc(uint32_t r, int mip_mode, int storage, bool alpha_chains = true) {
    release();
    const int L = std::min(kMaxLevels, ilog2(r) + 1);
    const int nmaps = mip_mode == VCT_MIP_ISO ? 1 : (mip_mode == VCT_MIP_BOTH ? 7 : 6);
    const cudaChannelFormatDesc desc = storage == VCT_STORAGE_RGBA16F
                                           ? cudaCreateChannelDesc(16, 16, 16, 16, cudaChannelFormatKindFloat)
                                           : cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
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
    td.readMode = storage == VCT_STORAGE_RGBA16F ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
    td.normalizedCoords = 1;
    td.mipmapFilterMode = cudaFilterModeLinear;
    VCT_CUDA(cudaCreateTextureObject(&ms.l0_tex, &rd, &td, nullptr));
    for (int d = 0; d < nmaps && L > 1; ++d) VCT_CHECK(chain(r, L, desc, td, &dir_arr[d], ms.surf[d], &ms.tex[d]));
    if (alpha_chains && nmaps >= 6 && storage == VCT_STORAGE_RGBA8 && L > 1) {
      const cudaChannelFormatDesc d4 = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
      const cudaChannelFormatDesc d2 = cudaCreateChannelDesc(8, 8, 0, 0, cudaChannelFormatKindUnsigned);
      VCT_CHECK(chain(r, L, d4, td, &alpha_arr[0], ms.alpha_surf[0], &ms.alpha_tex[0]));
      VCT_CHECK(chain(r, L, d2, td, &alpha_arr[1], ms.alpha_surf[1], &ms.alpha_tex[1]));
    }
    ms.N = (int)r;
    ms.L = L;
    ms.nmaps = nmaps;
    ms.storage = storage;
    if (L > 1) {
      // occupancy: raw bytes for every level (the first pass writes levels
      // 1..occ_k, the tail passes the rest), packed and dilated bits
      ms.occ_k = std::min(L - 1, 4);
      ms.occ_l1_packed = L - 1 >= 4 ? 1 : 0;
      size_t bytes = 0;
      for (int c = 1; c < L; ++c) bytes += (size_t)(r >> c) * (r >> c) * (r >> c);
      bytes = (bytes + 255) & ~(size_t)255;
      const size_t raw_bytes = bytes;
      for (int c = 1; c < L; ++c) {
        const size_t s = r >> c;
        ms.occ_wpr[c] = (int)((s + 31) / 32);
        bytes += 3 * s * s * (size_t)ms.occ_wpr[c] * 4;  // packed + box + dilated
      }
      VCT_CUDA(cudaMalloc(&occ_mem, bytes));
      unsigned char* base = static_cast<unsigned char*>(occ_mem);
      size_t o = 0;
      for (int c = 1; c < L; ++c) {
        ms.occ_raw[c] = base + o;
        o += (size_t)(r >> c) * (r >> c) * (r >> c);
      }
      o = raw_bytes;
      for (int c = 1; c < L; ++c) {
        const size_t s = r >> c;
        ms.occ[c] = reinterpret_cast<uint32_t*>(base + o);
        o += s * s * (size_t)ms.occ_wpr[c] * 4;
        ms.occ_pack[c] = reinterpret_cast<uint32_t*>(base + o);
        o += s * s * (size_t)ms.occ_wpr[c] * 4;
        ms.occ3[c] = reinterpret_cast<uint32_t*>(base + o);
        o += s * s * (size_t)ms.occ_wpr[c] * 4;
      }
    }
    set_full_march(false);
    return VCT_OK;
  }

  // Cones stop 3/4 of the coarsest texel outside the grid and skip samples
  // in empty space (both exact), or march and sample every step.
  void set_full_march(bool full) {
    ms.skip_empty = (!full && occ_mem) ? 1 : 0;
    ms.exit_margin = full ? std::numeric_limits<float>::infinity() : 0.75f * (float)(1 << (ms.L - 1)) / (float)ms.N;
  }
};

struct vct_renderer {
  int W = 0, H = 0;
  vct_config cfg;
  // resources (renderer.h:168-171)
  std::vector<vct_material_data> materials;
  std::vector<vct_draw_obj> objs;
  std::vector<std::unique_ptr<Model>> models;
  uint64_t next_shader = 0;
  bool materials_dirty = true, objs_dirty = true;
  uint64_t scene_version = 0;  // bumped by every material / draw-object change
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
  cudaStream_t gb_stream = nullptr;  // G-buffer raster + learned diffuse term (lowest priority)
  cudaStream_t vx_stream = nullptr;  // voxelize + mipmap beside it (highest priority)
  cudaEvent_t ev_vjoin = nullptr;
  cudaEvent_t ev_start = nullptr;
  cudaEvent_t ev[5] = {};
  cudaEvent_t evg[3] = {};
  cudaEvent_t ev_join = nullptr;
  cudaEvent_t ev_staged = nullptr;
  cudaEvent_t ev_done = nullptr;   // after the frame's status copy
  MapStore maps;
  MapSet& ms = maps.ms;
  DevBuf<unsigned char> l0_lin;  // level 0 also in linear memory (the MipBuilder's TMA source)
  CUtensorMap l0_map;
  bool have_l0_map = false;
  DevBuf<uint8_t> brick_dirty;  // BrickMips::dirty
  bool dirty_unknown = true;
  DevBuf<vct_material_data> d_materials;
  DevBuf<uint32_t> d_obj_material;
  DevBuf<DevInstance> d_inst;
  HostBuf<DevInstance> h_inst;
  DevBuf<uint32_t> brick_count, brick_offset, brick_cursor, pair_list, scan_tmp, counts;
  DevBuf<BinRec> bin_big;           // large-triangle binning records
  DevBuf<uint2> bin_rec;            // per triangle: counting pass -> filling pass
  DevBuf<uint32_t> bin_big_count;
  uint32_t bin_big_cap = 0;
  HeavyStore heavy;                 // dense bricks split across CTAs
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
  // deferred light injection: attribute grids + the geometry they hold
  bool inject = false;
  cudaArray_t inj_arr[3] = {};
  InjGrids inj_g = {};
  std::vector<unsigned char> inj_key;
  bool inj_valid = false;
  bool last_revoxelized = true;
  // learned diffuse term
  int diffuse_mode = VCT_DIFFUSE_CONES;
  // The judge of the learned term: frames that evaluate the network also
  // trace the nine cones at one pixel per judge_stride^2 tile and compare;
  // below judge_min_psnr the frame is rendered again with the cones and
  // later frames keep the cones until the network is trained again.
  int judge_stride = 16;  // 8,100 judged pixels of a 1080p frame
  bool infer_ran = false;  // the last frame evaluated the learned term
  float judge_min_psnr = 40.0f;
  uint32_t judge_frame = 0;
  bool judge_pending = false;
  float judge_last_psnr = -1.0f;
  uint32_t judge_last_n = 0;
  uint32_t judge_fallbacks = 0;
  MlpState mlp;
  DevBuf<float4> diffuse_px;
  SceneParams last_sp;  // scene of the last encoded frame (training samples come from it)
  bool have_sp = false;

  ~vct_renderer() {
    if (gb_stream) cudaStreamSynchronize(gb_stream);
    if (vx_stream) cudaStreamSynchronize(vx_stream);
    if (stream) cudaStreamSynchronize(stream);
    free_maps();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : evg)
      if (e) cudaEventDestroy(e);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_vjoin) cudaEventDestroy(ev_vjoin);
    if (ev_staged) cudaEventDestroy(ev_staged);
    if (ev_done) cudaEventDestroy(ev_done);
    if (gb_stream) cudaStreamDestroy(gb_stream);
    if (vx_stream) cudaStreamDestroy(vx_stream);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  void free_maps() {
    maps.release();
    free_inj();
  }

  void free_inj() {
    cudaSurfaceObject_t* s[3] = {&inj_g.albedo, &inj_g.normal, &inj_g.emission};
    for (int k = 0; k < 3; ++k) {
      if (*s[k]) cudaDestroySurfaceObject(*s[k]);
      *s[k] = 0;
      if (inj_arr[k]) cudaFreeArray(inj_arr[k]);
      inj_arr[k] = nullptr;
    }
    inj_valid = false;
  }

  // The three RGBA8 attribute grids of light injection at the current grid.
  vct_status alloc_inj() {
    free_inj();
    const cudaChannelFormatDesc desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
    cudaSurfaceObject_t* s[3] = {&inj_g.albedo, &inj_g.normal, &inj_g.emission};
    for (int k = 0; k < 3; ++k) {
      VCT_CUDA(cudaMalloc3DArray(&inj_arr[k], &desc, make_cudaExtent(res, res, res), cudaArraySurfaceLoadStore));
      cudaResourceDesc rd;
      std::memset(&rd, 0, sizeof(rd));
      rd.resType = cudaResourceTypeArray;
      rd.res.array.array = inj_arr[k];
      VCT_CUDA(cudaCreateSurfaceObject(s[k], &rd));
    }
    return VCT_OK;
  }

  // What the attribute grids depend on: queued models and their matrices,
  // cube size, grid, coverage rule and the material / draw-object tables.
  std::vector<unsigned char> voxel_key(const FrameInputs& fi) const {
    std::vector<unsigned char> k;
    auto put = [&k](const void* p, size_t n) {
      const unsigned char* c = static_cast<const unsigned char*>(p);
      k.insert(k.end(), c, c + n);
    };
    for (const Queued& q : fi.queue) {
      put(&q.model, sizeof(q.model));
      put(q.M, sizeof(q.M));
    }
    put(&fi.cube_size, sizeof(fi.cube_size));
    put(&res, sizeof(res));
    put(&cfg.vox_mode, sizeof(cfg.vox_mode));
    put(&scene_version, sizeof(scene_version));
    return k;
  }

  // set_grid_resolution (renderer.cpp:178-188): six 3D textures of `levels`
  // mip levels.  Here: level 0 once + one chain (levels 1..L-1) per map.
  vct_status alloc_maps(uint32_t r) {
    if (gb_stream) VCT_CUDA(cudaStreamSynchronize(gb_stream));
    if (vx_stream) VCT_CUDA(cudaStreamSynchronize(vx_stream));
    if (stream) VCT_CUDA(cudaStreamSynchronize(stream));
    free_inj();
    VCT_CHECK(maps.alloc(r, cfg.mip_mode, cfg.storage, cfg.shadow_from_maps == 0 && cfg.sampler == VCT_SAMPLER_HW));
    maps.set_full_march(cfg.full_march != 0);
    const int L = ms.L;
    const uint32_t tb = cfg.storage == VCT_STORAGE_RGBA16F ? 8u : 4u;
    have_l0_map = false;
    dirty_unknown = true;
    if (r >= 16) {
      VCT_CHECK(l0_lin.ensure((size_t)r * r * r * tb));
      VCT_CHECK(encode_box_map(&l0_map, l0_lin.p, r, tb));
      have_l0_map = true;
    }
    res = r;
    levels = L;
    const size_t nb = (size_t)(r / kBrick) * (r / kBrick) * (r / kBrick);
    VCT_CHECK(brick_count.ensure(nb));
    VCT_CHECK(brick_offset.ensure(nb + 1));
    VCT_CHECK(brick_cursor.ensure(nb));
    VCT_CHECK(brick_dirty.ensure(nb));
    VCT_CHECK(scan_tmp.ensure(scan_tmp_words(nb)));
    VCT_CHECK(heavy.reserve(nb, 256, 16384, stream));
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
    // With overlap_raster the G-buffer raster fills what voxelize and
    // mipmap leave idle: their stream has the highest priority, the
    // raster's the lowest, so the stages that the metric times are delayed
    // as little as possible.
    int prio_least = 0, prio_greatest = 0;
    VCT_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    VCT_CUDA(cudaStreamCreateWithPriority(&gb_stream, cudaStreamNonBlocking, prio_least));
    VCT_CUDA(cudaStreamCreateWithPriority(&vx_stream, cudaStreamNonBlocking, prio_greatest));
    VCT_CUDA(cudaEventCreateWithFlags(&ev_vjoin, cudaEventDisableTiming));
    for (auto& e : ev) VCT_CUDA(cudaEventCreate(&e));
    for (auto& e : evg) VCT_CUDA(cudaEventCreate(&e));
    VCT_CUDA(cudaEventCreate(&ev_start));
    VCT_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
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
    VCT_CHECK(grow_bin_big(1 << 12));
    return alloc_maps((uint32_t)cfg.grid_res);
  }

  vct_status grow_bin_big(uint32_t cap) {
    VCT_CHECK(bin_big.ensure(cap));
    VCT_CHECK(bin_big_count.ensure(1));
    bin_big_cap = cap;
    return VCT_OK;
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
    sp.radiance_max = cfg.radiance_max > 0.0f ? cfg.radiance_max : 1.0f;
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
    VCT_CHECK(bin_rec.ensure(std::max<size_t>(total, 1)));

    VoxBuffers vb;
    vb.brick_count = brick_count.p;
    vb.brick_offset = brick_offset.p;
    vb.brick_cursor = brick_cursor.p;
    vb.pair_list = pair_list.p;
    vb.pair_cap = (uint32_t)pair_list.n;
    vb.scan_tmp = scan_tmp.p;
    vb.counts = cfg.keep_counts ? counts.p : nullptr;
    vb.status = d_status.p;
    vb.big = bin_big.p;
    vb.big_cap = bin_big_cap;
    vb.big_count = bin_big_count.p;
    vb.level0_lin = have_l0_map ? (void*)l0_lin.p : nullptr;
    vb.heavy = kHeavySplit ? heavy.view() : HeavyBricks{};
    vb.bin_rec = bin_rec.p;
    // Anisotropic maps: the brick kernel writes mip levels 1-3 itself (not
    // for light injection, whose level 0 comes from k_inject).
    BrickMips bm;
    std::memset(&bm, 0, sizeof(bm));
    const bool fuse = kFuseBrickMips && !inject && cfg.mip_mode == VCT_MIP_ANISO && ms.L >= 4;
    if (fuse) {
      for (int d = 0; d < 6; ++d)
        for (int l = 1; l <= 3; ++l) bm.surf[d][l] = ms.surf[d][l];
      bm.has_alpha = ms.alpha_tex[0] != 0;
      for (int k = 0; k < 2 && bm.has_alpha; ++k)
        for (int l = 1; l <= 3; ++l) bm.alpha[k][l] = ms.alpha_surf[k][l];
      for (int l = 1; l <= 3 && ms.skip_empty; ++l) bm.occ_raw[l] = ms.occ_raw[l];
      vb.mips = &bm;
      vb.level0_lin = nullptr;  // no TMA-staged first pass to read it
    } else {
      vb.mips = nullptr;
    }
    if (!inject) {
      if (dirty_unknown) {  // new maps, or light injection wrote level 0: every brick writes
        const size_t nb = (size_t)(res / kBrick) * (res / kBrick) * (res / kBrick);
        VCT_CUDA(cudaMemsetAsync(brick_dirty.p, 1, nb, stream));
        dirty_unknown = false;
      }
      vb.dirty = brick_dirty.p;
    } else {
      vb.dirty = nullptr;
      dirty_unknown = true;
    }

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
    VCT_CUDA(cudaEventRecord(ev_start, stream));
    // The G-buffer raster reads only the scene and the camera, and the
    // learned diffuse term only the G-buffer: with overlap_raster both run
    // on a second stream beside voxelize and mipmap, and the trace waits
    // for them.
    const bool side = cfg.overlap_raster != 0;
    cudaStream_t gs = side ? gb_stream : stream;
    if (side) VCT_CUDA(cudaStreamWaitEvent(gb_stream, ev_start, 0));
    VCT_CUDA(cudaEventRecord(evg[0], gs));
    VCT_CUDA(launch_gbuffer(sp, cp, rb, gs, &launches));
    VCT_CUDA(cudaEventRecord(evg[1], gs));
    TraceParams tp = fi.tp;
    tp.diffuse_in = nullptr;
    if (diffuse_mode == VCT_DIFFUSE_MLP && mlp.trained && tp.enable_diffuse && tp.view_voxel_dir >= 7) {
      // The learned term replaces the nine diffuse cones (its time counts as trace time).
      VCT_CHECK(diffuse_px.ensure((size_t)W * H));
      VCT_CUDA(launch_mlp_infer(mlp.params(), sp, gb_pos.p, gb_nrm.p, W * H, diffuse_px.p, gs, mlp.tc, d_status.p));
      ++launches;
      tp.diffuse_in = diffuse_px.p;
    }
    VCT_CUDA(cudaEventRecord(evg[2], gs));
    infer_ran = tp.diffuse_in != nullptr;
    if (side) VCT_CUDA(cudaEventRecord(ev_join, gb_stream));
    cudaStream_t vs = side ? vx_stream : stream;  // voxelize + mipmap
    if (side) VCT_CUDA(cudaStreamWaitEvent(vx_stream, ev_start, 0));
    VCT_CUDA(cudaEventRecord(ev[0], vs));
    if (inject) {
      // Re-voxelize the attribute grids only when the geometry changed;
      // light changes cost one injection pass.
      std::vector<unsigned char> key = voxel_key(fi);
      last_revoxelized = !inj_valid || key != inj_key;
      if (last_revoxelized) {
        if (!inj_arr[0]) VCT_CHECK(alloc_inj());
        VCT_CUDA(launch_voxelize(sp, (int)res, cfg.vox_mode, cfg.storage, vb, ms.l0_surf, vs, &launches,
                                 &inj_g));
        inj_key.swap(key);
        inj_valid = true;
      }
      VCT_CUDA(launch_inject(sp, (int)res, inj_g, ms.l0_surf, have_l0_map ? (uchar4*)l0_lin.p : nullptr, vs,
                             &launches));
    } else {
      last_revoxelized = true;
      VCT_CUDA(launch_voxelize(sp, (int)res, cfg.vox_mode, cfg.storage, vb, ms.l0_surf, vs, &launches));
    }
    VCT_CUDA(cudaEventRecord(ev[1], vs));
    if (fuse) {
      MapSet m3 = ms;
      m3.occ_k = 3;          // the levels whose occupancy bytes the brick kernel wrote
      m3.occ_l1_packed = 0;  // (as bytes)
      VCT_CUDA(launch_mipmap(m3, cfg.mip_mode, vs, &launches, nullptr, d_status.p, 3));
    } else {
      VCT_CUDA(launch_mipmap(ms, cfg.mip_mode, vs, &launches, have_l0_map ? &l0_map : nullptr, d_status.p));
    }
    VCT_CUDA(cudaEventRecord(ev[2], vs));
    if (side) {
      VCT_CUDA(cudaEventRecord(ev_vjoin, vx_stream));
      VCT_CUDA(cudaStreamWaitEvent(stream, ev_vjoin, 0));
      VCT_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
    }
    VCT_CUDA(cudaEventRecord(ev[3], stream));
    VCT_CUDA(launch_trace(sp, cp, ms, tp, gb_pos.p, gb_nrm.p, frame.p, cfg.keep_float_frame ? frame_f32.p : nullptr,
                          stream, &launches));
    judge_pending = tp.diffuse_in != nullptr && judge_stride > 0;
    if (judge_pending) {
      const int ox = (int)((judge_frame * 5u) % (uint32_t)judge_stride);
      const int oy = (int)((judge_frame * 3u) % (uint32_t)judge_stride);
      ++judge_frame;
      VCT_CUDA(launch_judge_diffuse(sp, cp, ms, tp, gb_pos.p, gb_nrm.p, tp.diffuse_in, judge_stride, ox, oy,
                                    d_status.p, stream));
      ++launches;
    }
    last_sp = sp;
    have_sp = true;
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
      if (s.async_timeout) return set_error(VCT_ERR_CUDA, "an asynchronous copy or tensor-core group did not complete");
      VCT_CHECK(heavy.grow(s, brick_count.n, stream));  // exact either way: no redo
      bool redo = false;
      if (s.pair_total > pair_list.n) {
        VCT_CHECK(pair_list.ensure((size_t)s.pair_total + s.pair_total / 4 + 4096));
        redo = true;
      }
      if (s.big_total > big_cap) {
        VCT_CHECK(grow_big(s.big_total + s.big_total / 4 + 1024));
        redo = true;
      }
      if (s.bigtri_total > bin_big_cap) {
        VCT_CHECK(grow_bin_big(s.bigtri_total + s.bigtri_total / 4 + 256));
        redo = true;
      }
      if (!redo && judge_pending) {
        judge_pending = false;
        if (s.judge_n) {
          const double mse = (double)s.judge_sse / (3.0 * s.judge_n);
          judge_last_psnr = mse > 0.0 ? (float)(10.0 * std::log10(1.0 / mse)) : 999.0f;
          judge_last_n = s.judge_n;
          if (judge_last_psnr < judge_min_psnr) {
            // the network no longer predicts its cones: fall back to them
            diffuse_mode = VCT_DIFFUSE_CONES;
            ++judge_fallbacks;
            redo = true;
          }
        }
      }
      if (!redo) return VCT_OK;
      if (!have_last) return VCT_OK;
      inj_valid = false;  // the attribute grids of the overflowed frame are incomplete
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
    tp.diffuse_in = nullptr;
    tp.far_share = cfg.far_share;
    tp.tile_rows = cfg.trace_tile_rows;
    return tp;
  }
};
