// vct_internal.h -- structures shared by the host renderer and the kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vct.h"

namespace vct {

constexpr int kMaxLights = 10;   // MAX_POINT_LIGHTS, voxelize.frag:40,128
constexpr int kMaxLevels = 7;    // create_tex_3d(res,res,res,7), renderer.cpp:186
constexpr int kBrick = 8;        // voxelizer brick edge (voxels)
constexpr int kMaxMaps = 7;  // six directional maps + the isotropic one (VCT_MIP_BOTH)
// Internal storage mode of the voxelizer: per-voxel attribute grids for
// deferred light injection instead of shaded level-0 radiance.
constexpr int kStorageAttr = 2;

// The attribute grids of light injection (RGBA8, N^3 each): mean albedo x
// transmittance + mean alpha; mean normal as 0.5 n + 0.5; mean emission x
// transmittance + occupancy flag (a = 1 where any triangle contributes).
struct InjGrids {
  cudaSurfaceObject_t albedo, normal, emission;
};

// One queued model instance of the frame (queue_model captures the model
// matrix, renderer.cpp:209-218).
struct DevInstance {
  float M[16];            // column-major model matrix
  float NM[9];            // mat3(transpose(inverse(M))), row-major
  uint32_t tri_base;      // first frame-global triangle id
  uint32_t n_tris;
  const vct_vert_data* verts;
  const uint32_t* indices;
  const uint32_t* tri_obj;  // per-triangle global draw-object id
  uint32_t n_verts;
  uint32_t pad;
};

// Scene data every stage reads; passed by value to kernels.
struct SceneParams {
  const DevInstance* inst;
  const vct_material_data* materials;
  const uint32_t* obj_material;   // draw object -> material id
  uint32_t n_obj;                 // entries of obj_material (0: ids not clamped)
  uint32_t n_instances;
  uint32_t total_tris;
  uint32_t n_materials;
  int32_t n_lights;
  float cube_size;
  float radiance_max;  // clamp of voxel radiance (1 = the reference's)
  vct_point_light lights[kMaxLights];
};

// Device-side status of one frame, copied to pinned host memory at the end.
struct FrameStatus {
  uint32_t pair_total;      // (triangle, brick) pairs needed
  uint32_t big_total;       // raster work records needed
  uint32_t big_tiles;       // raster tiles of the big-triangle pass
  uint32_t rejected_tris;   // non-finite / out-of-range triangles
  uint32_t count_saturated; // voxels with > 65535 contributions
  uint32_t bigtri_total;    // large-triangle binning records needed
  uint32_t async_timeout;   // a bounded wait for a bulk copy gave up (never expected)
  uint32_t heavy_total;     // dense bricks split across CTAs (accumulator slots needed)
  uint32_t extra_total;     // extra chunk work items of the split bricks
  uint32_t bad_ids;         // out-of-range vertex indices / material ids (device-side meshes)
  float judge_sse;          // learned diffuse term vs its nine cones: summed squared error
  uint32_t judge_n;         //   over this many judged pixels (3 channels each)
};

// Dense bricks: a brick with more than kHeavyChunk (triangle, brick) pairs
// is split into chunks of kHeavyChunk pairs processed by different CTAs of
// the same launch.  Every chunk adds its sums atomically into the brick's
// global accumulator slot (integer sums: exact and order-free); the CTA that
// finishes the last chunk (a per-slot counter) writes the brick's texels and
// zeroes the slot and its counter again, so slots are zero between frames.
// A brick that gets no slot (the lists are full) is processed whole by one
// CTA, which is also exact.
constexpr uint32_t kHeavyChunk = 1024;
#ifndef VCT_HEAVY_SPLIT
#define VCT_HEAVY_SPLIT 1  // build with -DVCT_HEAVY_SPLIT=0 to time whole-brick CTAs only
#endif
constexpr bool kHeavySplit = VCT_HEAVY_SPLIT != 0;
struct HeavyBricks {
  int32_t* slot;       // per brick: accumulator slot, -1 = one CTA takes the whole brick
  uint32_t* brick;     // per slot: its brick (0xffffffff = unused)
  uint32_t* done;      // per slot: chunks finished in this frame
  void* acc;           // per slot: the brick's sums (the voxelizer's accumulator type)
  uint2* items;        // (brick, chunk >= 1), (0xffffffff, 0) = unused
  uint32_t* counters;  // [0] slots taken, [1] items taken, [2] next item to run
  uint32_t slot_cap, item_cap;
};

// A triangle with many candidate bricks, binned by k_bin_big.
struct BinRec {
  float v[3][3];    // vertices in voxel units
  int blo[3], bhi[3];
  uint32_t t, vol;  // frame triangle id, candidate bricks
  uint32_t scene;   // scene of a batch (0 for one renderer)
  uint32_t pad;
};

// The voxel maps of a renderer: level 0 once, plus one chain per map.
struct MapSet {
  int N, L, nmaps, storage;
  cudaSurfaceObject_t l0_surf;
  cudaTextureObject_t l0_tex;                    // linear, normalized coords, border 0
  cudaSurfaceObject_t surf[kMaxMaps][kMaxLevels];  // level l >= 1 of map d
  cudaTextureObject_t tex[kMaxMaps];             // mipmapped chain (base = level 1)
  // Alpha-only copies of the six chains for shadow cones (anisotropic RGBA8;
  // 0 when absent): levels 1..L-1 of (a-x, a+x, a-y, a+y) as RGBA8 in
  // alpha_tex[0] and of (a-z, a+z) as RG8 in alpha_tex[1].
  cudaSurfaceObject_t alpha_surf[2][kMaxLevels];
  cudaTextureObject_t alpha_tex[2];
  // A cone moving away from the grid stops once its sample position is more
  // than this far outside [0,1] along that axis (+inf: never).
  float exit_margin;
  // Empty-space skipping (skip_empty != 0).  occ_raw[c], c = 2..K (K = the
  // levels of the MipBuilder's first pass; level 1 goes straight to
  // occ_pack): one byte per level-c cell, 1 when its block of 2^c level-0
  // voxels holds a non-zero texel.  occ_pack[c]: those bits packed along x
  // in occ_wpr[c] words per row; occ[c], c = 1..L-1: bit k = OR over the
  // 2x2x2 cells k..k+1 -- the texels a trilinear lookup at level c reads when
  // its lower texel is k (the finer level's texels lie inside them), so an
  // unset bit means the sample reads only zeros; occ3[c]: the OR over the
  // 3x3x3 cells around k (a cheaper, coarser test: the texels read lie within
  // one cell of floor(u * (N >> c))).
  int skip_empty;
  int occ_k;
  int occ_l1_packed;  // level 1 written as packed bits by the first pass (16^3 regions), not as bytes
  uint8_t* occ_raw[kMaxLevels];
  uint32_t* occ_pack[kMaxLevels];  // undilated occupancy bits (same layout as occ)
  uint32_t* occ[kMaxLevels];
  uint32_t* occ3[kMaxLevels];
  int occ_wpr[kMaxLevels];
};

// Levels 1-3 of the six RGBA8 directional chains written by the brick
// kernel itself (the MipBuilder then starts from level 3): the chains'
// surfaces, the alpha-only chains and the occupancy bytes of those levels.
#ifndef VCT_FUSE_BRICK_MIPS
#define VCT_FUSE_BRICK_MIPS 1  // -DVCT_FUSE_BRICK_MIPS=0: the MipBuilder builds every level
#endif
constexpr bool kFuseBrickMips = VCT_FUSE_BRICK_MIPS != 0;
struct BrickMips {
  cudaSurfaceObject_t surf[6][4];   // [map][level 1..3]
  cudaSurfaceObject_t alpha[2][4];  // [chain][level 1..3] (has_alpha)
  uint8_t* occ_raw[4];              // [level 1..3] (null: no occupancy)
  uint8_t* dirty;  // (set by launch_voxelize from VoxBuffers::dirty)
  int has_alpha;
};

struct VoxBuffers {
  uint32_t* brick_count;   // n_bricks
  uint32_t* brick_offset;  // n_bricks + 1
  uint32_t* brick_cursor;  // n_bricks
  uint32_t* pair_list;     // capacity
  uint32_t pair_cap;
  uint32_t* scan_tmp;      // block sums
  uint32_t* counts;        // N^3 or nullptr
  FrameStatus* status;
  BinRec* big;             // large-triangle records (nullptr: bin them in-warp)
  uint32_t big_cap;
  uint32_t* big_count;
  void* level0_lin;        // level 0 also in linear memory (x fastest), or null
  HeavyBricks heavy;       // dense-brick splitting (heavy.slot null: off)
  uint2* bin_rec;          // per triangle: the counting pass's bricks, replayed
                           // by the filling pass (total_tris; null: recompute)
  const BrickMips* mips;   // anisotropic maps: the brick kernel writes levels 1-3 too (null: off)
  // Per brick: 1 when its level-0 texels (and linear copy, and fused levels
  // 1-3 and occupancy bytes) may hold non-zero data from an earlier frame;
  // a brick empty in this frame and not dirty holds zeros already and
  // writes nothing.  Null: every brick writes.
  uint8_t* dirty;
};

struct RasterBuffers {
  unsigned long long* vis;  // W*H (depth bits << 32 | triangle id)
  void* big;                // raster work records
  uint32_t big_cap;
  uint32_t* big_count;      // [0] records, [1] tiles
  uint32_t* big_offset;     // tile prefix per record (big_cap + 1)
  uint32_t* scan_tmp;
  float4* gb_pos;           // world position, material id bits in .w
  float4* gb_nrm;           // world normal, triangle id bits in .w
  FrameStatus* status;
};

struct CameraParams {
  float PV[16];       // projection * view (FP32, fixed order)
  float cam_pos[3];   // column 3 of the view matrix (renderer.cpp:279)
  int W, H;
};

struct TraceParams {
  int enable_direct, enable_diffuse, enable_specular, enable_shadow;
  int view_voxel_dir;
  float view_voxel_lod;
  int cone_set;
  int sampler;
  int mip_mode;
  // Per-pixel trace_diffuse from the learned term (null: trace the cones).
  const float4* diffuse_in;
  // Texture-unit sampler: pixel groups share the far fields of their diffuse
  // cones (vct_config::far_share).
  int far_share;
  // Rows of a CTA's 16-pixel-wide tile of the shared-far-field tracer: 8,
  // 16 (0 means 16) or 32.  The frame is the same for every value.
  int tile_rows;
};

// ---- batched rendering (api_batch.cu) --------------------------------------
// One scene of a batch, device-resident.  Scenes own their voxel maps; the
// per-frame work arrays are batch-wide, each scene using the slice that
// starts at its base index.
struct BatchScene {
  SceneParams sp;
  MapSet ms;
  TraceParams tp;
  int N;
  int W, H;
  uint32_t brick_base;  // first brick in the batch-wide brick arrays
  uint32_t pad;
  size_t px_base;       // first pixel in the batch-wide vis / G-buffer / frame arrays
};

// Work of one batched launch: the scene of global work item g is the s with
// prefix[s] <= g < prefix[s + 1] (per-scene ranges padded so that a warp,
// or a CTA, never straddles two scenes).
struct BatchWork {
  const BatchScene* scenes;
  const CameraParams* cams;  // per scene (updated per frame)
  int n;
  const uint32_t* prefix;    // n + 1 entries
  uint32_t total;            // prefix[n]
  uint32_t* queue;           // dynamic scheduling counter (or null: static stride)
};

__device__ __forceinline__ int batch_scene_of(const BatchWork& w, uint32_t g) {
  int lo = 0, hi = w.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(w.prefix + mid) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// batch_scene_of for a whole warp (all 32 lanes): the lanes test 32 scenes'
// prefixes at a time, so the lookup takes one round of loads per 32 scenes
// instead of a chain of dependent loads.  The prefixes are non-decreasing,
// so the scene is the number of prefixes <= g, minus one.
__device__ __forceinline__ int batch_scene_of_warp(const BatchWork& w, uint32_t g) {
  const int lane = threadIdx.x & 31;
  int count = 0;
  for (int base = 0; base < w.n; base += 32) {
    const int i = base + lane;
    const uint32_t m = __ballot_sync(0xffffffffu, i < w.n && __ldg(w.prefix + i) <= g);
    count += __popc(m);
    if (m != 0xffffffffu) break;  // warp-uniform
  }
  return count - 1;
}

// Batch-wide work arrays.
struct BatchBuffers {
  uint32_t* brick_count;
  uint32_t* brick_offset;
  uint32_t* brick_cursor;
  uint32_t* pair_list;
  uint32_t pair_cap;
  BinRec* big;
  uint32_t big_cap;
  uint32_t* big_count;
  FrameStatus* status;
  RasterBuffers rb;       // vis / gb_pos / gb_nrm point at pixel 0 of the batch
  uchar4* frame;
  HeavyBricks heavy;      // over the batch-wide (global) brick indices
  uint2* bin_rec;         // per (padded) batch triangle, as VoxBuffers::bin_rec
  uint8_t* dirty;         // per batch brick (global index), as VoxBuffers::dirty
  const BrickMips* mips;  // per scene: the brick kernel writes levels 1-3 too (null: off)
};

// Tunable launch shapes of the batched kernels (chosen by the autotuner).
struct BatchShape {
  int bin_ctas_per_sm;
  int bricks_ctas_per_sm;
  int trace_ctas_per_sm;
  int trace_dynamic;   // 1: tiles from an atomic queue; 0: static stride
  int trace_per_scene; // 1: one launch of the one-scene trace kernel per scene
  int trace_tile_rows; // 8, 16 or 32: CTA tile rows of the per-scene shared-far-field trace
};

// ---- learned diffuse term (k_mlp.cu) --------------------------------------
constexpr int kMlpLevels = 16;
constexpr int kMlpWeights = 5 * 64 * 64;  // W1..W4 64x64, W5 16x64 (padded to 64 rows)

struct MlpParams {
  const void* table_bf;     // [levels][2^log2_table] bf16 feature pairs
  float2* table_grad;       // [levels][2^log2_table] (training)
  const __nv_bfloat16* w_bf;  // [5][64][64] [out][in]
  float* w_grad;            // [5][64][64] (training)
  int log2_table;
  int dense_mask;           // bit l: level l is indexed densely
  int res[kMlpLevels];      // grid resolution of each level
};

// A training batch: rows of 12 floats (texture-space position, normal,
// albedo, target RGB), `n` rows starting at row `first` (mod `total`).
struct MlpBatch {
  const float* samples;
  int first, n, total;
};

struct AdamStep {
  float lr, beta1, beta2, eps, c1, c2, l2;  // c1 = 1/(1-beta1^t), c2 = 1/(1-beta2^t)
};

// ---- launchers (stream-ordered, no host synchronisation) ----------------
// `launches` (may be null) is incremented by the number of kernels enqueued.
// With `inj` the voxelizer writes the attribute grids instead of level 0.
cudaError_t launch_voxelize(const SceneParams& sp, int N, int mode, int storage, const VoxBuffers& vb,
                            cudaSurfaceObject_t l0, cudaStream_t st, int* launches, const InjGrids* inj = nullptr);
// Deferred light injection: level 0 (RGBA8) from the attribute grids and the
// scene's lights.
cudaError_t launch_inject(const SceneParams& sp, int N, const InjGrids& g, cudaSurfaceObject_t l0, uchar4* l0_lin,
                          cudaStream_t st, int* launches);
// The voxelizer writing RGBA8 level 0 to linear memory (x fastest).
cudaError_t launch_voxelize_linear(const SceneParams& sp, int N, int mode, const VoxBuffers& vb, uchar4* out,
                                   cudaStream_t st);
// `tmap` (a CUtensorMap over the linear level 0, or null): the first pass
// stages level 0 through TMA bulk-tensor copies; `status` receives timeouts.
// first_level 3: levels 1-3 are already written (BrickMips; then ms.occ_k
// must be 3, the levels whose occupancy bytes the brick kernel wrote).
cudaError_t launch_mipmap(const MapSet& ms, int mip_mode, cudaStream_t st, int* launches, const void* tmap = nullptr,
                          FrameStatus* status = nullptr, int first_level = 0);
cudaError_t launch_gbuffer(const SceneParams& sp, const CameraParams& cp, const RasterBuffers& rb,
                           cudaStream_t st, int* launches);
cudaError_t launch_trace(const SceneParams& sp, const CameraParams& cp, const MapSet& ms, const TraceParams& tp,
                         const float4* gb_pos, const float4* gb_nrm, uchar4* frame, float4* frame_f32,
                         cudaStream_t st, int* launches);
// Exclusive scan of n u32 values into out[0..n] (out[n] = total); tmp must
// hold scan_tmp_words(n) words.
size_t scan_tmp_words(size_t n);
// Work fused into the exclusive scan of the brick counts (no launches of
// its own): the dense-brick plan, one brick per thread of the add-back
// kernel, and a copy of the total.
struct ScanFuse {
  HeavyBricks hb;        // hb.slot null: no plan
  uint32_t cap;          // pair-list capacity (offsets beyond it are clamped)
  uint32_t slots;        // CTAs of the brick launch resident at once
  uint32_t* total_copy;  // also receives the total (or null)
};
cudaError_t launch_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t* copy_out, size_t n, uint32_t* tmp,
                                  cudaStream_t st, int* launches = nullptr, const ScanFuse* fuse = nullptr);

// The split plan of brick b with pairs [beg, end) of `pairs` in all: the
// brick is dense when it has more than kHeavyChunk pairs and more than the
// launch's pairs per resident CTA (a lighter brick cannot hold up the
// launch's end).  A dense brick gets an accumulator slot and one work item
// per extra chunk of kHeavyChunk pairs; every brick's slot is written (-1:
// not split).  A brick whose slot or items do not fit is left whole.
// counters[0..1] count the dense bricks and their extra chunks (all of
// them, also those that did not fit).
__device__ __forceinline__ void heavy_plan_brick(uint32_t b, uint32_t beg, uint32_t end, uint32_t pairs,
                                                 uint32_t slots, const HeavyBricks& hb) {
  const unsigned long long fair = ((unsigned long long)pairs + slots - 1) / (slots ? slots : 1u);
  const uint32_t dense = fair > kHeavyChunk ? (fair > 0xffffffffull ? 0xffffffffu : (uint32_t)fair) : kHeavyChunk;
  int32_t slot = -1;
  if (end - beg > dense) {
    const uint32_t nch = (end - beg + kHeavyChunk - 1) / kHeavyChunk;
    const uint32_t s = atomicAdd(&hb.counters[0], 1u);
    const uint32_t e = atomicAdd(&hb.counters[1], nch - 1);
    const bool ok = s < hb.slot_cap && e + (nch - 1) <= hb.item_cap;
    if (s < hb.slot_cap) hb.brick[s] = ok ? b : 0xffffffffu;
    for (uint32_t j = 1; j < nch; ++j)
      if (e + j - 1 < hb.item_cap) hb.items[e + j - 1] = ok ? make_uint2(b, j) : make_uint2(0xffffffffu, 0u);
    if (ok) slot = (int32_t)s;
  }
  hb.slot[b] = slot;
}
// Texture3D helpers.
cudaError_t launch_fill_rgba8(cudaSurfaceObject_t s, int w, int h, int d, uchar4 v, cudaStream_t st);
cudaError_t launch_box_mip_rgba8(cudaSurfaceObject_t src, int sw, int sh, int sd, cudaSurfaceObject_t dst, int dw,
                                 int dh, int dd, cudaStream_t st);

size_t big_record_bytes();
// Bytes of one dense-brick accumulator slot for a storage mode.
size_t heavy_slot_bytes(int storage);

// Batched stages (one launch per pass over all scenes of a batch).
cudaError_t launch_voxelize_batch(const BatchWork& tris, const BatchWork& bricks, uint32_t total_bricks, int mode,
                                  int storage, const BatchBuffers& bb, uint32_t* scan_tmp, const BatchShape& shape,
                                  int sms, cudaStream_t st, int* launches);
// Dilated occupancy words of a map set (0 without empty-space skipping) and
// their batch pass (one work item per word of every scene).
uint32_t occupancy_words(const MapSet& ms);
cudaError_t launch_occupancy_batch(const BatchWork& words, cudaStream_t st, int* launches);
// regions: the first pass's 16^3 regions of level 0 (levels 1-4; empty when
// the brick kernel wrote levels 1-3); tail[t]: the texels of level
// first_tail + t of every scene.
cudaError_t launch_mipmap_batch(const BatchWork& regions, const BatchWork* tail, int n_tail, int first_tail,
                                int storage, cudaStream_t st, int* launches);
cudaError_t launch_gbuffer_batch(const BatchWork& tris, const BatchWork& tiles, size_t total_px,
                                 const BatchBuffers& bb, int sms, cudaStream_t st, int* launches);
// share: every scene shares the far fields of its diffuse cones (the batch's
// far_share; k_trace_batch_share).
cudaError_t launch_trace_batch(const BatchWork& tiles, const BatchBuffers& bb, const BatchShape& shape, int sms,
                               cudaStream_t st, int* launches, bool share);

// Learned diffuse term.
cudaError_t launch_mlp_init(float* prm, __nv_bfloat16* prm_bf, size_t n, float scale, uint64_t seed, cudaStream_t st);
cudaError_t launch_mlp_train(const MlpParams& p, const MlpBatch& b, float* loss, cudaStream_t st);
cudaError_t launch_adam(float* prm, float* grad, float* m, float* v, __nv_bfloat16* prm_bf, size_t n,
                        const AdamStep& a, cudaStream_t st);
// Inference / evaluation of the network: on the 5th-generation tensor cores
// (tcgen05.mma, TMEM accumulators) when `tc`, else in mma.sync warp tiles.
cudaError_t launch_mlp_infer(const MlpParams& p, const SceneParams& sp, const float4* gb_pos, const float4* gb_nrm,
                             int n_px, float4* out, cudaStream_t st, bool tc, FrameStatus* status);
cudaError_t launch_mlp_eval(const MlpParams& p, const float* samples, int n, float* out, cudaStream_t st, bool tc,
                            FrameStatus* status);
// Training data: world-space area of every queued triangle; surface samples
// drawn from the area CDF (rows of 12 floats, see MlpBatch); their
// cone-traced diffuse targets (trace_diffuse with the texture-unit sampler).
cudaError_t launch_tri_area(const SceneParams& sp, float* area, cudaStream_t st);
cudaError_t launch_sample_surface(const SceneParams& sp, const float* cdf, int n, uint64_t seed, float* samples,
                                  cudaStream_t st);
// The judge of the learned diffuse term: at one pixel of every stride x
// stride tile (tile offset (ox, oy)), trace_diffuse's cones against the
// network's value in `net`; adds the squared error and the pixel count to
// status->judge_sse / judge_n.
cudaError_t launch_judge_diffuse(const SceneParams& sp, const CameraParams& cp, const MapSet& ms, const TraceParams& tp,
                                 const float4* gb_pos, const float4* gb_nrm, const float4* net, int stride, int ox,
                                 int oy, FrameStatus* status, cudaStream_t st);
cudaError_t launch_trace_points(const SceneParams& sp, const MapSet& ms, int mip_mode, int cone_set, float* samples,
                                int n, cudaStream_t st);

}  // namespace vct
