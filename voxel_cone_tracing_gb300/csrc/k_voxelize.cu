// k_voxelize.cu -- the Voxelizer: replaces voxelize.vert/.geom/.frag and the
// level-0 clear of Renderer::voxelize (renderer.cpp:316-353).
//
// Pipeline (all stream-ordered, no host synchronisation):
//   1. k_bin<false>: every queued triangle -> the 8^3-voxel bricks its
//      (margin-expanded) box test says it may touch; per-brick counts.
//   2. exclusive scan of the counts -> per-brick list offsets.
//   3. k_bin<true>: scatter triangle ids into the per-brick lists.
//   4. k_bricks: one CTA per brick.  Warps take 32 triangles at a time, set
//      them up in shared memory, expand (triangle, sample|voxel) work items
//      across lanes, decide coverage with the exact rule of the selected mode,
//      shade in FP32 (voxelize.frag:124-153) and add fixed-point colour sums
//      and counts into shared-memory accumulators.  The CTA then writes its
//      whole brick of level 0 (empty voxels = 0, which is the clear) as RGBA8
//      or RGBA16F through a surface -- level 0 is written exactly once.
//
// Coverage rules (the CPU oracle implements the same ones):
//   REF_RASTER2X -- the reference's method: dominant-axis projection
//     (voxelize.geom:27-51) rasterised on the 2N x 2N viewport
//     (renderer.cpp:339-340): vertices snapped to 1/256 sample pixel,
//     integer edge functions, top-left fill rule; sample depth = FP32
//     barycentric interpolation, voxel = int(N*(0.5*c+0.5)) (voxelize.frag
//     :156-157, truncation).
//   CONSERVATIVE -- exact separating-axis triangle/box test on vertices
//     snapped to 1/256 voxel (int64, the plane test in int128), colour at
//     the triangle point closest to the voxel centre.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <climits>
#include <type_traits>

#include "vct_internal.h"
#include "vct_math.cuh"
#include "vct_mip.cuh"
#include "vct_snap.h"

namespace vct {
namespace {

#ifndef VCT_BRICK_THREADS
#define VCT_BRICK_THREADS 128
#endif
constexpr int kThreads = VCT_BRICK_THREADS;  // threads of a brick CTA
constexpr int kWarps = kThreads / 32;
#ifndef VCT_BRICK_BALANCE
#define VCT_BRICK_BALANCE 1
#endif
// 1: a brick CTA spreads each round's samples over all its threads (a scan
// over the round's pairs); 0: each warp expands the samples of its own pairs.
constexpr bool kBrickBalance = VCT_BRICK_BALANCE != 0;
#ifndef VCT_BRICK_ROUND
#define VCT_BRICK_ROUND 0
#endif
// Pairs per round of the balanced expansion (0: one per thread); their
// triangle setups are the larger part of a brick CTA's shared memory.
constexpr int kRound = VCT_BRICK_ROUND > 0 ? VCT_BRICK_ROUND : kThreads;
static_assert(kRound % 32 == 0 && kRound <= kThreads, "round of whole warps, at most one pair per thread");
constexpr int kSetupSlots = kBrickBalance ? kRound : kThreads;
constexpr int kExclSlots = kBrickBalance ? kRound : kWarps * 33;
#ifndef VCT_BRICK_MIN_BLOCKS
#define VCT_BRICK_MIN_BLOCKS 0
#endif
// Resident brick CTAs per SM the kernels are compiled for (0: the default
// per coverage rule).  Both rules keep 7 per SM (30 KB of shared memory
// each); the conservative rule's kernel is held to the 72 registers that 7
// allow (unbounded it takes 98 and fits 5: 512^3 voxelize 1.47 -> 1.75 ms).
// Measured with 64-pair rounds (20 KB) at 8-10 per SM: the 512^3 raster
// rule gains 5%, the bench frame and the batch lose 4-8%.
template <int MODE>
constexpr int brick_min_blocks() {
  return VCT_BRICK_MIN_BLOCKS > 0 ? VCT_BRICK_MIN_BLOCKS : (MODE == VCT_VOX_CONSERVATIVE ? 7 : 1);
}
constexpr int kBrickVox = kBrick * kBrick * kBrick;
constexpr float kBinMargin = 0.25f;   // voxels; >> snapping and FP32 error
constexpr float kFix = 65535.0f;      // fixed-point scale of one contribution

// ------------------------------------------------------------ triangle load --
__device__ __forceinline__ int find_instance(const SceneParams& sp, uint32_t t) {
  int lo = 0, hi = (int)sp.n_instances - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sp.inst[mid].tri_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct TriLoad {
  float g[3][3];   // grid-space positions (voxelize.vert:26), FP32 fixed order
  V3 n[3];         // normalize(NM * normal) (voxelize.vert:28)
  uint32_t mat;
  bool ok;
};

template <bool NORMALS>
__device__ __forceinline__ void load_tri(const SceneParams& sp, uint32_t t, TriLoad& tl) {
  const DevInstance& in = sp.inst[find_instance(sp, t)];
  const uint32_t lt = t - in.tri_base;
  tl.ok = true;
  for (int k = 0; k < 3; ++k) {
    // Indices and material ids of host-side meshes are checked when they are
    // loaded; those of caller-owned device meshes are clamped here (and
    // counted by the caller's entry point), so that no id reads out of bounds.
    const uint32_t vi = min(__ldg(in.indices + 3 * (size_t)lt + k), in.n_verts - 1u);
    const float4* vp = reinterpret_cast<const float4*>(in.verts + vi);
    const float4 a = __ldg(vp), b = __ldg(vp + 1);
    for (int r = 0; r < 3; ++r) {
      float w = xform_row(in.M, r, a.x, a.y, a.z);
      float gv = rdiv(w, sp.cube_size);
      tl.g[k][r] = gv;
      if (!(fabsf(gv) <= 64.0f)) tl.ok = false;
    }
    if (NORMALS) tl.n[k] = normalize(nm_mul(in.NM, a.w, b.x, b.y));
  }
  if (NORMALS) tl.mat = __ldg(sp.obj_material + min(__ldg(in.tri_obj + lt), sp.n_obj - 1u));
}

// ------------------------------------------------ conservative brick test --
// Triangle / axis-aligned box overlap in FP32 (box normals, plane, 9 edge
// axes).  Only used for binning, with boxes grown by kBinMargin, so FP32
// rounding can only add candidates.
__device__ bool tri_box_f32(const float v[3][3], const float c[3], const float h[3]) {
  float u[3][3];
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) u[k][d] = v[k][d] - c[d];
  for (int d = 0; d < 3; ++d) {
    float mn = fminf(u[0][d], fminf(u[1][d], u[2][d])), mx = fmaxf(u[0][d], fmaxf(u[1][d], u[2][d]));
    if (mn > h[d] || mx < -h[d]) return false;
  }
  float f[3][3];
  for (int d = 0; d < 3; ++d) {
    f[0][d] = u[1][d] - u[0][d];
    f[1][d] = u[2][d] - u[1][d];
    f[2][d] = u[0][d] - u[2][d];
  }
  float n0 = f[0][1] * f[1][2] - f[0][2] * f[1][1];
  float n1 = f[0][2] * f[1][0] - f[0][0] * f[1][2];
  float n2 = f[0][0] * f[1][1] - f[0][1] * f[1][0];
  float dd = n0 * u[0][0] + n1 * u[0][1] + n2 * u[0][2];
  float rr = h[0] * fabsf(n0) + h[1] * fabsf(n1) + h[2] * fabsf(n2);
  if (fabsf(dd) > rr * 1.0001f + 1e-6f) return false;
  for (int e = 0; e < 3; ++e) {
    const float fx = f[e][0], fy = f[e][1], fz = f[e][2];
    float p0, p1, p2, r;
    p0 = -fz * u[0][1] + fy * u[0][2]; p1 = -fz * u[1][1] + fy * u[1][2]; p2 = -fz * u[2][1] + fy * u[2][2];
    r = h[1] * fabsf(fz) + h[2] * fabsf(fy);
    if (fminf(p0, fminf(p1, p2)) > r * 1.0001f || fmaxf(p0, fmaxf(p1, p2)) < -r * 1.0001f) return false;
    p0 = fz * u[0][0] - fx * u[0][2]; p1 = fz * u[1][0] - fx * u[1][2]; p2 = fz * u[2][0] - fx * u[2][2];
    r = h[0] * fabsf(fz) + h[2] * fabsf(fx);
    if (fminf(p0, fminf(p1, p2)) > r * 1.0001f || fmaxf(p0, fmaxf(p1, p2)) < -r * 1.0001f) return false;
    p0 = -fy * u[0][0] + fx * u[0][1]; p1 = -fy * u[1][0] + fx * u[1][1]; p2 = -fy * u[2][0] + fx * u[2][1];
    r = h[0] * fabsf(fy) + h[1] * fabsf(fx);
    if (fminf(p0, fminf(p1, p2)) > r * 1.0001f || fmaxf(p0, fmaxf(p1, p2)) < -r * 1.0001f) return false;
  }
  return true;
}

// One (triangle, candidate brick) test of the binning passes.
template <bool FILL>
__device__ __forceinline__ bool bin_one(const float v[3][3], int bx, int by, int bz, int nb, bool test, uint32_t t,
                                        uint32_t* __restrict__ count, uint32_t* __restrict__ cursor,
                                        uint32_t* __restrict__ list, uint32_t cap) {
  if (test) {
    const int b3[3] = {bx, by, bz};
    float c[3], h[3];
    for (int d = 0; d < 3; ++d) {
      float lo = (float)(b3[d] * kBrick) - kBinMargin - (b3[d] == 0 ? 1.0f : 0.0f);
      float hi = (float)(b3[d] * kBrick + kBrick) + kBinMargin;
      c[d] = 0.5f * (lo + hi);
      h[d] = 0.5f * (hi - lo);
    }
    if (!tri_box_f32(v, c, h)) return false;
  }
  const uint32_t brick = ((uint32_t)bz * nb + by) * nb + bx;
  if (FILL) {
    uint32_t slot = atomicAdd(cursor + brick, 1u);
    if (slot < cap) list[slot] = t;
  } else {
    atomicAdd(count + brick, 1u);
  }
  return true;
}

constexpr int kSoloBricks = 8;  // candidate bricks a lane bins on its own
constexpr int kBigSplit = 8;     // CTAs that share one large triangle
// Bin record of a triangle (counting pass -> filling pass): x = first
// candidate brick (10 bits per axis), y = bits 0-7 which of its (at most
// kSoloBricks) candidates passed the triangle/box test, bits 8-16 the
// candidate extents - 1 (3 bits per axis), bit 31 = bin it again in the
// filling pass (triangles the warp bins together).  Triangles of large-
// triangle records and rejected ones have no bricks here.
constexpr uint32_t kRecAgain = 1u << 31;

// Bins every triangle to the bricks it may touch.  A lane handles its own
// triangle when it has few candidate bricks.  A triangle with more
// candidates (room walls span 1024 bricks at 256^3) is recorded by the
// counting pass in `big` and binned by k_bin_big, which spreads each record
// over several CTAs; without a record list (or when it is full) the warp
// bins it, the lanes splitting the candidate range.
// All 32 lanes of a warp call it together (each with its own triangle t of
// the same scene; t >= total_tris is an idle lane).
template <bool FILL>
__device__ __forceinline__ void bin_tri(const SceneParams& sp, int N, uint32_t t, uint32_t* __restrict__ count,
                                        uint32_t* __restrict__ cursor, uint32_t* __restrict__ list, uint32_t cap,
                                        FrameStatus* st, BinRec* __restrict__ big, uint32_t big_cap,
                                        uint32_t* __restrict__ big_count, uint32_t scene, uint2* __restrict__ rec) {
  const int lane = threadIdx.x & 31;
  const int nb = N / kBrick;
  float v[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
  int blo[3] = {0, 0, 0}, bhi[3] = {-1, -1, -1};
  int vol = 0;
  bool again = true;  // (filling pass) this lane's triangle is binned from scratch
  if (FILL && rec && t < sp.total_tris) {
    // Replay the counting pass's bricks (same pairs, no triangle reload).
    const uint2 r = rec[t];
    again = (r.y & kRecAgain) != 0u;
    if (!again) {
      const int x0 = (int)(r.x & 1023u), y0 = (int)((r.x >> 10) & 1023u), z0 = (int)(r.x >> 20);
      const int ex = (int)((r.y >> 8) & 7u) + 1, ey = (int)((r.y >> 11) & 7u) + 1;
      for (uint32_t m = r.y & 0xffu; m; m &= m - 1) {
        const int i = __ffs(m) - 1;
        const uint32_t brick = ((uint32_t)(z0 + i / (ex * ey)) * nb + (uint32_t)(y0 + (i / ex) % ey)) * nb +
                               (uint32_t)(x0 + i % ex);
        const uint32_t slot = atomicAdd(cursor + brick, 1u);
        if (slot < cap) list[slot] = t;
      }
    }
  }
  if (again && t < sp.total_tris) {
    TriLoad tl;
    load_tri<false>(sp, t, tl);
    if (!tl.ok) {
      if (!FILL) atomicAdd(&st->rejected_tris, 1u);
    } else {
      const float hv = 0.5f * (float)N;
      for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) v[k][d] = (tl.g[k][d] + 1.0f) * hv;  // voxel units
      bool inside = true;
      for (int d = 0; d < 3; ++d) {
        float lo = fminf(v[0][d], fminf(v[1][d], v[2][d])) - kBinMargin;
        float hi = fmaxf(v[0][d], fmaxf(v[1][d], v[2][d])) + kBinMargin;
        // Depth values in (-1, 0) voxel still land in voxel 0 (int() truncates).
        if (hi <= -1.0f - kBinMargin || lo >= (float)N) inside = false;
        blo[d] = max(0, (int)floorf(lo / kBrick));
        bhi[d] = min(nb - 1, (int)floorf(fmaxf(hi, 0.0f) / kBrick));
      }
      if (inside && bhi[0] >= blo[0] && bhi[1] >= blo[1] && bhi[2] >= blo[2])
        vol = (bhi[0] - blo[0] + 1) * (bhi[1] - blo[1] + 1) * (bhi[2] - blo[2] + 1);
    }
  }
  if (vol > 0 && vol <= kSoloBricks) {
    uint32_t mask = 0u;
    int i = 0;
    for (int bz = blo[2]; bz <= bhi[2]; ++bz)
      for (int by = blo[1]; by <= bhi[1]; ++by)
        for (int bx = blo[0]; bx <= bhi[0]; ++bx, ++i)
          if (bin_one<FILL>(v, bx, by, bz, nb, vol > 1, t, count, cursor, list, cap)) mask |= 1u << i;
    if (!FILL && rec)
      rec[t] = make_uint2((uint32_t)blo[0] | (uint32_t)blo[1] << 10 | (uint32_t)blo[2] << 20,
                          mask | (uint32_t)(bhi[0] - blo[0]) << 8 | (uint32_t)(bhi[1] - blo[1]) << 11 |
                              (uint32_t)(bhi[2] - blo[2]) << 14);
  } else if (!FILL && rec && t < sp.total_tris) {
    // no bricks, or a large triangle: binned by its record (k_bin_big) or by the warp
    rec[t] = make_uint2(0u, vol > kSoloBricks && !big ? kRecAgain : 0u);
  }
  bool in_warp = vol > kSoloBricks;
  if (in_warp && big) {
    // Counting pass records it; the filling pass leaves it to k_bin_big.
    // A full record list is reported (big_total > big_cap) and the frame is
    // encoded again with a larger one.
    in_warp = false;
    if (!FILL) {
      const uint32_t slot = atomicAdd(big_count, 1u);
      if (slot < big_cap) {
        BinRec r;
        for (int k = 0; k < 3; ++k)
          for (int d = 0; d < 3; ++d) r.v[k][d] = v[k][d];
        for (int d = 0; d < 3; ++d) { r.blo[d] = blo[d]; r.bhi[d] = bhi[d]; }
        r.t = t;
        r.vol = (uint32_t)vol;
        r.scene = scene;
        r.pad = 0;
        big[slot] = r;
      }
    }
  }
  unsigned warp_big = __ballot_sync(0xffffffffu, in_warp);
  while (warp_big) {
    const int src = __ffs(warp_big) - 1;
    warp_big &= warp_big - 1;
    float w[3][3];
    for (int k = 0; k < 3; ++k)
      for (int d = 0; d < 3; ++d) w[k][d] = __shfl_sync(0xffffffffu, v[k][d], src);
    const int x0 = __shfl_sync(0xffffffffu, blo[0], src), y0 = __shfl_sync(0xffffffffu, blo[1], src);
    const int z0 = __shfl_sync(0xffffffffu, blo[2], src);
    const int nx = __shfl_sync(0xffffffffu, bhi[0], src) - x0 + 1;
    const int ny = __shfl_sync(0xffffffffu, bhi[1], src) - y0 + 1;
    const int n = __shfl_sync(0xffffffffu, vol, src);
    const uint32_t ts = __shfl_sync(0xffffffffu, t, src);
    for (int i = lane; i < n; i += 32)
      bin_one<FILL>(w, x0 + i % nx, y0 + (i / nx) % ny, z0 + i / (nx * ny), nb, true, ts, count, cursor, list, cap);
  }
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_bin(SceneParams sp, int N, uint32_t* __restrict__ count,
                                             uint32_t* __restrict__ cursor, uint32_t* __restrict__ list,
                                             uint32_t cap, FrameStatus* st, BinRec* __restrict__ big,
                                             uint32_t big_cap, uint32_t* __restrict__ big_count,
                                             uint2* __restrict__ rec) {
  bin_tri<FILL>(sp, N, blockIdx.x * blockDim.x + threadIdx.x, count, cursor, list, cap, st, big, big_cap, big_count,
                0u, rec);
}

// Every scene's triangles in one persistent launch; scene triangle ranges
// are padded to multiples of 32, so a warp bins one scene.
template <bool FILL>
__global__ void __launch_bounds__(256) k_bin_batch(BatchWork w, BatchBuffers bb) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < w.total; g += gridDim.x * blockDim.x) {
    const int s = batch_scene_of(w, g);
    const BatchScene& S = w.scenes[s];
    const uint32_t t = g - __ldg(w.prefix + s);
    bin_tri<FILL>(S.sp, S.N, t, FILL ? nullptr : bb.brick_count + S.brick_base,
                  FILL ? bb.brick_cursor + S.brick_base : nullptr, bb.pair_list, bb.pair_cap, bb.status, bb.big,
                  bb.big_cap, bb.big_count, (uint32_t)s,
                  bb.bin_rec ? bb.bin_rec + (g - t) : nullptr);
  }
}

// Large-triangle records: CTA (x, y) takes records x, x + gridDim.x, ... and
// the candidate bricks y*256 + tid, stepping by kBigSplit*256.  With
// `scenes` (a batch) each record bins into its own scene's brick slice.
template <bool FILL>
__global__ void __launch_bounds__(256) k_bin_big(int N, const BinRec* __restrict__ big, uint32_t big_cap,
                                                 const uint32_t* __restrict__ big_count, uint32_t* __restrict__ count,
                                                 uint32_t* __restrict__ cursor, uint32_t* __restrict__ list,
                                                 uint32_t cap, const BatchScene* __restrict__ scenes) {
  const uint32_t n = min(*big_count, big_cap);
  for (uint32_t r = blockIdx.x; r < n; r += gridDim.x) {
    const BinRec& rec = big[r];
    int nb = N / kBrick;
    uint32_t* cnt = count;
    uint32_t* cur = cursor;
    if (scenes) {
      const BatchScene& S = scenes[rec.scene];
      nb = S.N / kBrick;
      if (cnt) cnt += S.brick_base;
      if (cur) cur += S.brick_base;
    }
    float v[3][3];
    for (int k = 0; k < 3; ++k)
      for (int d = 0; d < 3; ++d) v[k][d] = rec.v[k][d];
    const int nx = rec.bhi[0] - rec.blo[0] + 1, ny = rec.bhi[1] - rec.blo[1] + 1;
    for (uint32_t i = blockIdx.y * blockDim.x + threadIdx.x; i < rec.vol; i += gridDim.y * blockDim.x)
      bin_one<FILL>(v, rec.blo[0] + (int)(i % nx), rec.blo[1] + (int)((i / nx) % ny), rec.blo[2] + (int)(i / (nx * ny)),
                    nb, true, rec.t, cnt, cur, list, cap);
  }
}

// ------------------------------------------------------------- shading -----
// voxelize.frag:124-153 in FP32.
__device__ __forceinline__ float4 voxel_color(const SceneParams& sp, const vct_material_data& m, V3 pos, V3 nrm) {
  V3 color = v3(0.f, 0.f, 0.f);
  const V3 nn = normalize(nrm);
  const int nl = min(sp.n_lights, kMaxLights);
  for (int i = 0; i < nl; ++i) {
    const vct_point_light& L = sp.lights[i];
    const V3 lp = v3(L.position[0] / sp.cube_size, L.position[1] / sp.cube_size, L.position[2] / sp.cube_size);
    const V3 dl = lp - pos;
    const V3 dir = normalize(dl);
    const float d = length(dl);
    const float a = 1.0f / (1.0f + d * d);  // attenuate(1, 0, 1, d)
    const float cs = fmaxf(dot(nn, dir), 0.0f);
    color = color + v3(L.color[0], L.color[1], L.color[2]) * (cs * a * L.intensity);
  }
  color = mulv(v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]), color) + v3(m.emission[0], m.emission[1], m.emission[2]);
  float alpha = 1.0f;
  if (m.illum == 4 || m.illum == 6 || m.illum == 7 || m.illum == 9) {
    color = mulv(color, v3(m.transmittance[0], m.transmittance[1], m.transmittance[2]));
    alpha = m.dissolve;
  }
  // clamp(vec4, 0, 1) (voxelize.frag:153); with HDR storage the colour clamps to
  // [0, radiance_max] instead (radiance_max = 1 is the reference).
  const float hi = sp.radiance_max;
  return make_float4(fminf(fmaxf(color.x, 0.0f), hi), fminf(fmaxf(color.y, 0.0f), hi),
                     fminf(fmaxf(color.z, 0.0f), hi), clamp01(alpha));
}

// Per-brick sums of the contributions.  RGBA8: 16-bit fixed point per
// contribution in u32 (exact for the 1/255 result).  RGBA16F: the colour
// divided by radiance_max in 32-bit fixed point, summed in u64, so the sum
// is exact, order-independent and far finer than half precision.  Attribute
// grids (light injection): ten unorm channels in 16-bit fixed point.
template <int STORAGE> struct AccT;
// A value of the global accumulator copy, read past L1 and zeroed.
template <class T>
__device__ __forceinline__ T take_cg(T& g) {
  const T v = __ldcg(&g);
  g = 0;
  return v;
}
// atomic_add_to: voxel i of these sums added into a global copy (the
// accumulator slot of a split brick); take_from: voxel i of the global copy
// read from L2 into these sums and zeroed there.
template <> struct AccT<VCT_STORAGE_RGBA8> {
  uint32_t c[4][kBrickVox];
  uint32_t n[kBrickVox];
  __device__ __forceinline__ void clear(int i) { c[0][i] = 0; c[1][i] = 0; c[2][i] = 0; c[3][i] = 0; n[i] = 0; }
  __device__ __forceinline__ void take_from(AccT& g, int i) {
    for (int k = 0; k < 4; ++k) c[k][i] = take_cg(g.c[k][i]);
    n[i] = take_cg(g.n[i]);
  }
  __device__ __forceinline__ void atomic_add_to(AccT& g, int i) const {
    if (!n[i]) return;
    for (int k = 0; k < 4; ++k)
      if (c[k][i]) atomicAdd(&g.c[k][i], c[k][i]);
    atomicAdd(&g.n[i], n[i]);
  }
  __device__ __forceinline__ void add(const SceneParams& sp, int v, const vct_material_data& m, V3 p, V3 nrm) {
    const float4 col = voxel_color(sp, m, p, nrm);
    atomicAdd(&c[0][v], __float2uint_rn(col.x * kFix));
    atomicAdd(&c[1][v], __float2uint_rn(col.y * kFix));
    atomicAdd(&c[2][v], __float2uint_rn(col.z * kFix));
    atomicAdd(&c[3][v], __float2uint_rn(col.w * kFix));
    atomicAdd(&n[v], 1u);
  }
};
template <> struct AccT<VCT_STORAGE_RGBA16F> {
  unsigned long long c[4][kBrickVox];
  uint32_t n[kBrickVox];
  __device__ __forceinline__ void clear(int i) { c[0][i] = 0; c[1][i] = 0; c[2][i] = 0; c[3][i] = 0; n[i] = 0; }
  __device__ __forceinline__ void take_from(AccT& g, int i) {
    for (int k = 0; k < 4; ++k) c[k][i] = take_cg(g.c[k][i]);
    n[i] = take_cg(g.n[i]);
  }
  __device__ __forceinline__ void atomic_add_to(AccT& g, int i) const {
    if (!n[i]) return;
    for (int k = 0; k < 4; ++k)
      if (c[k][i]) atomicAdd(&g.c[k][i], c[k][i]);
    atomicAdd(&g.n[i], n[i]);
  }
  __device__ __forceinline__ void add(const SceneParams& sp, int v, const vct_material_data& m, V3 p, V3 nrm) {
    const float4 col = voxel_color(sp, m, p, nrm);
    const float k = 4294967296.0f / sp.radiance_max;
    atomicAdd(&c[0][v], __float2ull_rn(col.x * k));
    atomicAdd(&c[1][v], __float2ull_rn(col.y * k));
    atomicAdd(&c[2][v], __float2ull_rn(col.z * k));
    atomicAdd(&c[3][v], __float2ull_rn(col.w * 4294967296.0f));
    atomicAdd(&n[v], 1u);
  }
};
// Light-injection attributes of one contribution (the factors of
// voxelize.frag:141-153 that do not depend on the lights): colour =
// t * (diffuse * lighting + emission), t = transmittance for transparent
// materials, else 1.
__device__ __forceinline__ void voxel_attrs(const vct_material_data& m, V3 nrm, float a[10]) {
  const bool tr = m.illum == 4 || m.illum == 6 || m.illum == 7 || m.illum == 9;
  const V3 t = tr ? v3(m.transmittance[0], m.transmittance[1], m.transmittance[2]) : v3(1.f, 1.f, 1.f);
  const V3 nn = normalize(nrm);
  a[0] = clamp01(m.diffuse[0] * t.x);
  a[1] = clamp01(m.diffuse[1] * t.y);
  a[2] = clamp01(m.diffuse[2] * t.z);
  a[3] = tr ? clamp01(m.dissolve) : 1.0f;
  a[4] = clamp01(0.5f * nn.x + 0.5f);
  a[5] = clamp01(0.5f * nn.y + 0.5f);
  a[6] = clamp01(0.5f * nn.z + 0.5f);
  a[7] = clamp01(m.emission[0] * t.x);
  a[8] = clamp01(m.emission[1] * t.y);
  a[9] = clamp01(m.emission[2] * t.z);
}
template <> struct AccT<kStorageAttr> {
  uint32_t c[10][kBrickVox];
  uint32_t n[kBrickVox];
  __device__ __forceinline__ void clear(int i) {
#pragma unroll
    for (int k = 0; k < 10; ++k) c[k][i] = 0;
    n[i] = 0;
  }
  __device__ __forceinline__ void take_from(AccT& g, int i) {
    for (int k = 0; k < 10; ++k) c[k][i] = take_cg(g.c[k][i]);
    n[i] = take_cg(g.n[i]);
  }
  __device__ __forceinline__ void atomic_add_to(AccT& g, int i) const {
    if (!n[i]) return;
    for (int k = 0; k < 10; ++k)
      if (c[k][i]) atomicAdd(&g.c[k][i], c[k][i]);
    atomicAdd(&g.n[i], n[i]);
  }
  __device__ __forceinline__ void add(const SceneParams&, int v, const vct_material_data& m, V3, V3 nrm) {
    float a[10];
    voxel_attrs(m, nrm, a);
#pragma unroll
    for (int k = 0; k < 10; ++k) atomicAdd(&c[k][v], __float2uint_rn(a[k] * kFix));
    atomicAdd(&n[v], 1u);
  }
};

// Mean of n 16-bit fixed-point contributions summing to c, as unorm8
// rounded to nearest (ties up).
__device__ __forceinline__ unsigned char unorm8_mean(uint32_t c, uint32_t n) {
  const unsigned long long v = ((unsigned long long)c * 510ull + (unsigned long long)n * 65535ull) /
                               (2ull * n * 65535ull);
  return (unsigned char)(v > 255ull ? 255ull : v);
}
typedef AccT<VCT_STORAGE_RGBA8> Acc;

// -------------------------------------------------- reference raster mode --
struct SetupRef {
  long long area;
  int A[3], B[3];
  float c[3];
  float farea;
  V3 gp[3], gn[3];
  uint32_t mat;
  int axis, tl;
  int i0, ni, j0, nj;
};

// Returns the number of samples of this triangle inside the brick's columns.
__device__ int setup_ref(const SceneParams& sp, int N, uint32_t t, const int b3[3], SetupRef& s) {
  TriLoad tl;
  load_tri<true>(sp, t, tl);
  if (!tl.ok) return 0;
  // Dominant axis, voxelize.geom:27-51 (FP32, fixed order).
  float e1[3], e2[3];
  for (int i = 0; i < 3; ++i) { e1[i] = rsub(tl.g[1][i], tl.g[0][i]); e2[i] = rsub(tl.g[2][i], tl.g[0][i]); }
  const float px = fabsf(rsub(rmul(e1[1], e2[2]), rmul(e2[1], e1[2])));
  const float py = fabsf(rsub(rmul(e1[2], e2[0]), rmul(e2[2], e1[0])));
  const float pz = fabsf(rsub(rmul(e1[0], e2[1]), rmul(e2[0], e1[1])));
  int axis;
  if (pz > px && pz > py) axis = 2;
  else if (px > py && px > pz) axis = 0;
  else axis = 1;
  const int ia = axis == 2 ? 0 : (axis == 0 ? 1 : 0);
  const int ib = axis == 2 ? 1 : 2;
  // Vertices snapped to 1/256 sample: round((g + 1) * N * 256), exactly,
  // in integer arithmetic (N is a power of two; vct_snap.h).
  const int shift = __ffs(N) - 1 + 8;
  int idx[3] = {0, 1, 2};
  long long A[3], B[3];
  float c[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = snap_fixed(tl.g[k][ia], shift);
    B[k] = snap_fixed(tl.g[k][ib], shift);
    c[k] = tl.g[k][axis];
  }
  long long area = (A[1] - A[0]) * (B[2] - B[0]) - (B[1] - B[0]) * (A[2] - A[0]);
  if (area == 0) return 0;
  if (area < 0) {
    long long tA = A[1]; A[1] = A[2]; A[2] = tA;
    long long tB = B[1]; B[1] = B[2]; B[2] = tB;
    float tc = c[1]; c[1] = c[2]; c[2] = tc;
    idx[1] = 2; idx[2] = 1;
    area = -area;
  }
  // Sample window: the triangle's sample bbox inside the brick's columns.
  const long long minA = min(A[0], min(A[1], A[2])), maxA = max(A[0], max(A[1], A[2]));
  const long long minB = min(B[0], min(B[1], B[2])), maxB = max(B[0], max(B[1], B[2]));
  const int sa0 = 2 * kBrick * b3[ia], sb0 = 2 * kBrick * b3[ib];
  const long long i0 = max((long long)sa0, ceil_div(minA - 128, 256));
  const long long i1 = min((long long)sa0 + 2 * kBrick - 1, floor_div(maxA - 128, 256));
  const long long j0 = max((long long)sb0, ceil_div(minB - 128, 256));
  const long long j1 = min((long long)sb0 + 2 * kBrick - 1, floor_div(maxB - 128, 256));
  if (i1 < i0 || j1 < j0) return 0;
  s.area = area;
  s.farea = __ll2float_rn(area);
  for (int k = 0; k < 3; ++k) {
    s.A[k] = (int)A[k];
    s.B[k] = (int)B[k];
    s.c[k] = c[k];
    const int o = idx[k];
    s.gp[k] = v3(tl.g[o][0], tl.g[o][1], tl.g[o][2]);
    s.gn[k] = tl.n[o];
  }
  s.tl = (top_left(A[1], B[1], A[2], B[2]) ? 1 : 0) | (top_left(A[2], B[2], A[0], B[0]) ? 2 : 0) |
         (top_left(A[0], B[0], A[1], B[1]) ? 4 : 0);
  s.mat = tl.mat;
  s.axis = axis;
  s.i0 = (int)i0; s.ni = (int)(i1 - i0 + 1);
  s.j0 = (int)j0; s.nj = (int)(j1 - j0 + 1);
  return s.ni * s.nj;
}

template <class A>
__device__ __forceinline__ void item_ref(const SceneParams& sp, int N, const int b3[3], const SetupRef& s, int local,
                                         A& acc) {
  const int i = s.i0 + local % s.ni, j = s.j0 + local / s.ni;
  const long long sx = 256LL * i + 128, sy = 256LL * j + 128;
  const long long w0 = edge_fn(s.A[1], s.B[1], s.A[2], s.B[2], sx, sy);
  const long long w1 = edge_fn(s.A[2], s.B[2], s.A[0], s.B[0], sx, sy);
  const long long w2 = edge_fn(s.A[0], s.B[0], s.A[1], s.B[1], sx, sy);
  if (!(w0 > 0 || (w0 == 0 && (s.tl & 1)))) return;
  if (!(w1 > 0 || (w1 == 0 && (s.tl & 2)))) return;
  if (!(w2 > 0 || (w2 == 0 && (s.tl & 4)))) return;
  const float b1 = rdiv(__ll2float_rn(w1), s.farea), b2 = rdiv(__ll2float_rn(w2), s.farea);
  float cz = radd(s.c[0], rmul(b1, rsub(s.c[1], s.c[0])));
  cz = radd(cz, rmul(b2, rsub(s.c[2], s.c[0])));
  const float Nf = (float)N;
  const float t = rmul(Nf, radd(rmul(0.5f, cz), 0.5f));
  if (!(t > -1.0f && t < Nf)) return;
  const int kd = __float2int_rz(t);
  int vx, vy, vz;
  if (s.axis == 2) { vx = i >> 1; vy = j >> 1; vz = kd; }
  else if (s.axis == 0) { vx = kd; vy = i >> 1; vz = j >> 1; }
  else { vx = i >> 1; vy = kd; vz = j >> 1; }
  const int lx = vx - b3[0] * kBrick, ly = vy - b3[1] * kBrick, lz = vz - b3[2] * kBrick;
  if ((unsigned)lx >= (unsigned)kBrick || (unsigned)ly >= (unsigned)kBrick || (unsigned)lz >= (unsigned)kBrick) return;
  const float l0 = __ll2float_rn(w0) / s.farea, l1 = __ll2float_rn(w1) / s.farea, l2 = __ll2float_rn(w2) / s.farea;
  const V3 p = s.gp[0] * l0 + s.gp[1] * l1 + s.gp[2] * l2;
  const V3 n = s.gn[0] * l0 + s.gn[1] * l1 + s.gn[2] * l2;
  acc.add(sp, (lz * kBrick + ly) * kBrick + lx, sp.materials[s.mat], p, n);
}

// ---------------------------------------------------- conservative mode ----
struct SetupSat {
  int V[3][3];
  V3 gp[3], gn[3];
  uint32_t mat;
  int x0, nx, y0, ny, z0, nz;
};

__device__ int setup_sat(const SceneParams& sp, int N, uint32_t t, const int b3[3], SetupSat& s) {
  TriLoad tl;
  load_tri<true>(sp, t, tl);
  if (!tl.ok) return 0;
  // Vertices snapped to 1/256 voxel: round((g + 1) * N * 128), exactly, in
  // integer arithmetic (N is a power of two; vct_snap.h).
  const int shift = __ffs(N) - 1 + 7;
  int lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    long long mn = LLONG_MAX, mx = LLONG_MIN;
    for (int k = 0; k < 3; ++k) {
      long long q = snap_fixed(tl.g[k][d], shift);
      s.V[k][d] = (int)q;
      mn = min(mn, q);
      mx = max(mx, q);
    }
    lo[d] = (int)max((long long)b3[d] * kBrick, ceil_div(mn, 256) - 1);
    hi[d] = (int)min((long long)b3[d] * kBrick + kBrick - 1, floor_div(mx, 256));
    if (hi[d] < lo[d]) return 0;
  }
  for (int k = 0; k < 3; ++k) {
    s.gp[k] = v3(tl.g[k][0], tl.g[k][1], tl.g[k][2]);
    s.gn[k] = tl.n[k];
  }
  s.mat = tl.mat;
  s.x0 = lo[0]; s.nx = hi[0] - lo[0] + 1;
  s.y0 = lo[1]; s.ny = hi[1] - lo[1] + 1;
  s.z0 = lo[2]; s.nz = hi[2] - lo[2] + 1;
  return s.nx * s.ny * s.nz;
}

__device__ __forceinline__ bool axis_sep(long long p0, long long p1, long long p2, long long r) {
  return min(p0, min(p1, p2)) > r || max(p0, max(p1, p2)) < -r;
}

// Exact closed-box SAT on integer coordinates (1/256 voxel units).
__device__ bool sat_exact(const int V[3][3], long long cx, long long cy, long long cz, long long h) {
  long long u[3][3];
  const long long c[3] = {cx, cy, cz};
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) u[k][d] = (long long)V[k][d] - c[d];
  for (int d = 0; d < 3; ++d) {
    long long mn = min(u[0][d], min(u[1][d], u[2][d])), mx = max(u[0][d], max(u[1][d], u[2][d]));
    if (mn > h || mx < -h) return false;
  }
  long long f[3][3];
  for (int d = 0; d < 3; ++d) {
    f[0][d] = u[1][d] - u[0][d];
    f[1][d] = u[2][d] - u[1][d];
    f[2][d] = u[0][d] - u[2][d];
  }
  const long long n0 = f[0][1] * f[1][2] - f[0][2] * f[1][1];
  const long long n1 = f[0][2] * f[1][0] - f[0][0] * f[1][2];
  const long long n2 = f[0][0] * f[1][1] - f[0][1] * f[1][0];
  const __int128 dd = (__int128)n0 * u[0][0] + (__int128)n1 * u[0][1] + (__int128)n2 * u[0][2];
  const __int128 rr = (__int128)h * ((__int128)llabs(n0) + (__int128)llabs(n1) + (__int128)llabs(n2));
  if (dd > rr || dd < -rr) return false;
  for (int e = 0; e < 3; ++e) {
    const long long fx = f[e][0], fy = f[e][1], fz = f[e][2];
    if (axis_sep(-fz * u[0][1] + fy * u[0][2], -fz * u[1][1] + fy * u[1][2], -fz * u[2][1] + fy * u[2][2],
                 h * (llabs(fz) + llabs(fy))))
      return false;
    if (axis_sep(fz * u[0][0] - fx * u[0][2], fz * u[1][0] - fx * u[1][2], fz * u[2][0] - fx * u[2][2],
                 h * (llabs(fz) + llabs(fx))))
      return false;
    if (axis_sep(-fy * u[0][0] + fx * u[0][1], -fy * u[1][0] + fx * u[1][1], -fy * u[2][0] + fx * u[2][1],
                 h * (llabs(fy) + llabs(fx))))
      return false;
  }
  return true;
}

// Barycentric weights of the closest triangle point to p (Voronoi-region
// classification of vertices, edges and face).
__device__ void closest_bary(V3 p, V3 a, V3 b, V3 c, float w[3]) {
  const V3 ab = b - a, ac = c - a, ap = p - a;
  const float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) { w[0] = 1.f; w[1] = 0.f; w[2] = 0.f; return; }
  const V3 bp = p - b;
  const float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.f && d4 <= d3) { w[0] = 0.f; w[1] = 1.f; w[2] = 0.f; return; }
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
    const float den = d1 - d3, v = den != 0.f ? d1 / den : 0.f;
    w[0] = 1.f - v; w[1] = v; w[2] = 0.f; return;
  }
  const V3 cp = p - c;
  const float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.f && d5 <= d6) { w[0] = 0.f; w[1] = 0.f; w[2] = 1.f; return; }
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
    const float den = d2 - d6, t = den != 0.f ? d2 / den : 0.f;
    w[0] = 1.f - t; w[1] = 0.f; w[2] = t; return;
  }
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
    const float den = (d4 - d3) + (d5 - d6), t = den != 0.f ? (d4 - d3) / den : 0.f;
    w[0] = 0.f; w[1] = 1.f - t; w[2] = t; return;
  }
  const float sum = va + vb + vc;
  if (!(sum != 0.f)) { w[0] = 1.f; w[1] = 0.f; w[2] = 0.f; return; }
  const float v = vb / sum, t = vc / sum;
  w[0] = 1.f - v - t; w[1] = v; w[2] = t;
}

template <class A>
__device__ __forceinline__ void item_sat(const SceneParams& sp, int N, const int b3[3], const SetupSat& s, int local,
                                         A& acc) {
  const int x = s.x0 + local % s.nx;
  const int y = s.y0 + (local / s.nx) % s.ny;
  const int z = s.z0 + local / (s.nx * s.ny);
  if (!sat_exact(s.V, 256LL * x + 128, 256LL * y + 128, 256LL * z + 128, 128)) return;
  const float inv = 2.0f / (float)N;
  const V3 vc = v3(((float)x + 0.5f) * inv - 1.0f, ((float)y + 0.5f) * inv - 1.0f, ((float)z + 0.5f) * inv - 1.0f);
  float w[3];
  closest_bary(vc, s.gp[0], s.gp[1], s.gp[2], w);
  const V3 p = s.gp[0] * w[0] + s.gp[1] * w[1] + s.gp[2] * w[2];
  const V3 n = s.gn[0] * w[0] + s.gn[1] * w[1] + s.gn[2] * w[2];
  const int lx = x - b3[0] * kBrick, ly = y - b3[1] * kBrick, lz = z - b3[2] * kBrick;
  acc.add(sp, (lz * kBrick + ly) * kBrick + lx, sp.materials[s.mat], p, n);
}

// ------------------------------------------------------------ brick CTA ----
template <int MODE>
using SetupOf = typename std::conditional<MODE == VCT_VOX_CONSERVATIVE, SetupSat, SetupRef>::type;

// Accumulates the (triangle, brick) pairs list[beg, end) of the brick at b3
// into acc (all threads of the CTA; cleared first, barrier at the end).
template <int MODE, int STORAGE>
__device__ __forceinline__ void brick_accumulate(const SceneParams& sp, int N, const int b3[3],
                                                 const uint32_t* __restrict__ list, uint32_t beg, uint32_t end,
                                                 AccT<STORAGE>& acc, SetupOf<MODE> (&setup)[kSetupSlots],
                                                 int (&excl)[kExclSlots]) {
  for (int i = threadIdx.x; i < kBrickVox; i += kThreads) acc.clear(i);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if constexpr (kBrickBalance) {
    // Rounds of up to kRound pairs: one setup per thread, an exclusive
    // scan of the pairs' sample counts, then every thread expands samples
    // it, it + kThreads, ... of the round (a triangle covering the whole
    // brick does not hold up one warp while the others wait).
    __shared__ int s_wsum[kWarps];
    SetupOf<MODE>* su = setup;
    int* ex = excl;
    for (uint32_t b0 = beg; b0 < end; b0 += kRound) {
      const uint32_t n = min((uint32_t)kRound, end - b0);
      int cnt = 0;
      if ((uint32_t)threadIdx.x < n) {
        if (MODE == VCT_VOX_CONSERVATIVE)
          cnt = setup_sat(sp, N, __ldg(list + b0 + threadIdx.x), b3, reinterpret_cast<SetupSat&>(su[threadIdx.x]));
        else
          cnt = setup_ref(sp, N, __ldg(list + b0 + threadIdx.x), b3, reinterpret_cast<SetupRef&>(su[threadIdx.x]));
      }
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      int off = 0, total = 0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        const int v = s_wsum[w];
        off += w < warp ? v : 0;
        total += v;
      }
      if (threadIdx.x < kRound) ex[threadIdx.x] = off + incl - cnt;
      __syncthreads();
      for (int it = threadIdx.x; it < total; it += kThreads) {
        int lo = 0, hi = (int)n - 1;  // owner = last pair with ex <= it
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ex[mid] <= it) lo = mid; else hi = mid - 1;
        }
        const int local = it - ex[lo];
        if (MODE == VCT_VOX_CONSERVATIVE)
          item_sat(sp, N, b3, reinterpret_cast<const SetupSat&>(su[lo]), local, acc);
        else
          item_ref(sp, N, b3, reinterpret_cast<const SetupRef&>(su[lo]), local, acc);
      }
      __syncthreads();  // the round's setups and offsets are free again
    }
  } else {
    // Rounds of up to kWarps * 32 pairs, split evenly between the warps (a
    // brick with a few dozen pairs keeps every warp busy expanding samples).
    for (uint32_t b0 = beg; b0 < end; b0 += kWarps * 32) {
      const uint32_t n = min((uint32_t)(kWarps * 32), end - b0);
      const uint32_t q = (n + kWarps - 1) / kWarps;
      const uint32_t k = warp * q + lane;
      const uint32_t e = b0 + k;
      int cnt = 0;
      if (lane < q && k < n) {
        if (MODE == VCT_VOX_CONSERVATIVE)
          cnt = setup_sat(sp, N, __ldg(list + e), b3, reinterpret_cast<SetupSat&>(setup[warp * 32 + lane]));
        else
          cnt = setup_ref(sp, N, __ldg(list + e), b3, reinterpret_cast<SetupRef&>(setup[warp * 32 + lane]));
      }
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      excl[warp * 33 + lane] = incl - cnt;
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      __syncwarp();
      for (int it = lane; it < total; it += 32) {
        int lo = 0, hi = 31;  // owner = last lane with excl <= it
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (excl[warp * 33 + mid] <= it) lo = mid; else hi = mid - 1;
        }
        const int local = it - excl[warp * 33 + lo];
        if (MODE == VCT_VOX_CONSERVATIVE)
          item_sat(sp, N, b3, reinterpret_cast<const SetupSat&>(setup[warp * 32 + lo]), local, acc);
        else
          item_ref(sp, N, b3, reinterpret_cast<const SetupRef&>(setup[warp * 32 + lo]), local, acc);
      }
      __syncwarp();
    }
    __syncthreads();
  }
}

// ---- fused mip levels 1-3 (six maps, RGBA8 or RGBA16F; BrickMips) ---------
// The brick holds whole 4^3, 2^3 and 1^3 blocks of levels 1-3, so its CTA
// writes them from its level-0 texels in shared memory with the MipBuilder's
// rule (vct_mip.cuh: exact integers for RGBA8, one fixed FP32 evaluation for
// RGBA16F), plus the alpha-only chains (RGBA8) and the occupancy bytes of
// those levels (a cell is occupied when its block of level 0 holds a
// non-zero texel); the MipBuilder then starts from level 3.  This replaces
// the first pass's re-read of level 0 (and the linear copy it read).
template <int STORAGE>
struct BrickMipScratchT {
  typedef typename std::conditional<STORAGE == VCT_STORAGE_RGBA16F, uint2, uint32_t>::type T;
  T l0[kBrick * kBrick * kBrick];
  T l1[6][64];
  T l2[6][8];
  T l3[6];
  uint8_t occ1[64];
  uint8_t occ2[8];
};
typedef BrickMipScratchT<VCT_STORAGE_RGBA8> BrickMipScratch;
__device__ __forceinline__ bool texel_nonzero(uint32_t v) { return v != 0u; }
__device__ __forceinline__ bool texel_nonzero(uint2 v) { return (v.x | v.y) != 0u; }

__device__ __forceinline__ void brick_alpha(const BrickMips& bm, int level, int x, int y, int z, const uint32_t* v,
                                            int stride) {
  surf3Dwrite(make_uchar4(v[0] >> 24, v[stride] >> 24, v[2 * stride] >> 24, v[3 * stride] >> 24),
              bm.alpha[0][level], x * 4, y, z);
  surf3Dwrite(make_uchar2(v[4 * stride] >> 24, v[5 * stride] >> 24), bm.alpha[1][level], x * 2, y, z);
}

__device__ __forceinline__ void brick_occ(const BrickMips& bm, int N, int level, int x, int y, int z, bool any) {
  if (!bm.occ_raw[level]) return;
  const int s = N >> level;
  bm.occ_raw[level][((size_t)z * s + y) * s + x] = any ? 1 : 0;
}

// Texel (x, y, z), map d, of the level above a cube of side s2 stored
// [z][y][x] at src (shared memory): one out-of-line copy of the rule for
// all three levels.
__device__ __noinline__ uint32_t brick_mip_texel(const uint32_t* src, int s2, int x, int y, int z, int d) {
  return aniso_rgba8_dir(d, [&](int k) { return src[mip_child(s2, x, y, z, k)]; });
}
__device__ __noinline__ uint2 brick_mip_texel(const uint2* src, int s2, int x, int y, int z, int d) {
  return aniso_rgba16f_dir(d, [&](int k) { return src[mip_child(s2, x, y, z, k)]; });
}

// Levels 1-3 of brick b3 from scr.l0 ([z][y][x], written and synchronised
// by the caller); all threads of the CTA.  Level 1 takes the whole CTA, one
// (texel, map) item per thread with the map a run-time index, so that the
// rule's code exists once (six unrolled copies made the kernel miss its
// instruction cache); levels 2 and 3 (48 and 6 items) and their occupancy
// and alpha copies are one warp's, which synchronises only itself.
template <int STORAGE>
__device__ void brick_mips(const BrickMips& bm, int N, const int b3[3], BrickMipScratchT<STORAGE>& scr) {
  static_assert(kThreads >= 96, "levels 2-3 are warp 2's");
  typedef typename BrickMipScratchT<STORAGE>::T T;
  constexpr int kB = sizeof(T);  // bytes per texel
  const int t = threadIdx.x;
  for (int i = t; i < 6 * 64; i += kThreads) {  // level 1: map i / 64 (warp-uniform), texel i % 64
    const int d = i >> 6, r = i & 63, x = r & 3, y = (r >> 2) & 3, z = r >> 4;
    const T v = brick_mip_texel(scr.l0, 8, x, y, z, d);
    surf3Dwrite(v, bm.surf[d][1], (b3[0] * 4 + x) * kB, b3[1] * 4 + y, b3[2] * 4 + z);
    scr.l1[d][r] = v;
  }
  if (t < 64) {  // occupancy of level 1: the texel's block of level 0
    const int x = t & 3, y = (t >> 2) & 3, z = t >> 4;
    bool any = false;
#pragma unroll
    for (int k = 0; k < 8; ++k) any |= texel_nonzero(scr.l0[mip_child(8, x, y, z, k)]);
    scr.occ1[t] = any ? 1 : 0;
    brick_occ(bm, N, 1, b3[0] * 4 + x, b3[1] * 4 + y, b3[2] * 4 + z, any);
  }
  __syncthreads();
  if (t < 64) {
    if constexpr (STORAGE == VCT_STORAGE_RGBA8)
      if (bm.has_alpha) brick_alpha(bm, 1, b3[0] * 4 + (t & 3), b3[1] * 4 + ((t >> 2) & 3), b3[2] * 4 + (t >> 4),
                                    &scr.l1[0][t], 64);
    return;
  }
  if (t >= 96) return;
  const int lane = t - 64;
  for (int j = lane; j < 48; j += 32) {  // level 2: texel r of map d from that map's level 1
    const int d = j >> 3, r = j & 7, x = r & 1, y = (r >> 1) & 1, z = r >> 2;
    const T v = brick_mip_texel(scr.l1[d], 4, x, y, z, d);
    surf3Dwrite(v, bm.surf[d][2], (b3[0] * 2 + x) * kB, b3[1] * 2 + y, b3[2] * 2 + z);
    scr.l2[d][r] = v;
  }
  if (lane < 8) {  // occupancy of level 2 from level 1's
    const int x = lane & 1, y = (lane >> 1) & 1, z = lane >> 2;
    bool any = false;
#pragma unroll
    for (int k = 0; k < 8; ++k) any |= scr.occ1[mip_child(4, x, y, z, k)] != 0;
    scr.occ2[lane] = any ? 1 : 0;
    brick_occ(bm, N, 2, b3[0] * 2 + x, b3[1] * 2 + y, b3[2] * 2 + z, any);
  }
  __syncwarp();
  if (lane < 8) {
    if constexpr (STORAGE == VCT_STORAGE_RGBA8)
      if (bm.has_alpha)
        brick_alpha(bm, 2, b3[0] * 2 + (lane & 1), b3[1] * 2 + ((lane >> 1) & 1), b3[2] * 2 + (lane >> 2),
                    &scr.l2[0][lane], 8);
  } else if (lane < 14) {  // level 3: the brick's one texel of map d
    const int d = lane - 8;
    const T v = brick_mip_texel(scr.l2[d], 2, 0, 0, 0, d);
    surf3Dwrite(v, bm.surf[d][3], b3[0] * kB, b3[1], b3[2]);
    scr.l3[d] = v;
  } else if (lane == 14) {
    bool any = false;
    for (int k = 0; k < 8; ++k) any |= scr.occ2[k] != 0;
    brick_occ(bm, N, 3, b3[0], b3[1], b3[2], any);
  }
  __syncwarp();
  if constexpr (STORAGE == VCT_STORAGE_RGBA8)
    if (lane == 0 && bm.has_alpha) brick_alpha(bm, 3, b3[0], b3[1], b3[2], scr.l3, 1);
}

// Levels 1-3 of an empty brick: zeros (the texels and the occupancy).
template <int STORAGE>
__device__ void brick_mips_zero(const BrickMips& bm, int N, const int b3[3]) {
  const int t = threadIdx.x;
  const uint32_t zero[6] = {0u, 0u, 0u, 0u, 0u, 0u};
  int level = 0, x = 0, y = 0, z = 0;
  if (t < 64) {
    level = 1;
    x = b3[0] * 4 + (t & 3);
    y = b3[1] * 4 + ((t >> 2) & 3);
    z = b3[2] * 4 + (t >> 4);
  } else if (t < 72) {
    level = 2;
    x = b3[0] * 2 + (t & 1);
    y = b3[1] * 2 + ((t >> 1) & 1);
    z = b3[2] * 2 + ((t >> 2) & 1);
  } else if (t == 72) {
    level = 3;
    x = b3[0];
    y = b3[1];
    z = b3[2];
  }
  if (!level) return;
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    if constexpr (STORAGE == VCT_STORAGE_RGBA16F) surf3Dwrite(make_uint2(0u, 0u), bm.surf[d][level], x * 8, y, z);
    else surf3Dwrite(0u, bm.surf[d][level], x * 4, y, z);
  }
  if constexpr (STORAGE == VCT_STORAGE_RGBA8)
    if (bm.has_alpha) brick_alpha(bm, level, x, y, z, zero, 1);
  brick_occ(bm, N, level, x, y, z, false);
}

// Writes the brick at b3 from its sums: order-independent mean, round to
// nearest (ties up); empty voxels = 0.  `acc` may be in shared or global
// memory.
template <int STORAGE>
__device__ __forceinline__ void brick_finalize(const SceneParams& sp, int N, const int b3[3], const AccT<STORAGE>& acc,
                                               cudaSurfaceObject_t l0, uint32_t* __restrict__ counts,
                                               FrameStatus* st, const InjGrids& inj, void* l0_lin,
                                               const BrickMips* bm = nullptr, void* scr_raw = nullptr) {
  using Scr = BrickMipScratchT<STORAGE == VCT_STORAGE_RGBA16F ? VCT_STORAGE_RGBA16F : VCT_STORAGE_RGBA8>;
  Scr* scr = static_cast<Scr*>(scr_raw);
  for (int i = threadIdx.x; i < kBrickVox; i += kThreads) {
    const uint32_t n = acc.n[i];
    const int lx = i & 7, ly = (i >> 3) & 7, lz = i >> 6;
    const int x = b3[0] * kBrick + lx, y = b3[1] * kBrick + ly, z = b3[2] * kBrick + lz;
    if (n > 65535u) atomicAdd(&st->count_saturated, 1u);
    if constexpr (STORAGE == kStorageAttr) {
      uchar4 a = make_uchar4(0, 0, 0, 0), nn = a, e = a;
      if (n) {
        a = make_uchar4(unorm8_mean(acc.c[0][i], n), unorm8_mean(acc.c[1][i], n), unorm8_mean(acc.c[2][i], n),
                        unorm8_mean(acc.c[3][i], n));
        nn = make_uchar4(unorm8_mean(acc.c[4][i], n), unorm8_mean(acc.c[5][i], n), unorm8_mean(acc.c[6][i], n), 0);
        e = make_uchar4(unorm8_mean(acc.c[7][i], n), unorm8_mean(acc.c[8][i], n), unorm8_mean(acc.c[9][i], n), 255);
      }
      surf3Dwrite(a, inj.albedo, x * 4, y, z);
      surf3Dwrite(nn, inj.normal, x * 4, y, z);
      surf3Dwrite(e, inj.emission, x * 4, y, z);
    } else if constexpr (STORAGE == VCT_STORAGE_RGBA8) {
      uchar4 o = make_uchar4(0, 0, 0, 0);
      if (n) o = make_uchar4(unorm8_mean(acc.c[0][i], n), unorm8_mean(acc.c[1][i], n), unorm8_mean(acc.c[2][i], n),
                             unorm8_mean(acc.c[3][i], n));
      surf3Dwrite(o, l0, x * 4, y, z);
      if (l0_lin) static_cast<uchar4*>(l0_lin)[((size_t)z * N + y) * N + x] = o;
      if (bm) scr->l0[i] = (uint32_t)o.x | (uint32_t)o.y << 8 | (uint32_t)o.z << 16 | (uint32_t)o.w << 24;
    } else {
      ushort4 o = make_ushort4(0, 0, 0, 0);
      if (n) {
        const float inv = 1.0f / ((float)n * 4294967296.0f), k = inv * sp.radiance_max;
        o = make_ushort4(__half_as_ushort(__float2half_rn((float)acc.c[0][i] * k)),
                         __half_as_ushort(__float2half_rn((float)acc.c[1][i] * k)),
                         __half_as_ushort(__float2half_rn((float)acc.c[2][i] * k)),
                         __half_as_ushort(__float2half_rn((float)acc.c[3][i] * inv)));
      }
      surf3Dwrite(o, l0, x * 8, y, z);
      if (l0_lin) static_cast<ushort4*>(l0_lin)[((size_t)z * N + y) * N + x] = o;
      if (bm) scr->l0[i] = make_uint2((uint32_t)o.x | (uint32_t)o.y << 16, (uint32_t)o.z | (uint32_t)o.w << 16);
    }
    if (counts) counts[((size_t)z * N + y) * N + x] = n;
  }
  if constexpr (STORAGE == VCT_STORAGE_RGBA8 || STORAGE == VCT_STORAGE_RGBA16F) {
    if (bm) {
      __syncthreads();
      brick_mips<STORAGE>(*bm, N, b3, *scr);
    }
  }
}

__device__ __forceinline__ void brick_coords(int N, uint32_t brick, int b3[3]) {
  const int nb = N / kBrick;
  b3[0] = (int)(brick % nb);
  b3[1] = (int)((brick / nb) % nb);
  b3[2] = (int)(brick / ((uint32_t)nb * nb));
}

// One unit of brick work, all threads of the CTA (the shared-memory arrays
// come from the caller, so that a persistent CTA reuses them unit after
// unit): the whole brick, or -- for a dense brick with an accumulator slot
// (hb->slot[slot_index] >= 0) -- its chunk `chunk` of kHeavyChunk pairs.
// A chunk adds its sums into the slot; the CTA that completes the brick's
// last chunk takes the sums back (zeroing the slot and its counter for the
// next frame) and writes the brick.  `item`: the unit is an extra chunk
// (>= 1) of a split brick.  Every kernel calls this from one place only,
// so that its code exists once per kernel (instruction-cache footprint).
template <int MODE, int STORAGE>
__device__ __forceinline__ void brick_unit(const SceneParams& sp, int N, uint32_t brick,
                                           const uint32_t* __restrict__ offset, const uint32_t* __restrict__ list,
                                           uint32_t cap, cudaSurfaceObject_t l0, uint32_t* __restrict__ counts,
                                           FrameStatus* st, AccT<STORAGE>& acc, SetupOf<MODE> (&setup)[kSetupSlots],
                                           int (&excl)[kExclSlots], const InjGrids& inj, void* l0_lin,
                                           const HeavyBricks* hb, uint32_t slot_index, uint32_t chunk, bool item,
                                           const BrickMips* bm = nullptr, uint8_t* dirty = nullptr) {
  static_assert(sizeof(BrickMipScratchT<VCT_STORAGE_RGBA16F>) <= sizeof(setup),
                "fused mips fit in the triangle setups' memory");
  __shared__ uint32_t s_last;
  int b3[3];
  brick_coords(N, brick, b3);
  const uint32_t beg0 = min(offset[brick], cap), end = min(offset[brick + 1], cap);
  if (beg0 == end) {
    // No triangle touches this brick (most of the grid): store cleared texels
    // without the accumulator or its barriers -- unless they are zero already
    // (`dirty`: per brick, 1 when its texels -- level 0, its linear copy and
    // any fused levels -- may be non-zero; the per-voxel counts are not
    // tracked by it).
    if (dirty && !counts) {
      if (!dirty[brick]) return;  // CTA-uniform
      __syncthreads();            // every thread has read the flag
      if (threadIdx.x == 0) dirty[brick] = 0;
    }
    for (int i = threadIdx.x; i < kBrickVox; i += kThreads) {
      const int x = b3[0] * kBrick + (i & 7), y = b3[1] * kBrick + ((i >> 3) & 7), z = b3[2] * kBrick + (i >> 6);
      if (STORAGE == kStorageAttr) {
        surf3Dwrite(make_uchar4(0, 0, 0, 0), inj.albedo, x * 4, y, z);
        surf3Dwrite(make_uchar4(0, 0, 0, 0), inj.normal, x * 4, y, z);
        surf3Dwrite(make_uchar4(0, 0, 0, 0), inj.emission, x * 4, y, z);
      } else if (STORAGE == VCT_STORAGE_RGBA8) {
        surf3Dwrite(make_uchar4(0, 0, 0, 0), l0, x * 4, y, z);
        if (l0_lin) static_cast<uchar4*>(l0_lin)[((size_t)z * N + y) * N + x] = make_uchar4(0, 0, 0, 0);
      } else {
        surf3Dwrite(make_ushort4(0, 0, 0, 0), l0, x * 8, y, z);
        if (l0_lin) static_cast<ushort4*>(l0_lin)[((size_t)z * N + y) * N + x] = make_ushort4(0, 0, 0, 0);
      }
      if (counts) counts[((size_t)z * N + y) * N + x] = 0u;
    }
    if constexpr (STORAGE == VCT_STORAGE_RGBA8 || STORAGE == VCT_STORAGE_RGBA16F)
      if (bm) brick_mips_zero<STORAGE>(*bm, N, b3);
    return;
  }
  // Only a dense brick looks up its slot.
  const int slot = (hb && hb->slot && (item || end - beg0 > kHeavyChunk)) ? hb->slot[slot_index] : -1;
  uint32_t beg = beg0, stop = end;
  if (slot >= 0) {
    beg = min(beg0 + chunk * kHeavyChunk, end);
    stop = min(beg + kHeavyChunk, end);
  }
  brick_accumulate<MODE, STORAGE>(sp, N, b3, list, beg, stop, acc, setup, excl);
  if (slot >= 0) {
    AccT<STORAGE>& g = static_cast<AccT<STORAGE>*>(hb->acc)[slot];
    for (int i = threadIdx.x; i < kBrickVox; i += kThreads) acc.atomic_add_to(g, i);
    __threadfence();  // this CTA's sums are in L2 before its chunk counts as done
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t nch = (end - beg0 + kHeavyChunk - 1) / kHeavyChunk;
      s_last = atomicAdd(&hb->done[slot], 1u) == nch - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int i = threadIdx.x; i < kBrickVox; i += kThreads) acc.take_from(g, i);
    if (threadIdx.x == 0) hb->done[slot] = 0;
    __syncthreads();
  }
  // (the triangle setups are done with: their memory holds the fused mips)
  if (dirty && threadIdx.x == 0) dirty[brick] = 1;
  brick_finalize<STORAGE>(sp, N, b3, acc, l0, counts, st, inj, l0_lin, bm, &setup[0]);
}

// One CTA per brick, after `n_extra` CTAs that run the extra chunks of
// split bricks from the launch-wide item queue (first in the grid, so that
// the dense bricks' chunks start with the first bricks, not in the tail).
// (FUSE: the fused mips' level-1 reduction holds 32 unpacked children; the
// kernel is held to the registers of 7 resident CTAs, as without it.)
template <int MODE, int STORAGE, bool FUSE = false>
__global__ void __launch_bounds__(kThreads, FUSE ? 7 : brick_min_blocks<MODE>()) k_bricks(SceneParams sp, int N, const uint32_t* __restrict__ offset,
                                                     const uint32_t* __restrict__ list, uint32_t cap,
                                                     cudaSurfaceObject_t l0, uint32_t* __restrict__ counts,
                                                     FrameStatus* st, InjGrids inj, void* l0_lin, HeavyBricks hb,
                                                     uint32_t n_extra, const __grid_constant__ BrickMips bm) {
  __shared__ AccT<STORAGE> acc;
  __shared__ SetupOf<MODE> setup[kSetupSlots];
  __shared__ int excl[kExclSlots];
  __shared__ uint32_t s_next;
  const bool extra = blockIdx.x < n_extra;
  const uint32_t n_items = extra ? min(hb.counters[1], hb.item_cap) : 0u;
  if (extra && blockIdx.x == 0 && threadIdx.x < 2) (&st->heavy_total)[threadIdx.x] = hb.counters[threadIdx.x];
  for (bool first = true;; first = false) {
    uint32_t brick, chunk = 0;
    if (!extra) {
      if (!first) return;
      brick = blockIdx.x - n_extra;
    } else {
      if (threadIdx.x == 0) s_next = atomicAdd(&hb.counters[2], 1u);
      __syncthreads();
      const uint32_t it = s_next;
      __syncthreads();  // s_next read by every thread before the next write
      if (it >= n_items) return;
      const uint2 w = hb.items[it];
      if (w.x == 0xffffffffu) continue;  // CTA-uniform
      brick = w.x;
      chunk = w.y;
    }
    brick_unit<MODE, STORAGE>(sp, N, brick, offset, list, cap, l0, counts, st, acc, setup, excl, inj, l0_lin, &hb,
                              brick, chunk, extra, FUSE ? &bm : nullptr, bm.dirty);
    __syncthreads();  // done with acc
  }
}

// Every scene's bricks in one persistent launch; a CTA takes its next unit
// from the atomic counter w.queue (brick costs range from an empty brick to
// thousands of triangle samples).  The queue hands out the extra chunks of
// the split bricks first (global brick indices), then the bricks.
template <int MODE, int STORAGE, bool FUSE = false>
__global__ void __launch_bounds__(kThreads, FUSE ? 7 : brick_min_blocks<MODE>())
    k_bricks_batch(BatchWork w, BatchBuffers bb) {
  __shared__ AccT<STORAGE> acc;
  __shared__ SetupOf<MODE> setup[kSetupSlots];
  __shared__ int excl[kExclSlots];
  __shared__ uint32_t s_next;
  const HeavyBricks& hb = bb.heavy;
  const uint32_t n_items = hb.slot ? min(hb.counters[1], hb.item_cap) : 0u;
  const uint32_t total = n_items + w.total;
  if (hb.slot && blockIdx.x == 0 && threadIdx.x < 2) (&bb.status->heavy_total)[threadIdx.x] = hb.counters[threadIdx.x];
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(w.queue, 1u);
    __syncthreads();
    const uint32_t q = s_next;
    __syncthreads();  // s_next read by every thread before the next write
    if (q >= total) return;
    uint32_t g, chunk = 0;
    const bool item = q < n_items;
    if (item) {
      const uint2 it = hb.items[q];
      if (it.x == 0xffffffffu) continue;  // CTA-uniform
      g = it.x;
      chunk = it.y;
    } else {
      g = q - n_items;
    }
    const int s = batch_scene_of(w, g);
    const BatchScene& S = w.scenes[s];
    brick_unit<MODE, STORAGE>(S.sp, S.N, g - __ldg(w.prefix + s), bb.brick_offset + S.brick_base, bb.pair_list,
                              bb.pair_cap, S.ms.l0_surf, nullptr, bb.status, acc, setup, excl, InjGrids{}, nullptr,
                              &hb, g, chunk, item, FUSE ? bb.mips + s : nullptr,
                              bb.dirty ? bb.dirty + S.brick_base : nullptr);
    __syncthreads();  // done with acc
  }
}

// Persistent grid of a batched kernel: `per_sm` CTAs per SM, but never more
// than fit on an SM at once (a CTA that waits for a slot would start its
// share of the work only after a whole resident CTA has finished).
template <class K>
unsigned resident_grid(K kern, int threads, size_t smem, int sms, int per_sm, uint32_t items) {
  int fit = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, threads, smem) != cudaSuccess || fit < 1) fit = 1;
  const int n = sms * std::min(std::max(per_sm, 1), fit);
  return (unsigned)std::max<uint32_t>(1u, std::min<uint32_t>((uint32_t)n, items));
}

// The same brick CTA writing RGBA8 level 0 into linear memory (x fastest)
// instead of a surface: the output of vct_voxelize_noalloc.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_bricks_linear(SceneParams sp, int N, const uint32_t* __restrict__ offset,
                                                            const uint32_t* __restrict__ list, uint32_t cap,
                                                            uchar4* __restrict__ out) {
  typedef typename std::conditional<MODE == VCT_VOX_CONSERVATIVE, SetupSat, SetupRef>::type Setup;
  __shared__ Acc acc;
  __shared__ Setup setup[kWarps][32];
  __shared__ int excl[kWarps][33];
  const int nb = N / kBrick;
  const uint32_t brick = blockIdx.x;
  const int b3[3] = {(int)(brick % nb), (int)((brick / nb) % nb), (int)(brick / ((uint32_t)nb * nb))};
  for (int i = threadIdx.x; i < kBrickVox; i += kThreads) acc.clear(i);
  __syncthreads();
  const uint32_t beg = min(offset[brick], cap), end = min(offset[brick + 1], cap);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (uint32_t base = beg + warp * 32; base < end; base += kWarps * 32) {
    const uint32_t e = base + lane;
    int cnt = 0;
    if (e < end) {
      if (MODE == VCT_VOX_CONSERVATIVE)
        cnt = setup_sat(sp, N, __ldg(list + e), b3, reinterpret_cast<SetupSat&>(setup[warp][lane]));
      else
        cnt = setup_ref(sp, N, __ldg(list + e), b3, reinterpret_cast<SetupRef&>(setup[warp][lane]));
    }
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    excl[warp][lane] = incl - cnt;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (int it = lane; it < total; it += 32) {
      int lo = 0, hi = 31;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (excl[warp][mid] <= it) lo = mid; else hi = mid - 1;
      }
      const int local = it - excl[warp][lo];
      if (MODE == VCT_VOX_CONSERVATIVE)
        item_sat(sp, N, b3, reinterpret_cast<const SetupSat&>(setup[warp][lo]), local, acc);
      else
        item_ref(sp, N, b3, reinterpret_cast<const SetupRef&>(setup[warp][lo]), local, acc);
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kBrickVox; i += kThreads) {
    const uint32_t n = acc.n[i];
    const int x = b3[0] * kBrick + (i & 7), y = b3[1] * kBrick + ((i >> 3) & 7), z = b3[2] * kBrick + (i >> 6);
    uchar4 o = make_uchar4(0, 0, 0, 0);
    if (n) {
      const unsigned long long den = 2ull * n * 65535ull;
      unsigned char q[4];
      for (int ch = 0; ch < 4; ++ch) {
        unsigned long long v = ((unsigned long long)acc.c[ch][i] * 510ull + (unsigned long long)n * 65535ull) / den;
        q[ch] = (unsigned char)(v > 255ull ? 255ull : v);
      }
      o = make_uchar4(q[0], q[1], q[2], q[3]);
    }
    out[((size_t)z * N + y) * N + x] = o;
  }
}

}  // namespace

cudaError_t launch_voxelize_linear(const SceneParams& sp, int N, int mode, const VoxBuffers& vb, uchar4* out,
                                   cudaStream_t st) {
  const int nb = N / kBrick;
  const size_t n_bricks = (size_t)nb * nb * nb;
  cudaError_t e = cudaMemsetAsync(vb.brick_count, 0, n_bricks * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const unsigned tri_blocks = (sp.total_tris + 255) / 256;
  if (tri_blocks)
    k_bin<false><<<tri_blocks, 256, 0, st>>>(sp, N, vb.brick_count, nullptr, nullptr, 0, vb.status, nullptr, 0,
                                             nullptr, nullptr);
  e = launch_exclusive_scan(vb.brick_count, vb.brick_offset, vb.brick_cursor, n_bricks, vb.scan_tmp, st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(&vb.status->pair_total, vb.brick_offset + n_bricks, sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                      st);
  if (e != cudaSuccess) return e;
  if (tri_blocks)
    k_bin<true><<<tri_blocks, 256, 0, st>>>(sp, N, nullptr, vb.brick_cursor, vb.pair_list, vb.pair_cap, vb.status,
                                            nullptr, 0, nullptr, nullptr);
  if (mode == VCT_VOX_CONSERVATIVE)
    k_bricks_linear<VCT_VOX_CONSERVATIVE><<<(unsigned)n_bricks, kThreads, 0, st>>>(sp, N, vb.brick_offset,
                                                                                 vb.pair_list, vb.pair_cap, out);
  else
    k_bricks_linear<VCT_VOX_REF_RASTER2X><<<(unsigned)n_bricks, kThreads, 0, st>>>(sp, N, vb.brick_offset,
                                                                                 vb.pair_list, vb.pair_cap, out);
  return cudaGetLastError();
}

// Calls f(mode tag, storage tag) for the brick kernel a frame uses.
template <class F>
void dispatch_bricks(int mode, int storage, bool attr, F&& f) {
  using RAS = std::integral_constant<int, VCT_VOX_REF_RASTER2X>;
  using SAT = std::integral_constant<int, VCT_VOX_CONSERVATIVE>;
  using R8 = std::integral_constant<int, VCT_STORAGE_RGBA8>;
  using F16 = std::integral_constant<int, VCT_STORAGE_RGBA16F>;
  using ATR = std::integral_constant<int, kStorageAttr>;
  if (mode == VCT_VOX_CONSERVATIVE) {
    if (attr) f(SAT(), ATR());
    else if (storage == VCT_STORAGE_RGBA8) f(SAT(), R8());
    else f(SAT(), F16());
  } else {
    if (attr) f(RAS(), ATR());
    else if (storage == VCT_STORAGE_RGBA8) f(RAS(), R8());
    else f(RAS(), F16());
  }
}

// CTAs of a kernel resident on one SM (cached per kernel).
template <class K>
int resident_per_sm(K kern) {
  int f = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, kern, kThreads, 0) != cudaSuccess || f < 1) f = 1;
  return f;
}

cudaError_t launch_voxelize(const SceneParams& sp, int N, int mode, int storage, const VoxBuffers& vb,
                            cudaSurfaceObject_t l0, cudaStream_t st, int* launches, const InjGrids* inj) {
  int nl = 0;
  const int nb = N / kBrick;
  const size_t n_bricks = (size_t)nb * nb * nb;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int fit = 1;
  dispatch_bricks(mode, storage, inj != nullptr, [&](auto mode_tag, auto storage_tag) {
    static const int f = resident_per_sm(k_bricks<decltype(mode_tag)::value, decltype(storage_tag)::value>);
    fit = f;
  });
  cudaError_t e = cudaMemsetAsync(vb.brick_count, 0, n_bricks * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const unsigned tri_blocks = (sp.total_tris + 255) / 256;
  const dim3 big_grid(128, kBigSplit);
  if (vb.big) {
    e = cudaMemsetAsync(vb.big_count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
  }
  if (tri_blocks) {
    k_bin<false><<<tri_blocks, 256, 0, st>>>(sp, N, vb.brick_count, nullptr, nullptr, 0, vb.status, vb.big,
                                             vb.big_cap, vb.big_count, vb.bin_rec);
    ++nl;
    if (vb.big) {
      k_bin_big<false><<<big_grid, 256, 0, st>>>(N, vb.big, vb.big_cap, vb.big_count, vb.brick_count, nullptr, nullptr,
                                                 0, nullptr);
      ++nl;
    }
  }
  // Offsets, pair_total <- offset[n_bricks], and the dense-brick plan
  // against the brick CTAs resident at once.
  const HeavyBricks& hb = vb.heavy;
  ScanFuse fuse;
  std::memset(&fuse, 0, sizeof(fuse));
  fuse.hb = hb;
  fuse.cap = vb.pair_cap;
  fuse.slots = (uint32_t)(sms * fit);
  fuse.total_copy = &vb.status->pair_total;
  e = launch_exclusive_scan(vb.brick_count, vb.brick_offset, vb.brick_cursor, n_bricks, vb.scan_tmp, st, &nl, &fuse);
  if (e != cudaSuccess) return e;
  if (vb.big) {
    e = cudaMemcpyAsync(&vb.status->bigtri_total, vb.big_count, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
  }
  if (tri_blocks) {
    k_bin<true><<<tri_blocks, 256, 0, st>>>(sp, N, nullptr, vb.brick_cursor, vb.pair_list, vb.pair_cap, vb.status,
                                            vb.big, vb.big_cap, vb.big_count, vb.bin_rec);
    ++nl;
    if (vb.big) {
      k_bin_big<true><<<big_grid, 256, 0, st>>>(N, vb.big, vb.big_cap, vb.big_count, nullptr, vb.brick_cursor,
                                                vb.pair_list, vb.pair_cap, nullptr);
      ++nl;
    }
  }
  const InjGrids g = inj ? *inj : InjGrids{};
  void* lin = inj ? nullptr : vb.level0_lin;
  const bool fuse_mips = vb.mips && !inj && (storage == VCT_STORAGE_RGBA8 || storage == VCT_STORAGE_RGBA16F);
  BrickMips bm;
  std::memset(&bm, 0, sizeof(bm));
  if (fuse_mips) bm = *vb.mips;
  bm.dirty = inj ? nullptr : vb.dirty;  // (kernel parameter of every brick kernel)
  // Before the bricks: two CTAs per SM that run the extra chunks.
  const uint32_t n_extra = hb.slot ? std::min<uint32_t>(hb.item_cap, (uint32_t)(sms * std::min(fit, 2))) : 0u;
  dispatch_bricks(mode, storage, inj != nullptr, [&](auto mode_tag, auto storage_tag) {
    constexpr int M = decltype(mode_tag)::value, S = decltype(storage_tag)::value;
    if constexpr (S == VCT_STORAGE_RGBA8 || S == VCT_STORAGE_RGBA16F) {
      if (fuse_mips) {
        k_bricks<M, S, true><<<(unsigned)(n_extra + n_bricks), kThreads, 0, st>>>(
            sp, N, vb.brick_offset, vb.pair_list, vb.pair_cap, l0, vb.counts, vb.status, g, lin, hb, n_extra, bm);
        return;
      }
    }
    k_bricks<M, S><<<(unsigned)(n_extra + n_bricks), kThreads, 0, st>>>(
        sp, N, vb.brick_offset, vb.pair_list, vb.pair_cap, l0, vb.counts, vb.status, g, lin, hb, n_extra, bm);
  });
  ++nl;
  if (launches) *launches += nl;
  return cudaGetLastError();
}

size_t heavy_slot_bytes(int storage) {
  return storage == kStorageAttr          ? sizeof(AccT<kStorageAttr>)
         : storage == VCT_STORAGE_RGBA16F ? sizeof(AccT<VCT_STORAGE_RGBA16F>)
                                          : sizeof(AccT<VCT_STORAGE_RGBA8>);
}

}  // namespace vct

namespace vct {

// Batched voxelizer: the same passes as launch_voxelize, each one launch
// over every scene of the batch (brick arrays concatenated, one scan).
cudaError_t launch_voxelize_batch(const BatchWork& tris, const BatchWork& bricks, uint32_t total_bricks, int mode,
                                  int storage, const BatchBuffers& bb, uint32_t* scan_tmp, const BatchShape& shape,
                                  int sms, cudaStream_t st, int* launches) {
  int nl = 0;
  const HeavyBricks& hb = bb.heavy;
  // The persistent brick grid (bricks + at most item_cap extra chunks).
  unsigned grid = 1;
  const bool fuse_mips = bb.mips != nullptr && storage == VCT_STORAGE_RGBA8;
  dispatch_bricks(mode, storage, false, [&](auto mode_tag, auto storage_tag) {
    constexpr int M = decltype(mode_tag)::value, S = decltype(storage_tag)::value;
    grid = fuse_mips ? resident_grid(k_bricks_batch<M, S, true>, kThreads, 0, sms, shape.bricks_ctas_per_sm,
                                bricks.total + (hb.slot ? hb.item_cap : 0u))
                : resident_grid(k_bricks_batch<M, S>, kThreads, 0, sms, shape.bricks_ctas_per_sm,
                                bricks.total + (hb.slot ? hb.item_cap : 0u));
  });
  cudaError_t e = cudaMemsetAsync(bb.brick_count, 0, (size_t)total_bricks * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(bb.big_count, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const unsigned bin_grid = resident_grid(k_bin_batch<false>, 256, 0, sms, shape.bin_ctas_per_sm,
                                          (tris.total + 255) / 256);
  const dim3 big_grid(128, kBigSplit);
  if (tris.total) {
    k_bin_batch<false><<<bin_grid, 256, 0, st>>>(tris, bb);
    k_bin_big<false><<<big_grid, 256, 0, st>>>(0, bb.big, bb.big_cap, bb.big_count, bb.brick_count, nullptr, nullptr,
                                               0, tris.scenes);
    nl += 2;
  }
  // Offsets, pair_total, and the dense-brick plan against the persistent
  // grid's CTAs.
  ScanFuse fuse;
  std::memset(&fuse, 0, sizeof(fuse));
  fuse.hb = hb;
  fuse.cap = bb.pair_cap;
  fuse.slots = grid;
  fuse.total_copy = &bb.status->pair_total;
  e = launch_exclusive_scan(bb.brick_count, bb.brick_offset, bb.brick_cursor, total_bricks, scan_tmp, st, &nl, &fuse);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(&bb.status->bigtri_total, bb.big_count, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (tris.total) {
    k_bin_batch<true><<<bin_grid, 256, 0, st>>>(tris, bb);
    k_bin_big<true><<<big_grid, 256, 0, st>>>(0, bb.big, bb.big_cap, bb.big_count, nullptr, bb.brick_cursor,
                                              bb.pair_list, bb.pair_cap, tris.scenes);
    nl += 2;
  }
  e = cudaMemsetAsync(bricks.queue, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  dispatch_bricks(mode, storage, false, [&](auto mode_tag, auto storage_tag) {
    constexpr int M = decltype(mode_tag)::value, S = decltype(storage_tag)::value;
    if (fuse_mips) k_bricks_batch<M, S, true><<<grid, kThreads, 0, st>>>(bricks, bb);
    else k_bricks_batch<M, S><<<grid, kThreads, 0, st>>>(bricks, bb);
  });
  ++nl;
  if (launches) *launches += nl;
  return cudaGetLastError();
}

}  // namespace vct

namespace vct {
namespace {

// Deferred light injection (no reference counterpart: the reference shades
// every fragment while voxelizing, voxelize.frag:124-153).  Each occupied
// voxel is lit at its centre (grid space (2x+1)/N - 1) with its mean normal
// and the same per-light terms as voxelize.frag:128-143:
//   colour = clamp(albedo * sum_i color_i * intensity_i * max(n.l_i, 0) /
//                  (1 + d_i^2) + emission, 0, 1),  alpha = mean alpha,
// stored as RGBA8 rounded to nearest.
__global__ void __launch_bounds__(256) k_inject(SceneParams sp, int N, InjGrids g, cudaSurfaceObject_t l0,
                                                uchar4* __restrict__ l0_lin) {
  const size_t total = (size_t)N * N * N;
  const float k = 1.0f / 255.0f, inv = 2.0f / (float)N;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((size_t)N * N));
    uchar4 e;
    surf3Dread(&e, g.emission, x * 4, y, z);
    if (e.w == 0) {
      surf3Dwrite(make_uchar4(0, 0, 0, 0), l0, x * 4, y, z);
      if (l0_lin) l0_lin[i] = make_uchar4(0, 0, 0, 0);
      continue;
    }
    uchar4 a, nq;
    surf3Dread(&a, g.albedo, x * 4, y, z);
    surf3Dread(&nq, g.normal, x * 4, y, z);
    const V3 nn = normalize(v3(nq.x * k * 2.0f - 1.0f, nq.y * k * 2.0f - 1.0f, nq.z * k * 2.0f - 1.0f));
    const V3 pos = v3(((float)x + 0.5f) * inv - 1.0f, ((float)y + 0.5f) * inv - 1.0f, ((float)z + 0.5f) * inv - 1.0f);
    V3 lit = v3(0.f, 0.f, 0.f);
    const int nl = min(sp.n_lights, kMaxLights);
    for (int l = 0; l < nl; ++l) {
      const vct_point_light& L = sp.lights[l];
      const V3 lp = v3(L.position[0] / sp.cube_size, L.position[1] / sp.cube_size, L.position[2] / sp.cube_size);
      const V3 dl = lp - pos;
      const float d = length(dl);
      const float cs = fmaxf(dot(nn, normalize(dl)), 0.0f);
      lit = lit + v3(L.color[0], L.color[1], L.color[2]) * (cs * (1.0f / (1.0f + d * d)) * L.intensity);
    }
    const V3 c = mulv(v3(a.x * k, a.y * k, a.z * k), lit) + v3(e.x * k, e.y * k, e.z * k);
    auto q = [](float v) { return (unsigned char)__float2uint_rz(clamp01(v) * 255.0f + 0.5f); };
    const uchar4 o = make_uchar4(q(c.x), q(c.y), q(c.z), a.w);
    surf3Dwrite(o, l0, x * 4, y, z);
    if (l0_lin) l0_lin[i] = o;
  }
}

}  // namespace

cudaError_t launch_inject(const SceneParams& sp, int N, const InjGrids& g, cudaSurfaceObject_t l0, uchar4* l0_lin,
                          cudaStream_t st, int* launches) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t total = (size_t)N * N * N;
  const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)sms * 16);
  k_inject<<<grid, 256, 0, st>>>(sp, N, g, l0, l0_lin);
  if (launches) ++*launches;
  return cudaGetLastError();
}

}  // namespace vct
