// k_mipmap.cu -- the MipBuilder: replaces Renderer::filter (renderer.cpp
// :283-314) and mipmap.comp.
//
// The reference dispatches one compute pass per level with a memory barrier
// in between, and every pass re-reads the level below from memory.  Here one
// CTA loads a B^3 region (B = 16) of the source level into shared memory once
// and produces up to four levels of all six directional maps from it (the
// intermediate levels never leave shared memory except for their own store).
// Level 0 is stored once and shared by the six maps, as in the reference
// (all six textures receive identical level-0 data, voxelize.frag:159-160).
// A second, tiny pass builds the remaining levels (5, 6) from level 4.
//
// RGBA8 texels are evaluated exactly: with texels k/255 the stored value of
// mean(alpha_blend(front, back)) (mipmap.comp:40-43,59-98) is
// round(S / 1020) with S = sum over the four pairs of (F*255 + (255-F.a)*B)
// per channel, ties up, clamped to 255 -- the exact real value of the GLSL
// expression, rounded to unorm8 as imageStore does.  RGBA16F texels use FP32
// maths and round-to-nearest-even to half.
#include <cuda_fp16.h>

#include <algorithm>

#include <cuda.h>

#include "vct_async.cuh"
#include "vct_internal.h"
#include "vct_mip.cuh"

namespace vct {
namespace {

constexpr int kThreads = 256;

// voxel_offsets, mipmap.comp:10-20.
__constant__ int c_off[8][3] = {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0},
                                {0, 1, 1}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
// (front, back) pairs per map (0:-x 1:+x 2:-y 3:+y 4:-z 5:+z), mipmap.comp:59-98.
__constant__ int c_pairs[6][4][2] = {
    {{0, 4}, {1, 5}, {2, 6}, {3, 7}}, {{4, 0}, {5, 1}, {6, 2}, {7, 3}},
    {{0, 2}, {1, 3}, {5, 7}, {4, 6}}, {{2, 0}, {3, 1}, {7, 5}, {6, 4}},
    {{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{1, 0}, {3, 2}, {5, 4}, {7, 6}}};
template <int STORAGE> struct Texel;
template <> struct Texel<VCT_STORAGE_RGBA8> {
  typedef uint32_t T;
  static constexpr int kBytes = 4;
};
template <> struct Texel<VCT_STORAGE_RGBA16F> {
  typedef uint2 T;
  static constexpr int kBytes = 8;
};

__device__ __forceinline__ uint32_t aniso_rgba8(const uint32_t* ch, int d) {
  uint32_t out = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint32_t S = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t f = ch[c_pairs[d][q][0]], b = ch[c_pairs[d][q][1]];
      S += ch8(f, c) * 255u + (255u - ch8(f, 3)) * ch8(b, c);
    }
    uint32_t v = (S + 510u) / 1020u;
    out |= (v > 255u ? 255u : v) << (8 * c);
  }
  return out;
}

__device__ __forceinline__ uint32_t iso_rgba8(const uint32_t* ch) {
  uint32_t out = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint32_t S = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) S += ch8(ch[i], c);
    out |= ((S + 4u) >> 3) << (8 * c);
  }
  return out;
}

__device__ __forceinline__ uint2 aniso_rgba16f(const uint2* ch, int d) {
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 4; ++q) blend16(acc, h2f(ch[c_pairs[d][q][0]]), h2f(ch[c_pairs[d][q][1]]));
  return finish16(acc);
}

__device__ __forceinline__ uint2 iso_rgba16f(const uint2* ch) {
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float4 v = h2f(ch[i]);
    acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
  }
  return f2h(make_float4(acc.x * 0.125f, acc.y * 0.125f, acc.z * 0.125f, acc.w * 0.125f));
}

template <int STORAGE>
__device__ __forceinline__ typename Texel<STORAGE>::T reduce(const typename Texel<STORAGE>::T* ch, int d, bool iso) {
  if constexpr (STORAGE == VCT_STORAGE_RGBA8) return iso ? iso_rgba8(ch) : aniso_rgba8(ch, d);
  else return iso ? iso_rgba16f(ch) : aniso_rgba16f(ch, d);
}

__device__ __forceinline__ void aniso6_rgba16f(const uint2* ch, uint2* out) {
  float4 c[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k] = h2f(ch[k]);
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int p = 0; p < 4; ++p) blend16(acc, c[c_pairs_h[d][p][0]], c[c_pairs_h[d][p][1]]);
    out[d] = finish16(acc);
  }
}

// Texel (x, y, z) of level `level` of the alpha-only chains from the six
// maps' RGBA8 texels v[0], v[stride], ..., v[5 * stride].
__device__ __forceinline__ void write_alpha(const MapSet& ms, int level, int x, int y, int z, const uint32_t* v,
                                            int stride) {
  surf3Dwrite(make_uchar4(v[0] >> 24, v[stride] >> 24, v[2 * stride] >> 24, v[3 * stride] >> 24),
              ms.alpha_surf[0][level], x * 4, y, z);
  surf3Dwrite(make_uchar2(v[4 * stride] >> 24, v[5 * stride] >> 24), ms.alpha_surf[1][level], x * 2, y, z);
}

// One pass: source level `src_level` (0 = the shared level 0) -> levels
// src_level+1 .. src_level+K of NMAPS maps, one CTA per B^3 source region.
// Levels src_level+1 .. src_level+K of the B^3 source region at (ox, oy, oz)
// held in shared memory at `src` ([map][z][y][x]); intermediate levels go to
// `lvl` (NMAPS * (B/2)^3, (B/4)^3, ...) and every level to its surfaces.
__device__ __forceinline__ bool nonzero(uint32_t v) { return v != 0u; }
__device__ __forceinline__ bool nonzero(uint2 v) { return (v.x | v.y) != 0u; }

// The eight children of destination texel (x, y, z) from a level of edge
// b2 (= 2 * the destination edge) at `src` in shared memory ([z][y][x]):
// the children at 2x and 2x+1 (c_off entries k+4 and k) are neighbours,
// and every row offset is even, so each pair is one aligned 8-byte (RGBA8)
// or 16-byte (RGBA16F) load.  Returns whether any child is non-zero.
__device__ __forceinline__ bool load_children(const uint32_t* src, int b2, int x, int y, int z, uint32_t* ch) {
  bool any = false;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint2 v = *reinterpret_cast<const uint2*>(src + ((2 * z + c_off[k][2]) * b2 + (2 * y + c_off[k][1])) * b2 +
                                                    2 * x);
    ch[k + 4] = v.x;
    ch[k] = v.y;
    any |= (v.x | v.y) != 0u;
  }
  return any;
}
__device__ __forceinline__ bool load_children(const uint2* src, int b2, int x, int y, int z, uint2* ch) {
  bool any = false;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint4 v = *reinterpret_cast<const uint4*>(src + ((2 * z + c_off[k][2]) * b2 + (2 * y + c_off[k][1])) * b2 +
                                                    2 * x);
    ch[k + 4] = make_uint2(v.x, v.y);
    ch[k] = make_uint2(v.z, v.w);
    any |= (v.x | v.y | v.z | v.w) != 0u;
  }
  return any;
}

// Occupancy of cell (x, y, z) (index r) of level l of the region at
// (ox, oy, oz): into the region's shared copy and to global memory -- level 1
// of 16^3 regions straight into the packed bits (a warp holds four rows of
// eight cells, each row one byte of its x-aligned word), other levels as
// bytes.  Called by every thread of a warp together for level 1.
template <int B>
__device__ __forceinline__ void occ_store(const MapSet& ms, int l, int ox, int oy, int oz, int x, int y, int z,
                                          int r, bool any, uint8_t* box) {
  box[r] = any ? 1 : 0;
  const int s = ms.N >> l;
  if (B == 16 && l == 1) {
    const uint32_t bits = __ballot_sync(0xffffffffu, any);
    if ((threadIdx.x & 7) == 0) {
      unsigned char* row = reinterpret_cast<unsigned char*>(
          ms.occ_pack[1] + ((size_t)((oz >> 1) + z) * s + (oy >> 1) + y) * ms.occ_wpr[1]);
      row[((ox >> 1) + x) >> 3] = (unsigned char)(bits >> (threadIdx.x & 31));
    }
  } else {
    ms.occ_raw[l][((size_t)((oz >> l) + z) * s + (oy >> l) + y) * s + (ox >> l) + x] = any ? 1 : 0;
  }
}

template <int NMAPS, bool FROM_L0, int K, int STORAGE>
__device__ __forceinline__ void mip_reduce(const MapSet& ms, int src_level, int ox, int oy, int oz,
                                           const typename Texel<STORAGE>::T* src, typename Texel<STORAGE>::T* lvl) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B = 1 << K;
  // Occupancy of the region's cells at levels 1..K (first pass only): a cell
  // is 1 when its block of level 0 holds a non-zero texel.
  __shared__ uint8_t occ_box[(B / 2) * (B / 2) * (B / 2) + (B / 4) * (B / 4) * (B / 4) + 16];
  const T* cur = src;
  int cur_b = B;
  bool cur_shared = FROM_L0;
  T* out = lvl;
  int occ_prev = 0, occ_off = 0;
#pragma unroll 1
  for (int l = 1; l <= K; ++l) {
    const int b = B >> l, b3 = b * b * b, cb3 = cur_b * cur_b * cur_b;
    if (FROM_L0 && ms.skip_empty && !(NMAPS >= 6 && l == 1)) {
      const int cb = b * 2;
      for (int r = threadIdx.x; r < b3; r += kThreads) {
        const int x = r % b, y = (r / b) % b, z = r / (b * b);
        bool any = false;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int ci = ((2 * z + c_off[k][2]) * cb + (2 * y + c_off[k][1])) * cb + (2 * x + c_off[k][0]);
          any |= l == 1 ? nonzero(src[ci]) : occ_box[occ_prev + ci] != 0;
        }
        occ_store<B>(ms, l, ox, oy, oz, x, y, z, r, any, occ_box + occ_off);
      }
    }
    if (!FROM_L0 && ms.skip_empty && ms.occ_raw[src_level + l]) {
      // Tail passes: the occupancy bytes of their levels, from the source
      // level's bytes (l = 1) and then from the region's shared copy.
      const int S = ms.N >> src_level, cb = b * 2, dl = src_level + l, sd = ms.N >> dl;
      for (int r = threadIdx.x; r < b3; r += kThreads) {
        const int x = r % b, y = (r / b) % b, z = r / (b * b);
        bool any = false;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int cx = 2 * x + c_off[k][0], cy = 2 * y + c_off[k][1], cz = 2 * z + c_off[k][2];
          any |= l == 1 ? __ldg(ms.occ_raw[src_level] + ((size_t)(oz + cz) * S + oy + cy) * S + ox + cx) != 0
                        : occ_box[occ_prev + (cz * cb + cy) * cb + cx] != 0;
        }
        occ_box[occ_off + r] = any ? 1 : 0;
        ms.occ_raw[dl][((size_t)((oz >> l) + z) * sd + (oy >> l) + y) * sd + (ox >> l) + x] = any ? 1 : 0;
      }
    }
    if (ms.skip_empty) {
      occ_prev = occ_off;
      occ_off += b3;
    }
    if (FROM_L0 && NMAPS >= 6 && l == 1) {
      // The six maps of level 1 read the same children: one thread per
      // destination texel evaluates all six directions (and, with the
      // isotropic map 6, the box mean too).
      for (int r = threadIdx.x; r < b3; r += kThreads) {
        const int x = r % b, y = (r / b) % b, z = r / (b * b);
        T ch[8], v6[6];
        const bool any = load_children(cur, cur_b, x, y, z, ch);
        // Eight zero children reduce to 0 in every direction (most of level
        // 0 is empty space): the blends are evaluated only where needed.
        if (any) {
          if constexpr (STORAGE == VCT_STORAGE_RGBA8) aniso6_rgba8(ch, v6);
          else aniso6_rgba16f(ch, v6);
        } else {
#pragma unroll
          for (int d = 0; d < 6; ++d) v6[d] = T{};
        }
        if (ms.skip_empty) occ_store<B>(ms, 1, ox, oy, oz, x, y, z, r, any, occ_box);
        const int dl = src_level + 1;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
          out[d * b3 + r] = v6[d];
          surf3Dwrite(v6[d], ms.surf[d][dl], ((ox >> 1) + x) * Texel<STORAGE>::kBytes, (oy >> 1) + y, (oz >> 1) + z);
        }
        if constexpr (NMAPS == 7) {
          const T v = any ? reduce<STORAGE>(ch, 0, true) : T{};
          out[6 * b3 + r] = v;
          surf3Dwrite(v, ms.surf[6][dl], ((ox >> 1) + x) * Texel<STORAGE>::kBytes, (oy >> 1) + y, (oz >> 1) + z);
        }
        if constexpr (STORAGE == VCT_STORAGE_RGBA8)
          if (ms.alpha_tex[0]) write_alpha(ms, dl, (ox >> 1) + x, (oy >> 1) + y, (oz >> 1) + z, v6, 1);
      }
      __syncthreads();
      cur = out;
      cur_b = b;
      cur_shared = false;
      out += NMAPS * b3;
      continue;
    }
    for (int i = threadIdx.x; i < NMAPS * b3; i += kThreads) {
      const int d = i / b3, r = i % b3;
      const int x = r % b, y = (r / b) % b, z = r / (b * b);
      const T* base = cur + (cur_shared ? 0 : d * cb3);
      T ch[8];
      const bool any = load_children(base, cur_b, x, y, z, ch);
      const T v = any ? reduce<STORAGE>(ch, d, NMAPS == 1 || d == 6) : T{};  // zero children reduce to 0
      out[i] = v;
      const int dl = src_level + l;
      surf3Dwrite(v, ms.surf[d][dl], ((ox >> l) + x) * Texel<STORAGE>::kBytes, (oy >> l) + y, (oz >> l) + z);
    }
    __syncthreads();
    if constexpr (NMAPS >= 6 && STORAGE == VCT_STORAGE_RGBA8) {
      if (ms.alpha_tex[0]) {
        // The alpha copies of this level, from the six maps in shared memory
        // (read only; the next level writes past them).
        for (int r = threadIdx.x; r < b3; r += kThreads) {
          const int x = r % b, y = (r / b) % b, z = r / (b * b);
          write_alpha(ms, src_level + l, (ox >> l) + x, (oy >> l) + y, (oz >> l) + z, out + r, b3);
        }
      }
    }
    cur = out;
    cur_b = b;
    cur_shared = false;
    out += NMAPS * b3;
  }
}

template <int NMAPS, bool FROM_L0, int K, int STORAGE>
__device__ __forceinline__ void mip_region(const MapSet& ms, int src_level, uint32_t region, unsigned char* smem_raw) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B = 1 << K;
  constexpr int B3 = B * B * B;
  constexpr int NSRC = FROM_L0 ? 1 : NMAPS;
  T* src = reinterpret_cast<T*>(smem_raw);
  T* lvl = src + NSRC * B3;  // level buffers follow, NMAPS * (B/2)^3, (B/4)^3, ...
  const int S = ms.N >> src_level;
  const int nbx = S / B;
  const int bx = region % nbx, by = (region / nbx) % nbx, bz = region / (nbx * nbx);
  const int ox = bx * B, oy = by * B, oz = bz * B;
  for (int i = threadIdx.x; i < NSRC * B3; i += kThreads) {
    const int m = i / B3, r = i % B3;
    const int x = r % B, y = (r / B) % B, z = r / (B * B);
    const cudaSurfaceObject_t s = FROM_L0 ? ms.l0_surf : ms.surf[m][src_level];
    T v;
    surf3Dread(&v, s, (ox + x) * Texel<STORAGE>::kBytes, oy + y, oz + z);
    src[i] = v;
  }
  __syncthreads();
  mip_reduce<NMAPS, FROM_L0, K, STORAGE>(ms, src_level, ox, oy, oz, src, lvl);
}

// ---- TMA-staged first pass --------------------------------------------------
// Level 0 in linear memory is read through a 3D tensor map, one 16^3 box per
// region, by cp.async.bulk.tensor into shared memory, completing on an
// mbarrier.  A persistent CTA double-buffers: while it reduces region i it
// has the copy of region i+1 in flight.  Every wait is bounded; a wait that
// gives up sets FrameStatus::async_timeout (the host reports an error),
// waits (bounded) for the copy it still has in flight and leaves.
#ifndef VCT_MIP_TMA_MIN_BLOCKS
#define VCT_MIP_TMA_MIN_BLOCKS 4  // resident CTAs per SM the RGBA8 TMA pass is compiled for
#endif
constexpr int kTmaBox = 16;
template <int NMAPS, int STORAGE>
__global__ void __launch_bounds__(kThreads, STORAGE == VCT_STORAGE_RGBA8 ? VCT_MIP_TMA_MIN_BLOCKS : 3) k_mip_tma(const __grid_constant__ CUtensorMap map, MapSet ms,
                                                      FrameStatus* status) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B3 = kTmaBox * kTmaBox * kTmaBox;
  constexpr uint32_t kBytes = B3 * sizeof(T);
  extern __shared__ __align__(128) unsigned char smem_tma[];
  __shared__ __align__(8) uint64_t bar[2];
  // Copy destinations 128-byte aligned (the launch adds 128 bytes of slack).
  unsigned char* base = smem_tma + ((128u - (smem_u32(smem_tma) & 127u)) & 127u);
  T* stage[2] = {reinterpret_cast<T*>(base), reinterpret_cast<T*>(base + kBytes)};
  T* lvl = reinterpret_cast<T*>(base + 2 * kBytes);
  const int nbx = ms.N / kTmaBox;
  const uint32_t total = (uint32_t)nbx * nbx * nbx;
  auto coords = [nbx](uint32_t r, int& x, int& y, int& z) {
    x = (int)(r % nbx) * kTmaBox;
    y = (int)((r / nbx) % nbx) * kTmaBox;
    z = (int)(r / ((uint32_t)nbx * nbx)) * kTmaBox;
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  uint32_t r = blockIdx.x;
  if (threadIdx.x == 0 && r < total) {
    int x, y, z;
    coords(r, x, y, z);
    tma_load_box3(&map, stage[0], &bar[0], kBytes, x, y, z);
  }
  for (uint32_t it = 0; r < total; r += gridDim.x, ++it) {
    const int s = (int)(it & 1);
    const uint32_t next = r + gridDim.x;
    if (threadIdx.x == 0 && next < total) {  // stage s^1 was released by the barrier ending iteration it-1
      int x, y, z;
      coords(next, x, y, z);
      tma_load_box3(&map, stage[s ^ 1], &bar[s ^ 1], kBytes, x, y, z);
    }
    const bool ok = mbar_wait(&bar[s], (it >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&status->async_timeout, 1u);
        if (next < total) mbar_wait(&bar[s ^ 1], ((it + 1) >> 1) & 1);  // the copy still in flight
      }
      __syncthreads();
      return;
    }
    int ox, oy, oz;
    coords(r, ox, oy, oz);
    mip_reduce<NMAPS, true, 4, STORAGE>(ms, 0, ox, oy, oz, stage[s], lvl);
    __syncthreads();  // every thread is done with stage s and the level buffers
  }
}

// One pass: source level `src_level` (0 = the shared level 0) -> levels
// src_level+1 .. src_level+K of NMAPS maps, one CTA per B^3 source region.
template <int NMAPS, bool FROM_L0, int K, int STORAGE>
__global__ void __launch_bounds__(kThreads) k_mip(MapSet ms, int src_level) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  mip_region<NMAPS, FROM_L0, K, STORAGE>(ms, src_level, blockIdx.x, smem_raw);
}

// The first pass (level 0 -> levels 1..4) of every scene of a batch in one
// persistent launch.
template <int NMAPS, int STORAGE>
__global__ void __launch_bounds__(kThreads, STORAGE == VCT_STORAGE_RGBA8 ? VCT_MIP_TMA_MIN_BLOCKS : 3) k_mip_batch(BatchWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (uint32_t g = blockIdx.x; g < w.total; g += gridDim.x) {
    const int s = batch_scene_of(w, g);
    mip_region<NMAPS, true, 4, STORAGE>(w.scenes[s].ms, 0, g - __ldg(w.prefix + s), smem_raw);
    __syncthreads();  // the next region overwrites the shared buffers
  }
}

// Level `level` (>= 2) of every scene of a batch from its level - 1, one
// thread per destination texel, all maps (the small last levels).
template <int NMAPS, int STORAGE>
__global__ void __launch_bounds__(kThreads) k_mip_level_batch(BatchWork w, int level) {
  typedef typename Texel<STORAGE>::T T;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < w.total; g += gridDim.x * blockDim.x) {
    const int s = batch_scene_of(w, g);
    const MapSet& ms = w.scenes[s].ms;
    const uint32_t r = g - __ldg(w.prefix + s);
    const int n = ms.N >> level;
    const int x = (int)(r % n), y = (int)((r / n) % n), z = (int)(r / ((uint32_t)n * n));
    T v[NMAPS];
#pragma unroll
    for (int d = 0; d < NMAPS; ++d) {
      T ch[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        surf3Dread(&ch[k], ms.surf[d][level - 1], (2 * x + c_off[k][0]) * Texel<STORAGE>::kBytes,
                   2 * y + c_off[k][1], 2 * z + c_off[k][2]);
      v[d] = reduce<STORAGE>(ch, d, NMAPS == 1);
      surf3Dwrite(v[d], ms.surf[d][level], x * Texel<STORAGE>::kBytes, y, z);
    }
    if constexpr (NMAPS == 6 && STORAGE == VCT_STORAGE_RGBA8)
      if (ms.alpha_tex[0]) write_alpha(ms, level, x, y, z, v, 1);
  }
}

template <int NMAPS, int STORAGE>
cudaError_t run_batch(const BatchWork& regions, const BatchWork* tail, int n_tail, int first_tail, cudaStream_t st,
                      int* launches) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B = 16;
  size_t smem = (size_t)B * B * B * sizeof(T);
  for (int l = 1; l <= 4; ++l) smem += (size_t)NMAPS * (B >> l) * (B >> l) * (B >> l) * sizeof(T);
  auto kern = k_mip_batch<NMAPS, STORAGE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int dev = 0, sms = 148, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (regions.total) {
    const unsigned grid = (unsigned)std::max(1, std::min<int>(sms * std::max(per_sm, 1), (int)regions.total));
    kern<<<grid, kThreads, smem, st>>>(regions);
    if (launches) ++*launches;
  }
  for (int t = 0; t < n_tail; ++t) {
    if (!tail[t].total) continue;
    const unsigned grid = (unsigned)std::min<uint32_t>((tail[t].total + kThreads - 1) / kThreads, (uint32_t)sms * 8);
    k_mip_level_batch<NMAPS, STORAGE><<<grid, kThreads, 0, st>>>(tail[t], first_tail + t);
    if (launches) ++*launches;
  }
  return cudaGetLastError();
}

template <int NMAPS, bool FROM_L0, int K, int STORAGE>
cudaError_t run_pass(const MapSet& ms, int src_level, cudaStream_t st) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B = 1 << K;
  constexpr int NSRC = FROM_L0 ? 1 : NMAPS;
  size_t smem = (size_t)NSRC * B * B * B * sizeof(T);
  for (int l = 1; l <= K; ++l) smem += (size_t)NMAPS * (B >> l) * (B >> l) * (B >> l) * sizeof(T);
  auto kern = k_mip<NMAPS, FROM_L0, K, STORAGE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int S = ms.N >> src_level;
  const unsigned grid = (unsigned)((S / B) * (S / B) * (S / B));
  kern<<<grid, kThreads, smem, st>>>(ms, src_level);
  return cudaGetLastError();
}

template <int NMAPS, bool FROM_L0, int STORAGE>
cudaError_t run_pass_k(const MapSet& ms, int src_level, int K, cudaStream_t st) {
  switch (K) {
    case 1: return run_pass<NMAPS, FROM_L0, 1, STORAGE>(ms, src_level, st);
    case 2: return run_pass<NMAPS, FROM_L0, 2, STORAGE>(ms, src_level, st);
    case 3: return run_pass<NMAPS, FROM_L0, 3, STORAGE>(ms, src_level, st);
    case 4: return run_pass<NMAPS, FROM_L0, 4, STORAGE>(ms, src_level, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int NMAPS, int STORAGE>
cudaError_t run_tma(const MapSet& ms, const CUtensorMap* map, FrameStatus* status, cudaStream_t st) {
  typedef typename Texel<STORAGE>::T T;
  constexpr int B = kTmaBox;
  size_t smem = 128 + 2 * (size_t)B * B * B * sizeof(T);
  for (int l = 1; l <= 4; ++l) smem += (size_t)NMAPS * (B >> l) * (B >> l) * (B >> l) * sizeof(T);
  auto kern = k_mip_tma<NMAPS, STORAGE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (STORAGE == VCT_STORAGE_RGBA8) {
    // shared memory for 4 CTAs per SM (the RGBA16F pass runs one per SM and
    // keeps the default split, which leaves more L1 for its surface reads)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
  }
  int dev = 0, sms = 148, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int nbx = ms.N / B;
  const int regions = nbx * nbx * nbx;
  kern<<<(unsigned)std::max(1, std::min(regions, sms * per_sm)), kThreads, smem, st>>>(*map, ms, status);
  return cudaGetLastError();
}

template <int NMAPS, int STORAGE>
cudaError_t run_all(const MapSet& ms, cudaStream_t st, int* launches, const CUtensorMap* map, FrameStatus* status,
                    int first_level) {
  cudaError_t e = cudaSuccess;
  int done = first_level;
  if (done == 0) {
    const int K1 = ms.L - 1 < 4 ? ms.L - 1 : 4;
    if (K1 < 1) return cudaSuccess;
    // The TMA-staged first pass needs four levels below a 16^3 box.
    e = (map && status && K1 == 4 && ms.N % kTmaBox == 0) ? run_tma<NMAPS, STORAGE>(ms, map, status, st)
                                                          : run_pass_k<NMAPS, true, STORAGE>(ms, 0, K1, st);
    if (e != cudaSuccess) return e;
    if (launches) ++*launches;
    done = K1;
  }
  // (seven RGBA16F source boxes of 16^3 would not fit in shared memory)
  constexpr int kTailMax = NMAPS == 7 && STORAGE == VCT_STORAGE_RGBA16F ? 3 : 4;
  while (done < ms.L - 1) {
    int K = ms.L - 1 - done;
    if (K > kTailMax) K = kTailMax;
    e = run_pass_k<NMAPS, false, STORAGE>(ms, done, K, st);
    if (e != cudaSuccess) return e;
    if (launches) ++*launches;
    done += K;
  }
  return cudaSuccess;
}

// ---- empty-space occupancy -------------------------------------------------
// Two passes over one 32-bit word per thread, every level of a map set in
// one launch each: (1) pack the raw occupancy of cells x0..x0+31 of a row
// into bits (occ_pack[c]; levels above the first pass's OR their block of
// level-occ_k bytes), (2) OR each cell with its +1 neighbours along x, y
// and z (occ[c]: the 2x2x2 block a trilinear lookup reads).

// Raw occupancy of cell (x, y, z) of level c (inside the grid).
__device__ __forceinline__ bool occ_raw_cell(const MapSet& ms, int c, int x, int y, int z) {
  if (c <= ms.occ_k) {
    const int s = ms.N >> c;
    return ms.occ_raw[c][((size_t)z * s + y) * s + x] != 0;
  }
  // The OR of the cell's f^3 block of level-k bytes: every row loaded
  // independently (no early exit, so the loads are in flight together).
  const int k = ms.occ_k, f = 1 << (c - k), sk = ms.N >> k;
  uint32_t any = 0u;
  for (int dz = 0; dz < f; ++dz)
    for (int dy = 0; dy < f; ++dy) {
      const uint8_t* row = ms.occ_raw[k] + ((size_t)(z * f + dz) * sk + (y * f + dy)) * sk + (size_t)x * f;
      if (f == 4) {
        any |= __ldg(reinterpret_cast<const uint32_t*>(row));  // 4-byte aligned: x * 4
      } else if (f == 8) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(row));  // 8-byte aligned: x * 8
        any |= v.x | v.y;
      } else if (f >= 16) {  // 16-byte aligned: x * f, and every row of level k holds a multiple of 16 bytes
        for (int dx = 0; dx < f; dx += 16) {
          const uint4 v = __ldg(reinterpret_cast<const uint4*>(row + dx));
          any |= v.x | v.y | v.z | v.w;
        }
      } else {
        for (int dx = 0; dx < f; ++dx) any |= __ldg(row + dx);
      }
    }
  return any != 0u;
}

__device__ void occ_pack_word(const MapSet& ms, int c, uint32_t w) {
  if (c == 1 && ms.occ_l1_packed) return;  // written packed by the first pass (16^3 regions)
  const int s = ms.N >> c, wpr = ms.occ_wpr[c];
  const int xw = (int)(w % wpr), y = (int)((w / wpr) % s), z = (int)(w / ((uint32_t)wpr * s));
  const int x0 = xw * 32;
  uint32_t bits = 0;
  if (c <= ms.occ_k && s >= 32) {
    // 32 bytes, 16-byte aligned (x0 and s are multiples of 32)
    const uint4* r = reinterpret_cast<const uint4*>(ms.occ_raw[c] + ((size_t)z * s + y) * s + x0);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const uint4 v4 = __ldg(r + j);
      const uint32_t v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) bits |= (((v[i] >> (8 * q)) & 0xffu) ? 1u : 0u) << (16 * j + 4 * i + q);
    }
  } else {
    for (int i = 0; i < 32 && x0 + i < s; ++i)
      if (occ_raw_cell(ms, c, x0 + i, y, z)) bits |= 1u << i;
  }
  ms.occ_pack[c][w] = bits;
}

// Bit i of word (x0 / 32) of row (y, z) of occ[c]: the OR over the 2x2x2
// cells x0+i .. x0+i+1, y .. y+1, z .. z+1 (the texels of one trilinear
// lookup whose lower texel is that cell); of occ3[c]: the OR over the
// 3x3x3 cells around it.
__device__ void occ_dilate_word(const MapSet& ms, int c, uint32_t w) {
  const int s = ms.N >> c, wpr = ms.occ_wpr[c];
  const int xw = (int)(w % wpr), y = (int)((w / wpr) % s), z = (int)(w / ((uint32_t)wpr * s));
  uint32_t box = 0, dil = 0;
  for (int dz = -1; dz <= 1; ++dz) {
    if ((unsigned)(z + dz) >= (unsigned)s) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      if ((unsigned)(y + dy) >= (unsigned)s) continue;
      const uint32_t* row = ms.occ_pack[c] + ((size_t)(z + dz) * s + (y + dy)) * wpr;
      const uint32_t cur = row[xw];
      const uint32_t lo = xw > 0 ? row[xw - 1] : 0u, hi = xw + 1 < wpr ? row[xw + 1] : 0u;
      const uint32_t up = cur | (cur >> 1) | (hi << 31);  // cells x0+i, x0+i+1
      dil |= up | (cur << 1) | (lo >> 31);                // and x0+i-1
      if (dz >= 0 && dy >= 0) box |= up;
    }
  }
  if (s - xw * 32 < 32) {
    box &= (1u << (s - xw * 32)) - 1u;
    dil &= (1u << (s - xw * 32)) - 1u;
  }
  ms.occ[c][w] = box;
  ms.occ3[c][w] = dil;
}

// Words of levels 1..L-1 of one map set, and the level of flat word g.
__host__ __device__ inline uint32_t occ_words(const MapSet& ms) {
  uint32_t t = 0;
  for (int c = 1; c < ms.L; ++c) t += (uint32_t)(ms.N >> c) * (uint32_t)(ms.N >> c) * (uint32_t)ms.occ_wpr[c];
  return t;
}
__device__ __forceinline__ int occ_level(const MapSet& ms, uint32_t& g) {
  for (int c = 1; c < ms.L; ++c) {
    const uint32_t n = (uint32_t)(ms.N >> c) * (uint32_t)(ms.N >> c) * (uint32_t)ms.occ_wpr[c];
    if (g < n) return c;
    g -= n;
  }
  return 0;
}

template <bool DILATE>
__global__ void __launch_bounds__(256) k_occupancy(MapSet ms, uint32_t total) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    uint32_t w = g;
    const int c = occ_level(ms, w);
    if (DILATE) occ_dilate_word(ms, c, w);
    else occ_pack_word(ms, c, w);
  }
}

template <bool DILATE>
__global__ void __launch_bounds__(256) k_occupancy_batch(BatchWork bw) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < bw.total; g += gridDim.x * blockDim.x) {
    const int s = batch_scene_of(bw, g);
    const MapSet& ms = bw.scenes[s].ms;
    if (!ms.skip_empty) continue;
    uint32_t w = g - __ldg(bw.prefix + s);
    const int c = occ_level(ms, w);
    if (DILATE) occ_dilate_word(ms, c, w);
    else occ_pack_word(ms, c, w);
  }
}

// ---- Texture3D helpers (create/clear/mip of standalone RGBA8 textures) ----
__global__ void k_fill_rgba8(cudaSurfaceObject_t s, int w, int h, int d, uchar4 v) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)w * h * d) return;
  const int x = (int)(i % w), y = (int)((i / w) % h), z = (int)(i / ((size_t)w * h));
  surf3Dwrite(v, s, x * 4, y, z);
}

// 2x2x2 box mean of the level below (glGenerateMipmap); for odd sizes the
// children are clamped to the source extent.
__global__ void k_box_mip_rgba8(cudaSurfaceObject_t src, int sw, int sh, int sd, cudaSurfaceObject_t dst, int dw,
                                int dh, int dd) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)dw * dh * dd) return;
  const int x = (int)(i % dw), y = (int)((i / dw) % dh), z = (int)(i / ((size_t)dw * dh));
  uint32_t S[4] = {0, 0, 0, 0};
  for (int k = 0; k < 8; ++k) {
    const int cx = min(2 * x + (k & 1), sw - 1), cy = min(2 * y + ((k >> 1) & 1), sh - 1),
              cz = min(2 * z + (k >> 2), sd - 1);
    uchar4 v;
    surf3Dread(&v, src, cx * 4, cy, cz);
    S[0] += v.x; S[1] += v.y; S[2] += v.z; S[3] += v.w;
  }
  surf3Dwrite(make_uchar4((S[0] + 4) >> 3, (S[1] + 4) >> 3, (S[2] + 4) >> 3, (S[3] + 4) >> 3), dst, x * 4, y, z);
}

}  // namespace

cudaError_t launch_mipmap(const MapSet& ms, int mip_mode, cudaStream_t st, int* launches, const void* tmap,
                          FrameStatus* status, int first_level) {
  const CUtensorMap* map = static_cast<const CUtensorMap*>(tmap);
  const int fl = first_level;
  cudaError_t e;
  if (mip_mode == VCT_MIP_ISO) {
    e = ms.storage == VCT_STORAGE_RGBA8 ? run_all<1, VCT_STORAGE_RGBA8>(ms, st, launches, map, status, fl)
                                        : run_all<1, VCT_STORAGE_RGBA16F>(ms, st, launches, map, status, fl);
  } else if (mip_mode == VCT_MIP_BOTH) {
    e = ms.storage == VCT_STORAGE_RGBA8 ? run_all<7, VCT_STORAGE_RGBA8>(ms, st, launches, map, status, fl)
                                        : run_all<7, VCT_STORAGE_RGBA16F>(ms, st, launches, map, status, fl);
  } else {
    e = ms.storage == VCT_STORAGE_RGBA8 ? run_all<6, VCT_STORAGE_RGBA8>(ms, st, launches, map, status, fl)
                                        : run_all<6, VCT_STORAGE_RGBA16F>(ms, st, launches, map, status, fl);
  }
  if (e != cudaSuccess || !ms.skip_empty || ms.L < 2) return e;
  // Every level now has its occupancy bytes (first pass or brick kernel,
  // then the tail passes).
  MapSet mo = ms;
  mo.occ_k = ms.L - 1;
  const uint32_t total = occ_words(mo);
  k_occupancy<false><<<(total + 255) / 256, 256, 0, st>>>(mo, total);
  k_occupancy<true><<<(total + 255) / 256, 256, 0, st>>>(mo, total);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

cudaError_t launch_occupancy_batch(const BatchWork& words, cudaStream_t st, int* launches) {
  if (!words.total) return cudaSuccess;
  k_occupancy_batch<false><<<(words.total + 255) / 256, 256, 0, st>>>(words);
  k_occupancy_batch<true><<<(words.total + 255) / 256, 256, 0, st>>>(words);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

uint32_t occupancy_words(const MapSet& ms) { return ms.skip_empty && ms.L > 1 ? occ_words(ms) : 0u; }

cudaError_t launch_mipmap_batch(const BatchWork& regions, const BatchWork* tail, int n_tail, int first_tail,
                                int storage, cudaStream_t st, int* launches) {
  // Every scene of a batch is anisotropic (6 maps); levels 1..4 in the first
  // launch (unless the brick kernel wrote 1-3), the tail levels (where a
  // scene has them) in one launch each.
  return storage == VCT_STORAGE_RGBA8
             ? run_batch<6, VCT_STORAGE_RGBA8>(regions, tail, n_tail, first_tail, st, launches)
             : run_batch<6, VCT_STORAGE_RGBA16F>(regions, tail, n_tail, first_tail, st, launches);
}

cudaError_t launch_fill_rgba8(cudaSurfaceObject_t s, int w, int h, int d, uchar4 v, cudaStream_t st) {
  const size_t n = (size_t)w * h * d;
  if (!n) return cudaSuccess;
  k_fill_rgba8<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, w, h, d, v);
  return cudaGetLastError();
}

cudaError_t launch_box_mip_rgba8(cudaSurfaceObject_t src, int sw, int sh, int sd, cudaSurfaceObject_t dst, int dw,
                                 int dh, int dd, cudaStream_t st) {
  const size_t n = (size_t)dw * dh * dd;
  if (!n) return cudaSuccess;
  k_box_mip_rgba8<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, sw, sh, sd, dst, dw, dh, dd);
  return cudaGetLastError();
}

}  // namespace vct
