// k_scan.cu -- device-wide exclusive prefix sum of u32 counts (brick list
// offsets of the voxelizer).  Three stream-ordered kernels: per-tile scan,
// scan of the tile totals in one CTA, add-back.
#include <cstring>

#include "vct_internal.h"

namespace vct {
namespace {

constexpr int kT = 1024;          // threads per tile
constexpr int kI = 4;             // items per thread
constexpr int kTile = kT * kI;

// Exclusive block scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t& excl) {
  __shared__ uint32_t warp_tot[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
    uint32_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    warp_tot[lane] = wi - w;  // exclusive warp offsets
  }
  __syncthreads();
  excl = warp_tot[warp] + incl - v;
  uint32_t total = __shfl_sync(0xffffffffu, incl, 31) + warp_tot[warp];
  total = __shfl_sync(0xffffffffu, total, 31);
  __shared__ uint32_t s_total;
  if (threadIdx.x == blockDim.x - 1) s_total = excl + v;
  __syncthreads();
  uint32_t r = s_total;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kT) k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                   uint32_t* __restrict__ tile_tot, size_t n) {
  const size_t base = (size_t)blockIdx.x * kTile + (size_t)threadIdx.x * kI;
  uint32_t v[kI];
  uint32_t s = 0;
  for (int i = 0; i < kI; ++i) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t ex;
  const uint32_t tot = block_excl_scan(s, ex);
  for (int i = 0; i < kI; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  if (threadIdx.x == 0) tile_tot[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kT) k_scan_top(uint32_t* __restrict__ tile_tot, size_t ntiles,
                                                 uint32_t* __restrict__ out_total, ScanFuse fuse) {
  uint32_t carry = 0;
  for (size_t b = 0; b < ntiles; b += kT) {
    const size_t i = b + threadIdx.x;
    const uint32_t v = i < ntiles ? tile_tot[i] : 0u;
    uint32_t ex;
    const uint32_t tot = block_excl_scan(v, ex);
    if (i < ntiles) tile_tot[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) {
    *out_total = carry;
    if (fuse.total_copy) *fuse.total_copy = carry;
  }
  if (fuse.hb.slot && threadIdx.x < 3) fuse.hb.counters[threadIdx.x] = 0u;  // the plan's counters, before k_scan_add
}

__global__ void __launch_bounds__(256) k_scan_add(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                  uint32_t* __restrict__ copy_out,
                                                  const uint32_t* __restrict__ tile_tot, size_t n, ScanFuse fuse) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = out[i] + tile_tot[i / kTile];
  out[i] = v;
  if (copy_out) copy_out[i] = v;
  if (fuse.hb.slot) {
    const uint32_t c = fuse.cap;
    heavy_plan_brick((uint32_t)i, min(v, c), min(v + in[i], c), min(out[n], c), fuse.slots, fuse.hb);
  }
}

}  // namespace

size_t scan_tmp_words(size_t n) { return (n + kTile - 1) / kTile + 1; }

cudaError_t launch_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t* copy_out, size_t n, uint32_t* tmp,
                                  cudaStream_t st, int* launches, const ScanFuse* fuse) {
  ScanFuse f;
  std::memset(&f, 0, sizeof(f));
  if (fuse) f = *fuse;
  if (n == 0) {
    // No bricks: nothing to plan (the counters still start at zero).
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess && f.total_copy) e = cudaMemsetAsync(f.total_copy, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess && f.hb.slot) e = cudaMemsetAsync(f.hb.counters, 0, 3 * sizeof(uint32_t), st);
    return e;
  }
  const size_t ntiles = (n + kTile - 1) / kTile;
  k_scan_tiles<<<(unsigned)ntiles, kT, 0, st>>>(in, out, tmp, n);
  k_scan_top<<<1, kT, 0, st>>>(tmp, ntiles, out + n, f);
  k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, copy_out, tmp, n, f);
  if (launches) *launches += 3;
  return cudaGetLastError();
}

}  // namespace vct
