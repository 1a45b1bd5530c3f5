// vct_snap.h -- exact fixed-point snapping of FP32 grid-space coordinates,
// in integer arithmetic (host and device).
//
// The voxelizers snap each vertex coordinate g (grid space, |g| <= 64) to
// round((g + 1) * 2^k), rounding half to even, with 2^k = N * 256 (the 2N x
// 2N raster's 1/256-sample grid) or N * 128 (the conservative rule's 1/256
// voxel).  The result is the exact value of that expression: g = m * 2^e
// with a 24-bit integer m, so (g + 1) * 2^k = 2^k + m * 2^(e + k); the
// second term is an integer or is rounded half to even by a shift, and
// adding the even integer 2^k does not change which neighbour is even.
// (It equals rounding the double (double)g + 1.0 scaled by 2^k: that sum is
// exact for |g| >= 2^-29, and for smaller g both give 2^k.)  No FP64
// arithmetic is involved.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define VCT_SNAP_HD __host__ __device__
#else
#define VCT_SNAP_HD
#endif

namespace vct {

// round-half-even((g + 1) * 2^k) for finite g with |g| <= 64 and 1 <= k <= 24.
VCT_SNAP_HD inline long long snap_fixed(float g, int k) {
#ifdef __CUDA_ARCH__
  const uint32_t bits = __float_as_uint(g);
#else
  uint32_t bits;
  std::memcpy(&bits, &g, sizeof(bits));
#endif
  const int exp = (int)((bits >> 23) & 0xffu);
  const long long base = 1LL << k;
  if (exp == 0) return base;  // zero or subnormal: |g * 2^k| < 1/2
  const uint32_t m = (bits & 0x7fffffu) | 0x800000u;
  const int s = exp - 150 + k;  // g * 2^k = m * 2^s
  long long q;
  if (s >= 0) {
    q = (long long)m << s;
  } else {
    const int sh = -s;
    if (sh > 24) {
      q = 0;  // m * 2^s < 1/2
    } else {
      const uint32_t rem = m & ((1u << sh) - 1u), half = 1u << (sh - 1);  // sh in [1, 24]
      q = (long long)(m >> sh);
      if (rem > half || (rem == half && (q & 1))) ++q;
    }
  }
  return (bits >> 31) ? base - q : base + q;
}

}  // namespace vct
