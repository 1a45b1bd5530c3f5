// vct_mip.cuh -- the exact RGBA8 anisotropic mip rule (mipmap.comp:40-98),
// shared by the MipBuilder (k_mipmap.cu) and the brick kernel's fused first
// levels (k_voxelize.cu).
//
// With texels k/255 the stored value of mean(alpha_blend(front, back)) over
// the four (front, back) child pairs of a direction is round(S / 1020) with
// S = sum over the pairs of (F*255 + (255-F.a)*B) per channel, ties up,
// clamped to 255 -- the exact real value of the GLSL expression, rounded to
// unorm8 as imageStore does.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace vct {

// voxel_offsets, mipmap.comp:10-20: child k of texel x is 2x + c_mip_off[k].
__device__ constexpr int c_mip_off[8][3] = {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0},
                                            {0, 1, 1}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
// (front, back) child pairs per map (0:-x 1:+x 2:-y 3:+y 4:-z 5:+z), mipmap.comp:59-98.
__device__ constexpr int c_pairs_h[6][4][2] = {
    {{0, 4}, {1, 5}, {2, 6}, {3, 7}}, {{4, 0}, {5, 1}, {6, 2}, {7, 3}},
    {{0, 2}, {1, 3}, {5, 7}, {4, 6}}, {{2, 0}, {3, 1}, {7, 5}, {6, 4}},
    {{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{1, 0}, {3, 2}, {5, 4}, {7, 6}}};

__device__ __forceinline__ uint32_t ch8(uint32_t t, int c) { return (t >> (8 * c)) & 0xffu; }

// All six directions of one destination texel from the same 8 children
// (level 1, where every map reads the shared level 0): each child's channels
// are unpacked once.
__device__ __forceinline__ void aniso6_rgba8(const uint32_t* ch, uint32_t* out) {
  uint32_t c[8][4];
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int q = 0; q < 4; ++q) c[k][q] = ch8(ch[k], q);
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    uint32_t o = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t S = 0;
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int f = c_pairs_h[d][p][0], b = c_pairs_h[d][p][1];
        S += c[f][q] * 255u + (255u - c[f][3]) * c[b][q];
      }
      const uint32_t v = (S + 510u) / 1020u;
      o |= (v > 255u ? 255u : v) << (8 * q);
    }
    out[d] = o;
  }
}

// Index of child k (as in c_mip_off) of destination texel (x, y, z) in a
// cube of side s2 = twice the destination's, stored [z][y][x].
__device__ __forceinline__ int mip_child(int s2, int x, int y, int z, int k) {
  return ((2 * z + 1 - (k & 1)) * s2 + 2 * y + 1 - ((k >> 1) & 1)) * s2 + 2 * x + 1 - ((k >> 2) & 1);
}

// Direction d (a run-time value: one code path for all six maps) of one
// destination texel whose children come from child(k).  The (front, back)
// pairs of map d are the children with d's axis bit (x: 4, y: 2, z: 1 in k)
// clear and set, front the clear one for the minus direction (c_pairs_h);
// S is a sum, so the pairs' order does not matter and the result equals
// the table's rule.
template <class Child>
__device__ __forceinline__ uint32_t aniso_rgba8_dir(int d, Child child) {
  const int bit = 4 >> (d >> 1), sel = (d & 1) ? bit : 0;
  uint32_t S[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int k = ((p & (bit - 1)) | ((p & ~(bit - 1)) << 1)) | sel;
    const uint32_t f = child(k), b = child(k ^ bit), fa = 255u - ch8(f, 3);
#pragma unroll
    for (int q = 0; q < 4; ++q) S[q] += ch8(f, q) * 255u + fa * ch8(b, q);
  }
  uint32_t o = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t v = (S[q] + 510u) / 1020u;
    o |= (v > 255u ? 255u : v) << (8 * q);
  }
  return o;
}

// ---- RGBA16F (half texels): the mean of the four blend(front, back) pairs
// in FP32, rounded to half -- one definition, each operation rounded once
// in a fixed order, so that the MipBuilder and the brick kernel's fused
// levels give the same bits.
__device__ __forceinline__ float4 h2f(uint2 t) {
  __half2 a = *reinterpret_cast<__half2*>(&t.x), b = *reinterpret_cast<__half2*>(&t.y);
  float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ uint2 f2h(float4 v) {
  __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
  return make_uint2(*reinterpret_cast<uint32_t*>(&a), *reinterpret_cast<uint32_t*>(&b));
}
// acc += f + (1 - f.a) * b
__device__ __forceinline__ void blend16(float4& acc, float4 f, float4 b) {
  const float k = __fsub_rn(1.0f, f.w);
  acc.x = __fadd_rn(acc.x, __fmaf_rn(k, b.x, f.x));
  acc.y = __fadd_rn(acc.y, __fmaf_rn(k, b.y, f.y));
  acc.z = __fadd_rn(acc.z, __fmaf_rn(k, b.z, f.z));
  acc.w = __fadd_rn(acc.w, __fmaf_rn(k, b.w, f.w));
}
__device__ __forceinline__ uint2 finish16(float4 acc) {
  return f2h(make_float4(__fmul_rn(acc.x, 0.25f), __fmul_rn(acc.y, 0.25f), __fmul_rn(acc.z, 0.25f),
                         __fmul_rn(acc.w, 0.25f)));
}
// Direction d (run-time) of one destination texel whose children come from
// child(k), the pairs summed in the order of c_pairs_h[d] (the order matters
// in floating point: for the y maps the table takes its last two pairs the
// other way round).
template <class Child>
__device__ __forceinline__ uint2 aniso_rgba16f_dir(int d, Child child) {
  const int bit = 4 >> (d >> 1), sel = (d & 1) ? bit : 0;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int pp = bit == 2 ? (p ^ (p >> 1)) : p;
    const int k = ((pp & (bit - 1)) | ((pp & ~(bit - 1)) << 1)) | sel;
    blend16(acc, h2f(child(k)), h2f(child(k ^ bit)));
  }
  return finish16(acc);
}

}  // namespace vct
