// vct_math.cuh -- small device vector helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vct {

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
// normalize(0) is undefined in GLSL; the engine (and the oracle) return 0.
__device__ __forceinline__ V3 normalize(V3 a) {
  float l2 = dot(a, a);
  if (!(l2 > 0.0f)) return v3(0.f, 0.f, 0.f);
  return a * rsqrtf(l2);
}
__device__ __forceinline__ V3 vabs(V3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// IEEE-rounded FP32 operations in a fixed order (no contraction into FMA):
// the coverage decisions that the oracle reproduces bit-for-bit use these.
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }

// (M * vec4(p, 1)).row r, column-major M, terms in column order.
__device__ __forceinline__ float xform_row(const float* M, int r, float px, float py, float pz) {
  float t = rmul(M[0 * 4 + r], px);
  t = radd(t, rmul(M[1 * 4 + r], py));
  t = radd(t, rmul(M[2 * 4 + r], pz));
  return radd(t, M[3 * 4 + r]);
}

__device__ __forceinline__ V3 nm_mul(const float* nm, float x, float y, float z) {
  return v3(nm[0] * x + nm[1] * y + nm[2] * z, nm[3] * x + nm[4] * y + nm[5] * z,
            nm[6] * x + nm[7] * y + nm[8] * z);
}

__device__ __forceinline__ long long edge_fn(long long ax, long long ay, long long bx, long long by, long long sx,
                                             long long sy) {
  return (bx - ax) * (sy - ay) - (by - ay) * (sx - ax);
}
// Fill rule for samples exactly on an edge (counter-clockwise, y up): keep
// left edges (dy < 0) and top edges (dy == 0, dx < 0).
__device__ __forceinline__ bool top_left(long long ax, long long ay, long long bx, long long by) {
  long long dy = by - ay, dx = bx - ax;
  return dy < 0 || (dy == 0 && dx < 0);
}

__device__ __forceinline__ long long floor_div(long long a, long long b) {
  long long q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}
__device__ __forceinline__ long long ceil_div(long long a, long long b) { return -floor_div(-a, b); }

}  // namespace vct
