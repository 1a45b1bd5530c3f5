// k_samples.cu -- training data of the learned diffuse term: points drawn
// uniformly by area over the queued triangles, with the attributes the
// G-buffer resolve produces for a visible pixel (texture-space position,
// interpolated world normal, material albedo).
#include "vct_internal.h"
#include "vct_math.cuh"

namespace vct {
namespace {

__device__ __forceinline__ int find_instance(const SceneParams& sp, uint32_t t) {
  int lo = 0, hi = (int)sp.n_instances - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sp.inst[mid].tri_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ float hash01(uint64_t key) {
  key ^= key >> 33; key *= 0xff51afd7ed558ccdull; key ^= key >> 33; key *= 0xc4ceb9fe1a85ec53ull; key ^= key >> 33;
  return ((float)(key >> 40) + 0.5f) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ V3 world_vertex(const DevInstance& in, uint32_t vi, V3* nrm) {
  const float4* vp = reinterpret_cast<const float4*>(in.verts + vi);
  const float4 a = __ldg(vp), b = __ldg(vp + 1);
  if (nrm) *nrm = normalize(nm_mul(in.NM, a.w, b.x, b.y));
  return v3(xform_row(in.M, 0, a.x, a.y, a.z), xform_row(in.M, 1, a.x, a.y, a.z), xform_row(in.M, 2, a.x, a.y, a.z));
}

__global__ void k_tri_area(SceneParams sp, float* __restrict__ area) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= sp.total_tris) return;
  const DevInstance& in = sp.inst[find_instance(sp, t)];
  const uint32_t lt = t - in.tri_base;
  V3 w[3];
  for (int k = 0; k < 3; ++k) w[k] = world_vertex(in, __ldg(in.indices + 3 * (size_t)lt + k), nullptr);
  area[t] = 0.5f * length(cross(w[1] - w[0], w[2] - w[0]));
}

__global__ void k_sample_surface(SceneParams sp, const float* __restrict__ cdf, int n, uint64_t seed,
                                 float* __restrict__ samples) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = (seed * 0x9e3779b97f4a7c15ull) ^ ((uint64_t)i * 0xd1b54a32d192ed03ull);
  const float total = cdf[sp.total_tris - 1];
  const float x = hash01(key) * total;
  int lo = 0, hi = (int)sp.total_tris - 1;  // first t with cdf[t] > x
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cdf[mid] > x) hi = mid; else lo = mid + 1;
  }
  const uint32_t t = (uint32_t)lo;
  const DevInstance& in = sp.inst[find_instance(sp, t)];
  const uint32_t lt = t - in.tri_base;
  V3 w[3], nn[3];
  for (int k = 0; k < 3; ++k) w[k] = world_vertex(in, __ldg(in.indices + 3 * (size_t)lt + k), &nn[k]);
  const float r1 = sqrtf(hash01(key + 1)), r2 = hash01(key + 2);
  const float b0 = 1.0f - r1, b1 = r1 * (1.0f - r2), b2 = r1 * r2;
  const V3 wp = w[0] * b0 + w[1] * b1 + w[2] * b2;
  const V3 nrm = nn[0] * b0 + nn[1] * b1 + nn[2] * b2;
  const uint32_t mat = __ldg(sp.obj_material + __ldg(in.tri_obj + lt));
  const vct_material_data& m = sp.materials[mat];
  const float ic = 1.0f / sp.cube_size;
  float* q = samples + (size_t)i * 12;
  q[0] = 0.5f * wp.x * ic + 0.5f;
  q[1] = 0.5f * wp.y * ic + 0.5f;
  q[2] = 0.5f * wp.z * ic + 0.5f;
  q[3] = nrm.x; q[4] = nrm.y; q[5] = nrm.z;
  q[6] = m.diffuse[0]; q[7] = m.diffuse[1]; q[8] = m.diffuse[2];
  q[9] = q[10] = q[11] = 0.f;
}

}  // namespace

cudaError_t launch_tri_area(const SceneParams& sp, float* area, cudaStream_t st) {
  if (!sp.total_tris) return cudaSuccess;
  k_tri_area<<<(sp.total_tris + 255) / 256, 256, 0, st>>>(sp, area);
  return cudaGetLastError();
}

cudaError_t launch_sample_surface(const SceneParams& sp, const float* cdf, int n, uint64_t seed, float* samples,
                                  cudaStream_t st) {
  if (n <= 0 || !sp.total_tris) return cudaSuccess;
  k_sample_surface<<<(n + 255) / 256, 256, 0, st>>>(sp, cdf, n, seed, samples);
  return cudaGetLastError();
}

}  // namespace vct
