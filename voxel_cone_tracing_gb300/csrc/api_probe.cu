// api_probe.cu -- vct_measure_texture_rate: the texture unit's throughput
// for the fetches the cone tracer issues, measured on the current device.
//
// The cone tracer (k_trace.cu) is bound by the texture unit, not by HBM: its
// texels are served from L1 (the whole mip chain of a 256^3 grid fits in
// L2, and a warp's neighbouring cones read the same cache lines).  The
// denominator of its roofline is therefore the rate at which one GPU filters
// 3D RGBA8 fetches when nothing else limits it: every lane of every warp
// fetching, texels L1-resident, enough independent fetches in flight.
//
// Kinds (the three fetch shapes of the tracer's texture-unit path):
//   0 -- tex3DLod of a mipmapped RGBA8 texture at a fractional lod: trilinear
//        within two levels and linear between them (16 texels);
//   1 -- tex3D of a non-mipmapped RGBA8 texture (the shared level 0):
//        trilinear (8 texels);
//   2 -- tex3DLod of the mipmapped texture at an integer lod: one level.
// The texture is 32^3 with 6 levels, the addressing and filtering those of
// the voxel maps (normalised coordinates, border 0, linear filters).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "api_common.h"

namespace vct {
namespace {

constexpr int kProbeRes = 32;
constexpr int kProbeLevels = 6;
constexpr int kProbeThreads = 256;
constexpr int kProbeUnroll = 4;

// Each warp samples a 4 x 8 footprint of positions 1/64 texel apart that
// drifts slowly through the texture, so that every fetch is an L1 hit and
// no two fetches of a thread are the same computation.
template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) k_tex_rate(cudaTextureObject_t tex, uint32_t iters, float lod,
                                                            float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float du = 1.0f / (64.0f * kProbeRes);
  float ux = 0.25f + (float)(lane & 3) * du + (float)(blockIdx.x & 7) * 0.04f;
  float uy = 0.25f + (float)(lane >> 2) * du + (float)((threadIdx.x >> 5) & 7) * 0.04f;
  float uz = 0.25f + (float)((blockIdx.x >> 3) & 7) * 0.04f;
  const float step = 1.0f / (256.0f * kProbeRes);
  float4 a[kProbeUnroll];
  for (int k = 0; k < kProbeUnroll; ++k) a[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (uint32_t i = 0; i < iters; i += kProbeUnroll) {
#pragma unroll
    for (int k = 0; k < kProbeUnroll; ++k) {
      const float z = uz + (float)k * du;
      float4 t;
      if (KIND == 1) t = tex3D<float4>(tex, ux, uy, z);
      else t = tex3DLod<float4>(tex, ux, uy, z, lod);
      a[k].x += t.x;
      a[k].y += t.y;
      a[k].z += t.z;
      a[k].w += t.w;
    }
    ux += step;
    uy += step;
  }
  float s = 0.0f;
  for (int k = 0; k < kProbeUnroll; ++k) s += a[k].x + a[k].y + a[k].z + a[k].w;
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

struct ProbeTexture {
  cudaMipmappedArray_t mip = nullptr;
  cudaArray_t flat = nullptr;
  cudaTextureObject_t tex = 0;
  ~ProbeTexture() {
    if (tex) cudaDestroyTextureObject(tex);
    if (mip) cudaFreeMipmappedArray(mip);
    if (flat) cudaFreeArray(flat);
  }
};

vct_status copy_level(cudaArray_t dst, int s, const std::vector<uint8_t>& src) {
  cudaMemcpy3DParms cp;
  std::memset(&cp, 0, sizeof(cp));
  cp.srcPtr = make_cudaPitchedPtr(const_cast<uint8_t*>(src.data()), (size_t)s * 4, s, s);
  cp.dstArray = dst;
  cp.extent = make_cudaExtent(s, s, s);
  cp.kind = cudaMemcpyHostToDevice;
  VCT_CUDA(cudaMemcpy3D(&cp));
  return VCT_OK;
}

vct_status make_texture(int kind, ProbeTexture& pt) {
  const cudaChannelFormatDesc desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
  std::vector<uint8_t> data((size_t)kProbeRes * kProbeRes * kProbeRes * 4);
  uint32_t x = 0x9e3779b9u;
  for (auto& b : data) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    b = (uint8_t)(x >> 24);
  }
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof(rd));
  if (kind == 1) {
    VCT_CUDA(cudaMalloc3DArray(&pt.flat, &desc, make_cudaExtent(kProbeRes, kProbeRes, kProbeRes)));
    VCT_CHECK(copy_level(pt.flat, kProbeRes, data));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = pt.flat;
  } else {
    VCT_CUDA(cudaMallocMipmappedArray(&pt.mip, &desc, make_cudaExtent(kProbeRes, kProbeRes, kProbeRes),
                                      kProbeLevels));
    for (int l = 0; l < kProbeLevels; ++l) {
      cudaArray_t la;
      VCT_CUDA(cudaGetMipmappedArrayLevel(&la, pt.mip, l));
      VCT_CHECK(copy_level(la, kProbeRes >> l, data));
    }
    rd.resType = cudaResourceTypeMipmappedArray;
    rd.res.mipmap.mipmap = pt.mip;
  }
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof(td));
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  td.mipmapFilterMode = cudaFilterModeLinear;
  td.minMipmapLevelClamp = 0.0f;
  td.maxMipmapLevelClamp = (float)(kProbeLevels - 1);
  VCT_CUDA(cudaCreateTextureObject(&pt.tex, &rd, &td, nullptr));
  return VCT_OK;
}

}  // namespace
}  // namespace vct

using namespace vct;

extern "C" vct_status vct_measure_texture_rate(int32_t kind, uint32_t iters, double* fetches_per_s, double* ms) {
  clear_error();
  if (kind < 0 || kind > 2) return set_error(VCT_ERR_INVALID_VALUE, "kind %d (0, 1 or 2)", kind);
  if (!fetches_per_s) return set_error(VCT_ERR_INVALID_VALUE, "fetches_per_s is NULL");
  // (at most 8192 fetches per thread: the footprint stays inside the texture)
  if (iters < kProbeUnroll || iters > 8192u) return set_error(VCT_ERR_INVALID_VALUE, "iters %u (4 .. 8192)", iters);
  iters -= iters % kProbeUnroll;
  int dev = 0, sms = 0;
  VCT_CUDA(cudaGetDevice(&dev));
  VCT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  ProbeTexture pt;
  VCT_CHECK(make_texture(kind, pt));
  int per_sm = 0;
  const void* fn = kind == 0 ? (const void*)k_tex_rate<0> : (kind == 1 ? (const void*)k_tex_rate<1>
                                                                        : (const void*)k_tex_rate<2>);
  VCT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kProbeThreads, 0));
  const unsigned blocks = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
  float* out = nullptr;
  VCT_CUDA(cudaMalloc(&out, (size_t)blocks * kProbeThreads * sizeof(float)));
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  const float lod = kind == 0 ? 1.5f : 1.0f;
  float best = 0.0f;
  for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {  // the first launch warms up
    err = cudaEventRecord(e0, st);
    if (err != cudaSuccess) break;
    if (kind == 0) k_tex_rate<0><<<blocks, kProbeThreads, 0, st>>>(pt.tex, iters, lod, out);
    else if (kind == 1) k_tex_rate<1><<<blocks, kProbeThreads, 0, st>>>(pt.tex, iters, lod, out);
    else k_tex_rate<2><<<blocks, kProbeThreads, 0, st>>>(pt.tex, iters, lod, out);
    err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    if (err == cudaSuccess && rep > 0 && (best == 0.0f || t < best)) best = t;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(out);
  if (err != cudaSuccess) return cuda_status(err, "texture rate probe");
  const double fetches = (double)blocks * kProbeThreads * (double)iters;
  *fetches_per_s = fetches / (best * 1e-3);
  if (ms) *ms = best;
  return VCT_OK;
}
