// api_common.h -- error reporting and small RAII helpers of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/vct.h"

namespace vct {

vct_status set_error(vct_status s, const char* fmt, ...);
void clear_error();
vct_status cuda_status(cudaError_t e, const char* what);

#define VCT_CUDA(expr)                                        \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) return ::vct::cuda_status(_e, #expr); \
  } while (0)

#define VCT_CHECK(expr)                 \
  do {                                  \
    vct_status _s = (expr);             \
    if (_s != VCT_OK) return _s;        \
  } while (0)

// Device buffer that only grows.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  vct_status ensure(size_t count) {
    if (count <= n && p) return VCT_OK;
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_status(e, "cudaMalloc");
    }
    n = count;
    return VCT_OK;
  }
};

// Pinned host buffer that only grows.
template <class T>
struct HostBuf {
  T* p = nullptr;
  size_t n = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
  vct_status ensure(size_t count) {
    if (count <= n && p) return VCT_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocHost(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_status(e, "cudaMallocHost");
    }
    n = count;
    return VCT_OK;
  }
};

vct_status ensure_device();

// Number of materials of a renderer (the next add_material id).
uint32_t material_count(const vct_renderer* r);

}  // namespace vct
