// api_tex3d.cu -- Texture3D helpers of include/vct.h (texture_3d.h:6-10):
// standalone RGBA8 3D textures with a mip chain, addressed by GL-style names.
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "api_common.h"
#include "vct_internal.h"

using namespace vct;

namespace {

struct Tex3D {
  cudaMipmappedArray_t arr = nullptr;
  int w = 0, h = 0, d = 0, levels = 0;
  std::vector<cudaSurfaceObject_t> surf;
  ~Tex3D() {
    for (auto s : surf)
      if (s) cudaDestroySurfaceObject(s);
    if (arr) cudaFreeMipmappedArray(arr);
  }
  int lw(int l) const { return std::max(1, w >> l); }
  int lh(int l) const { return std::max(1, h >> l); }
  int ld(int l) const { return std::max(1, d >> l); }
};

std::mutex g_mu;
std::unordered_map<uint32_t, std::unique_ptr<Tex3D>> g_tex;
uint32_t g_next = 1;
cudaStream_t g_stream = nullptr;

vct_status tex_stream() {
  if (!g_stream) VCT_CUDA(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
  return VCT_OK;
}

Tex3D* find(vct_tex3d t) {
  auto it = g_tex.find(t);
  return it == g_tex.end() ? nullptr : it->second.get();
}

vct_status copy_level(Tex3D* t, int level, void* host, bool upload) {
  cudaArray_t a;
  VCT_CUDA(cudaGetMipmappedArrayLevel(&a, t->arr, level));
  cudaMemcpy3DParms p;
  std::memset(&p, 0, sizeof(p));
  const size_t w = t->lw(level), h = t->lh(level), d = t->ld(level);
  if (upload) {
    p.srcPtr = make_cudaPitchedPtr(host, w * 4, w, h);
    p.dstArray = a;
    p.kind = cudaMemcpyHostToDevice;
  } else {
    p.srcArray = a;
    p.dstPtr = make_cudaPitchedPtr(host, w * 4, w, h);
    p.kind = cudaMemcpyDeviceToHost;
  }
  p.extent = make_cudaExtent(w, h, d);
  VCT_CUDA(cudaMemcpy3DAsync(&p, g_stream));
  VCT_CUDA(cudaStreamSynchronize(g_stream));
  return VCT_OK;
}

}  // namespace

extern "C" vct_tex3d vct_create_tex_3d(int32_t width, int32_t height, int32_t depth, int32_t levels) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  if (width <= 0 || height <= 0 || depth <= 0 || levels <= 0) {
    set_error(VCT_ERR_INVALID_VALUE, "bad texture size %dx%dx%d, %d levels", width, height, depth, levels);
    return 0;
  }
  // glTexStorage3D: levels <= floor(log2(max dimension)) + 1.
  int m = std::max(width, std::max(height, depth)), maxl = 1;
  while (m > 1) { m >>= 1; ++maxl; }
  if (levels > maxl) {
    set_error(VCT_ERR_INVALID_VALUE, "%d levels exceed the %d a %dx%dx%d texture has", levels, maxl, width, height,
              depth);
    return 0;
  }
  if (ensure_device() != VCT_OK || tex_stream() != VCT_OK) return 0;
  std::unique_ptr<Tex3D> t(new Tex3D());
  t->w = width; t->h = height; t->d = depth; t->levels = levels;
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
  cudaError_t e = cudaMallocMipmappedArray(&t->arr, &desc, make_cudaExtent(width, height, depth), levels,
                                           cudaArraySurfaceLoadStore);
  if (e != cudaSuccess) { cuda_status(e, "cudaMallocMipmappedArray"); return 0; }
  for (int l = 0; l < levels; ++l) {
    cudaArray_t a;
    cudaSurfaceObject_t s = 0;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    if ((e = cudaGetMipmappedArrayLevel(&a, t->arr, l)) != cudaSuccess) { cuda_status(e, "level"); return 0; }
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = a;
    if ((e = cudaCreateSurfaceObject(&s, &rd)) != cudaSuccess) { cuda_status(e, "surface"); return 0; }
    t->surf.push_back(s);
    // GL texture storage starts undefined; the engine starts at 0.
    if ((e = launch_fill_rgba8(s, t->lw(l), t->lh(l), t->ld(l), make_uchar4(0, 0, 0, 0), g_stream)) != cudaSuccess) {
      cuda_status(e, "fill");
      return 0;
    }
  }
  if ((e = cudaStreamSynchronize(g_stream)) != cudaSuccess) { cuda_status(e, "sync"); return 0; }
  const uint32_t id = g_next++;
  g_tex[id] = std::move(t);
  return id;
}

extern "C" void vct_destroy_tex_3d(vct_tex3d tex) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_tex.erase(tex);  // unknown names are ignored, as glDeleteTextures does
}

extern "C" vct_status vct_activate_tex_3d(uint32_t, vct_tex3d tex, uint32_t) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  if (!find(tex)) return set_error(VCT_ERR_INVALID_ID, "texture %u", tex);
  return VCT_OK;
}

static unsigned char to_unorm8(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 1.0f) return 255;
  return (unsigned char)std::floor(v * 255.0f + 0.5f);
}

extern "C" vct_status vct_clear_tex_3d(vct_tex3d tex, const float c[4]) {
  clear_error();
  if (!c) return set_error(VCT_ERR_INVALID_VALUE, "NULL colour");
  std::lock_guard<std::mutex> lk(g_mu);
  Tex3D* t = find(tex);
  if (!t) return set_error(VCT_ERR_INVALID_ID, "texture %u", tex);
  VCT_CUDA(launch_fill_rgba8(t->surf[0], t->w, t->h, t->d,
                             make_uchar4(to_unorm8(c[0]), to_unorm8(c[1]), to_unorm8(c[2]), to_unorm8(c[3])), g_stream));
  VCT_CUDA(cudaStreamSynchronize(g_stream));
  return VCT_OK;
}

extern "C" vct_status vct_mip_tex_3d(vct_tex3d tex) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  Tex3D* t = find(tex);
  if (!t) return set_error(VCT_ERR_INVALID_ID, "texture %u", tex);
  for (int l = 1; l < t->levels; ++l)
    VCT_CUDA(launch_box_mip_rgba8(t->surf[l - 1], t->lw(l - 1), t->lh(l - 1), t->ld(l - 1), t->surf[l], t->lw(l),
                                  t->lh(l), t->ld(l), g_stream));
  VCT_CUDA(cudaStreamSynchronize(g_stream));
  return VCT_OK;
}

extern "C" vct_status vct_tex3d_upload(vct_tex3d tex, int32_t level, const void* rgba8) {
  clear_error();
  if (!rgba8) return set_error(VCT_ERR_INVALID_VALUE, "NULL data");
  std::lock_guard<std::mutex> lk(g_mu);
  Tex3D* t = find(tex);
  if (!t) return set_error(VCT_ERR_INVALID_ID, "texture %u", tex);
  if (level < 0 || level >= t->levels) return set_error(VCT_ERR_INVALID_VALUE, "level %d", level);
  return copy_level(t, level, const_cast<void*>(rgba8), true);
}

extern "C" vct_status vct_tex3d_download(vct_tex3d tex, int32_t level, void* rgba8) {
  clear_error();
  if (!rgba8) return set_error(VCT_ERR_INVALID_VALUE, "NULL data");
  std::lock_guard<std::mutex> lk(g_mu);
  Tex3D* t = find(tex);
  if (!t) return set_error(VCT_ERR_INVALID_ID, "texture %u", tex);
  if (level < 0 || level >= t->levels) return set_error(VCT_ERR_INVALID_VALUE, "level %d", level);
  return copy_level(t, level, rgba8, false);
}
