// api_noalloc.cu -- vct_voxelize_noalloc: the voxelizer for callers that
// cannot allocate device memory.
//
// Some callers of this library own every byte of device memory themselves:
// a host application (a game engine, a plugin host, a render farm worker)
// that hands its components fixed heaps and forbids allocation inside its
// frame loop, because cudaMalloc / cudaFree can synchronise the whole device
// and stall the frame, or may simply be disallowed by the host's memory
// manager.  The renderer API allocates its work buffers as it goes; this entry
// point allocates nothing.  The caller passes its inputs (meshes, materials,
// lights) and its output buffer; every intermediate the voxelizer needs (the
// per-brick triangle counts, offsets and cursors, the triangle-brick pair
// list, the instance records and the status word) lives in one file-scope
// device array below, which exists once per GPU for as long as the library
// is loaded.
//
// Limits (calls beyond them fail with VCT_ERR_INVALID_VALUE): grid
// resolution <= 256, <= 64 meshes, <= 4096 materials, <= 2^21
// (triangle, 8^3-brick) pairs -- the last one is only known after binning,
// so such a call reports the error after the work ran (its output is then
// incomplete).
//
// The first call on a device looks up the device address of the array
// (cudaGetSymbolAddress, once per device, with that device current).  All
// calls share the array and it keeps the last call's contents; everything
// that must start at zero is cleared by each call.  Calls whose GPU work
// overlaps (other streams, other host threads) race on the array: issue them
// one after another.
#include <cstring>
#include <mutex>

#include "renderer_state.h"

namespace {

constexpr int kNaMaxGrid = 256;
constexpr int kNaMaxBricks = (kNaMaxGrid / kBrick) * (kNaMaxGrid / kBrick) * (kNaMaxGrid / kBrick);
constexpr uint32_t kNaMaxPairs = 1u << 21;
constexpr uint32_t kNaMaxMeshes = 64;
constexpr uint32_t kNaMaxMaterials = 4096;
constexpr int kNaScanTmp = kNaMaxBricks / 4096 + 8;
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
  uint32_t brick_count[kNaMaxBricks];
  uint32_t brick_offset[kNaMaxBricks + 1];
  uint32_t brick_cursor[kNaMaxBricks];
  uint32_t scan_tmp[kNaScanTmp];
  uint32_t pairs[kNaMaxPairs];
  uint32_t material_of_id[kNaMaxMaterials];  // identity: triangle material id -> material
  DevInstance inst[kNaMaxMeshes];
  FrameStatus status;
};

static __device__ __align__(256) unsigned char g_scratch[sizeof(NoAllocScratch)];

std::mutex g_mu;
NoAllocScratch* g_scratch_ptr[kNaMaxDevices] = {};
uint32_t g_identity[kNaMaxMaterials];

// Device address of the scratch array on the current device (set up once
// per device).
vct_status scratch_on_device(NoAllocScratch** out) {
  int dev = 0;
  VCT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) return set_error(VCT_ERR_UNSUPPORTED, "device %d", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(voxelizer scratch)");
    g_scratch_ptr[dev] = static_cast<NoAllocScratch*>(p);
    for (uint32_t i = 0; i < kNaMaxMaterials; ++i) g_identity[i] = i;
  }
  *out = g_scratch_ptr[dev];
  return VCT_OK;
}

}  // namespace

extern "C" vct_status vct_voxelize_noalloc(const vct_device_mesh* meshes, uint32_t n_meshes,
                                           const vct_material_data* materials, uint32_t n_materials,
                                           const vct_point_light* lights, uint32_t n_lights, float cube_size,
                                           int32_t grid_res, int32_t vox_mode, void* level0_rgba8, void* stream) {
  clear_error();
  if (!level0_rgba8 || !materials || (n_meshes && !meshes) || (n_lights && !lights))
    return set_error(VCT_ERR_INVALID_VALUE, "NULL pointer argument");
  if (!is_pow2((uint32_t)grid_res) || grid_res < 8 || grid_res > kNaMaxGrid)
    return set_error(VCT_ERR_INVALID_VALUE, "grid_res %d: this entry point takes a power of two in [8, %d]", grid_res,
                     kNaMaxGrid);
  if (n_meshes > kNaMaxMeshes)
    return set_error(VCT_ERR_INVALID_VALUE, "%u meshes: this entry point takes at most %u", n_meshes, kNaMaxMeshes);
  if (n_materials == 0 || n_materials > kNaMaxMaterials)
    return set_error(VCT_ERR_INVALID_VALUE, "%u materials: this entry point takes 1..%u", n_materials,
                     kNaMaxMaterials);
  if (vox_mode != VCT_VOX_REF_RASTER2X && vox_mode != VCT_VOX_CONSERVATIVE)
    return set_error(VCT_ERR_INVALID_VALUE, "vox_mode %d", vox_mode);
  if (!(cube_size > 0.0f) || !std::isfinite(cube_size))
    return set_error(VCT_ERR_INVALID_VALUE, "cube_size %g", (double)cube_size);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n_meshes; ++i) {
    if (meshes[i].n_tris && (!meshes[i].verts || !meshes[i].indices || !meshes[i].tri_material))
      return set_error(VCT_ERR_INVALID_VALUE, "mesh %u: NULL device pointer", i);
    total += meshes[i].n_tris;
  }
  if (total > kNaMaxPairs)
    return set_error(VCT_ERR_INVALID_VALUE, "%llu triangles: this entry point bins at most %u triangle-brick pairs",
                     (unsigned long long)total, kNaMaxPairs);
  NoAllocScratch* s = nullptr;
  VCT_CHECK(scratch_on_device(&s));
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  DevInstance inst[kNaMaxMeshes];
  std::memset(inst, 0, sizeof(inst));
  uint32_t base = 0;
  for (uint32_t i = 0; i < n_meshes; ++i) {
    std::memcpy(inst[i].M, meshes[i].model, sizeof(inst[i].M));
    normal_matrix(meshes[i].model, inst[i].NM);
    inst[i].tri_base = base;
    inst[i].n_tris = meshes[i].n_tris;
    inst[i].verts = meshes[i].verts;
    inst[i].indices = meshes[i].indices;
    inst[i].tri_obj = meshes[i].tri_material;
    inst[i].n_verts = meshes[i].n_verts;
    base += meshes[i].n_tris;
  }
  if (n_meshes)
    VCT_CUDA(cudaMemcpyAsync(s->inst, inst, n_meshes * sizeof(DevInstance), cudaMemcpyHostToDevice, st));
  VCT_CUDA(cudaMemcpyAsync(s->material_of_id, g_identity, n_materials * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  VCT_CUDA(cudaMemsetAsync(&s->status, 0, sizeof(FrameStatus), st));

  SceneParams sp;
  std::memset(&sp, 0, sizeof(sp));
  sp.inst = s->inst;
  sp.materials = materials;
  sp.obj_material = s->material_of_id;
  sp.n_instances = n_meshes;
  sp.total_tris = (uint32_t)total;
  sp.n_materials = n_materials;
  sp.n_lights = (int32_t)std::min<uint32_t>(n_lights, kMaxLights);
  sp.cube_size = cube_size;
  sp.radiance_max = 1.0f;
  for (int i = 0; i < sp.n_lights; ++i) sp.lights[i] = lights[i];

  VoxBuffers vb;
  std::memset(&vb, 0, sizeof(vb));
  vb.brick_count = s->brick_count;
  vb.brick_offset = s->brick_offset;
  vb.brick_cursor = s->brick_cursor;
  vb.pair_list = s->pairs;
  vb.pair_cap = kNaMaxPairs;
  vb.scan_tmp = s->scan_tmp;
  vb.counts = nullptr;
  vb.status = &s->status;
  VCT_CUDA(launch_voxelize_linear(sp, grid_res, vox_mode, vb, static_cast<uchar4*>(level0_rgba8), st));

  FrameStatus hs;
  VCT_CUDA(cudaMemcpyAsync(&hs, &s->status, sizeof(hs), cudaMemcpyDeviceToHost, st));
  VCT_CUDA(cudaStreamSynchronize(st));
  if (hs.pair_total > kNaMaxPairs)
    return set_error(VCT_ERR_INVALID_VALUE,
                     "the scene needs %u triangle-brick pairs; this entry point holds at most %u (output incomplete)",
                     hs.pair_total, kNaMaxPairs);
  return VCT_OK;
}
