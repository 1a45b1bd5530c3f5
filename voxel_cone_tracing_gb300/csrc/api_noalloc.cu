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
// Every call looks up the device address of the array on the current device
// (cudaGetSymbolAddress, with that device current); on a device's first call
// that lookup loads the library's device code, so make the first call on a
// device before any stream capture.  All calls share the array and it keeps
// the last call's contents; everything that must start at zero is cleared by
// each call.  Calls whose GPU work overlaps (other streams, other host
// threads) race on the array: issue them one after another.
//
// Vertex indices and material ids live in caller memory on the device, so
// they cannot be checked before the launch: the kernels clamp them (no read
// leaves the caller's buffers) and a small kernel counts the ones out of
// range, which makes the call fail with VCT_ERR_INVALID_VALUE after the work
// ran (its output is then not the meshes' voxelization).
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

std::once_flag g_identity_once;
uint32_t g_identity[kNaMaxMaterials];

// Device address of the scratch array on the current device.
vct_status scratch_on_device(NoAllocScratch** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(voxelizer scratch)");
  std::call_once(g_identity_once, [] {
    for (uint32_t i = 0; i < kNaMaxMaterials; ++i) g_identity[i] = i;
  });
  *out = static_cast<NoAllocScratch*>(p);
  return VCT_OK;
}

// Counts the vertex indices >= n_verts and material ids >= n_materials of
// one device mesh into *bad.
__global__ void k_count_bad_ids(const uint32_t* __restrict__ indices, const uint32_t* __restrict__ tri_material,
                                uint32_t n_tris, uint32_t n_verts, uint32_t n_materials, uint32_t* bad) {
  uint32_t nb = 0;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tris; t += gridDim.x * blockDim.x) {
    nb += __ldg(tri_material + t) >= n_materials;
    for (int k = 0; k < 3; ++k) nb += __ldg(indices + 3 * (size_t)t + k) >= n_verts;
  }
  for (int o = 16; o > 0; o >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, o);
  if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bad, nb);
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
  if (n_lights > (uint32_t)kMaxLights)
    return set_error(VCT_ERR_INVALID_VALUE, "%u lights: this entry point takes at most %d", n_lights, kMaxLights);
  if (!(cube_size > 0.0f) || !std::isfinite(cube_size))
    return set_error(VCT_ERR_INVALID_VALUE, "cube_size %g", (double)cube_size);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n_meshes; ++i) {
    if (meshes[i].n_tris && (!meshes[i].verts || !meshes[i].indices || !meshes[i].tri_material))
      return set_error(VCT_ERR_INVALID_VALUE, "mesh %u: NULL device pointer", i);
    if (meshes[i].n_tris && !meshes[i].n_verts)
      return set_error(VCT_ERR_INVALID_VALUE, "mesh %u: %u triangles and no vertices", i, meshes[i].n_tris);
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
  for (uint32_t i = 0; i < n_meshes; ++i) {
    if (!meshes[i].n_tris) continue;
    const unsigned blocks = std::min<unsigned>((meshes[i].n_tris + 255) / 256, 1024u);
    k_count_bad_ids<<<blocks, 256, 0, st>>>(meshes[i].indices, meshes[i].tri_material, meshes[i].n_tris,
                                            meshes[i].n_verts, n_materials, &s->status.bad_ids);
  }

  SceneParams sp;
  std::memset(&sp, 0, sizeof(sp));
  sp.inst = s->inst;
  sp.materials = materials;
  sp.obj_material = s->material_of_id;
  sp.n_obj = n_materials;
  sp.n_instances = n_meshes;
  sp.total_tris = (uint32_t)total;
  sp.n_materials = n_materials;
  sp.n_lights = (int32_t)n_lights;
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
  if (hs.bad_ids)
    return set_error(VCT_ERR_INVALID_VALUE,
                     "%u vertex indices / material ids out of range (indices < n_verts, ids < n_materials)",
                     hs.bad_ids);
  if (hs.pair_total > kNaMaxPairs)
    return set_error(VCT_ERR_INVALID_VALUE,
                     "the scene needs %u triangle-brick pairs; this entry point holds at most %u (output incomplete)",
                     hs.pair_total, kNaMaxPairs);
  return VCT_OK;
}
