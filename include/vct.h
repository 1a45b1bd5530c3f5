/*
 * vct.h -- C ABI of the GB300 voxel cone tracing engine.
 *
 * Drop-in boundary for the voxelize -> mipmap -> cone-trace path of
 * latencyhiding/voxel_cone_tracing: every entry point below replaces one
 * method of `struct Renderer` (src/renderer.h:122-196) or one Texture3D
 * helper (src/texture_3d.h:6-10).  Plain C types only; matrices are
 * column-major float[16] exactly as glm::mat4 stores them; GL object names
 * become opaque handles.  include/vct_renderer.hpp wraps this ABI in a C++
 * `Renderer` with the reference's method names and signatures.
 *
 * All GPU work of a renderer runs on one CUDA stream (its own, or one set
 * with vct_set_stream).  vct_render() only enqueues work; the read-back
 * calls and vct_synchronize() wait for it.  A renderer is not thread-safe,
 * like the reference (single GL context thread).
 */
#ifndef VCT_H
#define VCT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ types ---- */

/* model_id_t / shader_id_t / material_id_t are size_t (renderer.h:23-25). */
typedef uint64_t vct_model_id;
typedef uint64_t vct_shader_id;
typedef uint64_t vct_material_id;
/* INVALID_ID (~0), renderer.h:22. */
#define VCT_INVALID_ID (~(uint64_t)0)

/* point_light_t, renderer.h:87-92 (28 bytes). */
typedef struct {
  float position[3];
  float color[3];
  float intensity;
} vct_point_light;

/* material_data_t, renderer.h:94-120 (packed, 128 bytes). */
typedef struct {
  float ambient[4];
  float diffuse[4];
  float specular[4];
  float transmittance[4];
  float emission[3];
  float shininess;
  float ior;
  float dissolve;
  int32_t illum;
  float roughness;
  float metallic;
  float sheen;
  float clearcoat_thickness;
  float clearcoat_roughness;
  float anisotropy;
  float anisotropy_rotation;
  float pad[2];
} vct_material_data;

/* vert_data_t, renderer.cpp:23-35 (packed, 32 bytes). */
typedef struct {
  float pos[3];
  float norm[3];
  float tex[2];
} vct_vert_data;

/* One draw object of a model: a run of indices drawn with one material
 * (draw_obj_t, renderer.h:57-64; built in renderer.cpp:519-556). */
typedef struct {
  uint32_t first_index;
  uint32_t index_count;
  uint32_t material_id;
} vct_draw_obj;

typedef enum {
  VCT_OK = 0,
  VCT_ERR_INVALID_VALUE = 1,   /* bad argument (size, resolution, pointer) */
  VCT_ERR_INVALID_ID = 2,      /* unknown model / material / texture id    */
  VCT_ERR_CUDA = 3,            /* CUDA runtime error (see vct_last_error)   */
  VCT_ERR_OUT_OF_MEMORY = 4,
  VCT_ERR_IO = 5,              /* file could not be read / parsed          */
  VCT_ERR_UNSUPPORTED = 6,
  VCT_ERR_NO_DEVICE = 7
} vct_status;

enum { VCT_VOX_REF_RASTER2X = 0, VCT_VOX_CONSERVATIVE = 1 };
/* VCT_MIP_BOTH: the six directional chains (traced, as VCT_MIP_ANISO) and an
 * isotropic chain (map 6: the box mean of VCT_MIP_ISO), built in one pass
 * from the same staged children; view_voxel_dir 6 shows the isotropic chain. */
enum { VCT_MIP_ANISO = 0, VCT_MIP_ISO = 1, VCT_MIP_BOTH = 2 };
enum { VCT_STORAGE_RGBA8 = 0, VCT_STORAGE_RGBA16F = 1 };
enum { VCT_SAMPLER_HW = 0, VCT_SAMPLER_EXACT = 1 };
enum { VCT_CONES_REF9 = 0, VCT_CONES_SIX60 = 1 };
enum { VCT_FRAME_RGBA8 = 0, VCT_FRAME_RGBA32F = 1 };

/* Engine settings the reference hard-codes (7 mip levels, renderer.cpp:186;
 * 6-direction mips, mipmap.comp; 9 diffuse cones, voxel_cone_tracing.frag
 * :140-168) plus the engine's own choices. */
typedef struct {
  int32_t grid_res;     /* initial set_grid_resolution (reference: 128)    */
  int32_t vox_mode;     /* VCT_VOX_*: coverage rule of the voxelizer        */
  int32_t mip_mode;     /* VCT_MIP_*                                        */
  int32_t storage;      /* VCT_STORAGE_*: texel format of the voxel maps    */
  int32_t sampler;      /* VCT_SAMPLER_*: texture-unit or FP32 filtering    */
  int32_t cone_set;     /* VCT_CONES_*                                      */
  int32_t keep_counts;  /* keep per-voxel contribution counts (debug)       */
  int32_t keep_float_frame; /* also write the unclamped RGBA32F frame       */
  float radiance_max;   /* upper clamp of voxel radiance (voxelize.frag:153
                         * clamps to 1).  0 or 1: the reference's clamp;
                         * > 1 (HDR, e.g. 16) needs VCT_STORAGE_RGBA16F      */
  int32_t shadow_from_maps; /* 0 (default): shadow cones of the texture-unit
                         * sampler read packed alpha-only copies of the six
                         * maps' chains (two fetches per step instead of
                         * three, identical values); 1: the six maps       */
  int32_t full_march;   /* 1: cones march their full length also outside the
                         * grid, as the reference's loop does; 0 (default):
                         * a cone stops once every further sample can only
                         * read border texels (identical results)          */
  int32_t overlap_raster; /* 1: the G-buffer raster (and the learned
                         * diffuse term) run on a second stream beside
                         * voxelize and mipmap, which they do not depend on:
                         * a shorter frame, longer voxelize and mipmap
                         * stages; 0 (default): one stream, one stage
                         * after the other                                */
  int32_t far_share;    /* texture-unit sampler: 1 (default): the pixels of
                         * a 4x2 group with matching normals and positions
                         * share their diffuse cones after the first sample
                         * (the far field, marched once per group by the
                         * lanes of the warp together); 0: every pixel
                         * marches all of its cones (the reference's rule).
                         * The FP32 software sampler always marches per
                         * pixel                                           */
  int32_t trace_tile_rows; /* shared-far-field tracer: rows of a CTA's
                         * 16-pixel-wide tile, 8, 16 or 32; 0 (default): 16.
                         * The frame is the same for every value          */
  int32_t reserved[2];
} vct_config;

typedef struct vct_renderer vct_renderer;

/* Per-stage device times of the last rendered frame, milliseconds. */
typedef struct {
  float voxelize;   /* clear + bin + voxelize level 0                     */
  float mipmap;     /* levels 1..L-1                                       */
  float gbuffer;    /* forward raster + attribute resolve (with
                     * overlap_raster it runs beside voxelize and mipmap,
                     * and the stages can add up to more than total)      */
  float trace;      /* cone-trace shading (+ the learned diffuse term's
                     * inference when it replaces the diffuse cones)      */
  float total;      /* first to last event of the frame                    */
  uint32_t kernel_launches; /* engine kernels launched for the frame       */
  uint32_t voxelized;       /* 1: the frame voxelized its geometry; 0: light
                             * injection reused the attribute grids        */
  uint32_t split_bricks;    /* dense bricks (> 1024 triangle pairs) whose
                             * pairs were spread over several CTAs         */
  float infer;              /* the learned diffuse term's inference (part of
                             * trace; 0 without it)                        */
} vct_stage_times;

/* --------------------------------------------------- error reporting --- */

/* Message of the last failing call on this thread ("" if none). */
const char* vct_last_error(void);
const char* vct_status_string(vct_status s);

/* ------------------------------------------------ Renderer lifetime ---- */

void vct_config_default(vct_config* cfg);

/* Renderer::Renderer(int width, int height), renderer.cpp:100-147.
 * cfg may be NULL (defaults). */
vct_status vct_renderer_create(int32_t width, int32_t height, const vct_config* cfg,
                               vct_renderer** out);
/* Renderer::~Renderer, renderer.cpp:149-165. */
void vct_renderer_destroy(vct_renderer* r);

/* ----------------------------------------------------- resources ------- */

/* Renderer::load_model, renderer.cpp:407-603, with the OBJ already parsed:
 * vertices, u32 indices and draw-object runs are copied to the device.
 * Writes the new model id to *out (VCT_INVALID_ID on failure). */
vct_status vct_load_mesh(vct_renderer* r, const vct_vert_data* verts, uint32_t n_verts,
                         const uint32_t* indices, uint32_t n_indices,
                         const vct_draw_obj* objs, uint32_t n_objs, vct_model_id* out);
/* Renderer::load_model(const char*), renderer.cpp:407-603: parses a
 * Wavefront OBJ (+ MTL) file.  Returns VCT_INVALID_ID on failure. */
vct_model_id vct_load_model(vct_renderer* r, const char* filename);
/* Renderer::load_shader, renderer.cpp:605-641.  GLSL programs do not exist
 * here; kept for source compatibility, returns a new id and does nothing. */
vct_shader_id vct_load_shader(vct_renderer* r, const char* vertex_shader_name,
                              const char* fragment_shader_name,
                              const char* geometry_shader_name);
/* Renderer::add_material, renderer.cpp:653-665. */
vct_material_id vct_add_material(vct_renderer* r, const vct_material_data* material_data);
/* Renderer::upload_material_data, renderer.cpp:643-651. */
vct_status vct_upload_material_data(vct_renderer* r, const vct_material_data* material_data,
                                    vct_material_id material_id);
/* Renderer::set_model_material, renderer.cpp:667-677. */
vct_status vct_set_model_material(vct_renderer* r, vct_material_id material_id,
                                  vct_model_id model_id);
/* Renderer::get_model_dimensions, renderer.cpp:173-176. */
vct_status vct_get_model_dimensions(vct_renderer* r, vct_model_id model, float out[3]);
/* Renderer::get_material, renderer.cpp:230-233: copies the material data. */
vct_status vct_get_material(vct_renderer* r, vct_material_id material_id,
                            vct_material_data* out);

/* ------------------------------------------------------- settings ------ */

/* Renderer::set_grid_resolution, renderer.cpp:178-188 (power of two,
 * 8..1024; levels = min(7, log2(res)+1)). */
vct_status vct_set_grid_resolution(vct_renderer* r, uint32_t res);
/* Renderer::set_grid_size, renderer.cpp:190-193 (cube_size). */
vct_status vct_set_grid_size(vct_renderer* r, float size);
/* Renderer::set_camera_transform, renderer.cpp:167-171. */
vct_status vct_set_camera_transform(vct_renderer* r, const float lookat[16],
                                    const float projection[16]);
/* Renderer::set_model_transform, renderer.cpp:225-228. */
vct_status vct_set_model_transform(vct_renderer* r, vct_model_id model_id,
                                   const float model_matrix[16]);
/* Renderer::set_rendering_phases, renderer.cpp:195-201. */
vct_status vct_set_rendering_phases(vct_renderer* r, int32_t direct, int32_t diffuse,
                                    int32_t specular, int32_t shadow);
/* Renderer::set_voxel_view_dir, renderer.cpp:203-207 (dir < 7 shows map
 * `dir` at `lod`; the constructor default is 0, like the reference). */
vct_status vct_set_voxel_view_dir(vct_renderer* r, int32_t dir, float lod);

/* --------------------------------------------------------- frame ------- */

/* Renderer::queue_model, renderer.cpp:209-218 (captures the model matrix;
 * unknown ids are ignored, as in the reference). */
vct_status vct_queue_model(vct_renderer* r, vct_model_id model_id);
/* Renderer::queue_point_light, renderer.cpp:220-223. */
vct_status vct_queue_point_light(vct_renderer* r, const vct_point_light* light);
/* Renderer::render, renderer.cpp:392-405: voxelize, mipmap, G-buffer,
 * cone-trace; clears the queues.  Enqueued on the renderer's stream. */
vct_status vct_render(vct_renderer* r);

/* --------------------------------------- streams, timing, read-back ---- */

/* Use `stream` (a cudaStream_t) for all further work; NULL restores the
 * renderer's own stream. */
vct_status vct_set_stream(vct_renderer* r, void* stream);
vct_status vct_synchronize(vct_renderer* r);
vct_status vct_get_stage_times(vct_renderer* r, vct_stage_times* out);
/* The presented frame, W*H texels, row 0 = bottom (glReadPixels order).
 * VCT_FRAME_RGBA8: 4 bytes per pixel; VCT_FRAME_RGBA32F: 16 bytes (needs
 * keep_float_frame).  dst is host memory. */
vct_status vct_read_frame(vct_renderer* r, void* dst, int32_t format);
/* Device pointer of the RGBA8 frame (valid until the next resize). */
vct_status vct_frame_device_ptr(vct_renderer* r, void** out);
/* Voxel map texels of `level` (0 = the shared level 0) of map 0..5
 * (-x,+x,-y,+y,-z,+z; iso mode: map 0).  (N>>level)^3 texels, x fastest,
 * 4 bytes (RGBA8) or 8 bytes (RGBA16F) each. */
vct_status vct_read_voxels(vct_renderer* r, int32_t level, int32_t map, void* dst);
/* Per-voxel contribution counts of the last frame (N^3 u32; keep_counts). */
vct_status vct_read_voxel_counts(vct_renderer* r, uint32_t* dst);
/* G-buffer of the last frame: visible triangle id (0xffffffff = none; ids
 * count queued triangles in queue order), world position, interpolated
 * world normal, material id.  Any pointer may be NULL. */
vct_status vct_read_gbuffer(vct_renderer* r, uint32_t* tri_id, float* pos, float* nrm,
                            uint32_t* mat);
/* Grid resolution and mip level count currently in use. */
vct_status vct_get_grid(vct_renderer* r, int32_t* res, int32_t* levels);

/* ------------------------------------------- learned diffuse term ----- */

/* No reference counterpart: an engine extension.  A small network (hash
 * encoding of the surface position + normal + albedo -> 4 x 64 ReLU MLP ->
 * RGB, BF16 tensor cores, FP32 accumulation) trained on the GPU to predict
 * trace_diffuse (voxel_cone_tracing.frag:140-168), the average of the nine
 * diffuse cones; with VCT_DIFFUSE_MLP a frame evaluates it instead of
 * tracing those cones.  The cone tracer stays the default and the reference
 * the network's per-pixel error is measured against. */
enum { VCT_DIFFUSE_CONES = 0, VCT_DIFFUSE_MLP = 1 };

typedef struct {
  int32_t levels;       /* hash-grid levels (16)                          */
  int32_t log2_table;   /* entries per level, log2 (19)                   */
  int32_t n_min, n_max; /* coarsest / finest level resolution (16, 512)   */
  uint32_t n_samples;   /* training samples drawn from the scene (2^24)   */
  uint32_t batch;       /* samples per optimiser step (2^18)              */
  uint32_t steps;       /* Adam steps (1000)                              */
  float lr;             /* Adam learning rate (1e-2); constant over the first
                         * half of the steps, then decaying geometrically to
                         * lr / 10 at the last step                       */
  uint64_t seed;
  uint32_t reserved[8];
} vct_mlp_desc;

typedef struct {
  float loss_first;     /* MSE of the first step                          */
  float loss_last;      /* mean MSE over the last tenth of the steps      */
  float ms_samples;     /* surface sampling + cone-traced targets (device)*/
  float ms_train;       /* optimiser steps (device)                       */
  uint32_t steps, n_samples;
} vct_mlp_report;

void vct_mlp_desc_default(vct_mlp_desc* d);
/* Allocate and initialise the network (seeded) without training. */
vct_status vct_mlp_init(vct_renderer* r, const vct_mlp_desc* d);
/* Train on the scene and voxel maps of the last rendered frame: draw
 * n_samples surface points (uniform by area), cone-trace their diffuse
 * targets, run `steps` Adam steps.  Synchronous. */
vct_status vct_mlp_train(vct_renderer* r, const vct_mlp_desc* d, vct_mlp_report* report);
/* VCT_DIFFUSE_CONES (default) or VCT_DIFFUSE_MLP (needs a trained network). */
vct_status vct_set_diffuse_mode(vct_renderer* r, int32_t mode);
/* Checkpoint: versioned binary file with the configuration, the FP32 hash
 * table and weights and the Adam state. */
vct_status vct_mlp_save(vct_renderer* r, const char* path);
vct_status vct_mlp_load(vct_renderer* r, const char* path);
/* Host copies of the FP32 parameters: table levels*2^log2_table*2 floats,
 * weights 5*64*64 floats (W1..W4 [out][in], W5 rows 0..15 then zeros). */
vct_status vct_mlp_get_params(vct_renderer* r, float* table, float* weights);
vct_status vct_mlp_set_params(vct_renderer* r, const float* table, const float* weights);
/* Rows of 12 floats (texture-space position, normal, albedo, target RGB). */
vct_status vct_mlp_eval(vct_renderer* r, const float* samples, uint32_t n, float* rgb_out);
/* One forward + backward pass over the rows (no parameter update): MSE
 * loss and its gradients (same layouts as vct_mlp_get_params). */
vct_status vct_mlp_gradients(vct_renderer* r, const float* samples, uint32_t n, float* loss,
                             float* dweights, float* dtable);
/* Train on explicit rows instead of scene samples. */
/* Kernels of the network's forward pass (inference and vct_mlp_eval):
 * 1 = tcgen05.mma with TMEM accumulators, warp-specialised (encoder warps
 * fill 128-row tiles, epilogue warps drain the accumulators; the default),
 * 0 = mma.sync warp tiles (16 rows per warp).  Both give the same values.
 * Training always uses the warp tiles. */
vct_status vct_mlp_set_tensor_kernels(vct_renderer* r, int32_t use_tcgen05);
vct_status vct_mlp_train_samples(vct_renderer* r, const float* samples, uint32_t n,
                                 const vct_mlp_desc* d, vct_mlp_report* report);

/* The judge of the learned term: a frame that evaluates the network also
 * traces the nine diffuse cones (texture-unit sampler) at one pixel of every
 * stride x stride tile (the pixel within the tile changes from frame to
 * frame) and compares them with the network's prediction (PSNR over the
 * three channels, peak 1).  Below min_psnr_db the frame is rendered again
 * with the cones before render() returns, and later frames keep the cones
 * (vct_set_diffuse_mode(VCT_DIFFUSE_MLP) after training again re-enables
 * the network).  stride 0 turns the judge off; default 16 and 40 dB. */
vct_status vct_mlp_set_judge(vct_renderer* r, int32_t stride, float min_psnr_db);
typedef struct {
  float last_psnr_db;     /* judge's PSNR of the last judged frame (-1: none) */
  uint32_t judged_pixels; /* pixels it compared                              */
  uint32_t fallbacks;     /* frames it sent back to the cones                */
  int32_t diffuse_mode;   /* VCT_DIFFUSE_* now in effect                     */
  int32_t stride;
  float min_psnr_db;
  uint32_t reserved[4];
} vct_mlp_judge_report;
vct_status vct_mlp_get_judge(vct_renderer* r, vct_mlp_judge_report* out);

/* ------------------------------------------ allocation-free voxelizer --- */

/* No counterpart in the reference: an engine addition for callers that
 * cannot allocate device memory -- applications that own every device
 * allocation through their own heaps and forbid cudaMalloc / cudaFree inside
 * their frame loop (those calls can synchronise the device and stall the
 * frame, or are simply not theirs to make).  Everything below is caller
 * memory; the voxelizer's intermediates live in a fixed device array inside
 * the library (about 9 MB per GPU, held while the library is loaded).
 *
 * A mesh already on the device: vertices (vert_data_t layout), u32
 * indices, a material id per triangle (< n_materials), its model matrix. */
typedef struct {
  const vct_vert_data* verts;     /* device */
  const uint32_t* indices;        /* device, 3 per triangle */
  const uint32_t* tri_material;   /* device, one id per triangle */
  uint32_t n_verts;
  uint32_t n_tris;
  float model[16];                /* column-major, host */
} vct_device_mesh;

/* Voxelize meshes (host array of descriptors) into level0_rgba8 (device,
 * grid_res^3 x 4 bytes, x fastest, fully overwritten) with the same kernels
 * and coverage rules as vct_render's level 0.  materials: device array;
 * lights: host array.  Limits: grid_res a power of two in [8, 256], <= 64
 * meshes, <= 4096 materials, <= 10 lights, <= 2^21 (triangle, 8^3-voxel
 * brick) pairs; beyond them the call fails with VCT_ERR_INVALID_VALUE.  Two
 * failures are known only after the GPU work, which then leaves the output
 * incomplete: more pairs than the limit, and vertex indices >= n_verts or
 * material ids >= n_materials (the kernels clamp such ids, so they read
 * nothing outside the caller's buffers).  Every call looks up the library's
 * device array on the current device (the first lookup on a device loads
 * the library's device code: make that call before any stream capture);
 * calls share that array, so calls whose GPU work overlaps (other streams /
 * threads) race -- serialise them.  Synchronises `stream` (a cudaStream_t,
 * NULL = default stream) before returning. */
vct_status vct_voxelize_noalloc(const vct_device_mesh* meshes, uint32_t n_meshes,
                                const vct_material_data* materials, uint32_t n_materials,
                                const vct_point_light* lights, uint32_t n_lights,
                                float cube_size, int32_t grid_res, int32_t vox_mode,
                                void* level0_rgba8, void* stream);

/* ------------------------------------------- Deferred light injection --- */
/* No reference counterpart: the reference shades every fragment while it
 * voxelizes, so any light change re-voxelizes the scene (renderer.cpp
 * :316-353 runs every frame).  With injection on, the voxelizer stores per
 * voxel the mean albedo x transmittance and alpha, the mean normal and the
 * mean emission x transmittance (three RGBA8 grids), and every frame lights
 * the voxels at their centres from those grids (the per-light terms of
 * voxelize.frag:128-143).  Frames whose queued models, matrices, cube size,
 * grid and materials equal the previous frame's skip voxelization: a light
 * change costs one injection pass.  The lighting is evaluated from voxel
 * means at the voxel centre instead of per fragment, an approximation of
 * the reference's shading.  RGBA8 storage only. */
vct_status vct_set_light_injection(vct_renderer* r, int32_t enable);
/* The three attribute grids (N^3 RGBA8 each, x fastest): albedo, normal
 * (0.5 n + 0.5), emission (a = 255 where occupied). */
vct_status vct_read_injection_grids(vct_renderer* r, void* albedo, void* normal, void* emission);

/* ------------------------------------------------------- Texture3D ----- */

typedef uint32_t vct_tex3d;   /* 0 = no texture, like a GL name */

/* create_tex_3d, texture_3d.cpp:3-25: RGBA8, `levels` mip levels,
 * clamp-to-border, trilinear mip filtering. 0 on failure. */
vct_tex3d vct_create_tex_3d(int32_t width, int32_t height, int32_t depth, int32_t levels);
/* destroy_tex_3d, texture_3d.cpp:27-30. */
void vct_destroy_tex_3d(vct_tex3d tex);
/* activate_tex_3d, texture_3d.cpp:32-37: texture-unit binding has no
 * counterpart (kernels take texture objects); validates the handle. */
vct_status vct_activate_tex_3d(uint32_t program, vct_tex3d tex, uint32_t unit);
/* clear_tex_3d, texture_3d.cpp:39-44: fills level 0 with clear_color. */
vct_status vct_clear_tex_3d(vct_tex3d tex, const float clear_color[4]);
/* mip_tex_3d, texture_3d.cpp:46-51 (glGenerateMipmap): levels 1.. as the
 * 2x2x2 box mean of the level below. */
vct_status vct_mip_tex_3d(vct_tex3d tex);
/* Host <-> level copies (glTexSubImage3D / glGetTexImage counterparts). */
vct_status vct_tex3d_upload(vct_tex3d tex, int32_t level, const void* rgba8);
vct_status vct_tex3d_download(vct_tex3d tex, int32_t level, void* rgba8);

/* ------------------------------------------------- Batched rendering --- */
/* No reference counterpart: the reference renders one scene per frame
 * (Renderer::render, renderer.cpp:392-405).  A batch renders many
 * independent scenes of different grid, mesh and frame sizes per frame with
 * the same maths as a Renderer (each scene's frame and voxel maps equal a
 * Renderer's on the same scene, bit for bit), but each stage pass is one
 * persistent kernel launch over all scenes, and the frame can be captured
 * once in a CUDA graph and replayed.  Geometry, materials and lights are
 * fixed at creation; cameras can change every frame.  RGBA8 anisotropic
 * maps, texture-unit sampler. */

typedef struct {
  const vct_vert_data* verts;
  uint32_t n_verts;
  const uint32_t* indices;       /* 3 * n_tris */
  uint32_t n_tris;
  const uint32_t* tri_material;  /* per triangle, index into the scene's materials */
  float model[16];               /* column-major model matrix */
} vct_batch_mesh;

typedef struct {
  int32_t width, height;
  int32_t grid_res;              /* power of two, 16..256 */
  int32_t cone_set;              /* VCT_CONES_REF9 (9 cones) or VCT_CONES_SIX60 (6) */
  float cube_size;
  const vct_batch_mesh* meshes;
  uint32_t n_meshes;
  const vct_material_data* materials;  /* >= 1 */
  uint32_t n_materials;
  const vct_point_light* lights;       /* <= 10 */
  uint32_t n_lights;
  float view[16], proj[16];
} vct_batch_scene;

typedef struct {
  int32_t vox_mode;   /* VCT_VOX_* for every scene */
  int32_t use_graph;  /* capture the frame once in a CUDA graph, then replay it */
  int32_t far_share;  /* 1: shared far fields of the diffuse cones, as
                       * vct_config.far_share (vct_batch_config_default sets
                       * it); 0: every pixel marches all its cones          */
  int32_t reserved[5];
} vct_batch_config;

/* vox_mode VCT_VOX_REF_RASTER2X, no graph, far_share 1 (a Renderer's default). */
void vct_batch_config_default(vct_batch_config* cfg);

/* Launch shapes of the batched kernels: persistent CTAs per SM of the
 * binning, brick and trace launches (trace 1-3, or 0: one launch with one
 * CTA per 16 x 16 tile of every scene, not persistent), the persistent
 * trace's tile scheduling (1 = atomic tile queue, 0 = static stride), the
 * trace's form: 0 = one launch over all scenes, 1 = one launch of the
 * one-scene trace kernel per scene, spread over parallel streams (graph
 * branches), and the tile of the per-scene shared-far-field trace.  Every
 * shape renders the same frames. */
typedef struct {
  int32_t bin_ctas_per_sm;
  int32_t bricks_ctas_per_sm;
  int32_t trace_ctas_per_sm;
  int32_t trace_dynamic;
  int32_t trace_per_scene;
  int32_t trace_tile_rows;  /* per-scene shared-far-field trace: CTA tile 16 x 8,
                             * 16 x 16 or 16 x 32 pixels (the same frame) */
} vct_batch_shape;

typedef struct vct_batch vct_batch;

vct_status vct_batch_create(const vct_batch_scene* scenes, uint32_t n_scenes, const vct_batch_config* cfg,
                            vct_batch** out);
void vct_batch_destroy(vct_batch* b);
vct_status vct_batch_set_camera(vct_batch* b, uint32_t scene, const float view[16], const float proj[16]);
/* One frame of every scene, enqueued on the batch's stream. */
vct_status vct_batch_render(vct_batch* b);
vct_status vct_batch_synchronize(vct_batch* b);
vct_status vct_batch_set_stream(vct_batch* b, void* stream);
/* RGBA8 frame of one scene, row 0 = bottom. */
vct_status vct_batch_read_frame(vct_batch* b, uint32_t scene, void* rgba8);
/* One level of one voxel map of one scene (level 0: map ignored). */
vct_status vct_batch_read_voxels(vct_batch* b, uint32_t scene, int32_t level, int32_t map, void* rgba8);
/* Stage times of the last frame, all scenes together. */
vct_status vct_batch_stage_times(vct_batch* b, vct_stage_times* out);
vct_status vct_batch_get_shape(vct_batch* b, vct_batch_shape* out);
vct_status vct_batch_set_shape(vct_batch* b, const vct_batch_shape* shape);
/* The autotuner: times `frames` frames of each candidate launch shape on
 * this batch (coordinate search over the fields of vct_batch_shape), keeps
 * the fastest, and reports it with the frame times before and after. */
vct_status vct_batch_autotune(vct_batch* b, int32_t frames, vct_batch_shape* best, float* ms_before,
                              float* ms_after);

/* ------------------------------------------------------- measurement --- */

/* No counterpart in the reference: a measurement helper.  The cone tracer is
 * bound by the texture unit, so its roofline is the rate at which the
 * current device filters 3D RGBA8 fetches with every lane fetching and the
 * texels L1-resident.  kind 0: tex3DLod of a mipmapped texture at a
 * fractional lod (two levels, 16 texels); 1: tex3D of a non-mipmapped
 * texture (8 texels); 2: tex3DLod at an integer lod (one level).  Runs
 * iters (4..8192) fetches per thread on every SM, timed with CUDA events
 * (best of 3 launches after a warm-up); returns fetches per second and the
 * launch time in ms.  Allocates and frees its own 32^3 texture. */
vct_status vct_measure_texture_rate(int32_t kind, uint32_t iters, double* fetches_per_s, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* VCT_H */
