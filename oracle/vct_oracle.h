/*
 * vct_oracle.h -- C interface of the CPU oracle for the voxelize -> mipmap ->
 * cone-trace path of latencyhiding/voxel_cone_tracing.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark do, and only as the checker / the timed CPU restatement.
 *
 * Parity unpinned: the reference ships no tests, golden images or known-answer
 * vectors, and it cannot be built or run on these machines (it is an OpenGL
 * 4.5 program whose GLSL runs in a GL driver).  The oracle is a restatement of
 * the reference's shader and host maths; the known-answer cases in tests/ are
 * hand-derived from that maths.
 *
 * Layouts (all arrays dense, x fastest):
 *   level 0          : N^3 RGBA8 texels, index (z*N + y)*N + x, R in byte 0
 *   directional chain: for map d in 0..5 (-x,+x,-y,+y,-z,+z) the levels
 *                      1..L-1 concatenated, level l holding (N>>l)^3 texels;
 *                      the isotropic chain is one such map
 *   frame            : H rows (row 0 = bottom, as glReadPixels) of W RGBA
 */
#ifndef VCT_ORACLE_H
#define VCT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* point_light_t, renderer.h:87-92 (glm::vec3 is 12 bytes, no padding). */
typedef struct {
  float position[3];
  float color[3];
  float intensity;
} orc_point_light;

/* material_data_t, renderer.h:94-120 (packed, 128 bytes, std140 layout of
 * the GLSL `material` block in voxelize.frag:10-31 and
 * voxel_cone_tracing.frag:3-24). */
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
  float roughness, metallic, sheen, clearcoat_thickness, clearcoat_roughness;
  float anisotropy, anisotropy_rotation;
  float pad[2];
} orc_material;

/* One queued model: vert_data_t vertices (renderer.cpp:23-35: pos3 norm3
 * uv2, 32 bytes), u32 triangle indices, a material id per triangle (the
 * draw-object runs of renderer.cpp:519-556 flattened) and the model matrix
 * captured at queue time (renderer.cpp:209-218), column-major. */
typedef struct {
  const float* verts;
  const uint32_t* indices;
  const uint32_t* tri_material;
  uint32_t n_verts;
  uint32_t n_tris;
  float model[16];
} orc_instance;

typedef struct {
  const orc_instance* instances;
  const orc_material* materials;
  const orc_point_light* lights;
  uint32_t n_instances;
  uint32_t n_materials;
  uint32_t n_lights;
  float cube_size;
  float view[16];
  float proj[16];
} orc_scene;

enum { ORC_VOX_REF_RASTER2X = 0, ORC_VOX_CONSERVATIVE = 1 };
enum { ORC_MIP_ANISO = 0, ORC_MIP_ISO = 1 };
enum { ORC_CONES_REF9 = 0, ORC_CONES_SIX60 = 1 };

typedef struct {
  int32_t grid_res;         /* N, power of two, 8..1024 */
  int32_t levels;           /* L = min(7, log2(N)+1) */
  int32_t vox_mode;         /* ORC_VOX_* */
  int32_t mip_mode;         /* ORC_MIP_* */
  int32_t width, height;
  int32_t enable_direct, enable_diffuse, enable_specular, enable_shadow;
  int32_t view_voxel_dir;   /* < 7 selects the voxel debug view */
  float view_voxel_lod;
  int32_t cone_set;         /* ORC_CONES_* */
  int32_t threads;          /* host threads, >= 1 */
  float radiance_max;       /* voxel colour clamp: rgb to [0, radiance_max]
                             * (<= 0 means 1, the reference's clamp) */
  int32_t far_share;        /* 0: every pixel marches all its cones (the
                             * reference); W > 0: the engine's shared far
                             * fields in groups of W x 2 pixels (see
                             * trace_diffuse) */
} orc_params;

/* Number of texels in one directional chain (levels 1..L-1). */
uint64_t orc_chain_texels(int32_t N, int32_t L);

/* Voxelize: level 0 (N^3 RGBA8) and the per-voxel contribution count.
 * Returns the number of triangles rejected as non-finite / out of range. */
int64_t orc_voxelize(const orc_scene* s, const orc_params* p,
                     uint8_t* level0, uint32_t* counts);

/* Informational: level 0 as the reference's running average
 * (imageAtomicRGBA8Avg, voxelize.frag:62-119) leaves it when the frame's
 * contributions (FP32 shading) arrive one at a time in a fixed order: 0 =
 * draw order, 1 = reverse, 2 = a permutation drawn from `seed`.  Bytes keep
 * the 4-bit count in their low bits, as the reference's maps do. */
int64_t orc_voxelize_cas(const orc_scene* s, const orc_params* p, int32_t order, uint64_t seed,
                         uint8_t* level0);
/* The same running average of n RGBA contributions (rgba: n x 4 floats in
 * [0, 1]) arriving in order at a cleared voxel; returns the stored word. */
uint32_t orc_cas_avg(const float* rgba, int32_t n);

/* Voxelize with FP32 shading (the timed CPU restatement).  counts may be 0. */
int64_t orc_voxelize_f32(const orc_scene* s, const orc_params* p,
                         uint8_t* level0, uint32_t* counts);

/* Voxelize, FP64, writing the unrounded mean as float RGBA (HDR storage:
 * the GPU rounds the same mean to half). */
int64_t orc_voxelize_hdr(const orc_scene* s, const orc_params* p,
                         float* level0, uint32_t* counts);

/* Light injection (no reference counterpart): the attribute grids (N^3
 * RGBA8 each: mean albedo x transmittance + alpha; mean normal as 0.5 n +
 * 0.5; mean emission x transmittance + occupancy 255), with the coverage and
 * averaging rule of orc_voxelize; then level 0 lit from them. */
int64_t orc_voxelize_attr(const orc_scene* s, const orc_params* p, uint8_t* albedo,
                          uint8_t* normal, uint8_t* emission, uint32_t* counts);
void orc_inject(const orc_scene* s, const orc_params* p, const uint8_t* albedo,
                const uint8_t* normal, const uint8_t* emission, uint8_t* level0);

/* One mip level in FP64 from float texels: src holds src_maps (1 = the shared
 * level 0, or 6) maps of edge `n_src`; dst receives 6 maps (aniso) or 1 map
 * (iso) of edge n_src/2. */
void orc_mip_level_f(int32_t n_src, int32_t src_maps, const float* src,
                     int32_t mip_mode, float* dst);

/* orc_trace over float voxel maps (level 0: N^3 RGBA floats; chains in the
 * layout above, RGBA floats). */
void orc_trace_hdr(const orc_scene* s, const orc_params* p, const float* level0,
                   const float* chains, const uint32_t* tri_id, const double* pos,
                   const double* nrm, const uint32_t* mat, int32_t row_stride,
                   float* out);

/* Mip chains from level 0: aniso -> 6 chains, iso -> 1 chain. */
void orc_mipmap(const orc_params* p, const uint8_t* level0, uint8_t* chains);

/* G-buffer raster: visible triangle id per pixel (0xffffffff = none), world
 * position, interpolated (unnormalised) world normal, material id. */
void orc_gbuffer(const orc_scene* s, const orc_params* p, uint32_t* tri_id,
                 double* pos, double* nrm, uint32_t* mat);

/* Cone-trace shading of a G-buffer.  rows: trace only rows y with
 * (y % row_stride) == 0 (others untouched); out is W*H*4 floats. */
void orc_trace(const orc_scene* s, const orc_params* p, const uint8_t* level0,
               const uint8_t* chains, const uint32_t* tri_id,
               const double* pos, const double* nrm, const uint32_t* mat,
               int32_t row_stride, float* out);
void orc_trace_f32(const orc_scene* s, const orc_params* p,
                   const uint8_t* level0, const uint8_t* chains,
                   const uint32_t* tri_id, const double* pos,
                   const double* nrm, const uint32_t* mat, int32_t row_stride,
                   float* out);

/* orc_trace with instrumentation: stats[0..3] cones, [4..7] march steps,
 * [8..11] steps with lod < 1, per class (diffuse, specular, shadow,
 * refraction); [12..19] steps of all classes with lod in [k, k+1), k = 0..6,
 * and lod >= 7; [20..23] per class the steps taken more than 3/4 of the
 * coarsest texel outside [0,1] along an axis the cone moves away on (border
 * texels only); [24..27] per class the other steps whose texels are all 0
 * by the engine's occupancy rule, [28..31] those of them with lod < 1;
 * [32..35] and [36..39] per class the one-level and two-level texture
 * fetches the engine's texture-unit path issues for the steps it takes
 * (with far_share, a shared far field is counted once, by the group's
 * representative).  stats holds 40 entries.  row_stride < -1 traces pairs
 * of rows (k |row_stride|, k |row_stride| + 1), i.e. whole 2x2 quads.  Not
 * thread-safe against concurrent orc_trace_stats. */
void orc_trace_stats(const orc_scene* s, const orc_params* p, const uint8_t* level0,
                     const uint8_t* chains, const uint32_t* tri_id, const double* pos,
                     const double* nrm, const uint32_t* mat, int32_t row_stride,
                     float* out, uint64_t* stats);

/* One GL texture sample, textureLod(map d, u, lod) with GL_LINEAR_MIPMAP_LINEAR
 * and CLAMP_TO_BORDER(0) (for the known-answer tests). */
void orc_texture_lod(const orc_params* p, const uint8_t* level0,
                     const uint8_t* chains, int32_t map, const double* u,
                     double lod, double* rgba);

/* One cone march, trace_cone() of voxel_cone_tracing.frag:88-119. */
void orc_trace_cone(const orc_params* p, const uint8_t* level0,
                    const uint8_t* chains, const double* origin,
                    const double* dir, double aperture, double max_dist,
                    double* rgba, int32_t* steps);

/* ---- learned diffuse term (vct_oracle_mlp.cpp) ----
 * Hash table: levels x 2^log2_table x 2 floats; weights: 5 x 64 x 64 floats
 * (W1..W4 [out][in] 64x64, W5 rows 0..15 of [out][in], rows >= 3 unused). */
typedef struct {
  int32_t levels;      /* 16 */
  int32_t log2_table;  /* 19 */
  int32_t n_min;       /* 16 */
  int32_t n_max;       /* finest grid resolution */
} orc_mlp_config;

int32_t orc_mlp_level_res(const orc_mlp_config* c, int32_t level);
void orc_mlp_forward(const orc_mlp_config* c, const float* table, const float* W, int32_t n,
                     const float* pos, const float* nrm, const float* alb, float* out);
/* MSE loss; dW (5*64*64 doubles) and dtable (levels*2^log2_table*2 doubles,
 * may be NULL) receive d loss / d parameter. */
double orc_mlp_grad(const orc_mlp_config* c, const float* table, const float* W, int32_t n,
                    const float* pos, const float* nrm, const float* alb, const float* target,
                    double* dW, double* dtable);

/* Timed CPU restatement of one frame (FP32 shading, p->threads threads):
 * voxelize + mip over the whole scene, trace over rows y % row_stride == 0.
 * ms[0..3] = voxelize, mip, gbuffer, trace (trace for the sampled rows). */
void orc_time_frame(const orc_scene* s, const orc_params* p, int32_t row_stride,
                    double* ms);

#ifdef __cplusplus
}
#endif
#endif
