// k_trace.cu -- the ConeTracer: replaces the per-fragment cone marching of
// voxel_cone_tracing.frag (main :246-275) over the G-buffer.
//
// One thread shades one visible pixel; a k_trace CTA covers a 16x8 pixel
// tile of 8x4 warp blocks, a shared-far-field CTA a 16x16 tile of them, so that neighbouring lanes march neighbouring, nearly
// parallel cones and hit the same texture-cache lines.
//
// This file is compiled with -fmad=false: a product and a sum are fused only
// where the code says so (__fmaf_rn), so the results do not depend on how
// the compiler arranges the code around them.
//
// Texture sampling is GL textureLod with GL_LINEAR_MIPMAP_LINEAR and
// CLAMP_TO_BORDER(0) over levels 0..L-1 (texture_3d.cpp:10-15).  Level 0 is
// one texture shared by the six maps (as in the reference, where all six
// maps hold identical level-0 data), so for lambda < 1 the three per-axis
// lookups of sample_voxel (:80-86) need one level-0 fetch:
//   sum_k a_k [(1-f) T0 + f T1_k] = (1-f) T0 sum_k a_k + f sum_k a_k T1_k.
// Two samplers:
//   VCT_SAMPLER_HW    -- the texture unit filters (trilinear within a level,
//                        linear between levels; 8-bit fixed-point weights);
//   VCT_SAMPLER_EXACT -- FP32 trilinear / mip-linear filtering in software
//                        from surface reads (the accuracy reference).
#include <cuda_fp16.h>

#include <algorithm>

#include "vct_internal.h"
#include "vct_math.cuh"

namespace vct {
namespace {

__device__ __forceinline__ float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
__device__ __forceinline__ float4 operator+(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 operator*(float4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
// a * s and a * s + c with one rounding each, spelled out so that the alpha
// channel is computed identically by the RGBA and the alpha-only paths.
__device__ __forceinline__ float4 mul4(float4 a, float s) {
  return f4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ float4 fma4(float4 a, float s, float4 c) {
  return f4(__fmaf_rn(a.x, s, c.x), __fmaf_rn(a.y, s, c.y), __fmaf_rn(a.z, s, c.z), __fmaf_rn(a.w, s, c.w));
}

#ifndef VCT_TRACE_ROWS
#define VCT_TRACE_ROWS 8
#endif
#ifndef VCT_TRACE_MIN_BLOCKS
#define VCT_TRACE_MIN_BLOCKS 12
#endif
// A k_trace CTA shades a 16 x kTraceRows pixel tile (each warp a
// kTraceWarpW x (32 / kTraceWarpW) block); the texture-unit variant is compiled for kTraceMinBlocks resident
// CTAs per SM (register budget 65536 / (16 * rows * blocks) per thread).
// Measured on the 1080p bench frame (trace ms): 128 threads x 12 CTAs (40
// registers, 48 warps per SM) 2.59; x 9 (56 registers) 2.64; 256 threads
// x 4 (64 registers) 2.71, x 6 (40) 2.62; 32 registers 3.77 (spills);
// 64-thread CTAs x 22 2.98. Warps of 8x4 pixels instead of 16x2 strips:
// 2.536 vs 2.543 alternating on one GPU, within noise across GPUs (same frame).
constexpr int kTraceRows = VCT_TRACE_ROWS;
constexpr int kTraceThreads = 16 * kTraceRows;
constexpr int kTraceMinBlocks = VCT_TRACE_MIN_BLOCKS;
#ifndef VCT_TRACE_WARP_W
#define VCT_TRACE_WARP_W 8
#endif
constexpr int kTraceWarpW = VCT_TRACE_WARP_W;
static_assert((kTraceWarpW == 8 || kTraceWarpW == 16) && kTraceRows % (32 / kTraceWarpW) == 0,
              "a k_trace tile holds whole warp blocks");
#ifndef VCT_TRACE_BATCH_MIN_BLOCKS
#define VCT_TRACE_BATCH_MIN_BLOCKS 3
#endif
// The batched trace keeps a scene's descriptor in shared memory and its
// values in registers, so it is compiled for its own occupancy.
constexpr int kTraceBatchMinBlocks = VCT_TRACE_BATCH_MIN_BLOCKS;

constexpr float kTan22_5 = 0.55785173935f;      // TAN_22_5 (:136), kept verbatim
constexpr float kMaxDistance = 1.73205080757f;  // MAX_DISTANCE (:138)

// ---------------------------------------------------------------- samplers --
template <int STORAGE>
__device__ __forceinline__ float4 fetch_texel(cudaSurfaceObject_t s, int x, int y, int z) {
  if (STORAGE == VCT_STORAGE_RGBA8) {
    uchar4 v;
    surf3Dread(&v, s, x * 4, y, z, cudaBoundaryModeZero);
    const float k = 1.0f / 255.0f;
    return f4(v.x * k, v.y * k, v.z * k, v.w * k);
  } else {
    uint2 v;
    surf3Dread(&v, s, x * 8, y, z, cudaBoundaryModeZero);
    const float2 a = __half22float2(*reinterpret_cast<__half2*>(&v.x));
    const float2 b = __half22float2(*reinterpret_cast<__half2*>(&v.y));
    return f4(a.x, a.y, b.x, b.y);
  }
}

template <int STORAGE>
__device__ float4 trilinear_exact(const MapSet& m, int level, int map, V3 u) {
  const int s = m.N >> level;
  const cudaSurfaceObject_t surf = level == 0 ? m.l0_surf : m.surf[map][level];
  const float tx = u.x * (float)s - 0.5f, ty = u.y * (float)s - 0.5f, tz = u.z * (float)s - 0.5f;
  const float fx = floorf(tx), fy = floorf(ty), fz = floorf(tz);
  const float ax = tx - fx, ay = ty - fy, az = tz - fz;
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
    const float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay) * (dz ? az : 1.0f - az);
    const int X = ix + dx, Y = iy + dy, Z = iz + dz;
    if ((unsigned)X < (unsigned)s && (unsigned)Y < (unsigned)s && (unsigned)Z < (unsigned)s)
      acc = acc + fetch_texel<STORAGE>(surf, X, Y, Z) * w;
  }
  return acc;
}

__device__ __forceinline__ bool u_sane(V3 u) {
  return fabsf(u.x) < 1.0e6f && fabsf(u.y) < 1.0e6f && fabsf(u.z) < 1.0e6f;
}

template <int STORAGE>
__device__ float4 texture_lod_exact(const MapSet& m, int map, V3 u, float lod) {
  if (!u_sane(u)) return f4(0.f, 0.f, 0.f, 0.f);
  if (!(lod > 0.0f)) return trilinear_exact<STORAGE>(m, 0, map, u);
  const int q = m.L - 1;
  if (lod >= (float)q) return trilinear_exact<STORAGE>(m, q, map, u);
  const float fl = floorf(lod);
  const int d1 = (int)fl;
  const float f = lod - fl;
  return trilinear_exact<STORAGE>(m, d1, map, u) * (1.0f - f) + trilinear_exact<STORAGE>(m, d1 + 1, map, u) * f;
}

// sum_k a_k * textureLod(chain idx_k, u, l) from the texture unit.  A map
// whose weight is exactly 0 is not fetched: its term 0 * texel is 0 for every
// finite texel, so the sum is unchanged.  Cones along an axis-aligned normal
// (every wall pixel) have one or two such weights.
__device__ __forceinline__ float4 aniso_fetch(const MapSet& m, V3 u, int ix, int iy, int iz, V3 ad, float l) {
  float4 r = f4(0.f, 0.f, 0.f, 0.f);
  if (ad.x != 0.0f) r = mul4(tex3DLod<float4>(m.tex[ix], u.x, u.y, u.z, l), ad.x);
  if (ad.y != 0.0f) r = fma4(tex3DLod<float4>(m.tex[iy], u.x, u.y, u.z, l), ad.y, r);
  if (ad.z != 0.0f) r = fma4(tex3DLod<float4>(m.tex[iz], u.x, u.y, u.z, l), ad.z, r);
  return r;
}

// The alpha channel of aniso_fetch from the alpha-only chains: one fetch
// covers the x and y maps (a-x, a+x, a-y, a+y), one the z maps (a-z, a+z).
// The texture unit filters every channel with the same weights, so each
// term equals the alpha of the corresponding map's fetch bit for bit.
__device__ __forceinline__ float aniso_alpha(const MapSet& m, V3 u, int ix, int iy, int iz, V3 ad, float l) {
  float r = 0.0f;
  if (ad.x != 0.0f || ad.y != 0.0f) {
    const float4 a = tex3DLod<float4>(m.alpha_tex[0], u.x, u.y, u.z, l);
    if (ad.x != 0.0f) r = __fmul_rn(ix == 0 ? a.x : a.y, ad.x);
    if (ad.y != 0.0f) r = __fmaf_rn(iy == 2 ? a.z : a.w, ad.y, r);
  }
  if (ad.z != 0.0f) {
    const float2 b = tex3DLod<float2>(m.alpha_tex[1], u.x, u.y, u.z, l);
    r = __fmaf_rn(iz == 4 ? b.x : b.y, ad.z, r);
  }
  return r;
}

// sum_k a_k * textureLod(map idx_k, u, lod), lod >= 0.  Positions with a
// coordinate of magnitude >= 1e6 (or not finite) sample 0; CHECK = false
// when the caller knows the position is sane.
template <int SAMPLER, bool ISO, int STORAGE, bool CHECK = true>
__device__ __forceinline__ float4 sample_voxel(const MapSet& m, V3 u, int ix, int iy, int iz, V3 ad, float lod) {
  if (SAMPLER == VCT_SAMPLER_EXACT) {
    if (ISO) return texture_lod_exact<STORAGE>(m, 0, u, lod) * (ad.x + ad.y + ad.z);
    return texture_lod_exact<STORAGE>(m, ix, u, lod) * ad.x + texture_lod_exact<STORAGE>(m, iy, u, lod) * ad.y +
           texture_lod_exact<STORAGE>(m, iz, u, lod) * ad.z;
  }
  if (CHECK && !u_sane(u)) return f4(0.f, 0.f, 0.f, 0.f);
  const float wsum = ad.x + ad.y + ad.z;
  if (lod < 1.0f) {
    const float4 t0 = tex3D<float4>(m.l0_tex, u.x, u.y, u.z);
    if (!(lod > 0.0f)) return mul4(t0, wsum);
    float4 t1;
    if (ISO) t1 = tex3DLod<float4>(m.tex[0], u.x, u.y, u.z, 0.0f) * wsum;
    else t1 = aniso_fetch(m, u, ix, iy, iz, ad, 0.0f);
    return fma4(t1, lod, mul4(t0, __fmul_rn(1.0f - lod, wsum)));
  }
  const float l = lod - 1.0f;
  if (ISO) return tex3DLod<float4>(m.tex[0], u.x, u.y, u.z, l) * wsum;
  return aniso_fetch(m, u, ix, iy, iz, ad, l);
}

// The alpha of sample_voxel (texture unit, anisotropic RGBA8 maps) from the
// alpha-only chains, with the same arithmetic as the alpha channel there.
__device__ __forceinline__ float sample_alpha(const MapSet& m, V3 u, int ix, int iy, int iz, V3 ad, float lod) {
  const float wsum = ad.x + ad.y + ad.z;
  if (lod < 1.0f) {
    const float t0 = tex3D<float4>(m.l0_tex, u.x, u.y, u.z).w;
    if (!(lod > 0.0f)) return __fmul_rn(t0, wsum);
    const float t1 = aniso_alpha(m, u, ix, iy, iz, ad, 0.0f);
    return __fmaf_rn(t1, lod, __fmul_rn(t0, __fmul_rn(1.0f - lod, wsum)));
  }
  return aniso_alpha(m, u, ix, iy, iz, ad, lod - 1.0f);
}

// ------------------------------------------------------------ cone march ----
// Exact early exit: a sample whose position lies more than half the coarsest
// texel outside [0,1] along an axis reads only border texels (0) at every
// level -- a filtered fetch at level l reads texels whose centres lie within
// one texel (2^l / N) of the position, and the coarsest level is L-1.  A cone
// moving away from the volume along an axis is past margin = 3/4 of the
// coarsest texel (MapSet::exit_margin, set by the host) beyond
// `exit_distance`, and adds exact zeros from there on, so its march ends
// there (the extra quarter texel absorbs the rounding of the division).
// Diffuse cones that pass the room's walls (their alpha stays below 1 at the
// coarse levels) otherwise march on to sqrt(3) outside the grid.
__device__ __forceinline__ float exit_distance(const MapSet& m, V3 origin, V3 dir, float max_dist) {
  const float lo = -m.exit_margin, hi = 1.0f + m.exit_margin;
  float d = max_dist;
  if (dir.x > 0.0f) d = fminf(d, (hi - origin.x) / dir.x);
  if (dir.x < 0.0f) d = fminf(d, (lo - origin.x) / dir.x);
  if (dir.y > 0.0f) d = fminf(d, (hi - origin.y) / dir.y);
  if (dir.y < 0.0f) d = fminf(d, (lo - origin.y) / dir.y);
  if (dir.z > 0.0f) d = fminf(d, (hi - origin.z) / dir.z);
  if (dir.z < 0.0f) d = fminf(d, (lo - origin.z) / dir.z);
  return d;  // (+inf margin: max_dist)
}

// Exact empty-space skip: true when every texel the sample at u with this
// lod reads is 0 (MapSet::occ).  Its coarser quadrilinear level is c (level
// 1 when lod < 1, where level 0 and level 1 are read); there the lookup reads
// texels k .. k+1 along each axis, k = floor(u * (N >> c) - 0.5), and the
// finer level's texels lie inside them, so the occ bit of k decides.  Within
// 1/64 texel of a texel boundary the texture unit's fixed-point coordinate
// could pick the neighbouring pair: such samples are fetched.  The test runs
// in 8.8 fixed point: q = floor(256 t) (t scaled by a power of two, so the
// same rounding), k = q >> 8, and the fraction's top byte q & 255 in
// [252, 255] or [0, 3] marks the band (a superset of |frac - 0| < 1/64 and
// frac > 1 - 1/64: conservative).  A pair outside
// the grid is tested at the nearest cell inside it (conservative: border
// texels are 0, and cones leaving the grid stop at exit_distance).  (A position
// that is not finite or is huge ends up clamped or fetched; the texture path
// returns 0 for it either way.)
__device__ __forceinline__ bool sample_empty(const MapSet& m, V3 u, float lod) {
  const int c = min((int)lod + 1, m.L - 1);  // lod >= 0
  const int s = m.N >> c;
  const float fs = (float)(s << 8);
  // (huge or non-finite coordinates saturate or give 0: clamped or fetched)
  const int qx = __float2int_rd(__fmaf_rn(u.x, fs, -128.0f)), qy = __float2int_rd(__fmaf_rn(u.y, fs, -128.0f)),
            qz = __float2int_rd(__fmaf_rn(u.z, fs, -128.0f));
  if ((((uint32_t)qx + 4u) & 255u) < 8u || (((uint32_t)qy + 4u) & 255u) < 8u || (((uint32_t)qz + 4u) & 255u) < 8u)
    return false;
  const int kx = min(max(qx >> 8, 0), s - 1), ky = min(max(qy >> 8, 0), s - 1), kz = min(max(qz >> 8, 0), s - 1);
  const uint32_t w = __ldg(m.occ[c] + ((uint32_t)kz * s + ky) * m.occ_wpr[c] + (kx >> 5));
  return ((w >> (kx & 31)) & 1u) == 0u;
}

// The coarser test (MapSet::occ3): the texels the sample reads at level c
// lie within one cell of floor(u * (N >> c)) along each axis, under any
// rounding of the texture unit's coordinate (positions outside the grid are
// tested at the nearest cell inside, conservatively).  Cheaper than
// sample_empty (no boundary test); it finds nearly all the empty steps of
// the narrow shadow cones.
// (sample_empty3 in two parts: the occupancy word is loaded a step ahead by
// the pipelined shadow march; the word shifted right by `bit` holds the bit.)
__device__ __forceinline__ uint32_t empty3_word(const MapSet& m, V3 u, float lod, uint32_t& bit) {
  const int c = min((int)lod + 1, m.L - 1);  // lod >= 0
  const int s = m.N >> c;
  const float fs = (float)s;
  const int kx = min(max(__float2int_rd(u.x * fs), 0), s - 1), ky = min(max(__float2int_rd(u.y * fs), 0), s - 1),
            kz = min(max(__float2int_rd(u.z * fs), 0), s - 1);
  bit = (uint32_t)kx & 31u;
  return __ldg(m.occ3[c] + ((uint32_t)kz * s + ky) * m.occ_wpr[c] + (kx >> 5));
}

__device__ __forceinline__ bool sample_empty3(const MapSet& m, V3 u, float lod) {
  uint32_t bit;
  const uint32_t w = empty3_word(m, u, lod, bit);
  return ((w >> bit) & 1u) == 0u;
}

#ifndef VCT_SKIP_EMPTY_RGBA
#define VCT_SKIP_EMPTY_RGBA 1
#endif
constexpr bool kSkipEmptyRGBA = VCT_SKIP_EMPTY_RGBA != 0;  // also in the RGBA cones (else shadow cones only)
#ifndef VCT_SKIP_MAX_LOD
#define VCT_SKIP_MAX_LOD 5.0f
#endif
// RGBA cones test for empty space only below this lod: coarser samples are
// fetched without the test (the coarse cells are rarely empty; fetching a
// sample that is empty adds the same exact zeros).  Measured on the 1080p
// bench frame (trace ms): no cap 2.580, below 6 2.552, 5.5 2.550, 5 2.540,
// 4 2.572; the frames are bit-identical.
constexpr float kSkipMaxLod = VCT_SKIP_MAX_LOD;

// The lod of a march step, max(log2(diam * N), 0) with the fast log2
// (lg2.approx).  Its argument is at least 3 * aperture >= 0.05 (the first
// step is at 3 voxels and apertures are >= 0.0174533), never subnormal, so
// the flush-to-zero form gives the same result without the subnormal path.
#ifndef VCT_LOD_FTZ
#define VCT_LOD_FTZ 1
#endif
__device__ __forceinline__ float cone_lod(float x) {
#if VCT_LOD_FTZ
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return fmaxf(r, 0.0f);
#else
  return fmaxf(__log2f(x), 0.0f);
#endif
}

// The sample position origin + dir * dist of a march step, one rounding per
// coordinate (an explicit fused multiply-add, so that it does not depend on
// how the compiler arranges the step loop).
__device__ __forceinline__ V3 march_pos(V3 origin, V3 dir, float dist) {
  return v3(__fmaf_rn(dir.x, dist, origin.x), __fmaf_rn(dir.y, dist, origin.y), __fmaf_rn(dir.z, dist, origin.z));
}

// Whether every position of a march from `origin` along unit `dir` up to
// `stop` is sane (|coordinate| < 1e6, finite); then the step loop needs no
// per-sample check.
__device__ __forceinline__ bool march_sane(V3 origin, V3 dir, float stop) {
  const float reach = fmaxf(fabsf(origin.x), fmaxf(fabsf(origin.y), fabsf(origin.z))) + fmaxf(stop, 0.0f);
  return reach < 1.0e6f && isfinite(dir.x + dir.y + dir.z);
}

#ifndef VCT_TRACE_PIPE
#define VCT_TRACE_PIPE 1
#endif
// Step loop of the texture-unit anisotropic march: 0 = one step after the
// other; 1 = the next step's position, lod and empty-space test (with its
// occupancy load) run while this step's texture fetches are in flight;
// 2 = also the next step's fetches are issued before this step's results
// are used (two sets of results live).  Same samples, same arithmetic.
constexpr int kTracePipe = VCT_TRACE_PIPE;

// The raw texture results of one step of the anisotropic march (the
// fetches of sample_voxel, texture unit, anisotropic maps).
struct Taps {
  float4 t0, x, y, z;
};

__device__ __forceinline__ void issue_taps(const MapSet& m, V3 u, int ix, int iy, int iz, V3 ad, float lod, Taps& t) {
  float l = lod - 1.0f;
  if (lod < 1.0f) {
    t.t0 = tex3D<float4>(m.l0_tex, u.x, u.y, u.z);
    if (!(lod > 0.0f)) return;
    l = 0.0f;
  }
  if (ad.x != 0.0f) t.x = tex3DLod<float4>(m.tex[ix], u.x, u.y, u.z, l);
  if (ad.y != 0.0f) t.y = tex3DLod<float4>(m.tex[iy], u.x, u.y, u.z, l);
  if (ad.z != 0.0f) t.z = tex3DLod<float4>(m.tex[iz], u.x, u.y, u.z, l);
}

// sample_voxel<HW, aniso> from the step's taps, operation for operation.
__device__ __forceinline__ float4 combine_taps(const Taps& t, V3 ad, float lod) {
  const float wsum = ad.x + ad.y + ad.z;
  if (lod < 1.0f && !(lod > 0.0f)) return mul4(t.t0, wsum);
  float4 r = f4(0.f, 0.f, 0.f, 0.f);
  if (ad.x != 0.0f) r = mul4(t.x, ad.x);
  if (ad.y != 0.0f) r = fma4(t.y, ad.y, r);
  if (ad.z != 0.0f) r = fma4(t.z, ad.z, r);
  if (lod < 1.0f) return fma4(r, lod, mul4(t.t0, __fmul_rn(1.0f - lod, wsum)));
  return r;
}

// trace_cone for the texture unit and anisotropic maps with the step loop
// software-pipelined (kTracePipe): the march, the samples taken and the
// accumulation are those of the plain loop in trace_cone.
__device__ float4 trace_cone_pipe(const MapSet& m, V3 origin, V3 dir, float aperture, float max_dist) {
  dir = normalize(dir);
  const int ix = dir.x < 0.0f ? 0 : 1, iy = dir.y < 0.0f ? 2 : 3, iz = dir.z < 0.0f ? 4 : 5;
  const V3 ad = vabs(dir);
  const float cube_res = (float)m.N;
  const float voxel_size = 1.0f / cube_res;
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
  float dist = 3.0f * voxel_size;
  float diam = dist * aperture;
  V3 sp = march_pos(origin, dir, dist);
  const float stop = exit_distance(m, origin, dir, max_dist);
  const bool check = !march_sane(origin, dir, stop);
  if (!(dist < stop)) return acc;
  float mip = cone_lod(diam * cube_res);
  bool live = !(kSkipEmptyRGBA && m.skip_empty && mip < kSkipMaxLod && sample_empty(m, sp, mip)) && !(check && !u_sane(sp));
  Taps t;
  if (live) issue_taps(m, sp, ix, iy, iz, ad, mip, t);
  while (true) {
    // the next step (taken only while this one leaves alpha below 1)
    const float step = fmaxf(diam * 0.5f, voxel_size);
    dist += step;
    diam = dist * aperture;
    sp = march_pos(origin, dir, dist);
    const bool more = dist < stop;
    const float mip_n = cone_lod(diam * cube_res);
    const bool live_n =
        more && !(kSkipEmptyRGBA && m.skip_empty && mip_n < kSkipMaxLod && sample_empty(m, sp, mip_n)) && !(check && !u_sane(sp));
    if (kTracePipe >= 2) {
      Taps tn;
      if (live_n) issue_taps(m, sp, ix, iy, iz, ad, mip_n, tn);
      if (live) acc = fma4(combine_taps(t, ad, mip), 1.0f - acc.w, acc);
      if (!(acc.w < 1.0f) || !more) break;
      t = tn;
    } else {
      if (live) acc = fma4(combine_taps(t, ad, mip), 1.0f - acc.w, acc);
      if (!(acc.w < 1.0f) || !more) break;
      if (live_n) issue_taps(m, sp, ix, iy, iz, ad, mip_n, t);
    }
    mip = mip_n;
    live = live_n;
  }
  return acc;
}

// trace_cone, voxel_cone_tracing.frag:88-119.
template <int SAMPLER, bool ISO, int STORAGE>
__device__ float4 trace_cone(const MapSet& m, V3 origin, V3 dir, float aperture, float max_dist) {
  if (kTracePipe > 0 && SAMPLER == VCT_SAMPLER_HW && !ISO) return trace_cone_pipe(m, origin, dir, aperture, max_dist);
  dir = normalize(dir);
  const int ix = dir.x < 0.0f ? 0 : 1, iy = dir.y < 0.0f ? 2 : 3, iz = dir.z < 0.0f ? 4 : 5;
  const V3 ad = vabs(dir);
  const float cube_res = (float)m.N;
  const float voxel_size = 1.0f / cube_res;
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
  float dist = 3.0f * voxel_size;
  float diam = dist * aperture;
  V3 sp = march_pos(origin, dir, dist);
  const float stop = exit_distance(m, origin, dir, max_dist);
  const bool check = !march_sane(origin, dir, stop);
  while (acc.w < 1.0f && dist < stop) {
    const float mip = cone_lod(diam * cube_res);
    if (!(kSkipEmptyRGBA && m.skip_empty && mip < kSkipMaxLod && sample_empty(m, sp, mip)) && !(check && !u_sane(sp))) {
      // (an empty or insane sample adds exact zeros)
      const float4 s = sample_voxel<SAMPLER, ISO, STORAGE, false>(m, sp, ix, iy, iz, ad, mip);
      acc = fma4(s, 1.0f - acc.w, acc);
    }
    const float step = fmaxf(diam * 0.5f, voxel_size);
    dist += step;
    diam = dist * aperture;
    sp = march_pos(origin, dir, dist);
  }
  return acc;
}

// trace_cone(...).a (trace_shadow, :121-124) with the texture unit over the
// alpha-only chains: the same march and the same alpha arithmetic, two
// texture fetches per step instead of three.
__device__ float trace_alpha_pipe(const MapSet& m, V3 origin, V3 dir, float aperture, float max_dist);
__device__ float trace_alpha(const MapSet& m, V3 origin, V3 dir, float aperture, float max_dist) {
  if (kTracePipe > 0) return trace_alpha_pipe(m, origin, dir, aperture, max_dist);
  dir = normalize(dir);
  const int ix = dir.x < 0.0f ? 0 : 1, iy = dir.y < 0.0f ? 2 : 3, iz = dir.z < 0.0f ? 4 : 5;
  const V3 ad = vabs(dir);
  const float cube_res = (float)m.N;
  const float voxel_size = 1.0f / cube_res;
  float a = 0.0f;
  float dist = 3.0f * voxel_size;
  float diam = dist * aperture;
  V3 sp = march_pos(origin, dir, dist);
  const float stop = exit_distance(m, origin, dir, max_dist);
  const bool check = !march_sane(origin, dir, stop);
  while (a < 1.0f && dist < stop) {
    const float mip = cone_lod(diam * cube_res);
    if (!(m.skip_empty && sample_empty3(m, sp, mip)) && !(check && !u_sane(sp)))
      a = __fmaf_rn(sample_alpha(m, sp, ix, iy, iz, ad, mip), 1.0f - a, a);
    const float step = fmaxf(diam * 0.5f, voxel_size);
    dist += step;
    diam = dist * aperture;
    sp = march_pos(origin, dir, dist);
  }
  return a;
}

// trace_alpha with the occupancy word of the next step loaded while this
// step is sampled (kTracePipe > 0): the same samples and arithmetic.
__device__ float trace_alpha_pipe(const MapSet& m, V3 origin, V3 dir, float aperture, float max_dist) {
  dir = normalize(dir);
  const int ix = dir.x < 0.0f ? 0 : 1, iy = dir.y < 0.0f ? 2 : 3, iz = dir.z < 0.0f ? 4 : 5;
  const V3 ad = vabs(dir);
  const float cube_res = (float)m.N;
  const float voxel_size = 1.0f / cube_res;
  const bool skip = m.skip_empty != 0;
  float a = 0.0f;
  float dist = 3.0f * voxel_size;
  float diam = dist * aperture;
  V3 sp = march_pos(origin, dir, dist);
  const float stop = exit_distance(m, origin, dir, max_dist);
  const bool check = !march_sane(origin, dir, stop);
  if (!(dist < stop)) return a;
  float mip = cone_lod(diam * cube_res);
  uint32_t bit = 0, w = skip ? empty3_word(m, sp, mip, bit) : 1u;
  while (true) {
    const float step = fmaxf(diam * 0.5f, voxel_size);
    const float dist_n = dist + step;
    const float diam_n = dist_n * aperture;
    const V3 sp_n = march_pos(origin, dir, dist_n);
    const bool more = dist_n < stop;
    const float mip_n = cone_lod(diam_n * cube_res);
    uint32_t bit_n = 0, w_n = 1u;
    if (skip && more) w_n = empty3_word(m, sp_n, mip_n, bit_n);
    if (((w >> bit) & 1u) != 0u && !(check && !u_sane(sp)))
      a = __fmaf_rn(sample_alpha(m, sp, ix, iy, iz, ad, mip), 1.0f - a, a);
    if (!(a < 1.0f) || !more) break;
    dist = dist_n;
    diam = diam_n;
    sp = sp_n;
    mip = mip_n;
    w = w_n;
    bit = bit_n;
  }
  return a;
}

// tangent, :126-134.
__device__ __forceinline__ V3 tangent(V3 n) {
  const V3 t1 = cross(n, v3(0.f, 0.f, 1.f)), t2 = cross(n, v3(0.f, 1.f, 0.f));
  return length(t1) > length(t2) ? normalize(t1) : normalize(t2);
}
__device__ __forceinline__ V3 mixv(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }

// trace_diffuse, :140-168 (9 equal-weight cones); cone set SIX60 (no
// reference counterpart): the normal plus 5 cones 60 degrees off it in the
// same tangent frame, aperture 2 tan(30 deg), equal weights.
template <int SAMPLER, bool ISO, int STORAGE>
__device__ V3 trace_diffuse(const MapSet& m, int cone_set, V3 origin, V3 n) {
  const V3 o1 = normalize(tangent(n));
  const V3 o2 = normalize(cross(o1, n));
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
  if (cone_set == VCT_CONES_SIX60) {
    const float ap = 1.15470053838f;  // 2 tan(30 deg)
    const V3 nn = normalize(n);
    acc = trace_cone<SAMPLER, ISO, STORAGE>(m, origin, nn, ap, kMaxDistance);
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {
      float sphi, cphi;
      sincosf(6.28318530717958648f * (float)k / 5.0f, &sphi, &cphi);
      const V3 d = nn * 0.5f + (o1 * cphi + o2 * sphi) * 0.86602540378f;
      acc = acc + trace_cone<SAMPLER, ISO, STORAGE>(m, origin, d, ap, kMaxDistance);
    }
    return v3(acc.x, acc.y, acc.z) * (1.0f / 6.0f);
  }
  const V3 c1 = (o1 + o2) * 0.5f, c2 = (o1 - o2) * 0.5f;
  acc = trace_cone<SAMPLER, ISO, STORAGE>(m, origin, n, kTan22_5, kMaxDistance);
  // Side cones o1, -o1, o2, -o2, c1, -c1, c2, -c2 (:156-165), selected
  // arithmetically so that no local-memory array is needed.
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    const V3 b = k < 2 ? o1 : (k < 4 ? o2 : (k < 6 ? c1 : c2));
    const V3 side = (k & 1) ? -b : b;
    acc = acc + trace_cone<SAMPLER, ISO, STORAGE>(m, origin, mixv(n, side, 0.5f), kTan22_5, kMaxDistance);
  }
  return v3(acc.x, acc.y, acc.z) * (1.0f / 9.0f);
}

// ------------------------------------------------- shared far fields ------
// Far-field sharing (TraceParams::far_share, texture-unit sampler).  The
// diffuse cones of neighbouring pixels on one surface start a fraction of a
// voxel apart in nearly the same directions, and after their first sample
// (3 voxels out, lod log2(3 aperture)) their samples are coarse texels whose
// filtered values barely differ across a few pixels.  So every diffuse cone
// is split after its first step: each pixel takes that sample itself, and the
// rest of the march (the "far field") is done once per group of kShareW x 2
// pixels, along the cones of one pixel of the group (its representative),
// by the lanes of the warp together (far_fields below).  The split is exact
// front-to-back compositing: a march that continues from the first sample s
// equals s + (1 - s.a) * far, where far is the march of the remaining steps
// from zero, and both stop at the same step (alpha reaching 1).  Only the
// representative's positions and directions stand in for the other
// pixels'.  A pixel shares only when its normal is within kShareCos of the
// representative's and its surface point within kShareDist voxels along
// every axis; others march their own cones.  Measured against the FP64
// oracle on the 1080p bench frame (sharing alone, the texture unit's 8-bit
// filter weights being 71 dB): 2x2 groups 80.6 dB, 4x2 groups 73.1 dB, with
// the diffuse cones' two-level texture fetches cut from 238 to 60 and 31
// per pixel.
constexpr float kShareCos = 0.99f;
constexpr float kShareDist = 2.0f;  // voxels
#ifndef VCT_FAR_PIPE
#define VCT_FAR_PIPE 1
#endif
constexpr bool kFarPipe = VCT_FAR_PIPE != 0;  // software-pipelined far-field march
#ifndef VCT_FIRST_UNROLL
#define VCT_FIRST_UNROLL 1  // the per-pixel first samples of the diffuse cones: cones in flight together
#endif
#define VCT_STR(x) #x
#define VCT_UNROLL_N(n) _Pragma(VCT_STR(unroll n))
#ifndef VCT_SHARE_GROUP_W
#define VCT_SHARE_GROUP_W 4
#endif
// A sharing group is kShareW x 2 pixels of a warp's 8x4-pixel block.
constexpr int kShareW = VCT_SHARE_GROUP_W;
static_assert(kShareW == 2 || kShareW == 4 || kShareW == 8, "group width divides the 8-pixel block row");
constexpr int kShareQuads = 16 / kShareW;  // groups of a warp
constexpr int kShareCones = 9;
constexpr int kShareJobs = kShareQuads * kShareCones;

// Order of a warp's far-field jobs: 1 = the jobs that start after the
// first 32 (the last lanes to finish wait for them) are those with the
// shortest exit distance, so the warp's tail is short; 0 = cone-major order.
#ifndef VCT_FAR_SHORT_TAIL
#define VCT_FAR_SHORT_TAIL 1
#endif
constexpr bool kFarShortTail = VCT_FAR_SHORT_TAIL != 0;

struct FarWarp {
  float4 far[kShareJobs];   // far field of cone k of group slot q at q * K + k
  float4 job[kShareJobs];   // job j = k * nq + q: unit direction, exit distance
  float origin[kShareQuads][3];  // representative's texture-space position
  float normal[kShareQuads][3];  // and normal
  uint8_t order[kShareJobs];     // the job handed out n-th
};

// Direction (unnormalised) and aperture of diffuse cone k, as trace_diffuse
// computes them from the normal n and its frame o1, o2.
__device__ __forceinline__ V3 diffuse_dir(int cone_set, V3 n, V3 o1, V3 o2, int k, float& ap) {
  if (cone_set == VCT_CONES_SIX60) {
    ap = 1.15470053838f;
    const V3 nn = normalize(n);
    if (k == 0) return nn;
    float sphi, cphi;
    sincosf(6.28318530717958648f * (float)(k - 1) / 5.0f, &sphi, &cphi);
    return nn * 0.5f + (o1 * cphi + o2 * sphi) * 0.86602540378f;
  }
  ap = kTan22_5;
  if (k == 0) return n;
  const int j = k - 1;
  const V3 c1 = (o1 + o2) * 0.5f, c2 = (o1 - o2) * 0.5f;
  const V3 b = j < 2 ? o1 : (j < 4 ? o2 : (j < 6 ? c1 : c2));
  const V3 side = (j & 1) ? -b : b;
  return mixv(n, side, 0.5f);
}

// The far fields of a warp's nq groups.  Job j = k * nq + q is cone k of group
// slot q (neighbouring lanes start on the same cone of neighbouring groups,
// which read neighbouring texels).  The lanes first set up every job's
// direction and exit distance together (fw.job), then march: a lane whose
// cone ends (alpha 1, the grid's edge) takes the next job while the others
// march on.  The march starts at the second step of the schedule (dist1,
// diam1) with nothing accumulated.  Results go to fw.far[q * K + k].
template <bool ISO>
__device__ void far_fields(const MapSet& m, FarWarp& fw, int cone_set, int nq, float dist1, float diam1) {
  const int lane = threadIdx.x & 31;
  const int K = cone_set == VCT_CONES_SIX60 ? 6 : 9;
  const int n_jobs = nq * K;
  for (int j = lane; j < n_jobs; j += 32) {
    const int k = j / nq, q = j - k * nq;
    const V3 n = v3(fw.normal[q][0], fw.normal[q][1], fw.normal[q][2]);
    const V3 o1 = normalize(tangent(n));
    const V3 o2 = normalize(cross(o1, n));
    float ap;
    const V3 d = normalize(diffuse_dir(cone_set, n, o1, o2, k, ap));
    const V3 o = v3(fw.origin[q][0], fw.origin[q][1], fw.origin[q][2]);
    fw.job[j] = f4(d.x, d.y, d.z, exit_distance(m, o, d, kMaxDistance));
  }
  __syncwarp();
  {
    // Jobs 0..31 start together; the n_jobs - 32 handed out after them
    // (kShareJobs - 32 at most) are swapped for the jobs of shortest exit
    // distance -- the cones that reach least far, nearly always the shortest
    // marches -- picked by warp min-reductions of (distance, job) keys.
    // Which lane marches a job changes nothing in its result.
    static_assert(kShareJobs <= 64, "job index in 6 bits");
    const int n_tail = n_jobs - 32;
    uint64_t tail = 0;  // warp-uniform: the jobs chosen for the tail
    if (kFarShortTail && n_tail > 0) {
      auto key = [&](int j) {
        return j < n_jobs ? (__float_as_uint(fmaxf(fw.job[j].w, 0.0f)) & ~63u) | (unsigned)j : ~0u;
      };
      unsigned k0 = key(lane), k1 = key(lane + 32);
      for (int t = 0; t < n_tail; ++t) {
        const unsigned mn = __reduce_min_sync(0xffffffffu, min(k0, k1));
        tail |= 1ull << (mn & 63u);
        if (k0 == mn) k0 = ~0u;
        if (k1 == mn) k1 = ~0u;
      }
    }
    // chosen jobs among 0..31 trade places, in order, with the jobs at 32..
    // that were not chosen
    // (no choice made: a = b = 0, every job keeps its place)
    const uint32_t a = (uint32_t)tail;
    const uint32_t b = tail ? ~(uint32_t)(tail >> 32) & ((1u << n_tail) - 1u) : 0u;
    auto nth = [](uint32_t mask, int i) {  // the i-th set bit of mask
      for (; i > 0; --i) mask &= mask - 1u;
      return __ffs(mask) - 1;
    };
    for (int j = lane; j < n_jobs; j += 32) {
      int o = j;
      if (j < 32 && ((a >> j) & 1u)) o = 32 + nth(b, __popc(a & ((1u << j) - 1u)));
      if (j >= 32 && ((b >> (j - 32)) & 1u)) o = nth(a, __popc(b & ((1u << (j - 32)) - 1u)));
      fw.order[j] = (uint8_t)o;
    }
  }
  __syncwarp();
  const float ap = cone_set == VCT_CONES_SIX60 ? 1.15470053838f : kTan22_5;
  const float cube_res = (float)m.N;
  const float voxel_size = 1.0f / cube_res;
  int next = 0;  // warp-uniform: next job to hand out
  int res = 0;
  bool active = false;
  V3 origin = v3(0.f, 0.f, 0.f), dir = v3(0.f, 0.f, 1.f), ad = v3(0.f, 0.f, 1.f);
  int ix = 1, iy = 3, iz = 5;
  float dist = 0.f, diam = 0.f, stop = 0.f;
  bool check = false;
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
  if constexpr (kFarPipe && !ISO) {
    // Software-pipelined like trace_cone_pipe (anisotropic maps; the
    // isotropic march below samples one chain): a lane computes its next step
    // (position, lod, empty-space test with its occupancy load) while the
    // current step's texture fetches are in flight, and issues the next
    // step's fetches as soon as the current one is added.  Same samples, same
    // arithmetic as the loop below.
    float mip = 0.f;
    bool live = false;
    Taps t;
    for (;;) {
      const unsigned need = __ballot_sync(0xffffffffu, !active);
      if (need && next < n_jobs) {
        const int job = next + __popc(need & ((1u << lane) - 1u));
        if (!active && job < n_jobs) {
          const int jo = fw.order[job];
          const int k = jo / nq, q = jo - k * nq;
          res = q * K + k;
          const float4 jb = fw.job[jo];
          dir = v3(jb.x, jb.y, jb.z);
          stop = jb.w;
          origin = v3(fw.origin[q][0], fw.origin[q][1], fw.origin[q][2]);
          ix = dir.x < 0.0f ? 0 : 1;
          iy = dir.y < 0.0f ? 2 : 3;
          iz = dir.z < 0.0f ? 4 : 5;
          ad = vabs(dir);
          dist = dist1;
          diam = diam1;
          check = !march_sane(origin, dir, stop);
          acc = f4(0.f, 0.f, 0.f, 0.f);
          active = dist < stop;
          if (!active) {
            fw.far[res] = acc;
          } else {
            const V3 sp = march_pos(origin, dir, dist);
            mip = cone_lod(diam * cube_res);
            live = !(kSkipEmptyRGBA && m.skip_empty && mip < kSkipMaxLod && sample_empty(m, sp, mip)) &&
                   !(check && !u_sane(sp));
            if (live) issue_taps(m, sp, ix, iy, iz, ad, mip, t);
          }
        }
        next += __popc(need);
      }
      if (!__any_sync(0xffffffffu, active)) break;
      if (active) {
        const float step = fmaxf(diam * 0.5f, voxel_size);
        const float dist_n = dist + step;
        const float diam_n = dist_n * ap;
        const V3 sp_n = march_pos(origin, dir, dist_n);
        const bool more = dist_n < stop;
        const float mip_n = cone_lod(diam_n * cube_res);
        const bool live_n = more &&
                            !(kSkipEmptyRGBA && m.skip_empty && mip_n < kSkipMaxLod && sample_empty(m, sp_n, mip_n)) &&
                            !(check && !u_sane(sp_n));
        if (live) acc = fma4(combine_taps(t, ad, mip), 1.0f - acc.w, acc);
        if (!(acc.w < 1.0f) || !more) {
          fw.far[res] = acc;
          active = false;
        } else {
          dist = dist_n;
          diam = diam_n;
          mip = mip_n;
          live = live_n;
          if (live) issue_taps(m, sp_n, ix, iy, iz, ad, mip, t);
        }
      }
    }
  } else {
    for (;;) {
      const unsigned need = __ballot_sync(0xffffffffu, !active);
      if (need && next < n_jobs) {
        const int job = next + __popc(need & ((1u << lane) - 1u));
        if (!active && job < n_jobs) {
          const int jo = fw.order[job];
          const int k = jo / nq, q = jo - k * nq;
          res = q * K + k;
          const float4 jb = fw.job[jo];
          dir = v3(jb.x, jb.y, jb.z);
          stop = jb.w;
          origin = v3(fw.origin[q][0], fw.origin[q][1], fw.origin[q][2]);
          ix = dir.x < 0.0f ? 0 : 1;
          iy = dir.y < 0.0f ? 2 : 3;
          iz = dir.z < 0.0f ? 4 : 5;
          ad = vabs(dir);
          dist = dist1;
          diam = diam1;
          check = !march_sane(origin, dir, stop);
          acc = f4(0.f, 0.f, 0.f, 0.f);
          active = dist < stop;
          if (!active) fw.far[res] = acc;
        }
        next += __popc(need);
      }
      if (!__any_sync(0xffffffffu, active)) break;
      if (active) {
        const V3 sp = march_pos(origin, dir, dist);
        const float mip = cone_lod(diam * cube_res);
        if (!(kSkipEmptyRGBA && m.skip_empty && mip < kSkipMaxLod && sample_empty(m, sp, mip)) &&
            !(check && !u_sane(sp))) {
          const float4 smp = sample_voxel<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8, false>(m, sp, ix, iy, iz, ad, mip);
          acc = fma4(smp, 1.0f - acc.w, acc);
        }
        const float step = fmaxf(diam * 0.5f, voxel_size);
        dist += step;
        diam = dist * ap;
        if (!(acc.w < 1.0f) || !(dist < stop)) {
          fw.far[res] = acc;
          active = false;
        }
      }
    }
  }
}

// trace_diffuse with the group's far fields (far: this group's K results):
// each cone takes its first sample (step 0 of trace_cone) itself, then the
// far field behind it.
template <bool ISO>
__device__ V3 trace_diffuse_shared(const MapSet& m, int cone_set, V3 origin, V3 n, const float4* far) {
  const V3 o1 = normalize(tangent(n));
  const V3 o2 = normalize(cross(o1, n));
  const int K = cone_set == VCT_CONES_SIX60 ? 6 : 9;
  const float cube_res = (float)m.N;
  float4 acc = f4(0.f, 0.f, 0.f, 0.f);
  VCT_UNROLL_N(VCT_FIRST_UNROLL)
  for (int k = 0; k < K; ++k) {
    float ap;
    const V3 dir = normalize(diffuse_dir(cone_set, n, o1, o2, k, ap));
    const float dist = 3.0f * (1.0f / cube_res);
    const float diam = dist * ap;
    // (the origin is a surface point inside the grid and the first step
    // three voxels: the sample position is sane, and one beyond the grid's
    // exit margin reads border texels, 0, as the unshortened march would)
    float4 c = f4(0.f, 0.f, 0.f, 0.f);
    const V3 sp = march_pos(origin, dir, dist);
    const float mip = cone_lod(diam * cube_res);
    if (!(kSkipEmptyRGBA && m.skip_empty && mip < kSkipMaxLod && sample_empty(m, sp, mip))) {
      const int ix = dir.x < 0.0f ? 0 : 1, iy = dir.y < 0.0f ? 2 : 3, iz = dir.z < 0.0f ? 4 : 5;
      const float4 smp = sample_voxel<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8, false>(m, sp, ix, iy, iz, vabs(dir), mip);
      c = fma4(smp, 1.0f, c);
    }
    if (c.w < 1.0f) c = fma4(far[k], 1.0f - c.w, c);
    acc = acc + c;
  }
  return v3(acc.x, acc.y, acc.z) * (1.0f / (float)K);
}

__device__ __forceinline__ V3 refract(V3 I, V3 N, float eta) {
  const float d = dot(N, I);
  const float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return v3(0.f, 0.f, 0.f);
  return I * eta - N * (eta * d + sqrtf(k));
}
__device__ __forceinline__ V3 reflect(V3 I, V3 N) { return I - N * (2.0f * dot(N, I)); }

__device__ __forceinline__ V3 mat3v(const float* f) { return v3(f[0], f[1], f[2]); }

// direct_light, :175-218.
template <int SAMPLER, bool ISO, int STORAGE>
__device__ V3 direct_light(const SceneParams& sp, const MapSet& m, int enable_shadow, const vct_material_data& mat,
                           V3 pos, V3 nrm, V3 view_dir) {
  V3 result = v3(0.f, 0.f, 0.f);
  const int nl = min(sp.n_lights, kMaxLights);
  for (int i = 0; i < nl; ++i) {
    const vct_point_light& L = sp.lights[i];
    V3 lp = v3(L.position[0] / sp.cube_size, L.position[1] / sp.cube_size, L.position[2] / sp.cube_size);
    lp = lp * 0.5f + v3(0.5f, 0.5f, 0.5f);
    V3 ld = lp - pos;
    const float d = length(ld);
    ld = normalize(ld);
    const float cs = fmaxf(dot(nrm, ld), 0.0f);
    const V3 lc = v3(L.color[0], L.color[1], L.color[2]) * ((1.0f / (1.0f + d * d)) * cs * L.intensity);
    float shadow = 1.0f;
    if (enable_shadow) {
      float occ;
      if constexpr (SAMPLER == VCT_SAMPLER_HW && !ISO && STORAGE == VCT_STORAGE_RGBA8)
        occ = m.alpha_tex[0] ? trace_alpha(m, pos, ld, 0.1f, d) : trace_cone<SAMPLER, ISO, STORAGE>(m, pos, ld, 0.1f, d).w;
      else
        occ = trace_cone<SAMPLER, ISO, STORAGE>(m, pos, ld, 0.1f, d).w;
      shadow = fmaxf(0.0f, 1.0f - occ);
    }
    const float lambert = fmaxf(dot(ld, nrm), 0.0f);
    float refract_angle = 0.0f;
    if (mat.dissolve <= 0.1f) {
      const V3 rf = refract(view_dir, nrm, 1.0f / mat.ior);
      refract_angle = fmaxf((1.0f - mat.dissolve) * dot(rf, ld), 0.0f);
    }
    const V3 hv = normalize(ld + view_dir);
    float sa = fmaxf(dot(hv, nrm), 0.0f);
    sa = fmaxf(sa, refract_angle);
    const float sc = powf(sa, mat.shininess);
    const V3 term = mat3v(mat.diffuse) * lambert + mat3v(mat.specular) * sc;
    result = result + mulv(term, lc) * (shadow + 0.04f);
  }
  return result + v3(clamp01(mat.emission[0]), clamp01(mat.emission[1]), clamp01(mat.emission[2]));
}

__device__ __forceinline__ float specular_aperture(float shininess) {  // :220-227
  const float r = sqrtf(2.0f / (shininess + 2.0f));
  const float a = tanf(1.57079f * r);
  return fminf(fmaxf(a, 0.0174533f), 3.14159265f);
}

__device__ __forceinline__ unsigned char unorm8(float v) {
  return (unsigned char)__float2uint_rz(clamp01(v) * 255.0f + 0.5f);
}

// Shades pixel (px, py) of one frame (main, voxel_cone_tracing.frag:246-275).
template <int SAMPLER, bool ISO, int STORAGE, bool SHARE = false>
__device__ __forceinline__ void trace_px(const SceneParams& sp, const CameraParams& cp, const MapSet& m,
                                         const TraceParams& tp, const float4* __restrict__ gb_pos,
                                         const float4* __restrict__ gb_nrm, uchar4* __restrict__ frame,
                                         float4* __restrict__ frame_f32, int px, int py,
                                         const float4* far = nullptr) {
  if (px >= cp.W || py >= cp.H) return;
  const size_t p = (size_t)py * cp.W + px;
  float4 out = f4(0.15f, 0.25f, 0.25f, 1.0f);  // glClearColor, renderer.cpp:398
  const float4 g0 = gb_pos[p], g1 = gb_nrm[p];
  if (__float_as_uint(g1.w) != 0xffffffffu) {
    const V3 world = v3(g0.x, g0.y, g0.z);
    const V3 nrm = v3(g1.x, g1.y, g1.z);
    const vct_material_data& mat = sp.materials[__float_as_uint(g0.w)];
    const V3 pos = v3(world.x / sp.cube_size, world.y / sp.cube_size, world.z / sp.cube_size) * 0.5f +
                   v3(0.5f, 0.5f, 0.5f);
    // within_cube(pos, 0) (:61-64, 250): a fragment outside returns without
    // writing; the pixel keeps the clear colour.
    if (fabsf(pos.x) < 1.0f && fabsf(pos.y) < 1.0f && fabsf(pos.z) < 1.0f) {
      if (tp.view_voxel_dir < 7) {  // voxel debug view, :253-257
        // (map 6: the isotropic chain of VCT_MIP_BOTH; no such map otherwise)
        if (tp.view_voxel_dir >= 0 && (tp.view_voxel_dir <= 5 || (tp.view_voxel_dir == 6 && m.nmaps == 7))) {
          const float lod = fmaxf(tp.view_voxel_lod, 0.0f);
          const V3 one = v3(1.f, 0.f, 0.f);
          const int d = ISO ? 0 : tp.view_voxel_dir;
          out = sample_voxel<SAMPLER, ISO, STORAGE>(m, pos, d, d, d, one, lod);
        } else {
          out = f4(0.f, 0.f, 0.f, 0.f);
        }
      } else {
        const V3 cam = v3(cp.cam_pos[0], cp.cam_pos[1], cp.cam_pos[2]);
        const V3 view_dir = normalize(world - cam);
        V3 fd = v3(0.f, 0.f, 0.f), fdir = v3(0.f, 0.f, 0.f), fs = v3(0.f, 0.f, 0.f);
        if (tp.enable_diffuse) {
          if (tp.diffuse_in) {
            const float4 d = tp.diffuse_in[p];
            fd = mulv(mat3v(mat.diffuse), v3(d.x, d.y, d.z));
          } else if (SHARE && far) {
            fd = mulv(mat3v(mat.diffuse), trace_diffuse_shared<ISO>(m, tp.cone_set, pos, nrm, far));
          } else {
            fd = mulv(mat3v(mat.diffuse), trace_diffuse<SAMPLER, ISO, STORAGE>(m, tp.cone_set, pos, nrm));
          }
        }
        if (tp.enable_direct)
          fdir = direct_light<SAMPLER, ISO, STORAGE>(sp, m, tp.enable_shadow, mat, pos, nrm, view_dir);
        const float sap = specular_aperture(mat.shininess);
        if (tp.enable_specular) {
          const V3 sd = normalize(reflect(-view_dir, nrm));
          const float4 c = trace_cone<SAMPLER, ISO, STORAGE>(m, pos, sd, sap, kMaxDistance);
          fs = mulv(mat3v(mat.specular), v3(c.x, c.y, c.z));
        }
        V3 f = fs + fd + fdir;
        if ((mat.illum == 4 || mat.illum == 6 || mat.illum == 7 || mat.illum == 9) && tp.enable_specular) {
          const V3 rd = refract(view_dir, nrm, 1.0f / mat.ior);
          const float4 c = trace_cone<SAMPLER, ISO, STORAGE>(m, pos, rd, sap, kMaxDistance);
          const V3 tr = mulv(mat3v(mat.transmittance), v3(c.x, c.y, c.z));
          f = tr * (1.0f - mat.dissolve) + f * mat.dissolve;
        }
        out = f4(f.x, f.y, f.z, 1.0f);
      }
    }
  }
  frame[p] = make_uchar4(unorm8(out.x), unorm8(out.y), unorm8(out.z), unorm8(out.w));
  if (frame_f32) frame_f32[p] = out;
}

template <int SAMPLER, bool ISO, int STORAGE>
__global__ void __launch_bounds__(kTraceThreads, SAMPLER == VCT_SAMPLER_HW ? kTraceMinBlocks : 1)
    k_trace(SceneParams sp, CameraParams cp, MapSet m, TraceParams tp, const float4* __restrict__ gb_pos,
            const float4* __restrict__ gb_nrm, uchar4* __restrict__ frame, float4* __restrict__ frame_f32) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  trace_px<SAMPLER, ISO, STORAGE>(
      sp, cp, m, tp, gb_pos, gb_nrm, frame, frame_f32,
      blockIdx.x * 16 + (w % (16 / kTraceWarpW)) * kTraceWarpW + lane % kTraceWarpW,
      blockIdx.y * kTraceRows + (w / (16 / kTraceWarpW)) * (32 / kTraceWarpW) + lane / kTraceWarpW);
}

#ifndef VCT_SHARE_MIN_BLOCKS
#define VCT_SHARE_MIN_BLOCKS 8
#endif
constexpr int kShareMinBlocks = VCT_SHARE_MIN_BLOCKS;

// The pixel of this lane in a 16-pixel-wide CTA tile at (x0, y0) of the
// shared-far-field kernels: a warp is a kShareWarpW x (32 / kShareWarpW)
// block (lane = x + kShareWarpW y), 16 / kShareWarpW blocks per row of
// blocks.  (Measured on the 1080p bench frame, trace ms: 16 x 2 strips
// 1.235, 8 x 4 blocks 1.217, 4 x 8 blocks 1.221; the same frame: the
// groups are the same aligned kShareW x 2 pixels whatever the block.)
#ifndef VCT_SHARE_WARP_W
#define VCT_SHARE_WARP_W 8
#endif
constexpr int kShareWarpW = VCT_SHARE_WARP_W;
static_assert((kShareWarpW == 4 || kShareWarpW == 8 || kShareWarpW == 16) && kShareWarpW % kShareW == 0,
              "a warp block holds whole groups");
__device__ __forceinline__ void share_tile_px(int x0, int y0, int& px, int& py) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  px = x0 + (w % (16 / kShareWarpW)) * kShareWarpW + lane % kShareWarpW;
  py = y0 + (w / (16 / kShareWarpW)) * (32 / kShareWarpW) + lane / kShareWarpW;
}

// One pixel of k_trace_share: the warp (a block of kShareW x 2 groups, its
// rows starting at an even frame row; share_tile_px) first picks each group's
// representative (its first pixel, row by row, whose diffuse cones are
// traced) and the pixels that share with it, marches the groups' far fields
// together (far_fields), then shades its pixels as k_trace does.  Called by
// all 32 lanes of a warp together; fw is the warp's shared-memory block.
template <bool ISO>
__device__ __forceinline__ void trace_px_share(const SceneParams& sp, const CameraParams& cp, const MapSet& m,
                                               const TraceParams& tp, const float4* __restrict__ gb_pos,
                                               const float4* __restrict__ gb_nrm, uchar4* __restrict__ frame,
                                               float4* __restrict__ frame_f32, int px, int py, FarWarp& fw) {
  const int lane = threadIdx.x & 31;
  bool valid = false;
  V3 pos = v3(0.f, 0.f, 0.f), nrm = v3(0.f, 0.f, 1.f);
  if (px < cp.W && py < cp.H) {
    const size_t p = (size_t)py * cp.W + px;
    const float4 g0 = gb_pos[p], g1 = gb_nrm[p];
    if (__float_as_uint(g1.w) != 0xffffffffu) {
      pos = v3(g0.x / sp.cube_size, g0.y / sp.cube_size, g0.z / sp.cube_size) * 0.5f + v3(0.5f, 0.5f, 0.5f);
      nrm = v3(g1.x, g1.y, g1.z);
      // the pixels whose diffuse cones trace_px traces (within_cube, :250)
      valid = fabsf(pos.x) < 1.0f && fabsf(pos.y) < 1.0f && fabsf(pos.z) < 1.0f;
    }
  }
  valid = valid && tp.enable_diffuse && tp.view_voxel_dir >= 7 && !tp.diffuse_in;
  const unsigned vmask = __ballot_sync(0xffffffffu, valid);
  // this lane's group: columns kShareW * gx .., rows 2 gy and 2 gy + 1 of the block
  const int gx = (lane % kShareWarpW) / kShareW, gy = lane / (2 * kShareWarpW);
  const unsigned grow = ((1u << kShareW) - 1u) << (kShareW * gx);
  const unsigned qv = vmask & ((grow << (2 * kShareWarpW * gy)) | (grow << (2 * kShareWarpW * gy + kShareWarpW)));
  const int rep = qv ? __ffs(qv) - 1 : lane;
  const V3 rpos = v3(__shfl_sync(0xffffffffu, pos.x, rep), __shfl_sync(0xffffffffu, pos.y, rep),
                     __shfl_sync(0xffffffffu, pos.z, rep));
  const V3 rn = v3(__shfl_sync(0xffffffffu, nrm.x, rep), __shfl_sync(0xffffffffu, nrm.y, rep),
                   __shfl_sync(0xffffffffu, nrm.z, rep));
  const unsigned repmask = __ballot_sync(0xffffffffu, valid && rep == lane);
  const int slot = __popc(repmask & ((1u << rep) - 1u));
  bool share = false;
  if (valid) {
    const float lim = kShareDist / (float)m.N;
    share = dot(normalize(nrm), normalize(rn)) >= kShareCos && fabsf(pos.x - rpos.x) <= lim &&
            fabsf(pos.y - rpos.y) <= lim && fabsf(pos.z - rpos.z) <= lim;
  }
  if (valid && rep == lane) {
    fw.origin[slot][0] = pos.x;
    fw.origin[slot][1] = pos.y;
    fw.origin[slot][2] = pos.z;
    fw.normal[slot][0] = nrm.x;
    fw.normal[slot][1] = nrm.y;
    fw.normal[slot][2] = nrm.z;
  }
  __syncwarp();
  const int K = tp.cone_set == VCT_CONES_SIX60 ? 6 : 9;
  // the second step of the march schedule (trace_cone's recurrence)
  const float ap = tp.cone_set == VCT_CONES_SIX60 ? 1.15470053838f : kTan22_5;
  const float voxel_size = 1.0f / (float)m.N;
  const float dist0 = 3.0f * voxel_size;
  const float dist1 = dist0 + fmaxf(dist0 * ap * 0.5f, voxel_size);
  if (repmask) far_fields<ISO>(m, fw, tp.cone_set, __popc(repmask), dist1, dist1 * ap);
  __syncwarp();
  trace_px<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8, true>(sp, cp, m, tp, gb_pos, gb_nrm, frame, frame_f32, px, py,
                                                         share ? fw.far + slot * K : nullptr);
  __syncwarp();  // fw is free for the warp's next use
}

// k_trace with shared far fields: a CTA shades a 16 x ROWS tile (8 or 16
// rows: the same warps, 8x4 blocks, so the same frame either way).
template <bool ISO, int ROWS>
__global__ void __launch_bounds__(16 * ROWS, kShareMinBlocks * 8 / ROWS)
    k_trace_share(SceneParams sp, CameraParams cp, MapSet m, TraceParams tp, const float4* __restrict__ gb_pos,
                  const float4* __restrict__ gb_nrm, uchar4* __restrict__ frame, float4* __restrict__ frame_f32) {
  static_assert(ROWS % (32 / kShareWarpW) == 0 && ROWS % 2 == 0, "whole warp blocks");
  __shared__ FarWarp s_far[ROWS / 2];
  int px, py;
  share_tile_px(blockIdx.x * 16, blockIdx.y * ROWS, px, py);
  trace_px_share<ISO>(sp, cp, m, tp, gb_pos, gb_nrm, frame, frame_f32, px, py, s_far[threadIdx.x >> 5]);
}

// One pixel of a batch scene.  Called, not inlined, from the tile loop of
// k_trace_batch: inlined into a loop, the shading's loop-invariant loads
// (scene constants, texture handles) are hoisted out of the loop and held in
// registers across all tiles, which spills the march loop (measured: 4 KB of
// spill code against 0.2 KB for the one-scene kernel).
#ifdef VCT_TRACE_BATCH_INLINE
#define VCT_BATCH_PX_FN __forceinline__
#else
#define VCT_BATCH_PX_FN __noinline__
#endif
// The current scene of a k_trace_batch CTA, read by trace_batch_px at fixed
// shared-memory addresses.
__shared__ BatchScene s_batch_scene;
__shared__ CameraParams s_batch_cam;

template <bool ISO>
__device__ VCT_BATCH_PX_FN void trace_batch_px(const float4* __restrict__ gb_pos, const float4* __restrict__ gb_nrm,
                                            uchar4* __restrict__ frame, int px, int py) {
  trace_px<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8>(s_batch_scene.sp, s_batch_cam, s_batch_scene.ms,
                                                   s_batch_scene.tp, gb_pos, gb_nrm, frame, nullptr, px, py);
}

// trace_px_share on the CTA's current batch scene (k_trace_batch_share);
// called, not inlined, for the same reason as trace_batch_px.
__device__ VCT_BATCH_PX_FN void trace_batch_px_share(const float4* __restrict__ gb_pos,
                                                  const float4* __restrict__ gb_nrm, uchar4* __restrict__ frame,
                                                  int px, int py, FarWarp& fw) {
  trace_px_share<false>(s_batch_scene.sp, s_batch_cam, s_batch_scene.ms, s_batch_scene.tp, gb_pos, gb_nrm, frame,
                        nullptr, px, py, fw);
}

// The 16x16 tiles of every scene of a batch in one persistent launch.  With
// w.queue a CTA takes its next tile from an atomic counter (uneven scenes
// balance across SMs); without, tiles are strided by the grid.  The CTA
// keeps its current scene's descriptor and camera in shared memory, so the
// shading code addresses them at fixed offsets (as kernel parameters are in
// the one-scene kernel) instead of holding pointers in registers.
template <bool ISO>
__global__ void __launch_bounds__(256, kTraceBatchMinBlocks) k_trace_batch(BatchWork w, BatchBuffers bb) {
  __shared__ uint32_t s_next;
  __shared__ int s_cur;
  BatchScene& s_sc = s_batch_scene;
  CameraParams& s_cam = s_batch_cam;
  static_assert(sizeof(BatchScene) % 4 == 0 && sizeof(CameraParams) % 4 == 0, "word copies");
  uint32_t g = blockIdx.x;
  if (threadIdx.x == 0) s_cur = -1;
  if (w.queue) {
    if (threadIdx.x == 0) s_next = atomicAdd(w.queue, 1u);
    __syncthreads();
    g = s_next;
  }
  __syncthreads();
  while (g < w.total) {
    const int s = batch_scene_of(w, g);
    if (s != s_cur) {  // CTA-uniform
      __syncthreads();  // the previous tile is done with the old scene
      const uint32_t* src = reinterpret_cast<const uint32_t*>(w.scenes + s);
      for (int i = threadIdx.x; i < (int)(sizeof(BatchScene) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&s_sc)[i] = __ldg(src + i);
      const uint32_t* csrc = reinterpret_cast<const uint32_t*>(w.cams + s);
      for (int i = threadIdx.x; i < (int)(sizeof(CameraParams) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&s_cam)[i] = __ldg(csrc + i);
      __syncthreads();
      if (threadIdx.x == 0) s_cur = s;
    }
    const uint32_t lt = g - __ldg(w.prefix + s), tiles_x = (uint32_t)(s_sc.W + 15) / 16;
    trace_batch_px<ISO>(bb.rb.gb_pos + s_sc.px_base, bb.rb.gb_nrm + s_sc.px_base, bb.frame + s_sc.px_base,
                        (int)(lt % tiles_x) * 16 + (threadIdx.x & 15), (int)(lt / tiles_x) * 16 + (threadIdx.x >> 4));
    if (w.queue) {
      __syncthreads();  // every thread has read s_next
      if (threadIdx.x == 0) s_next = atomicAdd(w.queue, 1u);
      __syncthreads();
      g = s_next;
    } else {
      g += gridDim.x;
    }
  }
}

// k_trace_batch with shared far fields (the batch's far_share): every 16x16
// tile is eight 8x4 warps, as in k_trace_share, so each scene's frame equals
// a Renderer's with far_share 1.  Anisotropic maps (the batch's).
#ifndef VCT_TRACE_BATCH_SHARE_MIN_BLOCKS
#define VCT_TRACE_BATCH_SHARE_MIN_BLOCKS 4
#endif
constexpr int kTraceBatchShareMinBlocks = VCT_TRACE_BATCH_SHARE_MIN_BLOCKS;
__global__ void __launch_bounds__(256, kTraceBatchShareMinBlocks) k_trace_batch_share(BatchWork w, BatchBuffers bb) {
  __shared__ FarWarp s_far[8];
  __shared__ uint32_t s_next;
  __shared__ int s_cur;
  BatchScene& s_sc = s_batch_scene;
  CameraParams& s_cam = s_batch_cam;
  static_assert(sizeof(BatchScene) % 4 == 0 && sizeof(CameraParams) % 4 == 0, "word copies");
  uint32_t g = blockIdx.x;
  if (threadIdx.x == 0) s_cur = -1;
  if (w.queue) {
    if (threadIdx.x == 0) s_next = atomicAdd(w.queue, 1u);
    __syncthreads();
    g = s_next;
  }
  __syncthreads();
  while (g < w.total) {
    const int s = batch_scene_of(w, g);
    if (s != s_cur) {  // CTA-uniform
      __syncthreads();  // the previous tile is done with the old scene
      const uint32_t* src = reinterpret_cast<const uint32_t*>(w.scenes + s);
      for (int i = threadIdx.x; i < (int)(sizeof(BatchScene) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&s_sc)[i] = __ldg(src + i);
      const uint32_t* csrc = reinterpret_cast<const uint32_t*>(w.cams + s);
      for (int i = threadIdx.x; i < (int)(sizeof(CameraParams) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&s_cam)[i] = __ldg(csrc + i);
      __syncthreads();
      if (threadIdx.x == 0) s_cur = s;
    }
    const uint32_t lt = g - __ldg(w.prefix + s), tiles_x = (uint32_t)(s_sc.W + 15) / 16;
    int px, py;
    share_tile_px((int)(lt % tiles_x) * 16, (int)(lt / tiles_x) * 16, px, py);
    trace_batch_px_share(bb.rb.gb_pos + s_sc.px_base, bb.rb.gb_nrm + s_sc.px_base, bb.frame + s_sc.px_base, px, py,
                         s_far[threadIdx.x >> 5]);
    if (w.queue) {
      __syncthreads();  // every thread has read s_next
      if (threadIdx.x == 0) s_next = atomicAdd(w.queue, 1u);
      __syncthreads();
      g = s_next;
    } else {
      g += gridDim.x;
    }
  }
}

// One CTA per 16x16 tile of every scene of the batch, in one launch
// (BatchShape::trace_ctas_per_sm 0).  Without a tile loop the shading is
// inlined, as in the one-scene kernels, while the scene's descriptor and
// camera come from shared memory: a CTA looks up its scene, copies them
// there and traces its tile.
template <bool SHARE>
__global__ void __launch_bounds__(256, SHARE ? kTraceBatchShareMinBlocks : kTraceBatchMinBlocks)
    k_trace_batch_tiles(BatchWork w, BatchBuffers bb) {
  __shared__ FarWarp s_far[SHARE ? 8 : 1];
  BatchScene& s_sc = s_batch_scene;
  CameraParams& s_cam = s_batch_cam;
  const uint32_t g = blockIdx.x;
  const int s = batch_scene_of_warp(w, g);  // every warp finds it: no barrier before the copy
  const uint32_t* src = reinterpret_cast<const uint32_t*>(w.scenes + s);
  for (int i = threadIdx.x; i < (int)(sizeof(BatchScene) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(&s_sc)[i] = __ldg(src + i);
  const uint32_t* csrc = reinterpret_cast<const uint32_t*>(w.cams + s);
  for (int i = threadIdx.x; i < (int)(sizeof(CameraParams) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(&s_cam)[i] = __ldg(csrc + i);
  __syncthreads();
  const uint32_t lt = g - __ldg(w.prefix + s), tiles_x = (uint32_t)(s_sc.W + 15) / 16;
  int px, py;
  share_tile_px((int)(lt % tiles_x) * 16, (int)(lt / tiles_x) * 16, px, py);
  const float4* gp = bb.rb.gb_pos + s_sc.px_base;
  const float4* gn = bb.rb.gb_nrm + s_sc.px_base;
  uchar4* fr = bb.frame + s_sc.px_base;
  if constexpr (SHARE)
    trace_px_share<false>(s_sc.sp, s_cam, s_sc.ms, s_sc.tp, gp, gn, fr, nullptr, px, py, s_far[threadIdx.x >> 5]);
  else
    trace_px<VCT_SAMPLER_HW, false, VCT_STORAGE_RGBA8>(s_sc.sp, s_cam, s_sc.ms, s_sc.tp, gp, gn, fr, nullptr, px, py);
}

template <int SAMPLER, bool ISO, int STORAGE>
cudaError_t run(const SceneParams& sp, const CameraParams& cp, const MapSet& ms, const TraceParams& tp,
                const float4* gb_pos, const float4* gb_nrm, uchar4* frame, float4* frame_f32, cudaStream_t st) {
  dim3 grid((cp.W + 15) / 16, (cp.H + kTraceRows - 1) / kTraceRows);
  k_trace<SAMPLER, ISO, STORAGE><<<grid, kTraceThreads, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
  return cudaGetLastError();
}

// Training targets of the learned term: trace_diffuse (texture-unit sampler)
// at each sample's texture-space position and normal (rows of 12 floats;
// writes columns 9..11).
template <bool ISO>
__global__ void __launch_bounds__(256) k_trace_points(MapSet m, int cone_set, float* __restrict__ samples, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* q = samples + (size_t)i * 12;
  const V3 pos = v3(q[0], q[1], q[2]), nrm = v3(q[3], q[4], q[5]);
  const V3 d = trace_diffuse<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8>(m, cone_set, pos, nrm);
  q[9] = d.x;
  q[10] = d.y;
  q[11] = d.z;
}

// The judge of the learned diffuse term (launch_judge_diffuse): one pixel
// per stride x stride tile, the same visibility and within_cube test as
// trace_px, the cones of trace_diffuse with the texture unit against the
// network's prediction of them.  A CTA judges 32 pixels with one thread per
// (pixel, cone), so that the few judged pixels still fill the GPU; the
// cones of a pixel are summed in trace_diffuse's order.
constexpr int kJudgePixels = 32;
template <bool ISO>
__global__ void __launch_bounds__(kJudgePixels * 9) k_judge_diffuse(SceneParams sp, MapSet m, TraceParams tp, int W,
                                                                    int H, const float4* __restrict__ gb_pos,
                                                                    const float4* __restrict__ gb_nrm,
                                                                    const float4* __restrict__ net, int stride, int ox,
                                                                    int oy, int tw, int n_judged,
                                                                    FrameStatus* __restrict__ status) {
  __shared__ float4 s_cone[9][kJudgePixels];
  const int j = threadIdx.x % kJudgePixels, k = threadIdx.x / kJudgePixels;
  const int K = tp.cone_set == VCT_CONES_SIX60 ? 6 : 9;
  const int i = blockIdx.x * kJudgePixels + j;
  bool judged = false;
  size_t p = 0;
  if (i < n_judged) {
    const int px = (i % tw) * stride + ox, py = (i / tw) * stride + oy;
    if (px < W && py < H) {
      p = (size_t)py * W + px;
      const float4 g0 = gb_pos[p], g1 = gb_nrm[p];
      if (__float_as_uint(g1.w) != 0xffffffffu) {
        const V3 pos =
            v3(g0.x / sp.cube_size, g0.y / sp.cube_size, g0.z / sp.cube_size) * 0.5f + v3(0.5f, 0.5f, 0.5f);
        judged = fabsf(pos.x) < 1.0f && fabsf(pos.y) < 1.0f && fabsf(pos.z) < 1.0f;
        if (judged && k < K) {
          const V3 n = v3(g1.x, g1.y, g1.z);
          const V3 o1 = normalize(tangent(n));
          const V3 o2 = normalize(cross(o1, n));
          float ap;
          const V3 d = diffuse_dir(tp.cone_set, n, o1, o2, k, ap);
          s_cone[k][j] = trace_cone<VCT_SAMPLER_HW, ISO, VCT_STORAGE_RGBA8>(m, pos, d, ap, kMaxDistance);
        }
      }
    }
  }
  __syncthreads();
  if (k != 0) return;  // one warp sums
  float e = 0.0f;
  uint32_t n = 0;
  if (judged) {
    float4 acc = f4(0.f, 0.f, 0.f, 0.f);
    for (int c = 0; c < K; ++c) acc = acc + s_cone[c][j];
    const V3 d = v3(acc.x, acc.y, acc.z) * (1.0f / (float)K);
    const float4 q = net[p];
    e = (d.x - q.x) * (d.x - q.x) + (d.y - q.y) * (d.y - q.y) + (d.z - q.z) * (d.z - q.z);
    n = 1;
  }
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    n += __shfl_xor_sync(0xffffffffu, n, o);
  }
  if (threadIdx.x == 0 && n) {
    atomicAdd(&status->judge_sse, e);
    atomicAdd(&status->judge_n, n);
  }
}

}  // namespace

cudaError_t launch_judge_diffuse(const SceneParams& sp, const CameraParams& cp, const MapSet& ms, const TraceParams& tp,
                                 const float4* gb_pos, const float4* gb_nrm, const float4* net, int stride, int ox,
                                 int oy, FrameStatus* status, cudaStream_t st) {
  if (stride < 1) return cudaSuccess;
  const int tw = (cp.W - ox + stride - 1) / stride, th = (cp.H - oy + stride - 1) / stride;
  if (tw <= 0 || th <= 0) return cudaSuccess;
  const int n_judged = tw * th;
  const unsigned blocks = (unsigned)((n_judged + kJudgePixels - 1) / kJudgePixels);
  if (tp.mip_mode == VCT_MIP_ISO)
    k_judge_diffuse<true><<<blocks, kJudgePixels * 9, 0, st>>>(sp, ms, tp, cp.W, cp.H, gb_pos, gb_nrm, net, stride, ox,
                                                              oy, tw, n_judged, status);
  else
    k_judge_diffuse<false><<<blocks, kJudgePixels * 9, 0, st>>>(sp, ms, tp, cp.W, cp.H, gb_pos, gb_nrm, net, stride,
                                                               ox, oy, tw, n_judged, status);
  return cudaGetLastError();
}

cudaError_t launch_trace_points(const SceneParams&, const MapSet& ms, int mip_mode, int cone_set, float* samples,
                                int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (mip_mode == VCT_MIP_ISO) k_trace_points<true><<<grid, 256, 0, st>>>(ms, cone_set, samples, n);
  else k_trace_points<false><<<grid, 256, 0, st>>>(ms, cone_set, samples, n);
  return cudaGetLastError();
}

cudaError_t launch_trace_batch(const BatchWork& tiles, const BatchBuffers& bb, const BatchShape& shape, int sms,
                               cudaStream_t st, int* launches, bool share) {
  if (!tiles.total) return cudaSuccess;
  BatchWork w = tiles;
  if (shape.trace_ctas_per_sm == 0) {  // one CTA per tile
    if (share) k_trace_batch_tiles<true><<<tiles.total, 256, 0, st>>>(w, bb);
    else k_trace_batch_tiles<false><<<tiles.total, 256, 0, st>>>(w, bb);
    if (launches) ++*launches;
    return cudaGetLastError();
  }
  if (!shape.trace_dynamic) w.queue = nullptr;
  else {
    cudaError_t e = cudaMemsetAsync(w.queue, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
  }
  if (share) {
    const int per_sm = std::min(std::max(shape.trace_ctas_per_sm, 1), kTraceBatchShareMinBlocks);
    const unsigned grid = (unsigned)std::max(1, std::min<int>(sms * per_sm, (int)tiles.total));
    k_trace_batch_share<<<grid, 256, 0, st>>>(w, bb);
    if (launches) ++*launches;
    return cudaGetLastError();
  }
  const int per_sm = std::min(std::max(shape.trace_ctas_per_sm, 1), kTraceBatchMinBlocks);
  const unsigned grid = (unsigned)std::max(1, std::min<int>(sms * per_sm, (int)tiles.total));
  k_trace_batch<false><<<grid, 256, 0, st>>>(w, bb);
  if (launches) ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_trace(const SceneParams& sp, const CameraParams& cp, const MapSet& ms, const TraceParams& tp,
                         const float4* gb_pos, const float4* gb_nrm, uchar4* frame, float4* frame_f32,
                         cudaStream_t st, int* launches) {
  if (launches) ++*launches;
  const bool iso = tp.mip_mode == VCT_MIP_ISO;
  if (tp.sampler == VCT_SAMPLER_EXACT) {
    if (ms.storage == VCT_STORAGE_RGBA8)
      return iso ? run<VCT_SAMPLER_EXACT, true, VCT_STORAGE_RGBA8>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st)
                 : run<VCT_SAMPLER_EXACT, false, VCT_STORAGE_RGBA8>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st);
    return iso ? run<VCT_SAMPLER_EXACT, true, VCT_STORAGE_RGBA16F>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st)
               : run<VCT_SAMPLER_EXACT, false, VCT_STORAGE_RGBA16F>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st);
  }
  if (tp.far_share && tp.enable_diffuse && !tp.diffuse_in && tp.view_voxel_dir >= 7) {
    // (16 x 16 tiles by default: 5% faster than 16 x 8 on the 1080p bench
    // frame -- the eight warps of a CTA share their SM's texture cache)
    if (tp.tile_rows == 32) {
      dim3 grid((cp.W + 15) / 16, (cp.H + 31) / 32);
      if (iso) k_trace_share<true, 32><<<grid, 512, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
      else k_trace_share<false, 32><<<grid, 512, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
    } else if (tp.tile_rows != 8) {
      dim3 grid((cp.W + 15) / 16, (cp.H + 15) / 16);
      if (iso) k_trace_share<true, 16><<<grid, 256, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
      else k_trace_share<false, 16><<<grid, 256, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
    } else {
      dim3 grid((cp.W + 15) / 16, (cp.H + 7) / 8);
      if (iso) k_trace_share<true, 8><<<grid, 128, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
      else k_trace_share<false, 8><<<grid, 128, 0, st>>>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32);
    }
    return cudaGetLastError();
  }
  return iso ? run<VCT_SAMPLER_HW, true, VCT_STORAGE_RGBA8>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st)
             : run<VCT_SAMPLER_HW, false, VCT_STORAGE_RGBA8>(sp, cp, ms, tp, gb_pos, gb_nrm, frame, frame_f32, st);
}

}  // namespace vct
