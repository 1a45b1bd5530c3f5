// k_raster.cu -- G-buffer production: the forward raster of
// Renderer::visualize (renderer.cpp:355-390) with voxel_cone_tracing.vert
// :22-27, as CUDA kernels.
//
// The reference shades every fragment that passes GL_LESS at its time; the
// final image is the nearest surface (first drawn on equal depth).  Here the
// visible surface is found first and shaded once:
//   k_gb_setup  -- per triangle: world = M*p, clip = (P*V)*world (FP32, fixed
//                  order); triangles crossing the near plane or a guard band
//                  of |x|,|y| <= 16w are clipped (Sutherland-Hodgman) and
//                  fanned; vertices snapped to 1/256 pixel; triangles whose
//                  pixel box holds <= 32 pixels are rasterised right here,
//                  larger ones become records for the tiled pass.
//   k_gb_big_*  -- 16x16-pixel tiles of the large triangles, one pixel per
//                  thread.
//   coverage    -- integer edge functions at pixel centres, top-left rule;
//                  depth = FP32 z_window interpolated in screen space; the
//                  visibility buffer keeps min((depth bits << 32) | triangle
//                  id) via 64-bit atomicMin (ties -> earlier triangle).
//   k_gb_resolve -- per pixel: perspective-correct barycentrics of the
//                  visible triangle -> world position, interpolated world
//                  normal (not renormalised), material id.
#include <algorithm>

#include "vct_internal.h"
#include "vct_math.cuh"

namespace vct {
namespace {

constexpr int kSmallPixels = 32;
constexpr int kTile = 16;
constexpr float kGuard = 16.0f;

struct BigRec {
  long long area;
  int X[3], Y[3];
  float z[3];
  float farea;
  uint32_t tri;
  int tl;
  int x0, y0, x1, y1;  // pixel bbox (inclusive)
  int tw;              // tiles across
  uint32_t scene;      // scene of a batch (0 for one renderer)
};

__device__ __forceinline__ int find_instance(const SceneParams& sp, uint32_t t) {
  int lo = 0, hi = (int)sp.n_instances - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sp.inst[mid].tri_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct CV { float c[4]; };

__device__ __forceinline__ void vertex_clip(const DevInstance& in, const float* PV, uint32_t vi, float w[3], CV& cv,
                                            float4* a_out = nullptr, float4* b_out = nullptr) {
  const float4* vp = reinterpret_cast<const float4*>(in.verts + vi);
  const float4 a = __ldg(vp), b = __ldg(vp + 1);
  for (int r = 0; r < 3; ++r) w[r] = xform_row(in.M, r, a.x, a.y, a.z);
  for (int r = 0; r < 4; ++r) {
    float t = rmul(PV[0 * 4 + r], w[0]);
    t = radd(t, rmul(PV[1 * 4 + r], w[1]));
    t = radd(t, rmul(PV[2 * 4 + r], w[2]));
    cv.c[r] = radd(t, PV[3 * 4 + r]);
  }
  if (a_out) *a_out = a;
  if (b_out) *b_out = b;
}

__device__ __forceinline__ float plane_eval(int pl, const CV& v) {
  switch (pl) {
    case 0: return radd(v.c[2], v.c[3]);
    case 1: return rsub(rmul(kGuard, v.c[3]), v.c[0]);
    case 2: return radd(rmul(kGuard, v.c[3]), v.c[0]);
    case 3: return rsub(rmul(kGuard, v.c[3]), v.c[1]);
    default: return radd(rmul(kGuard, v.c[3]), v.c[1]);
  }
}

__device__ __forceinline__ void plot(unsigned long long* vis, int W, int px, int py, float zz, uint32_t tri) {
  if (!(zz < 1.0f)) return;
  if (!(zz > 0.0f)) zz = 0.0f;
  const unsigned long long key = ((unsigned long long)__float_as_uint(zz) << 32) | tri;
  unsigned long long* slot = vis + (size_t)py * W + px;
  if (key < *reinterpret_cast<volatile unsigned long long*>(slot)) atomicMin(slot, key);
}

__device__ __forceinline__ void pixel_test(const BigRec& r, unsigned long long* vis, int W, int px, int py) {
  const long long sx = 256LL * px + 128, sy = 256LL * py + 128;
  const long long w0 = edge_fn(r.X[1], r.Y[1], r.X[2], r.Y[2], sx, sy);
  const long long w1 = edge_fn(r.X[2], r.Y[2], r.X[0], r.Y[0], sx, sy);
  const long long w2 = edge_fn(r.X[0], r.Y[0], r.X[1], r.Y[1], sx, sy);
  if (!(w0 > 0 || (w0 == 0 && (r.tl & 1)))) return;
  if (!(w1 > 0 || (w1 == 0 && (r.tl & 2)))) return;
  if (!(w2 > 0 || (w2 == 0 && (r.tl & 4)))) return;
  const float b1 = rdiv(__ll2float_rn(w1), r.farea), b2 = rdiv(__ll2float_rn(w2), r.farea);
  float zz = radd(r.z[0], rmul(b1, rsub(r.z[1], r.z[0])));
  zz = radd(zz, rmul(b2, rsub(r.z[2], r.z[0])));
  plot(vis, W, px, py, zz, r.tri);
}

// Set up one (possibly clipped) screen triangle; raster it here if small.
__device__ void raster_subtri(const CV v[3], const CameraParams& cp, uint32_t tri, const RasterBuffers& rb,
                              uint32_t scene) {
  BigRec r;
  long long X[3], Y[3];
  for (int k = 0; k < 3; ++k) {
    if (!(v[k].c[3] > 0.0f)) return;
    const float nx = rdiv(v[k].c[0], v[k].c[3]), ny = rdiv(v[k].c[1], v[k].c[3]), nz = rdiv(v[k].c[2], v[k].c[3]);
    if (!(fabsf(nx) <= 64.0f) || !(fabsf(ny) <= 64.0f) || !(nz == nz)) return;
    X[k] = __double2ll_rn(__dmul_rn(__dadd_rn((double)nx, 1.0), (double)cp.W * 128.0));
    Y[k] = __double2ll_rn(__dmul_rn(__dadd_rn((double)ny, 1.0), (double)cp.H * 128.0));
    r.z[k] = radd(rmul(0.5f, nz), 0.5f);
  }
  long long area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
  if (area == 0) return;
  if (area < 0) {
    long long t = X[1]; X[1] = X[2]; X[2] = t;
    t = Y[1]; Y[1] = Y[2]; Y[2] = t;
    float tz = r.z[1]; r.z[1] = r.z[2]; r.z[2] = tz;
    area = -area;
  }
  const long long x0 = max(0LL, ceil_div(min(X[0], min(X[1], X[2])) - 128, 256));
  const long long x1 = min((long long)cp.W - 1, floor_div(max(X[0], max(X[1], X[2])) - 128, 256));
  const long long y0 = max(0LL, ceil_div(min(Y[0], min(Y[1], Y[2])) - 128, 256));
  const long long y1 = min((long long)cp.H - 1, floor_div(max(Y[0], max(Y[1], Y[2])) - 128, 256));
  if (x1 < x0 || y1 < y0) return;
  r.area = area;
  r.farea = __ll2float_rn(area);
  for (int k = 0; k < 3; ++k) { r.X[k] = (int)X[k]; r.Y[k] = (int)Y[k]; }
  r.tl = (top_left(X[1], Y[1], X[2], Y[2]) ? 1 : 0) | (top_left(X[2], Y[2], X[0], Y[0]) ? 2 : 0) |
         (top_left(X[0], Y[0], X[1], Y[1]) ? 4 : 0);
  r.tri = tri;
  r.x0 = (int)x0; r.x1 = (int)x1; r.y0 = (int)y0; r.y1 = (int)y1;
  const long long npx = (x1 - x0 + 1) * (y1 - y0 + 1);
  if (npx <= kSmallPixels) {
    for (int py = r.y0; py <= r.y1; ++py)
      for (int px = r.x0; px <= r.x1; ++px) pixel_test(r, rb.vis, cp.W, px, py);
    return;
  }
  r.tw = (r.x1 - r.x0 + kTile) / kTile;
  r.scene = scene;
  const uint32_t slot = atomicAdd(&rb.big_count[0], 1u);
  if (slot < rb.big_cap) reinterpret_cast<BigRec*>(rb.big)[slot] = r;
}

__device__ __forceinline__ void setup_tri(const SceneParams& sp, const CameraParams& cp, const RasterBuffers& rb,
                                          uint32_t t, uint32_t scene) {
  if (t >= sp.total_tris) return;
  const DevInstance& in = sp.inst[find_instance(sp, t)];
  const uint32_t lt = t - in.tri_base;
  CV cv[3];
  float w[3];
  for (int k = 0; k < 3; ++k) vertex_clip(in, cp.PV, __ldg(in.indices + 3 * (size_t)lt + k), w, cv[k]);
  bool all_in = true;
  for (int pl = 0; pl < 5; ++pl)
    for (int k = 0; k < 3; ++k)
      if (!(plane_eval(pl, cv[k]) >= 0.0f)) all_in = false;
  if (all_in) {
    raster_subtri(cv, cp, t, rb, scene);
    return;
  }
  CV a[10], b[10];
  int n = 3;
  for (int k = 0; k < 3; ++k) a[k] = cv[k];
  for (int pl = 0; pl < 5; ++pl) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
      const CV p0 = a[i], p1 = a[(i + 1) % n];
      const float d0 = plane_eval(pl, p0), d1 = plane_eval(pl, p1);
      const bool in0 = d0 >= 0.0f, in1 = d1 >= 0.0f;
      if (in0) b[m++] = p0;
      if (in0 != in1) {
        const float tt = rdiv(d0, rsub(d0, d1));
        CV q;
        for (int c = 0; c < 4; ++c) q.c[c] = radd(p0.c[c], rmul(tt, rsub(p1.c[c], p0.c[c])));
        b[m++] = q;
      }
    }
    n = m;
    for (int i = 0; i < n; ++i) a[i] = b[i];
    if (n < 3) return;
  }
  for (int k = 1; k + 1 < n; ++k) {
    const CV tri3[3] = {a[0], a[k], a[k + 1]};
    raster_subtri(tri3, cp, t, rb, scene);
  }
}

__global__ void __launch_bounds__(256) k_gb_setup(SceneParams sp, CameraParams cp, RasterBuffers rb) {
  setup_tri(sp, cp, rb, blockIdx.x * blockDim.x + threadIdx.x, 0u);
}

// The pixel slice of one batch scene in the batch-wide raster buffers.
__device__ __forceinline__ RasterBuffers scene_rb(const RasterBuffers& rb, const BatchScene& S) {
  RasterBuffers r = rb;
  r.vis = rb.vis + S.px_base;
  r.gb_pos = rb.gb_pos + S.px_base;
  r.gb_nrm = rb.gb_nrm + S.px_base;
  return r;
}

__global__ void __launch_bounds__(256) k_gb_setup_batch(BatchWork w, RasterBuffers rb) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < w.total; g += gridDim.x * blockDim.x) {
    const int s = batch_scene_of(w, g);
    const BatchScene& S = w.scenes[s];
    setup_tri(S.sp, w.cams[s], scene_rb(rb, S), g - __ldg(w.prefix + s), (uint32_t)s);
  }
}

// Tile counts of the large-triangle records -> exclusive prefix (one CTA).
__global__ void __launch_bounds__(1024) k_gb_big_scan(RasterBuffers rb) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t s_carry;
  const uint32_t n = min(rb.big_count[0], rb.big_cap);
  const BigRec* rec = reinterpret_cast<const BigRec*>(rb.big);
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t base = 0; base < n; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    uint32_t v = 0;
    if (i < n) v = (uint32_t)rec[i].tw * (uint32_t)((rec[i].y1 - rec[i].y0 + kTile) / kTile);
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t wv = warp_tot[lane], wi = wv;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += t;
      }
      warp_tot[lane] = wi - wv;
    }
    __syncthreads();
    const uint32_t carry = s_carry;
    if (i < n) rb.big_offset[i] = carry + warp_tot[warp] + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = carry + warp_tot[warp] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    rb.big_offset[n] = s_carry;
    rb.big_count[1] = s_carry;
    rb.status->big_total = rb.big_count[0];
    rb.status->big_tiles = s_carry;
  }
}

__global__ void __launch_bounds__(kTile * kTile) k_gb_big(RasterBuffers rb, int W, const BatchScene* scenes) {
  const uint32_t n = min(rb.big_count[0], rb.big_cap);
  const uint32_t total = rb.big_count[1];
  const BigRec* rec = reinterpret_cast<const BigRec*>(rb.big);
  for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
    int lo = 0, hi = (int)n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (rb.big_offset[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const BigRec& r = rec[lo];
    const uint32_t lt = t - rb.big_offset[lo];
    const int tx = (int)(lt % (uint32_t)r.tw), ty = (int)(lt / (uint32_t)r.tw);
    const int px = r.x0 + tx * kTile + (threadIdx.x % kTile), py = r.y0 + ty * kTile + (threadIdx.x / kTile);
    unsigned long long* vis = rb.vis;
    int w = W;
    if (scenes) {  // a batch: the record's scene
      vis += scenes[r.scene].px_base;
      w = scenes[r.scene].W;
    }
    if (px <= r.x1 && py <= r.y1) pixel_test(r, vis, w, px, py);
  }
}

__device__ __forceinline__ void resolve_px(const SceneParams& sp, const CameraParams& cp, const RasterBuffers& rb,
                                           int px, int py) {
  if (px >= cp.W || py >= cp.H) return;
  const size_t p = (size_t)py * cp.W + px;
  const unsigned long long key = rb.vis[p];
  if (key == ~0ull) {
    rb.gb_pos[p] = make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
    rb.gb_nrm[p] = make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
    return;
  }
  const uint32_t t = (uint32_t)(key & 0xffffffffull);
  const DevInstance& in = sp.inst[find_instance(sp, t)];
  const uint32_t lt = t - in.tri_base;
  CV cv[3];
  V3 wp[3], nn[3];
  for (int k = 0; k < 3; ++k) {
    float w[3];
    float4 a, b;
    vertex_clip(in, cp.PV, __ldg(in.indices + 3 * (size_t)lt + k), w, cv[k], &a, &b);
    wp[k] = v3(w[0], w[1], w[2]);
    nn[k] = normalize(nm_mul(in.NM, a.w, b.x, b.y));
  }
  // Perspective-correct barycentrics: sum b_k (x_k - px w_k) = 0, sum b_k
  // (y_k - py w_k) = 0, sum b_k = 1 (GL smooth interpolation).
  const float pxn = ((float)px + 0.5f) * 2.0f / (float)cp.W - 1.0f;
  const float pyn = ((float)py + 0.5f) * 2.0f / (float)cp.H - 1.0f;
  float u[3], v[3];
  for (int k = 0; k < 3; ++k) {
    u[k] = cv[k].c[0] - pxn * cv[k].c[3];
    v[k] = cv[k].c[1] - pyn * cv[k].c[3];
  }
  float b0 = u[1] * v[2] - u[2] * v[1], b1 = u[2] * v[0] - u[0] * v[2], b2 = u[0] * v[1] - u[1] * v[0];
  const float sb = b0 + b1 + b2;
  if (sb != 0.0f) {
    const float inv = 1.0f / sb;
    b0 *= inv; b1 *= inv; b2 *= inv;
  } else {
    b0 = b1 = b2 = 1.0f / 3.0f;
  }
  const V3 world = wp[0] * b0 + wp[1] * b1 + wp[2] * b2;
  const V3 nrm = nn[0] * b0 + nn[1] * b1 + nn[2] * b2;
  const uint32_t mat = __ldg(sp.obj_material + __ldg(in.tri_obj + lt));
  rb.gb_pos[p] = make_float4(world.x, world.y, world.z, __uint_as_float(mat));
  rb.gb_nrm[p] = make_float4(nrm.x, nrm.y, nrm.z, __uint_as_float(t));
}

__global__ void __launch_bounds__(256) k_gb_resolve(SceneParams sp, CameraParams cp, RasterBuffers rb) {
  resolve_px(sp, cp, rb, blockIdx.x * 16 + (threadIdx.x & 15), blockIdx.y * 16 + (threadIdx.x >> 4));
}

// 16x16-pixel tiles of every batch scene.
__global__ void __launch_bounds__(256) k_gb_resolve_batch(BatchWork w, RasterBuffers rb) {
  for (uint32_t g = blockIdx.x; g < w.total; g += gridDim.x) {
    const int s = batch_scene_of(w, g);
    const BatchScene& S = w.scenes[s];
    const uint32_t lt = g - __ldg(w.prefix + s), tiles_x = (uint32_t)(S.W + 15) / 16;
    resolve_px(S.sp, w.cams[s], scene_rb(rb, S), (int)(lt % tiles_x) * 16 + (threadIdx.x & 15),
               (int)(lt / tiles_x) * 16 + (threadIdx.x >> 4));
  }
}

}  // namespace

size_t big_record_bytes() { return sizeof(BigRec); }

cudaError_t launch_gbuffer(const SceneParams& sp, const CameraParams& cp, const RasterBuffers& rb, cudaStream_t st,
                           int* launches) {
  cudaError_t e = cudaMemsetAsync(rb.vis, 0xff, (size_t)cp.W * cp.H * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(rb.big_count, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (sp.total_tris) k_gb_setup<<<(sp.total_tris + 255) / 256, 256, 0, st>>>(sp, cp, rb);
  k_gb_big_scan<<<1, 1024, 0, st>>>(rb);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_gb_big<<<sms * 8, kTile * kTile, 0, st>>>(rb, cp.W, nullptr);
  dim3 grid((cp.W + 15) / 16, (cp.H + 15) / 16);
  k_gb_resolve<<<grid, 256, 0, st>>>(sp, cp, rb);
  if (launches) *launches += (sp.total_tris ? 1 : 0) + 3;
  return cudaGetLastError();
}

cudaError_t launch_gbuffer_batch(const BatchWork& tris, const BatchWork& tiles, size_t total_px,
                                 const BatchBuffers& bb, int sms, cudaStream_t st, int* launches) {
  const RasterBuffers& rb = bb.rb;
  cudaError_t e = cudaMemsetAsync(rb.vis, 0xff, total_px * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(rb.big_count, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  int nl = 0;
  if (tris.total) {
    const unsigned grid = (unsigned)std::max(1, std::min<int>(sms * 4, (int)((tris.total + 255) / 256)));
    k_gb_setup_batch<<<grid, 256, 0, st>>>(tris, rb);
    ++nl;
  }
  k_gb_big_scan<<<1, 1024, 0, st>>>(rb);
  k_gb_big<<<sms * 8, kTile * kTile, 0, st>>>(rb, 0, tris.scenes);
  const unsigned rgrid = (unsigned)std::max(1, std::min<int>(sms * 8, (int)tiles.total));
  k_gb_resolve_batch<<<rgrid, 256, 0, st>>>(tiles, rb);
  nl += 3;
  if (launches) *launches += nl;
  return cudaGetLastError();
}

}  // namespace vct
