// vct_oracle.cpp -- CPU oracle (test infrastructure only) for the
// voxelize -> mipmap -> cone-trace path of latencyhiding/voxel_cone_tracing.
//
// Parity unpinned: the reference has no tests or golden vectors and cannot be
// built or run here (OpenGL 4.5 + GLSL).  Every function below restates one
// piece of the reference and cites it.  Where the reference leaves a result to
// the GL implementation (raster coverage, fill rule, attribute interpolation,
// unorm rounding) the rule is fixed here and the CUDA kernels implement the
// same rule, so voxel occupancy, contribution counts, mip texels and visible
// triangle ids are compared bit-exactly:
//   * vertex transforms and the few interpolations that decide coverage run
//     in FP32 with one IEEE rounding per operation in a fixed order (this
//     file is compiled with -ffp-contract=off);
//   * coverage itself is decided on integer (fixed-point) coordinates with
//     exact integer edge functions / separating-axis tests;
//   * the anisotropic mip is evaluated in exact integer arithmetic.
// Shading values (voxel colours, cone-traced radiance) are computed in FP64
// (Real = double) and compared with a tolerance.  The Real = float
// instantiation is the timed CPU restatement.
//
// Built with:  g++ -O3 -std=c++17 -fPIC -shared -pthread -ffp-contract=off
#include "vct_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

typedef long long i64;
typedef __int128 i128;

// ---------------------------------------------------------------- helpers --
template <class R> struct V3 {
  R x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> static inline V3<R> operator+(V3<R> a, V3<R> b) { return V3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> static inline V3<R> operator-(V3<R> a, V3<R> b) { return V3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> static inline V3<R> operator-(V3<R> a) { return V3<R>(-a.x, -a.y, -a.z); }
template <class R> static inline V3<R> operator*(V3<R> a, R s) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> static inline V3<R> operator*(R s, V3<R> a) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> static inline V3<R> mulv(V3<R> a, V3<R> b) { return V3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> static inline V3<R> cross(V3<R> a, V3<R> b) {
  return V3<R>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <class R> static inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
// normalize(0) is undefined in GLSL; both this oracle and the kernels return 0.
template <class R> static inline V3<R> normalize(V3<R> a) {
  R l2 = dot(a, a);
  if (!(l2 > R(0))) return V3<R>();
  return a * (R(1) / std::sqrt(l2));
}
template <class R> static inline V3<R> vabs(V3<R> a) { return V3<R>(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
template <class R> static inline R clamp01(R v) { return v < R(0) ? R(0) : (v > R(1) ? R(1) : v); }
template <class R> static inline R fmaxr(R a, R b) { return a > b ? a : (b == b ? b : a); }

template <class R> struct V4 {
  R r, g, b, a;
  V4() : r(0), g(0), b(0), a(0) {}
  V4(R x, R y, R z, R w) : r(x), g(y), b(z), a(w) {}
};
template <class R> static inline V4<R> operator+(V4<R> p, V4<R> q) { return V4<R>(p.r + q.r, p.g + q.g, p.b + q.b, p.a + q.a); }
template <class R> static inline V4<R> operator*(V4<R> p, R s) { return V4<R>(p.r * s, p.g * s, p.b * s, p.a * s); }

static inline i64 floor_div(i64 a, i64 b) { i64 q = a / b; if ((a % b != 0) && ((a < 0) != (b < 0))) --q; return q; }
static inline i64 ceil_div(i64 a, i64 b) { return -floor_div(-a, b); }

template <class F> static void parallel_for(int threads, int n, F f) {
  if (threads <= 1 || n <= 1) { for (int i = 0; i < n; ++i) f(i); return; }
  std::atomic<int> next(0);
  std::vector<std::thread> pool;
  int t = std::min(threads, n);
  for (int k = 0; k < t; ++k)
    pool.emplace_back([&]() { for (;;) { int i = next.fetch_add(1); if (i >= n) break; f(i); } });
  for (auto& th : pool) th.join();
}

// ------------------------------------------------- FP32 fixed-order maths --
// These decide coverage, so the CUDA kernels evaluate exactly the same
// sequence of IEEE-rounded FP32 operations.

// (M * vec4(p, 1)).xyz, column-major, terms summed in column order.
static inline void xform_f32(const float* m, const float* p, float* o) {
  for (int r = 0; r < 3; ++r) {
    float t = m[0 * 4 + r] * p[0];
    t = t + m[1 * 4 + r] * p[1];
    t = t + m[2 * 4 + r] * p[2];
    o[r] = t + m[3 * 4 + r];
  }
}
// PV = P * V in FP32 (GLSL `projection * view`).
static inline void matmul_f32(const float* P, const float* V, float* o) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      float t = P[0 * 4 + r] * V[c * 4 + 0];
      t = t + P[1 * 4 + r] * V[c * 4 + 1];
      t = t + P[2 * 4 + r] * V[c * 4 + 2];
      o[c * 4 + r] = t + P[3 * 4 + r] * V[c * 4 + 3];
    }
}
static inline void clip_f32(const float* PV, const float* w, float* o) {
  for (int r = 0; r < 4; ++r) {
    float t = PV[0 * 4 + r] * w[0];
    t = t + PV[1 * 4 + r] * w[1];
    t = t + PV[2 * 4 + r] * w[2];
    o[r] = t + PV[3 * 4 + r];
  }
}

// mat3(transpose(inverse(M))) in double (voxelize.vert:28,
// voxel_cone_tracing.vert:26); nm[r*3+c] is row r, column c.
static void normal_matrix(const float* mf, double* nm) {
  double m[16], inv[16];
  for (int i = 0; i < 16; ++i) m[i] = mf[i];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  double id = det != 0.0 ? 1.0 / det : 0.0;
  // inverse element (row i, col j) = inv[j*4+i] * id; transpose -> (row r,
  // col c) = inverse(row c, col r) = inv[r*4+c].
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) nm[r * 3 + c] = inv[r * 4 + c] * id;
}

template <class R> static inline V3<R> mat3_mul(const double* nm, const float* n) {
  return V3<R>(R(nm[0] * n[0] + nm[1] * n[1] + nm[2] * n[2]),
               R(nm[3] * n[0] + nm[4] * n[1] + nm[5] * n[2]),
               R(nm[6] * n[0] + nm[7] * n[1] + nm[8] * n[2]));
}

template <class R> static inline V3<R> mat_of(const orc_material& m, int which) {
  const float* f = which == 0 ? m.diffuse : which == 1 ? m.specular : which == 2 ? m.transmittance : m.emission;
  return V3<R>(R(f[0]), R(f[1]), R(f[2]));
}
static inline bool illum_transparent(int illum) { return illum == 4 || illum == 6 || illum == 7 || illum == 9; }

// --------------------------------------------------------- voxelize.frag --
// Upper clamp of the voxel colour: 1 in the reference (voxelize.frag:153);
// orc_params.radiance_max for HDR storage.  Set by voxelize_impl before its
// worker threads start (the oracle runs one call at a time).
static double g_radiance_max = 1.0;
// What a contribution carries: 0 the shaded colour; for light injection 1
// albedo x transmittance + alpha, 2 the normal as 0.5 n + 0.5, 3 emission x
// transmittance + 1 (occupancy).  Set before voxelize_impl's threads start.
static int g_attr_mode = 0;

// Per-fragment colour, voxelize.frag:124-153.  pos is in grid space
// ([-1,1]^3 = world / cube_size), nrm the interpolated vertex normal.
template <class R>
static V4<R> voxel_fragment_color(const orc_scene* s, const orc_material& mat, V3<R> pos, V3<R> nrm) {
  V3<R> color;
  int nl = std::min<int>((int)s->n_lights, 10);  // MAX_POINT_LIGHTS, voxelize.frag:40,128
  R cube = R(s->cube_size);
  V3<R> nn = normalize(nrm);
  for (int i = 0; i < nl; ++i) {
    const orc_point_light& L = s->lights[i];
    V3<R> lp(R(L.position[0]) / cube, R(L.position[1]) / cube, R(L.position[2]) / cube);
    V3<R> dir = normalize(lp - pos);
    R d = length(lp - pos);
    R a = R(1) / (R(1) + R(0) * d + R(1) * d * d);  // attenuate(1,0,1,d), voxelize.frag:56-59,134
    R cs = fmaxr(dot(nn, dir), R(0));
    V3<R> lc(R(L.color[0]), R(L.color[1]), R(L.color[2]));
    color = color + lc * (cs * a * R(L.intensity));
  }
  color = mulv(mat_of<R>(mat, 0), color) + mat_of<R>(mat, 3);  // voxelize.frag:142-143
  V3<R> trans(R(1), R(1), R(1));
  R alpha = R(1);
  if (illum_transparent(mat.illum)) { trans = mat_of<R>(mat, 2); alpha = R(mat.dissolve); }  // voxelize.frag:145-151
  if (g_attr_mode) {
    const V3<R> t = illum_transparent(mat.illum) ? mat_of<R>(mat, 2) : V3<R>(R(1), R(1), R(1));
    if (g_attr_mode == 1) {
      const V3<R> a = mulv(mat_of<R>(mat, 0), t);
      return V4<R>(clamp01(a.x), clamp01(a.y), clamp01(a.z), clamp01(alpha));
    }
    if (g_attr_mode == 2)
      return V4<R>(clamp01(R(0.5) * nn.x + R(0.5)), clamp01(R(0.5) * nn.y + R(0.5)), clamp01(R(0.5) * nn.z + R(0.5)),
                   R(0));
    const V3<R> e = mulv(mat_of<R>(mat, 3), t);
    return V4<R>(clamp01(e.x), clamp01(e.y), clamp01(e.z), R(1));
  }
  V3<R> c = mulv(trans, color);
  const R hi = R(g_radiance_max);
  auto cl = [hi](R v) { return v < R(0) ? R(0) : (v > hi ? hi : v); };
  return V4<R>(cl(c.x), cl(c.y), cl(c.z), clamp01(alpha));  // voxelize.frag:153
}

// One voxel contribution: voxel index + clamped colour.
template <class R> struct Contrib { uint32_t voxel; R c[4]; };

struct TriVerts {
  float g[3][3];    // grid-space positions, FP32 (voxelize.vert:26)
  double nm[9];
};

// Edge function E(a->b, s) = (b - a) x (s - a) on integer coordinates.
static inline i64 edge_fn(i64 ax, i64 ay, i64 bx, i64 by, i64 sx, i64 sy) {
  return (bx - ax) * (sy - ay) - (by - ay) * (sx - ax);
}
// Fill rule for samples exactly on an edge (counter-clockwise triangles,
// y up): keep left edges (going down) and top edges (horizontal, going -x).
static inline bool top_left(i64 ax, i64 ay, i64 bx, i64 by) {
  i64 dy = by - ay, dx = bx - ax;
  return dy < 0 || (dy == 0 && dx < 0);
}
static inline bool edge_in(i64 e, bool tl) { return e > 0 || (e == 0 && tl); }

// Dominant axis of voxelize.geom:27-51: 2 -> project to (x,y), 0 -> (y,z),
// 1 -> (x,z).  Strict comparisons: ties fall through to the y projection.
static inline int dominant_axis(const float v[3][3]) {
  float e1[3], e2[3];
  for (int i = 0; i < 3; ++i) { e1[i] = v[1][i] - v[0][i]; e2[i] = v[2][i] - v[0][i]; }
  float cx = e1[1] * e2[2] - e2[1] * e1[2];
  float cy = e1[2] * e2[0] - e2[2] * e1[0];
  float cz = e1[0] * e2[1] - e2[0] * e1[1];
  float px = std::fabs(cx), py = std::fabs(cy), pz = std::fabs(cz);
  if (pz > px && pz > py) return 2;
  if (px > py && px > pz) return 0;
  return 1;
}

static inline bool coord_ok(float v) { return std::fabs(v) <= 64.0f; }  // also false for NaN

// ---- reference-raster coverage (renderer.cpp:339-347 + voxelize.geom/.frag)
// The 2N x 2N viewport puts 2x2 samples over every voxel column of the
// dominant projection.  A sample (i, j) sits at window (i + 0.5, j + 0.5);
// vertices are snapped to 1/256 of a sample pixel; the sample's depth is the
// FP32 barycentric interpolation of the vertex depths and its voxel is
// int(N * (0.5*c + 0.5)) (truncation, voxelize.frag:156-157).
template <class R>
static bool raster_tri_ref(const orc_scene* s, int N, const TriVerts& tv, const float* nrm_obj[3],
                           const orc_material& mat, std::vector<Contrib<R>>& out) {
  const int axis = dominant_axis(tv.g);
  const int ia = axis == 2 ? 0 : (axis == 0 ? 1 : 0);
  const int ib = axis == 2 ? 1 : 2;
  const int ic = axis;  // depth axis
  float a[3], b[3], c[3];
  int idx[3] = {0, 1, 2};
  for (int k = 0; k < 3; ++k) {
    a[k] = tv.g[k][ia]; b[k] = tv.g[k][ib]; c[k] = tv.g[k][ic];
    if (!coord_ok(tv.g[k][0]) || !coord_ok(tv.g[k][1]) || !coord_ok(tv.g[k][2])) return false;
  }
  const double scale = (double)N * 256.0;
  i64 A[3], B[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = std::llrint(((double)a[k] + 1.0) * scale);
    B[k] = std::llrint(((double)b[k] + 1.0) * scale);
  }
  i64 area = (A[1] - A[0]) * (B[2] - B[0]) - (B[1] - B[0]) * (A[2] - A[0]);
  if (area == 0) return true;
  if (area < 0) {
    std::swap(A[1], A[2]); std::swap(B[1], B[2]); std::swap(c[1], c[2]); std::swap(idx[1], idx[2]);
    area = -area;
  }
  const bool tl0 = top_left(A[1], B[1], A[2], B[2]);
  const bool tl1 = top_left(A[2], B[2], A[0], B[0]);
  const bool tl2 = top_left(A[0], B[0], A[1], B[1]);
  i64 minA = std::min({A[0], A[1], A[2]}), maxA = std::max({A[0], A[1], A[2]});
  i64 minB = std::min({B[0], B[1], B[2]}), maxB = std::max({B[0], B[1], B[2]});
  i64 i0 = std::max<i64>(0, ceil_div(minA - 128, 256)), i1 = std::min<i64>(2 * N - 1, floor_div(maxA - 128, 256));
  i64 j0 = std::max<i64>(0, ceil_div(minB - 128, 256)), j1 = std::min<i64>(2 * N - 1, floor_div(maxB - 128, 256));
  const float farea = (float)area;
  const float Nf = (float)N;
  V3<R> gp[3], gn[3];
  for (int k = 0; k < 3; ++k) {
    int o = idx[k];
    gp[k] = V3<R>(R(tv.g[o][0]), R(tv.g[o][1]), R(tv.g[o][2]));
    gn[k] = normalize(mat3_mul<R>(tv.nm, nrm_obj[o]));  // voxelize.vert:28
  }
  for (i64 j = j0; j <= j1; ++j) {
    const i64 sy = 256 * j + 128;
    for (i64 i = i0; i <= i1; ++i) {
      const i64 sx = 256 * i + 128;
      i64 w0 = edge_fn(A[1], B[1], A[2], B[2], sx, sy);
      i64 w1 = edge_fn(A[2], B[2], A[0], B[0], sx, sy);
      i64 w2 = edge_fn(A[0], B[0], A[1], B[1], sx, sy);
      if (!edge_in(w0, tl0) || !edge_in(w1, tl1) || !edge_in(w2, tl2)) continue;
      float b1 = (float)w1 / farea, b2 = (float)w2 / farea;
      float cz = c[0] + b1 * (c[1] - c[0]);
      cz = cz + b2 * (c[2] - c[0]);
      float t = Nf * (0.5f * cz + 0.5f);
      if (!(t > -1.0f && t < Nf)) continue;
      int kd = (int)t;
      int vi = (int)(i >> 1), vj = (int)(j >> 1);
      int vx, vy, vz;
      if (axis == 2) { vx = vi; vy = vj; vz = kd; }
      else if (axis == 0) { vx = kd; vy = vi; vz = vj; }
      else { vx = vi; vy = kd; vz = vj; }
      R l0 = R(w0) / R(area), l1 = R(w1) / R(area), l2 = R(w2) / R(area);
      V3<R> p = gp[0] * l0 + gp[1] * l1 + gp[2] * l2;
      V3<R> n = gn[0] * l0 + gn[1] * l1 + gn[2] * l2;
      V4<R> col = voxel_fragment_color<R>(s, mat, p, n);
      Contrib<R> ct;
      ct.voxel = (uint32_t)(((i64)vz * N + vy) * N + vx);
      ct.c[0] = col.r; ct.c[1] = col.g; ct.c[2] = col.b; ct.c[3] = col.a;
      out.push_back(ct);
    }
  }
  return true;
}

// ---- conservative coverage: exact triangle/box separating-axis test on
// vertices snapped to 1/256 voxel (box normals, triangle plane, 9 edge
// cross products; closed boxes, so touching counts as overlap).
struct I3 { i64 v[3]; };

static bool sat_overlap(const I3 V[3], const i64 c[3], i64 h) {
  i64 u[3][3];
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) u[k][d] = V[k].v[d] - c[d];
  for (int d = 0; d < 3; ++d) {
    i64 mn = std::min({u[0][d], u[1][d], u[2][d]}), mx = std::max({u[0][d], u[1][d], u[2][d]});
    if (mn > h || mx < -h) return false;
  }
  i64 f[3][3];
  for (int d = 0; d < 3; ++d) {
    f[0][d] = u[1][d] - u[0][d]; f[1][d] = u[2][d] - u[1][d]; f[2][d] = u[0][d] - u[2][d];
  }
  i64 n[3] = {f[0][1] * f[1][2] - f[0][2] * f[1][1], f[0][2] * f[1][0] - f[0][0] * f[1][2],
              f[0][0] * f[1][1] - f[0][1] * f[1][0]};
  i128 dd = (i128)n[0] * u[0][0] + (i128)n[1] * u[0][1] + (i128)n[2] * u[0][2];
  i128 rr = (i128)h * ((i128)std::llabs(n[0]) + std::llabs(n[1]) + std::llabs(n[2]));
  if (dd > rr || dd < -rr) return false;
  for (int e = 0; e < 3; ++e) {
    const i64 fx = f[e][0], fy = f[e][1], fz = f[e][2];
    // axis X x f = (0, -fz, fy)
    {
      i64 p0 = -fz * u[0][1] + fy * u[0][2], p1 = -fz * u[1][1] + fy * u[1][2], p2 = -fz * u[2][1] + fy * u[2][2];
      i64 r = h * (std::llabs(fz) + std::llabs(fy));
      if (std::min({p0, p1, p2}) > r || std::max({p0, p1, p2}) < -r) return false;
    }
    // axis Y x f = (fz, 0, -fx)
    {
      i64 p0 = fz * u[0][0] - fx * u[0][2], p1 = fz * u[1][0] - fx * u[1][2], p2 = fz * u[2][0] - fx * u[2][2];
      i64 r = h * (std::llabs(fz) + std::llabs(fx));
      if (std::min({p0, p1, p2}) > r || std::max({p0, p1, p2}) < -r) return false;
    }
    // axis Z x f = (-fy, fx, 0)
    {
      i64 p0 = -fy * u[0][0] + fx * u[0][1], p1 = -fy * u[1][0] + fx * u[1][1], p2 = -fy * u[2][0] + fx * u[2][1];
      i64 r = h * (std::llabs(fy) + std::llabs(fx));
      if (std::min({p0, p1, p2}) > r || std::max({p0, p1, p2}) < -r) return false;
    }
  }
  return true;
}

// Closest point on triangle (a,b,c) to p, returned as barycentric weights
// (region classification of the Voronoi regions of the vertices, edges and
// face; e.g. Ericson, Real-Time Collision Detection, sec. 5.1.5).
template <class R> static void closest_bary(V3<R> p, V3<R> a, V3<R> b, V3<R> c, R w[3]) {
  V3<R> ab = b - a, ac = c - a, ap = p - a;
  R d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= R(0) && d2 <= R(0)) { w[0] = 1; w[1] = 0; w[2] = 0; return; }
  V3<R> bp = p - b;
  R d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= R(0) && d4 <= d3) { w[0] = 0; w[1] = 1; w[2] = 0; return; }
  R vc = d1 * d4 - d3 * d2;
  if (vc <= R(0) && d1 >= R(0) && d3 <= R(0)) {
    R den = d1 - d3; R v = den != R(0) ? d1 / den : R(0);
    w[0] = R(1) - v; w[1] = v; w[2] = 0; return;
  }
  V3<R> cp = p - c;
  R d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= R(0) && d5 <= d6) { w[0] = 0; w[1] = 0; w[2] = 1; return; }
  R vb = d5 * d2 - d1 * d6;
  if (vb <= R(0) && d2 >= R(0) && d6 <= R(0)) {
    R den = d2 - d6; R t = den != R(0) ? d2 / den : R(0);
    w[0] = R(1) - t; w[1] = 0; w[2] = t; return;
  }
  R va = d3 * d6 - d5 * d4;
  if (va <= R(0) && (d4 - d3) >= R(0) && (d5 - d6) >= R(0)) {
    R den = (d4 - d3) + (d5 - d6); R t = den != R(0) ? (d4 - d3) / den : R(0);
    w[0] = 0; w[1] = R(1) - t; w[2] = t; return;
  }
  R sum = va + vb + vc;
  if (!(sum != R(0))) { w[0] = 1; w[1] = 0; w[2] = 0; return; }
  R v = vb / sum, t = vc / sum;
  w[0] = R(1) - v - t; w[1] = v; w[2] = t;
}

template <class R>
static bool sat_tri(const orc_scene* s, int N, const TriVerts& tv, const float* nrm_obj[3],
                    const orc_material& mat, std::vector<Contrib<R>>& out) {
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d)
      if (!coord_ok(tv.g[k][d])) return false;
  const double scale = (double)N * 128.0;
  I3 V[3];
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) V[k].v[d] = std::llrint(((double)tv.g[k][d] + 1.0) * scale);
  i64 lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    i64 mn = std::min({V[0].v[d], V[1].v[d], V[2].v[d]}), mx = std::max({V[0].v[d], V[1].v[d], V[2].v[d]});
    lo[d] = std::max<i64>(0, ceil_div(mn, 256) - 1);
    hi[d] = std::min<i64>(N - 1, floor_div(mx, 256));
  }
  V3<R> gp[3], gn[3];
  for (int k = 0; k < 3; ++k) {
    gp[k] = V3<R>(R(tv.g[k][0]), R(tv.g[k][1]), R(tv.g[k][2]));
    gn[k] = normalize(mat3_mul<R>(tv.nm, nrm_obj[k]));
  }
  for (i64 z = lo[2]; z <= hi[2]; ++z)
    for (i64 y = lo[1]; y <= hi[1]; ++y)
      for (i64 x = lo[0]; x <= hi[0]; ++x) {
        i64 c[3] = {256 * x + 128, 256 * y + 128, 256 * z + 128};
        if (!sat_overlap(V, c, 128)) continue;
        V3<R> vc(R(2) * (R(x) + R(0.5)) / R(N) - R(1), R(2) * (R(y) + R(0.5)) / R(N) - R(1),
                 R(2) * (R(z) + R(0.5)) / R(N) - R(1));
        R w[3];
        closest_bary(vc, gp[0], gp[1], gp[2], w);
        V3<R> p = gp[0] * w[0] + gp[1] * w[1] + gp[2] * w[2];
        V3<R> n = gn[0] * w[0] + gn[1] * w[1] + gn[2] * w[2];
        V4<R> col = voxel_fragment_color<R>(s, mat, p, n);
        Contrib<R> ct;
        ct.voxel = (uint32_t)((z * N + y) * N + x);
        ct.c[0] = col.r; ct.c[1] = col.g; ct.c[2] = col.b; ct.c[3] = col.a;
        out.push_back(ct);
      }
  return true;
}

struct TriRef { uint32_t inst, tri; };

static inline void tri_verts(const orc_scene* s, const orc_instance& in, uint32_t t, const double* nm,
                             TriVerts& tv, const float* nrm[3]) {
  for (int k = 0; k < 3; ++k) {
    uint32_t vi = in.indices[3 * t + k];
    const float* v = in.verts + 8 * (size_t)vi;
    float w[3];
    xform_f32(in.model, v, w);
    for (int d = 0; d < 3; ++d) tv.g[k][d] = w[d] / s->cube_size;  // voxelize.vert:26
    nrm[k] = v + 3;
  }
  std::memcpy(tv.nm, nm, sizeof(tv.nm));
}

// Voxelize (renderer.cpp:316-353): clear level 0, rasterize/test every
// queued triangle, order-independent mean of all contributions per voxel,
// stored RGBA8 with round-to-nearest.  Contributions are generated in
// triangle chunks and summed per voxel in global triangle order, so the
// result does not depend on the thread count.
// Every contribution of the frame, in triangle chunks of consecutive queued
// triangles: lists[0], lists[1], ... concatenated are in draw order
// (triangles in queue order, each triangle's samples in scan order).
template <class R>
static int64_t gather_contribs(const orc_scene* s, const orc_params* p, std::vector<std::vector<Contrib<R>>>& lists) {
  const int N = p->grid_res;
  g_radiance_max = p->radiance_max > 0.0f ? (double)p->radiance_max : 1.0;
  std::vector<TriRef> tris;
  std::vector<std::vector<double>> nms(s->n_instances, std::vector<double>(9));
  for (uint32_t i = 0; i < s->n_instances; ++i) {
    normal_matrix(s->instances[i].model, nms[i].data());
    for (uint32_t t = 0; t < s->instances[i].n_tris; ++t) tris.push_back({i, t});
  }
  const int nthreads = std::max(1, p->threads);
  const int chunks = std::max(1, std::min<int>(nthreads * 4, (int)std::max<size_t>(1, tris.size() / 64)));
  lists.assign(chunks, {});
  std::vector<int64_t> rejected(chunks, 0);
  parallel_for(nthreads, chunks, [&](int ch) {
    size_t b = tris.size() * ch / chunks, e = tris.size() * (ch + 1) / chunks;
    for (size_t k = b; k < e; ++k) {
      const orc_instance& in = s->instances[tris[k].inst];
      TriVerts tv;
      const float* nrm[3];
      tri_verts(s, in, tris[k].tri, nms[tris[k].inst].data(), tv, nrm);
      uint32_t mid = in.tri_material[tris[k].tri];
      const orc_material& mat = s->materials[mid < s->n_materials ? mid : 0];
      bool ok = p->vox_mode == ORC_VOX_CONSERVATIVE ? sat_tri<R>(s, N, tv, nrm, mat, lists[ch])
                                                    : raster_tri_ref<R>(s, N, tv, nrm, mat, lists[ch]);
      if (!ok) rejected[ch]++;
    }
  });
  int64_t rej = 0;
  for (int64_t r : rejected) rej += r;
  return rej;
}

template <class R>
static int64_t voxelize_impl(const orc_scene* s, const orc_params* p, uint8_t* level0, uint32_t* counts,
                             float* level0f = nullptr) {
  const int N = p->grid_res;
  const int nthreads = std::max(1, p->threads);
  std::vector<std::vector<Contrib<R>>> lists;
  const int64_t rej = gather_contribs<R>(s, p, lists);
  const int chunks = (int)lists.size();
  const size_t nvox = (size_t)N * N * N;
  const int parts = nthreads;
  parallel_for(nthreads, parts, [&](int part) {
    size_t vb = nvox * part / parts, ve = nvox * (part + 1) / parts;
    std::vector<R> sum((ve - vb) * 4, R(0));
    std::vector<uint32_t> cnt(ve - vb, 0);
    for (int ch = 0; ch < chunks; ++ch)
      for (const Contrib<R>& c : lists[ch]) {
        if (c.voxel < vb || c.voxel >= ve) continue;
        size_t o = c.voxel - vb;
        for (int q = 0; q < 4; ++q) sum[4 * o + q] += c.c[q];
        cnt[o]++;
      }
    for (size_t o = 0; o < ve - vb; ++o) {
      if (counts) counts[vb + o] = cnt[o];
      if (level0f) {  // HDR storage: the mean itself
        for (int q = 0; q < 4; ++q) level0f[4 * (vb + o) + q] = cnt[o] ? (float)(sum[4 * o + q] / R(cnt[o])) : 0.0f;
        continue;
      }
      uint8_t* t = level0 + 4 * (vb + o);
      for (int q = 0; q < 4; ++q) {
        if (!cnt[o]) { t[q] = 0; continue; }
        R mean = sum[4 * o + q] / R(cnt[o]);
        R v = std::floor(mean * R(255) + R(0.5));
        t[q] = (uint8_t)(v < R(0) ? 0 : (v > R(255) ? 255 : v));
      }
    }
  });
  return rej;
}

// ---- the reference's running average (informational) ----------------------
// imageAtomicRGBA8Avg and its helpers, voxelize.frag:62-119, for one
// contribution arriving at a voxel that holds `cur` (0 = cleared).  With one
// writer at a time the compare-and-swap loop runs its body once: the stored
// RGBA8 (the low bit of each byte masked off) times the 4-bit count n in those
// low bits, plus the new value (x 255), divided by n + 1, rounded to an even
// integer (round(x / 2) * 2; GLSL leaves the direction of a .5 tie to the
// implementation, here away from zero), each channel truncated to uint and
// masked to 8 bits (so 256 wraps to 0), and n + 1 stored back in the low bits
// (16 wraps to 0, restarting the average).  FP32 throughout, as in GLSL.
static inline uint32_t cas_pack(const float v[4]) {
  return ((uint32_t)v[3] & 0xFFu) << 24 | ((uint32_t)v[2] & 0xFFu) << 16 | ((uint32_t)v[1] & 0xFFu) << 8 |
         ((uint32_t)v[0] & 0xFFu);
}
static inline uint32_t cas_enc(uint32_t m, uint32_t n) {
  return (m & 0xFEFEFEFEu) | (n & 1u) | (n & 2u) << 7 | (n & 4u) << 14 | (n & 8u) << 21;
}
static inline uint32_t cas_dec(uint32_t m) {
  return (m & 1u) | (m & 0x100u) >> 7 | (m & 0x10000u) >> 14 | (m & 0x1000000u) >> 21;
}
static uint32_t cas_step(uint32_t cur, const float c[4]) {
  float val[4];
  for (int q = 0; q < 4; ++q) val[q] = c[q] * 255.0f;
  if (cur == 0) return cas_enc(cas_pack(val), 1u);  // the first compare-and-swap (expected 0) succeeds
  const uint32_t m = cur & 0xFEFEFEFEu;
  const uint32_t n = cas_dec(cur);
  float r[4];
  for (int q = 0; q < 4; ++q) {
    float x = (float)((m >> (8 * q)) & 0xFFu);
    x = x * (float)n + val[q];
    x = x / (float)(n + 1);
    r[q] = std::round(x / 2.0f) * 2.0f;
  }
  return cas_enc(cas_pack(r), n + 1);
}

// Level 0 as the reference's running average leaves it after the frame's
// contributions arrive one at a time in a fixed order: 0 = draw order,
// 1 = reverse draw order, 2 = a permutation drawn from `seed` (Fisher-Yates
// over a 64-bit linear congruential generator).  The stored bytes keep the
// count bits in their low bits, as the reference's maps do.
static int64_t voxelize_cas_impl(const orc_scene* s, const orc_params* p, int order, uint64_t seed,
                                 uint8_t* level0) {
  const int N = p->grid_res;
  std::vector<std::vector<Contrib<float>>> lists;
  const int64_t rej = gather_contribs<float>(s, p, lists);
  std::vector<const Contrib<float>*> seq;
  for (const auto& l : lists)
    for (const auto& c : l) seq.push_back(&c);
  if (order == 1) std::reverse(seq.begin(), seq.end());
  if (order == 2) {
    uint64_t x = seed * 2862933555777941757ull + 3037000493ull;
    for (size_t i = seq.size(); i > 1; --i) {
      x = x * 6364136223846793005ull + 1442695040888963407ull;
      std::swap(seq[i - 1], seq[(size_t)((x >> 33) % i)]);
    }
  }
  std::vector<uint32_t> state((size_t)N * N * N, 0u);
  for (const Contrib<float>* c : seq) state[c->voxel] = cas_step(state[c->voxel], c->c);
  for (size_t v = 0; v < state.size(); ++v)
    for (int q = 0; q < 4; ++q) level0[4 * v + q] = (uint8_t)(state[v] >> (8 * q));
  return rej;
}

// ------------------------------------------------------------ mipmap.comp --
// voxel_offsets, mipmap.comp:10-20.
static const int kOff[8][3] = {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0},
                               {0, 1, 1}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
// (front, back) pairs per map, mipmap.comp:59-98 (0:-x 1:+x 2:-y 3:+y 4:-z 5:+z).
static const int kPairs[6][4][2] = {
    {{0, 4}, {1, 5}, {2, 6}, {3, 7}}, {{4, 0}, {5, 1}, {6, 2}, {7, 3}},
    {{0, 2}, {1, 3}, {5, 7}, {4, 6}}, {{2, 0}, {3, 1}, {7, 5}, {6, 4}},
    {{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{1, 0}, {3, 2}, {5, 4}, {7, 6}}};

static uint64_t level_offset(int N, int l) {  // offset of level l (>=1) inside a chain
  uint64_t o = 0;
  for (int k = 1; k < l; ++k) { uint64_t s = (uint64_t)(N >> k); o += s * s * s; }
  return o;
}

// One destination texel of map d.  alpha_blend(f, b) = f + (1 - f.a) * b
// (mipmap.comp:40-43), mean of 4 pairs, stored as unorm8 (GL rounds to
// nearest).  Evaluated exactly: with texels k/255 the stored value is
// round(S / 1020), S = sum over pairs of (F*255 + (255 - F.a) * B), ties up,
// clamped to 255.
static void aniso_texel(const uint8_t* const child[8], int d, uint8_t* out) {
  for (int ch = 0; ch < 4; ++ch) {
    uint32_t S = 0;
    for (int q = 0; q < 4; ++q) {
      const uint8_t* f = child[kPairs[d][q][0]];
      const uint8_t* b = child[kPairs[d][q][1]];
      S += (uint32_t)f[ch] * 255u + (255u - f[3]) * (uint32_t)b[ch];
    }
    uint32_t v = (S + 510u) / 1020u;
    out[ch] = (uint8_t)(v > 255u ? 255u : v);
  }
}

// Renderer::filter (renderer.cpp:283-314): level l+1 of every map from level
// l (level 0 is the same texture for all six maps).
static void mipmap_impl(const orc_params* p, const uint8_t* level0, uint8_t* chains) {
  const int N = p->grid_res, L = p->levels;
  const uint64_t chain = orc_chain_texels(N, L);
  const int nmaps = p->mip_mode == ORC_MIP_ISO ? 1 : 6;
  for (int l = 1; l < L; ++l) {
    const int s = N >> l, ss = N >> (l - 1);
    parallel_for(std::max(1, p->threads), s, [&](int z) {
      for (int y = 0; y < s; ++y)
        for (int x = 0; x < s; ++x)
          for (int d = 0; d < nmaps; ++d) {
            const uint8_t* src = l == 1 ? level0 : chains + 4 * (d * chain + level_offset(N, l - 1));
            const uint8_t* child[8];
            for (int i = 0; i < 8; ++i) {
              int cx = 2 * x + kOff[i][0], cy = 2 * y + kOff[i][1], cz = 2 * z + kOff[i][2];
              child[i] = src + 4 * (((size_t)cz * ss + cy) * ss + cx);
            }
            uint8_t* dst = chains + 4 * (d * chain + level_offset(N, l) + ((size_t)z * s + y) * s + x);
            if (nmaps == 6) {
              aniso_texel(child, d, dst);
            } else {
              // Isotropic box mean of the 8 children (glGenerateMipmap-style),
              // round to nearest, ties up.
              for (int ch = 0; ch < 4; ++ch) {
                uint32_t S = 0;
                for (int i = 0; i < 8; ++i) S += child[i][ch];
                dst[ch] = (uint8_t)((S + 4u) / 8u);
              }
            }
          }
    });
  }
}

// One level of float maps in FP64: the same pairs / box mean as above
// without unorm8 rounding (RGBA16F storage).
static void mip_level_f(int n_src, int src_maps, const float* src, int mip_mode, float* dst, int threads) {
  const int s = n_src / 2;
  const int nmaps = mip_mode == ORC_MIP_ISO ? 1 : 6;
  const size_t src_n = (size_t)n_src * n_src * n_src, dst_n = (size_t)s * s * s;
  parallel_for(std::max(1, threads), s, [&](int z) {
    for (int y = 0; y < s; ++y)
      for (int x = 0; x < s; ++x)
        for (int d = 0; d < nmaps; ++d) {
          const float* base = src + 4 * (src_maps == 1 ? 0 : d) * src_n;
          const float* child[8];
          for (int i = 0; i < 8; ++i) {
            int cx = 2 * x + kOff[i][0], cy = 2 * y + kOff[i][1], cz = 2 * z + kOff[i][2];
            child[i] = base + 4 * (((size_t)cz * n_src + cy) * n_src + cx);
          }
          float* o = dst + 4 * (d * dst_n + ((size_t)z * s + y) * s + x);
          for (int ch = 0; ch < 4; ++ch) {
            double S = 0.0;
            if (nmaps == 6) {
              for (int q = 0; q < 4; ++q) {
                const float* f = child[kPairs[d][q][0]];
                const float* b = child[kPairs[d][q][1]];
                S += (double)f[ch] + (1.0 - (double)f[3]) * (double)b[ch];
              }
              o[ch] = (float)(S * 0.25);
            } else {
              for (int i = 0; i < 8; ++i) S += child[i][ch];
              o[ch] = (float)(S * 0.125);
            }
          }
        }
  });
}

// -------------------------------------------------- GL texture sampling ----
struct Maps {
  const uint8_t* level0;
  const uint8_t* chains;
  int N, L;
  uint64_t chain;
  bool iso;
  const float* level0f = nullptr;  // float maps (HDR storage) instead of RGBA8
  const float* chainsf = nullptr;
};

template <class R> static inline V4<R> texel(const Maps& m, int l, int map, int x, int y, int z) {
  int s = m.N >> l;
  if (x < 0 || y < 0 || z < 0 || x >= s || y >= s || z >= s) return V4<R>();  // CLAMP_TO_BORDER(0)
  if (m.level0f) {
    const float* f;
    if (l == 0) f = m.level0f + 4 * (((size_t)z * s + y) * s + x);
    else f = m.chainsf + 4 * ((m.iso ? 0 : map) * m.chain + level_offset(m.N, l) + ((size_t)z * s + y) * s + x);
    return V4<R>(R(f[0]), R(f[1]), R(f[2]), R(f[3]));
  }
  const uint8_t* t;
  if (l == 0) t = m.level0 + 4 * (((size_t)z * s + y) * s + x);
  else t = m.chains + 4 * ((m.iso ? 0 : map) * m.chain + level_offset(m.N, l) + ((size_t)z * s + y) * s + x);
  const R k = R(1) / R(255);
  return V4<R>(R(t[0]) * k, R(t[1]) * k, R(t[2]) * k, R(t[3]) * k);
}

// GL_LINEAR on one level: x = u * size - 0.5, 8 neighbours, border texels 0.
template <class R> static V4<R> trilinear(const Maps& m, int l, int map, V3<R> u) {
  int s = m.N >> l;
  R tx = u.x * R(s) - R(0.5), ty = u.y * R(s) - R(0.5), tz = u.z * R(s) - R(0.5);
  R fx = std::floor(tx), fy = std::floor(ty), fz = std::floor(tz);
  R ax = tx - fx, ay = ty - fy, az = tz - fz;
  int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  V4<R> acc;
  for (int c = 0; c < 8; ++c) {
    int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
    R w = (dx ? ax : R(1) - ax) * (dy ? ay : R(1) - ay) * (dz ? az : R(1) - az);
    acc = acc + texel<R>(m, l, map, ix + dx, iy + dy, iz + dz) * w;
  }
  return acc;
}

static inline bool u_sane(double v) { return v > -1.0e6 && v < 1.0e6; }

// textureLod with GL_LINEAR_MIPMAP_LINEAR (min) / GL_LINEAR (mag) over levels
// 0..L-1 (texture_3d.cpp:14-17; OpenGL 4.5 sec. 8.14): lambda <= 0 samples
// level 0, lambda >= L-1 the last level, otherwise the two levels around it
// blended by frac(lambda).
template <class R> static V4<R> texture_lod(const Maps& m, int map, V3<R> u, R lod) {
  if (!u_sane((double)u.x) || !u_sane((double)u.y) || !u_sane((double)u.z)) return V4<R>();
  if (!(lod > R(0))) return trilinear<R>(m, 0, map, u);
  const int q = m.L - 1;
  if (lod >= R(q)) return trilinear<R>(m, q, map, u);
  R fl = std::floor(lod);
  int d1 = (int)fl;
  R f = lod - fl;
  V4<R> t1 = trilinear<R>(m, d1, map, u), t2 = trilinear<R>(m, d1 + 1, map, u);
  return t1 * (R(1) - f) + t2 * f;
}

// --------------------------------------------------- voxel_cone_tracing ----
template <class R> struct ConeOut { V4<R> c; int steps; };

// Instrumentation for orc_trace_stats: per cone class (0 diffuse, 1
// specular, 2 shadow, 3 refraction) the cones traced, the march steps and
// the steps whose lod is < 1 (those read level 0 plus level 1); then, over
// all classes, the steps whose lod lies in [k, k+1) for k = 0..6 (k = 7:
// lod >= 7); then per class the steps taken once the cone has moved more
// than 3/4 of the coarsest texel outside [0,1] along an axis it travels
// away on (they read border texels only; the engine does not take them);
// then per class the other steps whose texels are all 0 by the engine's
// occupancy rule (below), and how many of those have lod < 1; then per
// class the texture fetches the engine's texture-unit path issues for the
// steps it takes, split into single-level (trilinear: the shared level 0,
// a chain at lod 0 when lod < 1, a chain clamped at its last level) and
// two-level (quadrilinear) fetches.  A map whose weight is exactly 0 is not
// fetched; shadow cones fetch the packed alpha chains (one fetch for the x
// and y maps, one for the z maps).
enum {
  kStatCones = 0, kStatSteps = 4, kStatLodLt1 = 8, kStatLodBand = 12, kStatBeyond = 20, kStatEmpty = 24,
  kStatEmptyLt1 = 28, kStatFetchTri = 32, kStatFetchQuad = 36, kStatN = 40
};
static std::atomic<uint64_t> g_stats[kStatN];
// The engine's empty-space rule (csrc/k_trace.cu sample_empty): per level c
// >= 1, cell occupancy (its block of level 0 holds a non-zero texel) ORed
// over the 2x2x2 cells k..k+1; a sample with lod is empty, for c = (lod < 1
// ? 1 : min(floor(lod) + 1, L - 1)) and k = floor(u * (N >> c) - 0.5)
// clamped into the grid, when no coordinate lies within 1/64 of a texel
// boundary and the ORed occupancy of k is 0.  Shadow cones use the coarser
// rule of sample_empty3: occupancy ORed over the 3x3x3 cells around k =
// floor(u * (N >> c)) clamped into the grid, empty when that is 0.
static std::vector<std::vector<uint8_t>> g_dilated, g_dilated3;
static void build_dilated(const uint8_t* level0, int N, int L) {
  std::vector<std::vector<uint8_t>> raw(1, std::vector<uint8_t>((size_t)N * N * N));
  for (size_t v = 0; v < (size_t)N * N * N; ++v)
    raw[0][v] = (level0[4 * v] | level0[4 * v + 1] | level0[4 * v + 2] | level0[4 * v + 3]) != 0;
  g_dilated.assign(L, {});
  g_dilated3.assign(L, {});
  for (int c = 1; c < L; ++c) {
    const int s = N >> c, p = 2 * s;
    std::vector<uint8_t> o((size_t)s * s * s, 0);
    for (int z = 0; z < s; ++z)
      for (int y = 0; y < s; ++y)
        for (int x = 0; x < s; ++x) {
          uint8_t a = 0;
          for (int k = 0; k < 8; ++k)
            a |= raw[c - 1][((size_t)(2 * z + (k >> 2)) * p + 2 * y + ((k >> 1) & 1)) * p + 2 * x + (k & 1)];
          o[((size_t)z * s + y) * s + x] = a;
        }
    raw.push_back(o);
    std::vector<uint8_t> d((size_t)s * s * s, 0);
    for (int z = 0; z < s; ++z)
      for (int y = 0; y < s; ++y)
        for (int x = 0; x < s; ++x) {
          uint8_t a = 0;
          for (int dz = 0; dz <= 1; ++dz)
            for (int dy = 0; dy <= 1; ++dy)
              for (int dx = 0; dx <= 1; ++dx) {
                const int X = x + dx, Y = y + dy, Z = z + dz;
                if (X >= 0 && Y >= 0 && Z >= 0 && X < s && Y < s && Z < s) a |= o[((size_t)Z * s + Y) * s + X];
              }
          d[((size_t)z * s + y) * s + x] = a;
        }
    g_dilated[c] = std::move(d);
    std::vector<uint8_t> d3((size_t)s * s * s, 0);
    for (int z = 0; z < s; ++z)
      for (int y = 0; y < s; ++y)
        for (int x = 0; x < s; ++x) {
          uint8_t a = 0;
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                const int X = x + dx, Y = y + dy, Z = z + dz;
                if (X >= 0 && Y >= 0 && Z >= 0 && X < s && Y < s && Z < s) a |= o[((size_t)Z * s + Y) * s + X];
              }
          d3[((size_t)z * s + y) * s + x] = a;
        }
    g_dilated3[c] = std::move(d3);
  }
}
template <class R> static bool sample_empty3_rule(int N, int L, V3<R> u, R lod) {
  const int c = lod < R(1) ? 1 : std::min((int)lod + 1, L - 1);
  const int s = N >> c;
  int k[3] = {(int)std::floor(u.x * R(s)), (int)std::floor(u.y * R(s)), (int)std::floor(u.z * R(s))};
  for (int a = 0; a < 3; ++a) k[a] = std::min(std::max(k[a], 0), s - 1);
  return g_dilated3[c][((size_t)k[2] * s + k[1]) * s + k[0]] == 0;
}
template <class R> static bool sample_empty_rule(int N, int L, V3<R> u, R lod) {
  const int c = lod < R(1) ? 1 : std::min((int)lod + 1, L - 1);
  const int s = N >> c;
  const R t[3] = {u.x * R(s) - R(0.5), u.y * R(s) - R(0.5), u.z * R(s) - R(0.5)};
  int k[3];
  for (int a = 0; a < 3; ++a) {
    // 8.8 fixed point: the top byte of the fraction within 4/256 of a
    // texel boundary marks a sample that is fetched
    const R q = std::floor(t[a] * R(256));
    const R fr = q - R(256) * std::floor(q / R(256));
    if (fr < R(4) || fr >= R(252)) return false;
    k[a] = std::min(std::max((int)std::floor(t[a]), 0), s - 1);
  }
  return g_dilated[c][((size_t)k[2] * s + k[1]) * s + k[0]] == 0;
}
static bool g_stats_on = false;
static thread_local int t_cone_class = 0;

// trace_cone, voxel_cone_tracing.frag:88-119 (face_indices :71-78,
// sample_voxel :80-86).
static thread_local bool t_stats_skip = false;  // (a shared far field counted by another pixel)

// start_dist > 0: the march starts at that step of the schedule (a far
// field, see trace_diffuse) with nothing accumulated.
template <class R>
static ConeOut<R> trace_cone(const Maps& m, V3<R> origin, V3<R> dir, R aperture, R max_dist, R start_dist = R(0)) {
  dir = normalize(dir);
  const int ix = dir.x < R(0) ? 0 : 1, iy = dir.y < R(0) ? 2 : 3, iz = dir.z < R(0) ? 4 : 5;
  const V3<R> ad = vabs(dir);
  const R cube_res = R(m.N);
  const R voxel_size = R(1) / cube_res;
  V4<R> acc;
  R dist = start_dist > R(0) ? start_dist : R(3) * voxel_size;
  R diam = dist * aperture;
  V3<R> sp = dir * dist + origin;
  int steps = 0, lod_lt1 = 0, beyond = 0, empty = 0, empty_lt1 = 0, f_tri = 0, f_quad = 0;
  const int maps_fetched = t_cone_class == 2 ? (ad.x != R(0) || ad.y != R(0)) + (ad.z != R(0))
                                             : (ad.x != R(0)) + (ad.y != R(0)) + (ad.z != R(0));
  const R margin = R(0.75) * R(1 << (m.L - 1)) / cube_res;
  auto outside = [&](R p, bool up) { return up ? p > R(1) + margin : p < -margin; };
  bool gone = false;
  while (acc.a < R(1) && dist < max_dist) {
    gone = gone || outside(sp.x, ix == 1) || outside(sp.y, iy == 3) || outside(sp.z, iz == 5);
    if (gone) ++beyond;
    R mip = fmaxr(R(std::log2(diam * cube_res)), R(0));
    if (g_stats_on && !t_stats_skip && !gone && !g_dilated.empty()) {
      if (t_cone_class == 2 ? sample_empty3_rule<R>(m.N, m.L, sp, mip)
                            : mip < R(5) && sample_empty_rule<R>(m.N, m.L, sp, mip)) {  // RGBA cones: lod < 5 only
        ++empty;
        if (mip < R(1)) ++empty_lt1;
      } else if (mip < R(1)) {
        f_tri += 1 + (mip > R(0) ? maps_fetched : 0);
      } else if (mip - R(1) >= R(m.L - 2) || mip == std::floor(mip)) {
        f_tri += maps_fetched;
      } else {
        f_quad += maps_fetched;
      }
    }
    V4<R> smp = texture_lod<R>(m, ix, sp, mip) * ad.x + texture_lod<R>(m, iy, sp, mip) * ad.y +
                texture_lod<R>(m, iz, sp, mip) * ad.z;
    acc = acc + smp * (R(1) - acc.a);
    R step = fmaxr(diam / R(2), voxel_size);
    dist += step;
    diam = dist * aperture;
    sp = dir * dist + origin;
    ++steps;
    if (mip < R(1)) ++lod_lt1;
    if (g_stats_on && !t_stats_skip) g_stats[kStatLodBand + (mip >= R(7) ? 7 : (int)mip)] += 1;
  }
  if (g_stats_on && !t_stats_skip) {
    g_stats[kStatCones + t_cone_class] += 1;
    g_stats[kStatSteps + t_cone_class] += (uint64_t)steps;
    g_stats[kStatLodLt1 + t_cone_class] += (uint64_t)lod_lt1;
    g_stats[kStatBeyond + t_cone_class] += (uint64_t)beyond;
    g_stats[kStatEmpty + t_cone_class] += (uint64_t)empty;
    g_stats[kStatEmptyLt1 + t_cone_class] += (uint64_t)empty_lt1;
    g_stats[kStatFetchTri + t_cone_class] += (uint64_t)f_tri;
    g_stats[kStatFetchQuad + t_cone_class] += (uint64_t)f_quad;
  }
  return {acc, steps};
}

// tangent, voxel_cone_tracing.frag:126-134.
template <class R> static V3<R> tangent(V3<R> n) {
  V3<R> t1 = cross(n, V3<R>(0, 0, 1)), t2 = cross(n, V3<R>(0, 1, 0));
  return length(t1) > length(t2) ? normalize(t1) : normalize(t2);
}
template <class R> static inline V3<R> mixv(V3<R> a, V3<R> b, R t) { return a * (R(1) - t) + b * t; }

static const double kTan22_5 = 0.55785173935;   // TAN_22_5, :136 (kept verbatim)
static const double kMaxDistance = 1.73205080757;  // MAX_DISTANCE, :138

// The engine's shared far fields (orc_params::far_share = the group width W;
// csrc/k_trace.cu k_trace_share), restated: the pixels of a W x 2 group
// (corner x0 a multiple of W, y0 even) take as representative the group's
// first pixel, in the order (x0,y0) .. (x0+W-1,y0), (x0,y0+1) ..
// (x0+W-1,y0+1), whose diffuse cones are traced.  A pixel shares when its normal is within cos 0.99 of the
// representative's and its texture-space position within 2 voxels along
// every axis.  A shared diffuse cone k takes its own first sample (step 0,
// 3 voxels out), then adds the representative's cone k marched from the
// second step of the schedule (distance far_dist) with nothing accumulated
// ("far field"): near + (1 - near.a) * far while near.a < 1.
template <class R> struct ShareQuad {
  bool on = false, count_far = false;
  V3<R> pos, n;  // representative's texture-space position and normal
  R far_dist = R(0);
};

template <class R> static R far_start_dist(int N, R ap) {  // the second step of trace_cone's schedule
  const R voxel = R(1) / R(N);
  const R dist = R(3) * voxel;
  return dist + fmaxr(dist * ap / R(2), voxel);
}

template <class R>
static V4<R> diffuse_cone(const Maps& m, V3<R> origin, V3<R> dir, V3<R> rep_dir, R ap, R md,
                          const ShareQuad<R>* sq) {
  if (!sq || !sq->on) return trace_cone<R>(m, origin, dir, ap, md).c;
  V4<R> near = trace_cone<R>(m, origin, dir, ap, sq->far_dist).c;
  t_stats_skip = !sq->count_far;
  V4<R> far = trace_cone<R>(m, sq->pos, rep_dir, ap, md, sq->far_dist).c;
  t_stats_skip = false;
  return near.a < R(1) ? near + far * (R(1) - near.a) : near;
}

// trace_diffuse, voxel_cone_tracing.frag:140-168 (9 cones, equal weights).
// cone_set SIX60 (no reference counterpart): the normal plus 5 cones 60
// degrees off it, evenly spaced in azimuth in the same tangent frame, each
// of aperture 2*tan(30 deg), equal weights.
template <class R> static V3<R> trace_diffuse(const Maps& m, int cone_set, V3<R> origin, V3<R> n,
                                              const ShareQuad<R>* sq = nullptr) {
  const V3<R> o1 = normalize(tangent(n));
  const V3<R> o2 = normalize(cross(o1, n));
  if (sq && sq->on) {
    const V3<R> rn = sq->n;
    const V3<R> q1 = normalize(tangent(rn)), q2 = normalize(cross(q1, rn));
    V4<R> acc;
    if (cone_set == ORC_CONES_SIX60) {
      const R ap = R(2) * R(std::tan(3.14159265358979323846 / 6.0));
      const V3<R> nn = normalize(n), rnn = normalize(rn);
      acc = acc + diffuse_cone<R>(m, origin, nn, rnn, ap, R(kMaxDistance), sq);
      for (int k = 0; k < 5; ++k) {
        R phi = R(2.0 * 3.14159265358979323846 * k / 5.0);
        const R c = R(std::cos(phi)), sn = R(std::sin(phi)), h = R(0.86602540378443864676);
        acc = acc + diffuse_cone<R>(m, origin, nn * R(0.5) + (o1 * c + o2 * sn) * h,
                                    rnn * R(0.5) + (q1 * c + q2 * sn) * h, ap, R(kMaxDistance), sq);
      }
      return V3<R>(acc.r, acc.g, acc.b) * (R(1) / R(6));
    }
    const R ap = R(kTan22_5), md = R(kMaxDistance), h = R(0.5);
    const V3<R> c1 = (o1 + o2) * R(0.5), c2 = (o1 - o2) * R(0.5);
    const V3<R> d1 = (q1 + q2) * R(0.5), d2 = (q1 - q2) * R(0.5);
    const V3<R> pb[4] = {o1, o2, c1, c2}, rb[4] = {q1, q2, d1, d2};
    acc = acc + diffuse_cone<R>(m, origin, n, rn, ap, md, sq);
    for (int j = 0; j < 8; ++j) {
      const R sgn = (j & 1) ? R(-1) : R(1);
      acc = acc + diffuse_cone<R>(m, origin, mixv(n, pb[j >> 1] * sgn, h), mixv(rn, rb[j >> 1] * sgn, h), ap, md, sq);
    }
    return V3<R>(acc.r, acc.g, acc.b) * (R(1) / R(9));
  }
  V4<R> acc;
  if (cone_set == ORC_CONES_SIX60) {
    const R ap = R(2) * R(std::tan(3.14159265358979323846 / 6.0));
    V3<R> nn = normalize(n);
    acc = acc + trace_cone<R>(m, origin, nn, ap, R(kMaxDistance)).c;
    for (int k = 0; k < 5; ++k) {
      R phi = R(2.0 * 3.14159265358979323846 * k / 5.0);
      V3<R> d = nn * R(0.5) + (o1 * R(std::cos(phi)) + o2 * R(std::sin(phi))) * R(0.86602540378443864676);
      acc = acc + trace_cone<R>(m, origin, d, ap, R(kMaxDistance)).c;
    }
    return V3<R>(acc.r, acc.g, acc.b) * (R(1) / R(6));
  }
  const R ap = R(kTan22_5), md = R(kMaxDistance), h = R(0.5);
  const V3<R> c1 = (o1 + o2) * R(0.5), c2 = (o1 - o2) * R(0.5);
  acc = acc + trace_cone<R>(m, origin, n, ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, o1, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, -o1, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, o2, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, -o2, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, c1, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, -c1, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, c2, h), ap, md).c;
  acc = acc + trace_cone<R>(m, origin, mixv(n, -c2, h), ap, md).c;
  return V3<R>(acc.r, acc.g, acc.b) * (R(1) / R(9));
}

// GLSL refract(I, N, eta).
template <class R> static V3<R> refract(V3<R> I, V3<R> N, R eta) {
  R d = dot(N, I);
  R k = R(1) - eta * eta * (R(1) - d * d);
  if (k < R(0)) return V3<R>();
  return I * eta - N * (eta * d + std::sqrt(k));
}
template <class R> static V3<R> reflect(V3<R> I, V3<R> N) { return I - N * (R(2) * dot(N, I)); }

template <class R> static R specular_aperture(const orc_material& mat) {  // voxel_cone_tracing.frag:220-227
  R r = std::sqrt(R(2) / (R(mat.shininess) + R(2)));
  R a = R(std::tan(R(1.57079) * r));
  const R lo = R(0.0174533), hi = R(3.14159265);
  return a < lo ? lo : (a > hi ? hi : a);
}

// direct_light, voxel_cone_tracing.frag:175-218.
template <class R>
static V3<R> direct_light(const orc_scene* s, const Maps& m, int enable_shadow, const orc_material& mat,
                          V3<R> pos, V3<R> nrm, V3<R> view_dir) {
  V3<R> result;
  int nl = std::min<int>((int)s->n_lights, 10);
  const R cube = R(s->cube_size);
  for (int i = 0; i < nl; ++i) {
    const orc_point_light& L = s->lights[i];
    V3<R> lp(R(L.position[0]) / cube, R(L.position[1]) / cube, R(L.position[2]) / cube);
    lp = lp * R(0.5) + V3<R>(R(0.5), R(0.5), R(0.5));  // scale_and_bias
    V3<R> ld = lp - pos;
    R d = length(ld);
    ld = normalize(ld);
    R cs = fmaxr(dot(nrm, ld), R(0));
    V3<R> lc = V3<R>(R(L.color[0]), R(L.color[1]), R(L.color[2])) *
               ((R(1) / (R(1) + R(0) * d + R(1) * d * d)) * cs * R(L.intensity));
    R shadow = R(1);
    t_cone_class = 2;
    if (enable_shadow) shadow = fmaxr(R(0), R(1) - trace_cone<R>(m, pos, ld, R(0.1), d).c.a);
    R lambert = fmaxr(dot(ld, nrm), R(0));
    R refract_angle = R(0);
    if (R(mat.dissolve) <= R(0.1f)) {
      V3<R> rf = refract(view_dir, nrm, R(1) / R(mat.ior));
      refract_angle = fmaxr((R(1) - R(mat.dissolve)) * dot(rf, ld), R(0));
    }
    V3<R> hv = normalize(ld + view_dir);
    R sa = fmaxr(dot(hv, nrm), R(0));
    sa = fmaxr(sa, refract_angle);
    R sc = std::pow(sa, R(mat.shininess));
    V3<R> term = mat_of<R>(mat, 0) * lambert + mat_of<R>(mat, 1) * sc;
    result = result + mulv(term, lc) * (shadow + R(0.04));
  }
  V3<R> e = mat_of<R>(mat, 3);
  return result + V3<R>(clamp01(e.x), clamp01(e.y), clamp01(e.z));
}

// main, voxel_cone_tracing.frag:246-275, for one visible surface point.
template <class R>
static V4<R> shade_pixel(const orc_scene* s, const orc_params* p, const Maps& m, V3<R> world, V3<R> nrm,
                         uint32_t mat_id, bool* written, const ShareQuad<R>* sq = nullptr) {
  const orc_material& mat = s->materials[mat_id < s->n_materials ? mat_id : 0];
  const R cube = R(s->cube_size);
  V3<R> pos = V3<R>(world.x / cube, world.y / cube, world.z / cube) * R(0.5) + V3<R>(R(0.5), R(0.5), R(0.5));
  *written = false;
  if (!(std::fabs(pos.x) < R(1) && std::fabs(pos.y) < R(1) && std::fabs(pos.z) < R(1))) return V4<R>();
  *written = true;
  if (p->view_voxel_dir < 7) {
    if (p->view_voxel_dir < 0 || p->view_voxel_dir > 5) return V4<R>();
    return texture_lod<R>(m, p->view_voxel_dir, pos, R(p->view_voxel_lod));
  }
  // camera_position = column 3 of the view matrix (renderer.cpp:279).
  V3<R> cam(R(s->view[12]), R(s->view[13]), R(s->view[14]));
  V3<R> view_dir = normalize(world - cam);
  V3<R> fd, fdir, fs;
  t_cone_class = 0;
  if (p->enable_diffuse) fd = mulv(mat_of<R>(mat, 0), trace_diffuse<R>(m, p->cone_set, pos, nrm, sq));
  if (p->enable_direct) fdir = direct_light<R>(s, m, p->enable_shadow, mat, pos, nrm, view_dir);
  R sap = specular_aperture<R>(mat);
  if (p->enable_specular) {
    V3<R> sd = normalize(reflect(-view_dir, nrm));
    t_cone_class = 1;
    ConeOut<R> c = trace_cone<R>(m, pos, sd, sap, R(kMaxDistance));
    fs = mulv(mat_of<R>(mat, 1), V3<R>(c.c.r, c.c.g, c.c.b));
  }
  V3<R> f = fs + fd + fdir;
  if (illum_transparent(mat.illum) && p->enable_specular) {
    V3<R> rd = refract(view_dir, nrm, R(1) / R(mat.ior));
    t_cone_class = 3;
    ConeOut<R> c = trace_cone<R>(m, pos, rd, sap, R(kMaxDistance));
    V3<R> tr = mulv(mat_of<R>(mat, 2), V3<R>(c.c.r, c.c.g, c.c.b));
    R a = R(mat.dissolve);
    f = tr * (R(1) - a) + f * a;
  }
  return V4<R>(f.x, f.y, f.z, R(1));
}

static const float kClear[4] = {0.15f, 0.25f, 0.25f, 1.0f};  // renderer.cpp:398

template <class R>
static void trace_impl(const orc_scene* s, const orc_params* p, const uint8_t* level0, const uint8_t* chains,
                       const uint32_t* tri_id, const double* pos, const double* nrm, const uint32_t* mat,
                       int row_stride, float* out, const float* level0f = nullptr, const float* chainsf = nullptr) {
  Maps m{level0, chains, p->grid_res, p->levels, orc_chain_texels(p->grid_res, p->levels), p->mip_mode == ORC_MIP_ISO,
         level0f, chainsf};
  const int W = p->width, H = p->height;
  // row_stride < 0: pairs of rows (k |row_stride|, k |row_stride| + 1), so
  // that sampled rows hold whole 2x2 quads (shared far fields)
  const bool pairs = row_stride < -1;
  if (pairs) row_stride = -row_stride;
  if (row_stride < 1) row_stride = 1;
  const int rows = pairs ? 2 * ((H + row_stride - 1) / row_stride) : (H + row_stride - 1) / row_stride;
  // Work items are 32-pixel runs of a traced row, so that every thread gets
  // a share of the frame whatever the row count (a sampled frame may have
  // fewer rows than threads).
  const int kRun = 32;
  const int runs = (W + kRun - 1) / kRun;
  // Shared far fields: which pixels' diffuse cones are traced (the quad's
  // candidates for representative), and the far fields' start distance.
  const double cube = s->cube_size;
  auto tex_pos = [&](size_t q, int a) { return pos[3 * q + a] / cube * 0.5 + 0.5; };
  auto diffuse_traced = [&](int x, int y) {
    if (x >= W || y >= H) return false;
    const size_t q = (size_t)y * W + x;
    if (tri_id[q] == 0xffffffffu || !p->enable_diffuse || p->view_voxel_dir < 7) return false;
    for (int a = 0; a < 3; ++a)
      if (!(std::fabs(tex_pos(q, a)) < 1.0)) return false;
    return true;
  };
  const bool share_on = p->far_share != 0 && p->view_voxel_dir >= 7;
  const R far_dist = far_start_dist<R>(p->grid_res, p->cone_set == ORC_CONES_SIX60
                                                        ? R(2) * R(std::tan(3.14159265358979323846 / 6.0))
                                                        : R(kTan22_5));
  parallel_for(std::max(1, p->threads), rows * runs, [&](int item) {
    const int ri = item / runs;
    const int y = pairs ? (ri >> 1) * row_stride + (ri & 1) : ri * row_stride;
    if (y >= H) return;
    const int x0 = (item % runs) * kRun, x1 = std::min(W, x0 + kRun);
    for (int x = x0; x < x1; ++x) {
      size_t px = (size_t)y * W + x;
      float* o = out + 4 * px;
      for (int q = 0; q < 4; ++q) o[q] = kClear[q];
      if (tri_id[px] == 0xffffffffu) continue;
      V3<R> w(R(pos[3 * px]), R(pos[3 * px + 1]), R(pos[3 * px + 2]));
      V3<R> n(R(nrm[3 * px]), R(nrm[3 * px + 1]), R(nrm[3 * px + 2]));
      ShareQuad<R> sq;
      if (share_on && diffuse_traced(x, y)) {
        const int gw = std::min(std::max(p->far_share, 1), 16);
        const int qx = x - x % gw, qy = y & ~1;
        int order[32][2];
        int no = 0;
        for (int r = 0; r < 2; ++r)
          for (int i = 0; i < gw; ++i) {
            order[no][0] = qx + i;
            order[no][1] = qy + r;
            ++no;
          }
        for (int oi = 0; oi < no; ++oi) {
          const int* c = order[oi];
          if (!diffuse_traced(c[0], c[1])) continue;
          const size_t rp = (size_t)c[1] * W + c[0];
          V3<double> na(nrm[3 * px], nrm[3 * px + 1], nrm[3 * px + 2]);
          V3<double> nb(nrm[3 * rp], nrm[3 * rp + 1], nrm[3 * rp + 2]);
          const double lim = 2.0 / p->grid_res;
          bool ok = dot(normalize(na), normalize(nb)) >= 0.99;
          for (int a = 0; a < 3; ++a) ok = ok && std::fabs(tex_pos(px, a) - tex_pos(rp, a)) <= lim;
          if (ok) {
            sq.on = true;
            sq.count_far = rp == px;
            sq.pos = V3<R>(R(tex_pos(rp, 0)), R(tex_pos(rp, 1)), R(tex_pos(rp, 2)));
            sq.n = V3<R>(R(nrm[3 * rp]), R(nrm[3 * rp + 1]), R(nrm[3 * rp + 2]));
            sq.far_dist = far_dist;
          }
          break;  // the first traced pixel is the representative
        }
      }
      bool written;
      V4<R> c = shade_pixel<R>(s, p, m, w, n, mat[px], &written, &sq);
      if (!written) continue;  // fragment returned without writing: keep the clear colour
      o[0] = (float)c.r; o[1] = (float)c.g; o[2] = (float)c.b; o[3] = (float)c.a;
    }
  });
}

// ---------------------------------------------------------- G-buffer -------
// Forward raster of Renderer::visualize (renderer.cpp:355-390) with
// voxel_cone_tracing.vert:22-27: GL_LESS depth test against a cleared depth
// of 1.0, culling off, draw order = queue order then index order (so on equal
// depth the earlier triangle stays).  Triangles are clipped to the near plane
// and to a guard band of |x|,|y| <= 16 w, snapped to 1/256 pixel, covered by
// the same integer edge functions and fill rule as the voxelizer; depth is
// FP32 z_window interpolated linearly in screen space.
struct ClipV { float c[4]; };

static inline float plane_eval(int pl, const ClipV& v) {
  const float G = 16.0f;
  switch (pl) {
    case 0: return v.c[2] + v.c[3];
    case 1: return G * v.c[3] - v.c[0];
    case 2: return G * v.c[3] + v.c[0];
    case 3: return G * v.c[3] - v.c[1];
    default: return G * v.c[3] + v.c[1];
  }
}

static int clip_polygon(const ClipV in[3], ClipV* out /* >= 9 */) {
  ClipV a[10], b[10];
  int n = 3;
  for (int k = 0; k < 3; ++k) a[k] = in[k];
  bool all_in = true;
  for (int pl = 0; pl < 5 && all_in; ++pl)
    for (int k = 0; k < 3; ++k)
      if (!(plane_eval(pl, in[k]) >= 0.0f)) { all_in = false; break; }
  if (all_in) { for (int k = 0; k < 3; ++k) out[k] = in[k]; return 3; }
  for (int pl = 0; pl < 5; ++pl) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
      const ClipV& p0 = a[i];
      const ClipV& p1 = a[(i + 1) % n];
      float d0 = plane_eval(pl, p0), d1 = plane_eval(pl, p1);
      bool in0 = d0 >= 0.0f, in1 = d1 >= 0.0f;
      if (in0) b[m++] = p0;
      if (in0 != in1) {
        float t = d0 / (d0 - d1);
        ClipV q;
        for (int c = 0; c < 4; ++c) q.c[c] = p0.c[c] + t * (p1.c[c] - p0.c[c]);
        b[m++] = q;
      }
    }
    n = m;
    for (int i = 0; i < n; ++i) a[i] = b[i];
    if (n < 3) return 0;
  }
  for (int i = 0; i < n; ++i) out[i] = a[i];
  return n;
}

static void raster_subtri(const ClipV v[3], int W, int H, int y_lo, int y_hi, uint32_t tid, uint64_t* zbuf) {
  i64 X[3], Y[3];
  float z[3];
  for (int k = 0; k < 3; ++k) {
    if (!(v[k].c[3] > 0.0f)) return;
    float nx = v[k].c[0] / v[k].c[3], ny = v[k].c[1] / v[k].c[3], nz = v[k].c[2] / v[k].c[3];
    if (!(std::fabs(nx) <= 64.0f) || !(std::fabs(ny) <= 64.0f) || !(nz == nz)) return;
    X[k] = std::llrint(((double)nx + 1.0) * ((double)W * 128.0));
    Y[k] = std::llrint(((double)ny + 1.0) * ((double)H * 128.0));
    z[k] = 0.5f * nz + 0.5f;
  }
  i64 area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
  if (area == 0) return;
  if (area < 0) { std::swap(X[1], X[2]); std::swap(Y[1], Y[2]); std::swap(z[1], z[2]); area = -area; }
  const bool tl0 = top_left(X[1], Y[1], X[2], Y[2]);
  const bool tl1 = top_left(X[2], Y[2], X[0], Y[0]);
  const bool tl2 = top_left(X[0], Y[0], X[1], Y[1]);
  i64 x0 = std::max<i64>(0, ceil_div(std::min({X[0], X[1], X[2]}) - 128, 256));
  i64 x1 = std::min<i64>(W - 1, floor_div(std::max({X[0], X[1], X[2]}) - 128, 256));
  i64 y0 = std::max<i64>(y_lo, ceil_div(std::min({Y[0], Y[1], Y[2]}) - 128, 256));
  i64 y1 = std::min<i64>(y_hi - 1, floor_div(std::max({Y[0], Y[1], Y[2]}) - 128, 256));
  const float fa = (float)area;
  for (i64 py = y0; py <= y1; ++py) {
    const i64 sy = 256 * py + 128;
    for (i64 px = x0; px <= x1; ++px) {
      const i64 sx = 256 * px + 128;
      i64 w0 = edge_fn(X[1], Y[1], X[2], Y[2], sx, sy);
      i64 w1 = edge_fn(X[2], Y[2], X[0], Y[0], sx, sy);
      i64 w2 = edge_fn(X[0], Y[0], X[1], Y[1], sx, sy);
      if (!edge_in(w0, tl0) || !edge_in(w1, tl1) || !edge_in(w2, tl2)) continue;
      float b1 = (float)w1 / fa, b2 = (float)w2 / fa;
      float zz = z[0] + b1 * (z[1] - z[0]);
      zz = zz + b2 * (z[2] - z[0]);
      if (!(zz < 1.0f)) continue;
      if (!(zz > 0.0f)) zz = 0.0f;
      uint32_t zb;
      std::memcpy(&zb, &zz, 4);
      uint64_t key = ((uint64_t)zb << 32) | tid;
      uint64_t& slot = zbuf[(size_t)py * W + px];
      if (key < slot) slot = key;
    }
  }
}

static void gbuffer_impl(const orc_scene* s, const orc_params* p, uint32_t* tri_id, double* pos, double* nrm,
                         uint32_t* mat) {
  const int W = p->width, H = p->height;
  float PV[16];
  matmul_f32(s->proj, s->view, PV);
  std::vector<uint64_t> zbuf((size_t)W * H, ~0ull);
  std::vector<uint32_t> base(s->n_instances + 1, 0);
  for (uint32_t i = 0; i < s->n_instances; ++i) base[i + 1] = base[i] + s->instances[i].n_tris;
  const int nthreads = std::max(1, p->threads);
  const int bands = std::max(1, std::min(H, nthreads * 2));
  parallel_for(nthreads, bands, [&](int band) {
    int ylo = H * band / bands, yhi = H * (band + 1) / bands;
    for (uint32_t i = 0; i < s->n_instances; ++i) {
      const orc_instance& in = s->instances[i];
      for (uint32_t t = 0; t < in.n_tris; ++t) {
        ClipV cv[3];
        for (int k = 0; k < 3; ++k) {
          const float* v = in.verts + 8 * (size_t)in.indices[3 * t + k];
          float w[4];
          xform_f32(in.model, v, w);
          w[3] = 1.0f;
          clip_f32(PV, w, cv[k].c);
        }
        ClipV poly[10];
        int n = clip_polygon(cv, poly);
        for (int k = 1; k + 1 < n; ++k) {
          ClipV tri[3] = {poly[0], poly[k], poly[k + 1]};
          raster_subtri(tri, W, H, ylo, yhi, base[i] + t, zbuf.data());
        }
      }
    }
  });
  std::vector<std::vector<double>> nms(s->n_instances, std::vector<double>(9));
  for (uint32_t i = 0; i < s->n_instances; ++i) normal_matrix(s->instances[i].model, nms[i].data());
  parallel_for(nthreads, H, [&](int y) {
    for (int x = 0; x < W; ++x) {
      size_t px = (size_t)y * W + x;
      uint64_t key = zbuf[px];
      if (key == ~0ull) {
        tri_id[px] = 0xffffffffu; mat[px] = 0xffffffffu;
        for (int c = 0; c < 3; ++c) { pos[3 * px + c] = 0; nrm[3 * px + c] = 0; }
        continue;
      }
      uint32_t t = (uint32_t)(key & 0xffffffffu);
      uint32_t i = (uint32_t)(std::upper_bound(base.begin(), base.end(), t) - base.begin()) - 1;
      const orc_instance& in = s->instances[i];
      uint32_t lt = t - base[i];
      double C[3][4], Wp[3][3], Nn[3][3];
      for (int k = 0; k < 3; ++k) {
        const float* v = in.verts + 8 * (size_t)in.indices[3 * lt + k];
        float w[4], c4[4];
        xform_f32(in.model, v, w);
        w[3] = 1.0f;
        clip_f32(PV, w, c4);
        for (int c = 0; c < 4; ++c) C[k][c] = c4[c];
        for (int c = 0; c < 3; ++c) Wp[k][c] = w[c];
        V3<double> nn = normalize(mat3_mul<double>(nms[i].data(), v + 3));
        Nn[k][0] = nn.x; Nn[k][1] = nn.y; Nn[k][2] = nn.z;
      }
      // Perspective-correct barycentrics of the pixel centre (GL smooth
      // interpolation): solve sum b_k (x_k - px w_k) = 0, sum b_k (y_k - py w_k) = 0.
      double pxn = (x + 0.5) * 2.0 / W - 1.0, pyn = (y + 0.5) * 2.0 / H - 1.0;
      double u[3], v[3];
      for (int k = 0; k < 3; ++k) { u[k] = C[k][0] - pxn * C[k][3]; v[k] = C[k][1] - pyn * C[k][3]; }
      double b[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
      double sb = b[0] + b[1] + b[2];
      if (sb != 0.0) { for (int k = 0; k < 3; ++k) b[k] /= sb; }
      else { b[0] = b[1] = b[2] = 1.0 / 3.0; }
      tri_id[px] = t;
      mat[px] = in.tri_material[lt];
      for (int c = 0; c < 3; ++c) {
        pos[3 * px + c] = b[0] * Wp[0][c] + b[1] * Wp[1][c] + b[2] * Wp[2][c];
        nrm[3 * px + c] = b[0] * Nn[0][c] + b[1] * Nn[1][c] + b[2] * Nn[2][c];
      }
    }
  });
}

}  // namespace

// ------------------------------------------------------------- C entry -----
extern "C" {

uint64_t orc_chain_texels(int32_t N, int32_t L) {
  uint64_t t = 0;
  for (int l = 1; l < L; ++l) { uint64_t s = (uint64_t)(N >> l); t += s * s * s; }
  return t;
}

int64_t orc_voxelize(const orc_scene* s, const orc_params* p, uint8_t* level0, uint32_t* counts) {
  return voxelize_impl<double>(s, p, level0, counts);
}
int64_t orc_voxelize_f32(const orc_scene* s, const orc_params* p, uint8_t* level0, uint32_t* counts) {
  return voxelize_impl<float>(s, p, level0, counts);
}

void orc_mipmap(const orc_params* p, const uint8_t* level0, uint8_t* chains) { mipmap_impl(p, level0, chains); }

int64_t orc_voxelize_cas(const orc_scene* s, const orc_params* p, int32_t order, uint64_t seed, uint8_t* level0) {
  return voxelize_cas_impl(s, p, order, seed, level0);
}

uint32_t orc_cas_avg(const float* rgba, int32_t n) {
  uint32_t cur = 0;
  for (int32_t i = 0; i < n; ++i) cur = cas_step(cur, rgba + 4 * i);
  return cur;
}

int64_t orc_voxelize_attr(const orc_scene* s, const orc_params* p, uint8_t* albedo, uint8_t* normal,
                          uint8_t* emission, uint32_t* counts) {
  uint8_t* out[3] = {albedo, normal, emission};
  int64_t rej = 0;
  for (int m = 1; m <= 3; ++m) {
    g_attr_mode = m;
    rej = voxelize_impl<double>(s, p, out[m - 1], m == 1 ? counts : nullptr);
  }
  g_attr_mode = 0;
  return rej;
}

// Deferred light injection (no reference counterpart), FP64: each occupied
// voxel lit at its centre from its mean attributes with the per-light terms
// of voxelize.frag:128-143; RGBA8 round to nearest.
void orc_inject(const orc_scene* s, const orc_params* p, const uint8_t* albedo, const uint8_t* normal,
                const uint8_t* emission, uint8_t* level0) {
  const int N = p->grid_res;
  const double k = 1.0 / 255.0, cube = (double)s->cube_size;
  const int nl = std::min<int>((int)s->n_lights, 10);
  parallel_for(std::max(1, p->threads), N, [&](int z) {
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const size_t i = 4 * (((size_t)z * N + y) * N + x);
        uint8_t* o = level0 + i;
        if (emission[i + 3] == 0) {
          o[0] = o[1] = o[2] = o[3] = 0;
          continue;
        }
        const V3<double> nn = normalize(V3<double>(normal[i] * k * 2.0 - 1.0, normal[i + 1] * k * 2.0 - 1.0,
                                                   normal[i + 2] * k * 2.0 - 1.0));
        const V3<double> pos((x + 0.5) * 2.0 / N - 1.0, (y + 0.5) * 2.0 / N - 1.0, (z + 0.5) * 2.0 / N - 1.0);
        V3<double> lit;
        for (int l = 0; l < nl; ++l) {
          const orc_point_light& L = s->lights[l];
          const V3<double> lp(L.position[0] / cube, L.position[1] / cube, L.position[2] / cube);
          const V3<double> dl = lp - pos;
          const double d = length(dl);
          const double cs = fmaxr(dot(nn, normalize(dl)), 0.0);
          lit = lit + V3<double>(L.color[0], L.color[1], L.color[2]) * (cs * (1.0 / (1.0 + d * d)) * L.intensity);
        }
        const V3<double> c = mulv(V3<double>(albedo[i] * k, albedo[i + 1] * k, albedo[i + 2] * k), lit) +
                             V3<double>(emission[i] * k, emission[i + 1] * k, emission[i + 2] * k);
        auto q = [](double v) { return (uint8_t)std::floor(clamp01(v) * 255.0 + 0.5); };
        o[0] = q(c.x);
        o[1] = q(c.y);
        o[2] = q(c.z);
        o[3] = albedo[i + 3];
      }
  });
}

int64_t orc_voxelize_hdr(const orc_scene* s, const orc_params* p, float* level0, uint32_t* counts) {
  return voxelize_impl<double>(s, p, nullptr, counts, level0);
}

void orc_mip_level_f(int32_t n_src, int32_t src_maps, const float* src, int32_t mip_mode, float* dst) {
  mip_level_f(n_src, src_maps, src, mip_mode, dst, (int)std::thread::hardware_concurrency());
}

void orc_trace_hdr(const orc_scene* s, const orc_params* p, const float* level0, const float* chains,
                   const uint32_t* tri_id, const double* pos, const double* nrm, const uint32_t* mat,
                   int32_t row_stride, float* out) {
  trace_impl<double>(s, p, nullptr, nullptr, tri_id, pos, nrm, mat, row_stride, out, level0, chains);
}

void orc_gbuffer(const orc_scene* s, const orc_params* p, uint32_t* tri_id, double* pos, double* nrm,
                 uint32_t* mat) {
  gbuffer_impl(s, p, tri_id, pos, nrm, mat);
}

void orc_trace(const orc_scene* s, const orc_params* p, const uint8_t* level0, const uint8_t* chains,
               const uint32_t* tri_id, const double* pos, const double* nrm, const uint32_t* mat,
               int32_t row_stride, float* out) {
  trace_impl<double>(s, p, level0, chains, tri_id, pos, nrm, mat, row_stride, out);
}
void orc_trace_f32(const orc_scene* s, const orc_params* p, const uint8_t* level0, const uint8_t* chains,
                   const uint32_t* tri_id, const double* pos, const double* nrm, const uint32_t* mat,
                   int32_t row_stride, float* out) {
  trace_impl<float>(s, p, level0, chains, tri_id, pos, nrm, mat, row_stride, out);
}

void orc_texture_lod(const orc_params* p, const uint8_t* level0, const uint8_t* chains, int32_t map,
                     const double* u, double lod, double* rgba) {
  Maps m{level0, chains, p->grid_res, p->levels, orc_chain_texels(p->grid_res, p->levels), p->mip_mode == ORC_MIP_ISO};
  V4<double> r = texture_lod<double>(m, map, V3<double>(u[0], u[1], u[2]), lod);
  rgba[0] = r.r; rgba[1] = r.g; rgba[2] = r.b; rgba[3] = r.a;
}

void orc_trace_cone(const orc_params* p, const uint8_t* level0, const uint8_t* chains, const double* origin,
                    const double* dir, double aperture, double max_dist, double* rgba, int32_t* steps) {
  Maps m{level0, chains, p->grid_res, p->levels, orc_chain_texels(p->grid_res, p->levels), p->mip_mode == ORC_MIP_ISO};
  ConeOut<double> c = trace_cone<double>(m, V3<double>(origin[0], origin[1], origin[2]),
                                         V3<double>(dir[0], dir[1], dir[2]), aperture, max_dist);
  rgba[0] = c.c.r; rgba[1] = c.c.g; rgba[2] = c.c.b; rgba[3] = c.c.a;
  if (steps) *steps = c.steps;
}

void orc_trace_stats(const orc_scene* s, const orc_params* p, const uint8_t* level0, const uint8_t* chains,
                     const uint32_t* tri_id, const double* pos, const double* nrm, const uint32_t* mat,
                     int32_t row_stride, float* out, uint64_t* stats) {
  for (auto& g : g_stats) g = 0;
  build_dilated(level0, p->grid_res, p->levels);
  g_stats_on = true;
  trace_impl<double>(s, p, level0, chains, tri_id, pos, nrm, mat, row_stride, out);
  g_stats_on = false;
  g_dilated.clear();
  g_dilated3.clear();
  for (int i = 0; i < kStatN; ++i) stats[i] = g_stats[i].load();
}

void orc_time_frame(const orc_scene* s, const orc_params* p, int32_t row_stride, double* ms) {
  typedef std::chrono::steady_clock clk;
  const int N = p->grid_res, W = p->width, H = p->height;
  std::vector<uint8_t> l0((size_t)N * N * N * 4);
  const int nm = p->mip_mode == ORC_MIP_ISO ? 1 : 6;
  std::vector<uint8_t> ch(4 * nm * orc_chain_texels(N, p->levels) + 4);
  std::vector<uint32_t> tid((size_t)W * H), mat((size_t)W * H);
  std::vector<double> pos((size_t)W * H * 3), nrm((size_t)W * H * 3);
  std::vector<float> out((size_t)W * H * 4);
  auto t0 = clk::now();
  voxelize_impl<float>(s, p, l0.data(), nullptr);
  auto t1 = clk::now();
  mipmap_impl(p, l0.data(), ch.data());
  auto t2 = clk::now();
  gbuffer_impl(s, p, tid.data(), pos.data(), nrm.data(), mat.data());
  auto t3 = clk::now();
  trace_impl<float>(s, p, l0.data(), ch.data(), tid.data(), pos.data(), nrm.data(), mat.data(), row_stride,
                    out.data());
  auto t4 = clk::now();
  ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
  ms[1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
  ms[2] = std::chrono::duration<double, std::milli>(t3 - t2).count();
  ms[3] = std::chrono::duration<double, std::milli>(t4 - t3).count();
}

}  // extern "C"
