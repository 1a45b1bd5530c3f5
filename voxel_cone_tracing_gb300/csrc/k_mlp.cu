// k_mlp.cu -- the learned diffuse term: a multiresolution hash encoding of
// the surface position plus normal and albedo, fed to a 4 x 64 ReLU MLP that
// predicts trace_diffuse (voxel_cone_tracing.frag:140-168) -- the average of
// the nine diffuse cones -- so that a frame can skip those cones.
//
// Network (the CPU oracle, oracle/vct_oracle_mlp.cpp, restates it in FP64):
//   input (64): 16 levels x 2 hash features, normalize(normal), albedo, 1, 0...
//   W1..W4: 64x64 + ReLU, W5: 16x64 (outputs 0..2 = RGB), no biases.
// Tensor cores: mma.sync m16n8k16 BF16 x BF16 -> FP32.  A warp owns 16 rows
// (samples / pixels); a layer's FP32 accumulator fragments are repacked in
// registers into the next layer's BF16 A fragments (the D layout of
// m16n8 tiles 2j, 2j+1 is the A layout of k-tile j), so activations never
// leave registers.  Weights live in shared memory as [out][in] (forward B
// operands) and [in][out] (backward B operands), rows padded to 72 bf16 so
// that the fragment loads are bank-conflict free.
// Training: per 16-row tile the warp runs forward, the MSE gradient, the
// backward pass (activation gradients by mma, ReLU masks from the stored
// forward fragments), the weight gradients dW_l = dH_l^T X_l by mma with
// movmatrix-transposed fragments (accumulated in shared memory, flushed once
// per CTA) and scatters the input gradient of the 32 hash features to the
// table gradient (float2 atomics).  Adam runs as a separate elementwise pass.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "vct_async.cuh"
#include "vct_internal.h"
#include "vct_math.cuh"

namespace vct {
namespace {

constexpr int kWS = 72;        // padded smem row stride of a 64-wide bf16 matrix
constexpr int kWSw = kWS / 2;  // ... in 32-bit words
constexpr int kW5TS = 24;      // padded row stride of W5^T ([64 in][16 out])
constexpr int kDWS = 72;       // padded row stride of the fp32 dW accumulators

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t trans8x8(uint32_t x) {
  uint32_t y;
  asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;\n" : "=r"(y) : "r"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

// Grid index of one corner of level l (dense when the level fits the table).
// Sparse levels use the spatial hash of the multiresolution hash encoding
// (Mueller, Evans, Schied, Keller: "Instant Neural Graphics Primitives with a
// Multiresolution Hash Encoding", SIGGRAPH 2022): per-axis primes 1,
// 2654435761, 805459861 combined by XOR, modulo the table size.
__device__ __forceinline__ uint32_t grid_index(const MlpParams& p, int l, int cx, int cy, int cz) {
  const int R = p.res[l];
  if ((p.dense_mask >> l) & 1) {
    cx = min(max(cx, 0), R);
    cy = min(max(cy, 0), R);
    cz = min(max(cz, 0), R);
    return (uint32_t)(cx + (R + 1) * (cy + (R + 1) * cz));
  }
  return ((uint32_t)cx * 1u ^ (uint32_t)cy * 2654435761u ^ (uint32_t)cz * 805459861u) & ((1u << p.log2_table) - 1u);
}

struct Corners {
  uint32_t idx[8];
  float w[8];
};

__device__ __forceinline__ void level_corners(const MlpParams& p, int l, V3 pos, Corners& c) {
  const float R = (float)p.res[l];
  const float x = pos.x * R, y = pos.y * R, z = pos.z * R;
  const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  const float ax = x - fx, ay = y - fy, az = z - fz;
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int bx = k & 1, by = (k >> 1) & 1, bz = k >> 2;
    c.idx[k] = grid_index(p, l, ix + bx, iy + by, iz + bz);
    c.w[k] = (bx ? ax : 1.0f - ax) * (by ? ay : 1.0f - ay) * (bz ? az : 1.0f - az);
  }
}

// Hash features of one (row, level) pair.
__device__ __forceinline__ float2 level_features(const MlpParams& p, int l, V3 pos) {
  Corners c;
  level_corners(p, l, pos, c);
  const size_t base = (size_t)l << p.log2_table;
  float f0 = 0.f, f1 = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t v = __ldg(reinterpret_cast<const unsigned int*>(p.table_bf) + base + c.idx[k]);
    f0 += c.w[k] * bf_lo(v);
    f1 += c.w[k] * bf_hi(v);
  }
  return make_float2(f0, f1);
}

// Shared-memory image of the network weights for the forward pass.
struct SmemW {
  uint32_t w[4][64 * kWSw];  // W1..W4 [out][in]
  uint32_t w5[16 * kWSw];    // W5 [out 16][in 64]
};
// ... and their transposes for the backward pass.
struct SmemWT {
  uint32_t wt[4][64 * kWSw];     // W1^T..W4^T [in][out]
  uint32_t w5t[64 * kW5TS / 2];  // W5^T [in 64][out 16]
};

__device__ void load_weights(const __nv_bfloat16* __restrict__ wg, SmemW& s, SmemWT* st) {
  const unsigned short* g = reinterpret_cast<const unsigned short*>(wg);
  unsigned short* w = reinterpret_cast<unsigned short*>(s.w);
  unsigned short* w5 = reinterpret_cast<unsigned short*>(s.w5);
  for (int i = threadIdx.x; i < 4 * 64 * 64; i += blockDim.x) {
    const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
    w[l * 64 * kWS + o * kWS + k] = g[i];
  }
  for (int i = threadIdx.x; i < 16 * 64; i += blockDim.x) w5[(i >> 6) * kWS + (i & 63)] = g[4 * 4096 + i];
  if (st) {
    unsigned short* wt = reinterpret_cast<unsigned short*>(st->wt);
    unsigned short* w5t = reinterpret_cast<unsigned short*>(st->w5t);
    for (int i = threadIdx.x; i < 4 * 64 * 64; i += blockDim.x) {
      const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
      wt[l * 64 * kWS + k * kWS + o] = g[i];
    }
    for (int i = threadIdx.x; i < 16 * 64; i += blockDim.x) w5t[(i & 63) * kW5TS + (i >> 6)] = g[4 * 4096 + i];
  }
}

// Fill the warp's 16 x 64 input tile E (bf16, stride kWS) for rows whose
// position / normal / albedo are given by get(row, pos, nrm, alb, valid).
template <class Get>
__device__ void build_inputs(const MlpParams& p, unsigned short* E, Get get) {
  const int lane = threadIdx.x & 31;
  const int row = lane & 15;
  V3 pos, nrm, alb;
  bool valid;
  get(row, pos, nrm, alb, valid);
  for (int l = (lane >> 4); l < 16; l += 2) {
    float2 f = valid ? level_features(p, l, pos) : make_float2(0.f, 0.f);
    const uint32_t v = pack_bf16(f.x, f.y);
    *reinterpret_cast<uint32_t*>(E + row * kWS + 2 * l) = v;
  }
  if (lane < 16) {
    const V3 n = normalize(nrm);
    float x[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) x[i] = 0.f;
    if (valid) {
      x[0] = n.x; x[1] = n.y; x[2] = n.z;
      x[3] = alb.x; x[4] = alb.y; x[5] = alb.z;
      x[6] = 1.0f;
    }
#pragma unroll
    for (int i = 0; i < 32; i += 2) *reinterpret_cast<uint32_t*>(E + row * kWS + 32 + i) = pack_bf16(x[i], x[i + 1]);
  }
  __syncwarp();
}

// The first layer's A fragments built directly in registers (no input tile
// in shared memory): lane (g, t) holds rows g and g + 8 of columns
// 16 kk + 2t, +1 (a[kk][0], a[kk][1]) and 16 kk + 8 + 2t, +1 (a[kk][2],
// a[kk][3]), i.e. hash levels t and t + 4 (kk 0), 8 + t and 12 + t (kk 1),
// inputs x[2t], x[2t + 1] (kk 2) and zeros.  The values and their bf16
// packing are those of build_inputs + load_a.
template <class Get>
__device__ __forceinline__ void build_a(const MlpParams& p, uint32_t (&a)[4][4], Get get) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    V3 pos, nrm, alb;
    bool valid;
    get(g + 8 * h, pos, nrm, alb, valid);
    const int lv[4] = {t, t + 4, 8 + t, 12 + t};
    uint32_t f[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2 v = valid ? level_features(p, lv[q], pos) : make_float2(0.f, 0.f);
      f[q] = pack_bf16(v.x, v.y);
    }
    a[0][h] = f[0];
    a[0][2 + h] = f[1];
    a[1][h] = f[2];
    a[1][2 + h] = f[3];
    float x0 = 0.f, x1 = 0.f;
    if (valid) {
      const V3 n = normalize(nrm);
      // x = (n.x, n.y, n.z, alb.x, alb.y, alb.z, 1, 0, 0, ...)
      x0 = t == 0 ? n.x : (t == 1 ? n.z : (t == 2 ? alb.y : 1.0f));
      x1 = t == 0 ? n.y : (t == 1 ? alb.x : (t == 2 ? alb.z : 0.0f));
    }
    a[2][h] = pack_bf16(x0, x1);
    a[2][2 + h] = pack_bf16(0.f, 0.f);
    a[3][h] = pack_bf16(0.f, 0.f);
    a[3][2 + h] = pack_bf16(0.f, 0.f);
  }
}

__device__ __forceinline__ void load_a(const unsigned short* E, uint32_t (&a)[4][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t* E32 = reinterpret_cast<const uint32_t*>(E);
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    a[kk][0] = E32[g * kWSw + 8 * kk + t];
    a[kk][1] = E32[(g + 8) * kWSw + 8 * kk + t];
    a[kk][2] = E32[g * kWSw + 8 * kk + 4 + t];
    a[kk][3] = E32[(g + 8) * kWSw + 8 * kk + 4 + t];
  }
}

// acc (16 x 64 fp32, D layout) = A (16 x 64) * W^T, W [out][in] rows stride kWSw words.
__device__ __forceinline__ void layer64(const uint32_t (&a)[4][4], const uint32_t* W, float (&acc)[8][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const uint32_t* r = W + (8 * nt + g) * kWSw + 8 * kk;
      mma16816(acc[nt], a[kk], r[t], r[4 + t]);
    }
}

// D fragments (16 x 64) -> A fragments, optionally through ReLU.
__device__ __forceinline__ void d_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4], bool relu) {
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const float* e = acc[2 * kk];
    const float* o = acc[2 * kk + 1];
    if (relu) {
      a[kk][0] = pack_bf16(fmaxf(e[0], 0.f), fmaxf(e[1], 0.f));
      a[kk][1] = pack_bf16(fmaxf(e[2], 0.f), fmaxf(e[3], 0.f));
      a[kk][2] = pack_bf16(fmaxf(o[0], 0.f), fmaxf(o[1], 0.f));
      a[kk][3] = pack_bf16(fmaxf(o[2], 0.f), fmaxf(o[3], 0.f));
    } else {
      a[kk][0] = pack_bf16(e[0], e[1]);
      a[kk][1] = pack_bf16(e[2], e[3]);
      a[kk][2] = pack_bf16(o[0], o[1]);
      a[kk][3] = pack_bf16(o[2], o[3]);
    }
  }
}

// Output layer: y (16 x 16 fp32, D layout, 2 n-tiles) = A * W5^T.
__device__ __forceinline__ void layer_out(const uint32_t (&a)[4][4], const uint32_t* W5, float (&y)[2][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) y[nt][0] = y[nt][1] = y[nt][2] = y[nt][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      const uint32_t* r = W5 + (8 * nt + g) * kWSw + 8 * kk;
      mma16816(y[nt], a[kk], r[t], r[4 + t]);
    }
}

// ------------------------------------------------------------- training ----
struct TrainSmem {
  SmemW w;
  SmemWT wt;
  float dw[4][64 * kDWS];
  float dw5[16 * kDWS];
  unsigned short E[8][16 * kWS];
  float pos[8][16][3];
};

// Weight gradient of one layer: dW[out][in] += dH^T (16 rows) * X.
__device__ __forceinline__ void accum_dw(const uint32_t (&dh)[4][4], const uint32_t (&x)[4][4], int m_tiles,
                                         float* dw) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t bx[8][2];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int kk = nt >> 1;
    bx[nt][0] = trans8x8(x[kk][(nt & 1) ? 2 : 0]);
    bx[nt][1] = trans8x8(x[kk][(nt & 1) ? 3 : 1]);
  }
  for (int mt = 0; mt < m_tiles; ++mt) {
    const uint32_t a[4] = {trans8x8(dh[mt][0]), trans8x8(dh[mt][2]), trans8x8(dh[mt][1]), trans8x8(dh[mt][3])};
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(acc, a, bx[nt][0], bx[nt][1]);
      float* r0 = dw + (16 * mt + g) * kDWS + 8 * nt + 2 * t;
      float* r1 = r0 + 8 * kDWS;
      atomicAdd(r0, acc[0]);
      atomicAdd(r0 + 1, acc[1]);
      atomicAdd(r1, acc[2]);
      atomicAdd(r1 + 1, acc[3]);
    }
  }
}

// Backward through one 64x64 layer: dX = dH * W (W^T stored [in][out] as wt),
// masked by (X > 0) when X is a ReLU output.
__device__ __forceinline__ void back64(const uint32_t (&dh)[4][4], const uint32_t* wt, const uint32_t (&xmask)[4][4],
                                       bool mask, float (&acc)[8][4]) {
  layer64(dh, wt, acc);
  if (!mask) return;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int kk = nt >> 1;
    const uint32_t m0 = xmask[kk][(nt & 1) ? 2 : 0], m1 = xmask[kk][(nt & 1) ? 3 : 1];
    if (!(bf_lo(m0) > 0.f)) acc[nt][0] = 0.f;
    if (!(bf_hi(m0) > 0.f)) acc[nt][1] = 0.f;
    if (!(bf_lo(m1) > 0.f)) acc[nt][2] = 0.f;
    if (!(bf_hi(m1) > 0.f)) acc[nt][3] = 0.f;
  }
}

__global__ void __launch_bounds__(256, 1) k_mlp_train(MlpParams p, MlpBatch b, float* __restrict__ loss_out) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
  load_weights(p.w_bf, S.w, &S.wt);
  for (int i = threadIdx.x; i < 4 * 64 * kDWS; i += blockDim.x) (&S.dw[0][0])[i] = 0.f;
  for (int i = threadIdx.x; i < 16 * kDWS; i += blockDim.x) S.dw5[i] = 0.f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int nwarps = blockDim.x >> 5;
  unsigned short* E = S.E[warp];
  float loss = 0.f;
  const float inv_n = 1.0f / (float)b.n;
  for (int tile = blockIdx.x * nwarps + warp; tile * 16 < b.n; tile += gridDim.x * nwarps) {
    const int row0 = tile * 16;
    build_inputs(p, E, [&](int row, V3& pos, V3& nrm, V3& alb, bool& valid) {
      const int s = row0 + row;
      valid = s < b.n;
      const int j = valid ? s : 0;
      const float* q = b.samples + (size_t)(b.first + j) % b.total * 12;
      pos = v3(q[0], q[1], q[2]);
      nrm = v3(q[3], q[4], q[5]);
      alb = v3(q[6], q[7], q[8]);
      if ((lane >> 4) == 0) {
        S.pos[warp][row][0] = pos.x; S.pos[warp][row][1] = pos.y; S.pos[warp][row][2] = pos.z;
      }
    });
    uint32_t x0[4][4], h1[4][4], h2[4][4], h3[4][4], h4[4][4];
    float acc[8][4];
    load_a(E, x0);
    layer64(x0, S.w.w[0], acc); d_to_a(acc, h1, true);
    layer64(h1, S.w.w[1], acc); d_to_a(acc, h2, true);
    layer64(h2, S.w.w[2], acc); d_to_a(acc, h3, true);
    layer64(h3, S.w.w[3], acc); d_to_a(acc, h4, true);
    float y[2][4];
    layer_out(h4, S.w.w5, y);
    // MSE gradient on the 3 valid outputs (cols 0..2 live in n-tile 0, t <= 1).
    float dy[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = row0 + g + (e >= 2 ? 8 : 0);
      const int c = 2 * t + (e & 1);
      if (c < 3 && r < b.n) {
        const float tg = b.samples[(size_t)(b.first + r) % b.total * 12 + 9 + c];
        const float d = y[0][e] - tg;
        loss += d * d * inv_n;
        dy[e] = 2.0f * d * inv_n;
      }
    }
    uint32_t dya[4][4];
    dya[0][0] = pack_bf16(dy[0], dy[1]);
    dya[0][1] = pack_bf16(dy[2], dy[3]);
    dya[0][2] = 0u;
    dya[0][3] = 0u;
    // dH4 = dY * W5 (masked by h4 > 0): one k-tile, B = W5^T [in][out].
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
      const uint32_t* r = S.wt.w5t + (8 * nt + g) * (kW5TS / 2);
      mma16816(acc[nt], dya[0], r[t], r[4 + t]);
      const int kk = nt >> 1;
      const uint32_t m0 = h4[kk][(nt & 1) ? 2 : 0], m1 = h4[kk][(nt & 1) ? 3 : 1];
      if (!(bf_lo(m0) > 0.f)) acc[nt][0] = 0.f;
      if (!(bf_hi(m0) > 0.f)) acc[nt][1] = 0.f;
      if (!(bf_lo(m1) > 0.f)) acc[nt][2] = 0.f;
      if (!(bf_hi(m1) > 0.f)) acc[nt][3] = 0.f;
    }
    accum_dw(dya, h4, 1, S.dw5);
    uint32_t dh[4][4];
    d_to_a(acc, dh, false);                  // dH4
    accum_dw(dh, h3, 4, S.dw[3]);
    back64(dh, S.wt.wt[3], h3, true, acc);    // dH3
    d_to_a(acc, dh, false);
    accum_dw(dh, h2, 4, S.dw[2]);
    back64(dh, S.wt.wt[2], h2, true, acc);    // dH2
    d_to_a(acc, dh, false);
    accum_dw(dh, h1, 4, S.dw[1]);
    back64(dh, S.wt.wt[1], h1, true, acc);    // dH1
    d_to_a(acc, dh, false);
    accum_dw(dh, x0, 4, S.dw[0]);
    back64(dh, S.wt.wt[0], x0, false, acc);   // dE (cols 0..31 = hash features)
    // Scatter: lane holds levels 4*nt + t (nt < 4) for rows g and g + 8.
#pragma unroll 1
    for (int nt = 0; nt < 4; ++nt) {
      const int l = 4 * nt + t;
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int row = g + 8 * h;
        if (row0 + row >= b.n) continue;
        const float d0 = acc[nt][2 * h], d1 = acc[nt][2 * h + 1];
        if (d0 == 0.f && d1 == 0.f) continue;
        Corners c;
        level_corners(p, l, v3(S.pos[warp][row][0], S.pos[warp][row][1], S.pos[warp][row][2]), c);
        float2* gl = p.table_grad + ((size_t)l << p.log2_table);
#pragma unroll
        for (int k = 0; k < 8; ++k) atomicAdd(gl + c.idx[k], make_float2(c.w[k] * d0, c.w[k] * d1));
      }
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 4 * 4096; i += blockDim.x) {
    const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
    const float v = S.dw[l][o * kDWS + k];
    if (v != 0.f) atomicAdd(p.w_grad + i, v);
  }
  for (int i = threadIdx.x; i < 16 * 64; i += blockDim.x) {
    const float v = S.dw5[(i >> 6) * kDWS + (i & 63)];
    if (v != 0.f) atomicAdd(p.w_grad + 4 * 4096 + i, v);
  }
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if (lane == 0 && loss_out) atomicAdd(loss_out, loss);
}

// Adam on a flat parameter array; refreshes the bf16 copy and clears grads.
__global__ void k_adam(float* __restrict__ prm, float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ prm_bf, size_t n, AdamStep a) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = grad[i] + a.l2 * prm[i];
    const float mi = a.beta1 * m[i] + (1.0f - a.beta1) * gi;
    const float vi = a.beta2 * v[i] + (1.0f - a.beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = prm[i] - a.lr * (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
    prm[i] = pi;
    grad[i] = 0.f;
    prm_bf[i] = __float2bfloat16_rn(pi);
  }
}

// Deterministic init: table U(-1e-4, 1e-4), weights U(-s, s), s = sqrt(6/fan_in)
// (hash-based generator, independent of launch shape).
__device__ __forceinline__ float uniform01(uint64_t key) {
  key ^= key >> 33; key *= 0xff51afd7ed558ccdull; key ^= key >> 33; key *= 0xc4ceb9fe1a85ec53ull; key ^= key >> 33;
  return (float)(key >> 40) * (1.0f / 16777216.0f);
}

__global__ void k_mlp_init(float* prm, __nv_bfloat16* prm_bf, size_t n, float scale, uint64_t seed) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float v = (2.0f * uniform01(seed * 0x9e3779b97f4a7c15ull + i) - 1.0f) * scale;
    prm[i] = v;
    prm_bf[i] = __float2bfloat16_rn(v);
  }
}

// ------------------------------------------------------------ inference ----
struct InferSmem {
  SmemW w;
  unsigned short E[8][16 * kWS];
};

__global__ void __launch_bounds__(256, 4) k_mlp_infer(MlpParams p, SceneParams sp, const float4* __restrict__ gb_pos,
                                                   const float4* __restrict__ gb_nrm, int n_px,
                                                   float4* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemW& W = *reinterpret_cast<SmemW*>(smem_raw);
  load_weights(p.w_bf, W, nullptr);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int nwarps = blockDim.x >> 5;
  const float inv_cube = 1.0f / sp.cube_size;
  for (int tile = blockIdx.x * nwarps + warp; tile * 16 < n_px; tile += gridDim.x * nwarps) {
    const int row0 = tile * 16;
    uint32_t x[4][4], h[4][4];
    build_a(p, x, [&](int row, V3& pos, V3& nrm, V3& alb, bool& valid) {
      const int px = row0 + row;
      valid = false;
      pos = nrm = alb = v3(0.f, 0.f, 0.f);
      if (px < n_px) {
        const float4 a = gb_pos[px], c = gb_nrm[px];
        if (__float_as_uint(c.w) != 0xffffffffu) {
          valid = true;
          pos = v3(a.x * inv_cube, a.y * inv_cube, a.z * inv_cube) * 0.5f + v3(0.5f, 0.5f, 0.5f);
          nrm = v3(c.x, c.y, c.z);
          const vct_material_data& m = sp.materials[__float_as_uint(a.w)];
          alb = v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
        }
      }
    });
    float acc[8][4];
    layer64(x, W.w[0], acc); d_to_a(acc, h, true);
    layer64(h, W.w[1], acc); d_to_a(acc, x, true);
    layer64(x, W.w[2], acc); d_to_a(acc, h, true);
    layer64(h, W.w[3], acc); d_to_a(acc, x, true);
    float y[2][4];
    layer_out(x, W.w5, y);
    // lanes t = 0 hold cols 0,1; t = 1 holds col 2 -> gather per row
    const float c2_lo = __shfl_sync(0xffffffffu, y[0][0], (lane & ~3) | 1);
    const float c2_hi = __shfl_sync(0xffffffffu, y[0][2], (lane & ~3) | 1);
    if (t == 0) {
      const int r0 = row0 + g, r1 = row0 + g + 8;
      if (r0 < n_px) out[r0] = make_float4(y[0][0], y[0][1], c2_lo, 0.f);
      if (r1 < n_px) out[r1] = make_float4(y[0][2], y[0][3], c2_hi, 0.f);
    }
    __syncwarp();
  }
}

// Forward of explicit samples (tests, evaluation): rows of 12 floats
// (pos, normal, albedo, ignored target).
__global__ void __launch_bounds__(256) k_mlp_eval(MlpParams p, const float* __restrict__ samples, int n,
                                                  float* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
  load_weights(p.w_bf, S.w, nullptr);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int nwarps = blockDim.x >> 5;
  unsigned short* E = S.E[warp];
  for (int tile = blockIdx.x * nwarps + warp; tile * 16 < n; tile += gridDim.x * nwarps) {
    const int row0 = tile * 16;
    build_inputs(p, E, [&](int row, V3& pos, V3& nrm, V3& alb, bool& valid) {
      const int s = row0 + row;
      valid = s < n;
      const float* q = samples + (size_t)(valid ? s : 0) * 12;
      pos = v3(q[0], q[1], q[2]);
      nrm = v3(q[3], q[4], q[5]);
      alb = v3(q[6], q[7], q[8]);
    });
    uint32_t x[4][4], h[4][4];
    float acc[8][4];
    load_a(E, x);
    layer64(x, S.w.w[0], acc); d_to_a(acc, h, true);
    layer64(h, S.w.w[1], acc); d_to_a(acc, x, true);
    layer64(x, S.w.w[2], acc); d_to_a(acc, h, true);
    layer64(h, S.w.w[3], acc); d_to_a(acc, x, true);
    float y[2][4];
    layer_out(x, S.w.w5, y);
    const float c2_lo = __shfl_sync(0xffffffffu, y[0][0], (lane & ~3) | 1);
    const float c2_hi = __shfl_sync(0xffffffffu, y[0][2], (lane & ~3) | 1);
    if (t == 0) {
      const int r0 = row0 + g, r1 = row0 + g + 8;
      if (r0 < n) { out[3 * r0] = y[0][0]; out[3 * r0 + 1] = y[0][1]; out[3 * r0 + 2] = c2_lo; }
      if (r1 < n) { out[3 * r1] = y[0][2]; out[3 * r1 + 1] = y[0][3]; out[3 * r1 + 2] = c2_hi; }
    }
    __syncwarp();
  }
}

// ---- forward on the 5th-generation tensor cores ----------------------------
// Warp-specialised, one persistent CTA per SM:
//  * 24 encoder warps in 3 groups of 8.  A group encodes one 128-row tile at
//    a time into a shared-memory stage (6 stages of 128 x 64 BF16): warp w of
//    the group encodes rows 16w..16w+15 with the lane layout of the warp-tile
//    kernels (lane (g, t): rows g and g + 8, hash levels t, t + 4, 8 + t,
//    12 + t), so each lane gathers what it gathers there; then every encoder
//    thread arrives on the stage's `full` barrier.  Group k takes the CTA's
//    tiles k, k + 3, k + 6, ...; an encoder never waits for the network,
//    only for a stage to be free again.
//  * 8 epilogue warps (two threads per row: warp e reads TMEM lanes
//    32(e%4)..+31, columns 32(e/4)..+31), one of whose threads issues the
//    MMAs.  They run the
//    network over batches of 3 tiles (one per group) with 3 TMEM
//    accumulators: for each layer and tile, wait for that tile's MMAs, read
//    the accumulator (tcgen05.ld), apply ReLU, pack to BF16 and write the
//    next layer's activations over the tile's stage (its MMAs are done with
//    it), synchronise the 128 epilogue threads, and issue the tile's next
//    layer -- which runs while the epilogue drains the next tile.  After the
//    last layer the stage goes back to its encoder group (`empty`).
// Operands in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices: element (r, k) at (r/8)*512 + (k/8)*64 +
// (r%8)*8 + k%8); one tcgen05.mma kind::f16 per K=16 step, M=128, N=64 (the
// output layer N=16, 3 columns used), FP32 accumulators.  Every wait is
// bounded: a wait that gives up sets FrameStatus::async_timeout and the CTA
// leaves after waiting (bounded) for its MMAs still in flight.
constexpr int kTcRows = 128;
constexpr int kWsGroups = 3;
constexpr int kWsEncThreads = kWsGroups * 256;
constexpr int kWsEpiThreads = 256;
constexpr int kWsThreads = kWsEncThreads + kWsEpiThreads;
constexpr int kWsStages = 2 * kWsGroups;
constexpr uint32_t kTcCols = 256;  // TMEM columns: 3 accumulators of 64
constexpr uint32_t kCoreLbo = 128, kCoreSbo = 1024;

__device__ __forceinline__ int umma_elem(int r, int k) { return (r >> 3) * 512 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); }

struct TcSmem {
  unsigned short w[4][64 * 64];                 // W1..W4 (rows = outputs), canonical layout
  unsigned short w5[16 * 64];                   // W5 (16 output rows, 3 used)
  unsigned short a[kWsStages][kTcRows * 64];    // per stage: a tile's inputs, then its activations
  uint64_t full[kWsStages];                     // encoder group -> issuer (256 arrivals)
  uint64_t empty[kWsStages];                    // issuer -> encoder group (1 arrival)
  uint64_t mma[kWsGroups];                      // tcgen05.commit of a batch slot's layer
  uint32_t tmem;
  int abort;
};

__device__ __forceinline__ uint4 pack8(const float* x) {
  return make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
}

// bar.sync of the epilogue threads (named barrier 1) with an OR of `v`.
__device__ __forceinline__ bool epi_sync_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.or.pred q, 1, 256, p;\n"
      " selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)v)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Input row `row` of the batch: texture-space position, normal, albedo.
template <bool FROM_GBUF>
__device__ __forceinline__ void tc_input(const SceneParams& sp, const float4* __restrict__ gb_pos,
                                         const float4* __restrict__ gb_nrm, const float* __restrict__ samples, int n,
                                         float inv_cube, int r, V3& pos, V3& nrm, V3& alb, bool& valid) {
  valid = false;
  pos = nrm = alb = v3(0.f, 0.f, 0.f);
  if (r >= n) return;
  if (FROM_GBUF) {
    const float4 a = gb_pos[r], c = gb_nrm[r];
    if (__float_as_uint(c.w) != 0xffffffffu) {
      valid = true;
      pos = v3(a.x * inv_cube, a.y * inv_cube, a.z * inv_cube) * 0.5f + v3(0.5f, 0.5f, 0.5f);
      nrm = v3(c.x, c.y, c.z);
      const vct_material_data& m = sp.materials[__float_as_uint(a.w)];
      alb = v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    }
  } else {
    const float* q = samples + (size_t)r * 12;
    valid = true;
    pos = v3(q[0], q[1], q[2]);
    nrm = v3(q[3], q[4], q[5]);
    alb = v3(q[6], q[7], q[8]);
  }
}

template <bool FROM_GBUF>
__global__ void __launch_bounds__(kWsThreads, 1)
    k_mlp_fwd_tc(MlpParams p, SceneParams sp, const float4* __restrict__ gb_pos, const float4* __restrict__ gb_nrm,
                 const float* __restrict__ samples, int n, float4* __restrict__ out4, float* __restrict__ out3,
                 FrameStatus* status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned short* gw = reinterpret_cast<const unsigned short*>(p.w_bf);
  for (int i = tid; i < 4 * 64 * 64; i += kWsThreads) {
    const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
    S.w[l][umma_elem(o, k)] = gw[i];
  }
  for (int i = tid; i < 16 * 64; i += kWsThreads) S.w5[umma_elem(i >> 6, i & 63)] = gw[4 * 4096 + i];
  if (tid == 0) {
    for (int s = 0; s < kWsStages; ++s) {
      mbar_init(&S.full[s], 256);
      mbar_init(&S.empty[s], 1);
    }
    for (int j = 0; j < kWsGroups; ++j) mbar_init(&S.mma[j], 1);
    S.abort = 0;
    mbar_init_fence();
  }
  const int epi_warp0 = kWsEncThreads / 32;
  if (warp == epi_warp0) tc_alloc(&S.tmem, kTcCols);
  fence_async_smem();  // the weights, for the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const int tiles = (n + kTcRows - 1) / kTcRows;
  const float inv_cube = 1.0f / sp.cube_size;
  // The CTA's it-th tile is blockIdx.x + it * gridDim.x; its stage it % 6.
  if (tid < kWsEncThreads) {
    // ---------------------------------------------------------- encoders --
    const int grp = warp >> 3, wi = warp & 7, g = lane >> 2, t = lane & 3;
    for (int it = grp;; it += kWsGroups) {
      const int tile = blockIdx.x + it * gridDim.x;
      if (tile >= tiles) break;
      const int s = it % kWsStages, use = it / kWsStages;
      if (use > 0 && !mbar_wait(&S.empty[s], (use - 1) & 1)) {
        atomicOr(&status->async_timeout, 1u);
        S.abort = 1;
        break;
      }
      if (*(volatile int*)&S.abort) break;
      uint32_t* a32 = reinterpret_cast<uint32_t*>(S.a[s]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = 16 * wi + g + 8 * h;
        V3 pos, nrm, alb;
        bool valid;
        tc_input<FROM_GBUF>(sp, gb_pos, gb_nrm, samples, n, inv_cube, tile * kTcRows + row, pos, nrm, alb, valid);
        const int lv[4] = {t, t + 4, 8 + t, 12 + t};
        uint32_t f[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float2 v = valid ? level_features(p, lv[q], pos) : make_float2(0.f, 0.f);
          f[q] = pack_bf16(v.x, v.y);
        }
        float x0 = 0.f, x1 = 0.f;
        if (valid) {
          const V3 nn = normalize(nrm);
          // x = (n.x, n.y, n.z, alb.x, alb.y, alb.z, 1, 0, 0, ...)
          x0 = t == 0 ? nn.x : (t == 1 ? nn.z : (t == 2 ? alb.y : 1.0f));
          x1 = t == 0 ? nn.y : (t == 1 ? alb.x : (t == 2 ? alb.z : 0.0f));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) a32[umma_elem(row, 2 * lv[q]) >> 1] = f[q];
        a32[umma_elem(row, 32 + 2 * t) >> 1] = pack_bf16(x0, x1);
#pragma unroll
        for (int c = 0; c < 3; ++c) a32[umma_elem(row, 40 + 8 * c + 2 * t) >> 1] = 0u;
      }
      fence_async_smem();
      mbar_arrive(&S.full[s]);
    }
  } else {
    // ---------------------------------------------------------- epilogue --
    const int e = tid - kWsEncThreads, ew = e >> 5, row = 32 * (ew & 3) + lane, ch = ew >> 2;
    const uint32_t tmem = S.tmem;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * (ew & 3)) << 16);
    const uint32_t idesc64 = tc_idesc_bf16(kTcRows, 64), idesc16 = tc_idesc_bf16(kTcRows, 16);
    uint32_t mma_phase = 0;  // bit j: parity of slot j's next commit (flipped by each completed wait)
    uint32_t pending = 0;    // bit j: an MMA group of slot j not yet waited for (issuer)
    bool bad = false;
    auto issue = [&](int j, int s, int layer) {  // issuer only
      tc_fence_after();
      const unsigned short* W = layer < 4 ? S.w[layer] : S.w5;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc_mma_bf16(tmem + 64u * j, tc_smem_desc(S.a[s] + 128 * kk, kCoreLbo, kCoreSbo),
                    tc_smem_desc(W + 128 * kk, kCoreLbo, kCoreSbo), layer < 4 ? idesc64 : idesc16, kk > 0 ? 1u : 0u);
      tc_commit(&S.mma[j]);
      pending |= 1u << j;
    };
    for (int b = 0; !bad; ++b) {
      int nb = 0;
      while (nb < kWsGroups && blockIdx.x + (kWsGroups * b + nb) * gridDim.x < tiles) ++nb;
      if (nb == 0) break;
      bool ok = true;
      if (e == 0) {
        for (int j = 0; j < nb && ok; ++j) {
          const int it = kWsGroups * b + j;
          ok = mbar_wait(&S.full[it % kWsStages], (it / kWsStages) & 1);
          if (ok) issue(j, it % kWsStages, 0);
        }
      }
      if (epi_sync_or(!ok)) {
        bad = true;
        break;
      }
      for (int layer = 0; layer < 5 && !bad; ++layer) {
        for (int j = 0; j < nb; ++j) {
          const int it = kWsGroups * b + j, s = it % kWsStages;
          ok = mbar_wait(&S.mma[j], (mma_phase >> j) & 1);
          if (ok) {
            mma_phase ^= 1u << j;
            pending &= ~(1u << j);
            tc_fence_after();
            const uint32_t acc = lane_addr + 64u * j;
            if (layer < 4) {
              float v[16], w[16];
              uint4* arow = reinterpret_cast<uint4*>(S.a[s]);
              tc_ld16(acc + 32 * ch, v);
              tc_ld16(acc + 32 * ch + 16, w);
              tc_wait_ld();
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                v[i] = fmaxf(v[i], 0.f);
                w[i] = fmaxf(w[i], 0.f);
              }
              arow[umma_elem(row, 32 * ch) / 8] = pack8(v);
              arow[umma_elem(row, 32 * ch + 8) / 8] = pack8(v + 8);
              arow[umma_elem(row, 32 * ch + 16) / 8] = pack8(w);
              arow[umma_elem(row, 32 * ch + 24) / 8] = pack8(w + 8);
              fence_async_smem();
            } else if (ch == 0) {
              float v[16];
              tc_ld16(acc, v);
              tc_wait_ld();
              const int r = (blockIdx.x + it * gridDim.x) * kTcRows + row;
              if (r < n) {
                if (FROM_GBUF) out4[r] = make_float4(v[0], v[1], v[2], 0.f);
                else {
                  out3[3 * r] = v[0];
                  out3[3 * r + 1] = v[1];
                  out3[3 * r + 2] = v[2];
                }
              }
            }
          }
          tc_fence_before();
          if (epi_sync_or(!ok)) {
            bad = true;
            break;
          }
          if (e == 0) {
            if (layer < 4) issue(j, s, layer + 1);
            else mbar_arrive(&S.empty[s]);  // the tile's last MMAs are done with its stage
          }
        }
      }
    }
    if (bad) {
      if (e == 0) atomicOr(&status->async_timeout, 1u);
      S.abort = 1;
    }
    if (e == 0)  // MMA groups still in flight
      for (int j = 0; j < kWsGroups; ++j)
        if ((pending >> j) & 1) mbar_wait(&S.mma[j], (mma_phase >> j) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == epi_warp0) {
    tc_fence_after();
    tc_dealloc(S.tmem, kTcCols);
  }
}

int sm_count() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

size_t mlp_train_smem() { return sizeof(TrainSmem); }
size_t mlp_infer_smem() { return sizeof(InferSmem); }

cudaError_t launch_mlp_init(float* prm, __nv_bfloat16* prm_bf, size_t n, float scale, uint64_t seed, cudaStream_t st) {
  k_mlp_init<<<sm_count() * 4, 256, 0, st>>>(prm, prm_bf, n, scale, seed);
  return cudaGetLastError();
}

cudaError_t launch_mlp_train(const MlpParams& p, const MlpBatch& b, float* loss, cudaStream_t st) {
  const size_t smem = sizeof(TrainSmem);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tiles = (b.n + 15) / 16;
  int grid = sm_count();
  if (grid * 8 > tiles) grid = (tiles + 7) / 8;
  if (grid < 1) grid = 1;
  k_mlp_train<<<grid, 256, smem, st>>>(p, b, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* prm, float* grad, float* m, float* v, __nv_bfloat16* prm_bf, size_t n,
                        const AdamStep& a, cudaStream_t st) {
  k_adam<<<sm_count() * 8, 256, 0, st>>>(prm, grad, m, v, prm_bf, n, a);
  return cudaGetLastError();
}

namespace {

template <bool FROM_GBUF>
cudaError_t run_fwd_tc(const MlpParams& p, const SceneParams& sp, const float4* gb_pos, const float4* gb_nrm,
                       const float* samples, int n, float4* out4, float* out3, cudaStream_t st, FrameStatus* status) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = sizeof(TcSmem) + 128;
  auto kern = k_mlp_fwd_tc<FROM_GBUF>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // One CTA per SM (it holds kTcCols of the SM's 512 TMEM columns).
  const int tiles = (n + kTcRows - 1) / kTcRows;
  kern<<<std::max(1, std::min(tiles, sm_count())), kWsThreads, smem, st>>>(p, sp, gb_pos, gb_nrm, samples, n, out4,
                                                                         out3, status);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_mlp_infer(const MlpParams& p, const SceneParams& sp, const float4* gb_pos, const float4* gb_nrm,
                             int n_px, float4* out, cudaStream_t st, bool tc, FrameStatus* status) {
  if (tc) return run_fwd_tc<true>(p, sp, gb_pos, gb_nrm, nullptr, n_px, out, nullptr, st, status);
  const size_t smem = sizeof(SmemW);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // Persistent: every CTA slot the SMs can hold (the gathers of the hash
  // encoding need the warps to hide their latency).
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_infer, 256, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  k_mlp_infer<<<sm_count() * per_sm, 256, smem, st>>>(p, sp, gb_pos, gb_nrm, n_px, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_eval(const MlpParams& p, const float* samples, int n, float* out, cudaStream_t st, bool tc,
                            FrameStatus* status) {
  if (tc) {
    SceneParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.cube_size = 1.0f;
    return run_fwd_tc<false>(p, sp, nullptr, nullptr, samples, n, nullptr, out, st, status);
  }
  const size_t smem = sizeof(InferSmem);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int grid = sm_count() * 2;
  const int tiles = (n + 15) / 16;
  if (grid * 8 > tiles) grid = (tiles + 7) / 8;
  if (grid < 1) grid = 1;
  k_mlp_eval<<<grid, 256, smem, st>>>(p, samples, n, out);
  return cudaGetLastError();
}

}  // namespace vct
