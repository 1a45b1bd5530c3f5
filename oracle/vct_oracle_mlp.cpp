// vct_oracle_mlp.cpp -- CPU oracle (test infrastructure only) of the learned
// diffuse term: multiresolution hash encoding of the surface position +
// normal + albedo -> 4 x 64 ReLU MLP -> RGB, its MSE loss and its exact FP64
// gradients.  The reference has no learned component (the MLP stands in for
// trace_diffuse, voxel_cone_tracing.frag:140-168); this file pins the CUDA
// training kernels' forward and backward passes.
//
// Encoding (per level l of 16): resolution N_l = floor(N_min * b^l),
// b = (N_max / N_min)^(1/15); x = p * N_l; the 8 corners of floor(x) are
// looked up densely (c.x + c.y (N_l+1) + c.z (N_l+1)^2, corners clamped to
// N_l) when (N_l+1)^3 <= T, else by the spatial hash
// (c.x * 1 ^ c.y * 2654435761 ^ c.z * 805459861) mod T of Mueller et al.,
// "Instant Neural Graphics Primitives" (SIGGRAPH 2022); trilinear weights
// from frac(x).  Input vector (64): 32 hash features, normalize(normal),
// albedo, a constant 1, zeros.  Layers: W1..W4 64x64 (ReLU), W5 16x64 (first
// 3 outputs used, linear).  No biases.  Loss = mean over samples of the sum
// over RGB of (y - target)^2.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "vct_oracle.h"

namespace {

struct Enc {
  uint32_t idx[16][8];
  double w[16][8];
};

inline int level_res(const orc_mlp_config* c, int l) {
  const double b = std::exp((std::log((double)c->n_max) - std::log((double)c->n_min)) / (c->levels - 1));
  return (int)std::floor((double)c->n_min * std::pow(b, l) + 1e-6);
}

void encode(const orc_mlp_config* c, const float* p, Enc& e) {
  const uint32_t T = 1u << c->log2_table;
  for (int l = 0; l < c->levels; ++l) {
    const int R = level_res(c, l);
    const bool dense = (uint64_t)(R + 1) * (R + 1) * (R + 1) <= T;
    double x[3], f[3];
    int i0[3];
    for (int d = 0; d < 3; ++d) {
      x[d] = (double)p[d] * R;
      double fl = std::floor(x[d]);
      i0[d] = (int)fl;
      f[d] = x[d] - fl;
    }
    for (int k = 0; k < 8; ++k) {
      int cc[3];
      double w = 1.0;
      for (int d = 0; d < 3; ++d) {
        const int bit = (k >> d) & 1;
        cc[d] = i0[d] + bit;
        w *= bit ? f[d] : 1.0 - f[d];
      }
      uint32_t idx;
      if (dense) {
        for (int d = 0; d < 3; ++d) cc[d] = cc[d] < 0 ? 0 : (cc[d] > R ? R : cc[d]);
        idx = (uint32_t)(cc[0] + (R + 1) * (cc[1] + (R + 1) * cc[2]));
      } else {
        idx = ((uint32_t)cc[0] * 1u ^ (uint32_t)cc[1] * 2654435761u ^ (uint32_t)cc[2] * 805459861u) & (T - 1);
      }
      e.idx[l][k] = idx;
      e.w[l][k] = w;
    }
  }
}

void input_vector(const orc_mlp_config* c, const float* table, const float* p, const float* n, const float* a,
                  const Enc& e, double* in) {
  const size_t T = (size_t)1 << c->log2_table;
  for (int i = 0; i < 64; ++i) in[i] = 0.0;
  for (int l = 0; l < c->levels; ++l)
    for (int k = 0; k < 8; ++k)
      for (int f = 0; f < 2; ++f) in[2 * l + f] += e.w[l][k] * table[((size_t)l * T + e.idx[l][k]) * 2 + f];
  double nn = std::sqrt((double)n[0] * n[0] + (double)n[1] * n[1] + (double)n[2] * n[2]);
  for (int d = 0; d < 3; ++d) {
    in[32 + d] = nn > 0 ? n[d] / nn : 0.0;
    in[35 + d] = a[d];
  }
  in[38] = 1.0;
  (void)p;
}

// Layer weights: W[l] row-major [out][in]; W1..W4 64x64, W5 16x64.
inline const float* wl(const float* W, int l) { return W + (size_t)l * 64 * 64; }

void forward(const float* W, const double* in, double h[5][64], double* y) {
  const double* x = in;
  for (int l = 0; l < 4; ++l) {
    for (int o = 0; o < 64; ++o) {
      double s = 0.0;
      for (int i = 0; i < 64; ++i) s += (double)wl(W, l)[o * 64 + i] * x[i];
      h[l][o] = s > 0.0 ? s : 0.0;
    }
    x = h[l];
  }
  for (int o = 0; o < 3; ++o) {
    double s = 0.0;
    for (int i = 0; i < 64; ++i) s += (double)wl(W, 4)[o * 64 + i] * x[i];
    y[o] = s;
  }
}

}  // namespace

extern "C" {

int32_t orc_mlp_level_res(const orc_mlp_config* c, int32_t level) { return level_res(c, level); }

void orc_mlp_forward(const orc_mlp_config* c, const float* table, const float* W, int32_t n, const float* pos,
                     const float* nrm, const float* alb, float* out) {
  for (int s = 0; s < n; ++s) {
    Enc e;
    encode(c, pos + 3 * s, e);
    double in[64], h[5][64], y[3];
    input_vector(c, table, pos + 3 * s, nrm + 3 * s, alb + 3 * s, e, in);
    forward(W, in, h, y);
    for (int k = 0; k < 3; ++k) out[3 * s + k] = (float)y[k];
  }
}

double orc_mlp_grad(const orc_mlp_config* c, const float* table, const float* W, int32_t n, const float* pos,
                    const float* nrm, const float* alb, const float* target, double* dW, double* dtable) {
  const size_t T = (size_t)1 << c->log2_table;
  std::memset(dW, 0, sizeof(double) * 5 * 64 * 64);
  if (dtable) std::memset(dtable, 0, sizeof(double) * c->levels * T * 2);
  double loss = 0.0;
  for (int s = 0; s < n; ++s) {
    Enc e;
    encode(c, pos + 3 * s, e);
    double in[64], h[5][64], y[3];
    input_vector(c, table, pos + 3 * s, nrm + 3 * s, alb + 3 * s, e, in);
    forward(W, in, h, y);
    double dy[64] = {0};
    for (int k = 0; k < 3; ++k) {
      const double r = y[k] - (double)target[3 * s + k];
      loss += r * r / n;
      dy[k] = 2.0 * r / n;
    }
    // W5 (16 x 64): only rows 0..2 are used.
    double g[64];
    for (int i = 0; i < 64; ++i) {
      double acc = 0.0;
      for (int o = 0; o < 3; ++o) {
        dW[4 * 4096 + o * 64 + i] += dy[o] * h[3][i];
        acc += (double)wl(W, 4)[o * 64 + i] * dy[o];
      }
      g[i] = h[3][i] > 0.0 ? acc : 0.0;
    }
    for (int l = 3; l >= 0; --l) {
      const double* x = l == 0 ? in : h[l - 1];
      double gx[64];
      for (int i = 0; i < 64; ++i) {
        double acc = 0.0;
        for (int o = 0; o < 64; ++o) {
          dW[l * 4096 + o * 64 + i] += g[o] * x[i];
          acc += (double)wl(W, l)[o * 64 + i] * g[o];
        }
        gx[i] = acc;
      }
      if (l > 0)
        for (int i = 0; i < 64; ++i) g[i] = h[l - 1][i] > 0.0 ? gx[i] : 0.0;
      else
        for (int i = 0; i < 64; ++i) g[i] = gx[i];
    }
    if (dtable)
      for (int l = 0; l < c->levels; ++l)
        for (int k = 0; k < 8; ++k)
          for (int f = 0; f < 2; ++f) dtable[((size_t)l * T + e.idx[l][k]) * 2 + f] += e.w[l][k] * g[2 * l + f];
  }
  return loss;
}

}  // extern "C"
