// Checks vct::snap_fixed (voxel_cone_tracing_gb300/csrc/vct_snap.h) against
// the FP64 rounding it replaces: llrint(((double)g + 1.0) * 2^k), rounding
// half to even.  Random coordinates over the valid range |g| <= 64, values
// near 0, exact ties (x + 1/2 after scaling) and their float neighbours,
// zeros, subnormals and the range ends.  Prints the count of mismatches and
// exits non-zero if there is one.
#include <cmath>
#include <cstdio>
#include <random>

#include "vct_snap.h"

int main(int argc, char** argv) {
  const long per_k = argc > 1 ? std::atol(argv[1]) : 200000;
  std::mt19937 rng(7);
  long long bad = 0, n = 0;
  auto check = [&](float g, int k) {
    const long long ref = std::llrint(((double)g + 1.0) * std::ldexp(1.0, k));
    const long long got = vct::snap_fixed(g, k);
    ++n;
    if (ref != got) {
      if (bad < 8) std::printf("g=%a k=%d ref=%lld got=%lld\n", (double)g, k, ref, got);
      ++bad;
    }
  };
  // k = log2(N) + 7 (conservative rule) or + 8 (2N raster), N in [8, 1024]
  for (int k = 10; k <= 18; ++k) {
    std::uniform_real_distribution<float> wide(-64.f, 64.f), unit(-1.5f, 1.5f);
    std::uniform_real_distribution<double> tiny_exp(-40.0, 0.0);
    for (long i = 0; i < per_k; ++i) {
      check(wide(rng), k);
      check(unit(rng), k);
      const float t = (float)std::ldexp(1.0, (int)tiny_exp(rng)) * unit(rng);
      check(t, k);
    }
    for (int j = -3000; j < 3000; ++j) {
      const float g = (float)(((double)j + 0.5) / std::ldexp(1.0, k) - 1.0);
      check(g, k);
      check(std::nextafter(g, 100.f), k);
      check(std::nextafter(g, -100.f), k);
      check(-g, k);
    }
    for (float g : {0.f, -0.f, 1e-40f, -1e-40f, 1e-30f, -1e-30f, 64.f, -64.f, 1.f, -1.f, 0.5f, -0.5f, -1.5f})
      check(g, k);
  }
  std::printf("%lld of %lld differ\n", bad, n);
  return bad != 0;
}
