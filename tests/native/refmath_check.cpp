// Host check of flip3d_gb300/csrc/refmath.h against the reference's own
// double-promoted expressions (src/kernel.cpp:4-10, src/utility.cpp:16-18,
// src/flip3D.cpp:884,1095). Prints mismatch counts per function.
#include "../../flip3d_gb300/csrc/refmath.h"
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <random>

using namespace refmath;

static float ref_sharp(float r2, float h) {
  return (float)std::fmax((double)(h * h) / std::fmax((double)r2, 1.0e-5) - 1.0, 0.0);
}
static float ref_smooth(float r2, float h) {
  return (float)std::fmax(1.0 - (double)(r2 / (h * h)), 0.0);
}

int main(int argc, char **argv) {
  long N = argc > 1 ? atol(argv[1]) : 2000000;
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<float> U(-1.0f, 1.0f);
  long bad_hyp = 0, bad_len = 0, bad_sharp = 0, bad_smooth = 0, bad_blend = 0, bad_axpy = 0, bad_add = 0;
  const float hs[3] = {1.4f, 0.5f / 32, 1.0f / 64};
  for (int t = 0; t < 3; t++) {
    float h = hs[t];
    float hh = h * h;
    float floor_ = nextafterf((float)1.0e-5, 1.0f);
    if ((double)floor_ <= 1e-5) floor_ = nextafterf(floor_, 1.0f);
    while ((double)nextafterf(floor_, 0.0f) >= 1e-5) floor_ = nextafterf(floor_, 0.0f);
    float small = (float)std::fmax((double)hh / 1.0e-5 - 1.0, 0.0);
    for (long i = 0; i < N; i++) {
      float a = U(rng) * h * 2, b = U(rng) * h * 2, c = U(rng) * h * 2;
      if (i % 7 == 0) { a *= 1e-3f; }
      if (hypotf(a, b) != hypot_ref(a, b)) bad_hyp++;
      if (hypotf(hypotf(a, b), c) != length_ref(a, b, c)) bad_len++;
      float r2 = hypot2_ref(a, b, c);
      if (i % 11 == 0) r2 *= 1e-4f;
      if (i % 13 == 0) r2 = hh * (1.0f - std::fabs(U(rng)) * 1e-5f);    /* q near 1 */
      if (ref_sharp(r2, h) != sharp_ref(r2, hh, floor_, small)) bad_sharp++;
      if (ref_smooth(r2, h) != smooth_ref(r2, hh)) bad_smooth++;
    }
  }
  const double alpha = 0.95, c1 = 1.0 - alpha, c2 = alpha;
  float c1h = (float)c1, c1l = (float)(c1 - (double)c1h), c2h = (float)c2, c2l = (float)(c2 - (double)c2h);
  const double dt = 0.6e-2;
  float dth = (float)dt, dtl = (float)(dt - (double)dth);
  const double g = -0.6e-2 * 9.8;
  float gh = (float)g, gl = (float)(g - (double)gh);
  std::normal_distribution<float> G(0.0f, 2.0f);
  for (long i = 0; i < N; i++) {
    float x = G(rng), y = G(rng);
    if (i % 5 == 0) y = -x * (float)(c1 / c2) * (1.0f + U(rng) * 1e-6f); /* blend cancels */
    if (i % 5 == 1) x = -(float)g * (1.0f + U(rng) * 1e-6f);              /* u + g cancels */
    if (i % 5 == 2) x = (float)(-0.3 / dt) * (1.0f + U(rng) * 1e-6f);     /* p + dt*v cancels */
    if ((float)(c1 * x + c2 * y) != blend_ref(x, y, c1h, c1l, c2h, c2l, c1, c2)) bad_blend++;
    float p = (i % 5 == 2) ? 0.3f : std::fabs(U(rng));
    if ((float)((double)p + dt * (double)x) != axpy_fd(p, x, dth, dtl, dt)) bad_axpy++;
    if ((float)((double)x + g) != add_fd(x, gh, gl, g)) bad_add++;
  }
  printf("hypot %ld length %ld sharp %ld smooth %ld blend %ld axpy %ld add %ld of %ld\n",
         bad_hyp, bad_len, bad_sharp, bad_smooth, bad_blend, bad_axpy, bad_add, 3 * N);
  return 0;
}
