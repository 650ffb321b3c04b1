// Host-side scene helpers: the seeded campfire layout and seeded floor spots.
#include <cmath>
#include <cstdint>
#include <cstring>
#include "../../include/fire_sim.h"

namespace {
uint32_t pcg1(uint32_t n) {   // src/shaders/lib.js:11-15
  uint32_t s = n * 747796405u + 2891336453u;
  uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
double rand2(uint32_t n, uint32_t m) { return (double)pcg1(n ^ pcg1(m)) / 4294967295.0; }
}  // namespace

extern "C" {

// buildCampfire (src/scene.js:21-42): LCG-seeded two base logs, a five-log teepee and a charred chunk;
// packLogs (src/scene.js:92-98) writes (a.xyz, r, b.xyz, burn) per log, zero-padded to max_logs.
int fire_build_campfire(uint32_t seed, float* out, int max_logs) {
  if (!out || max_logs <= 0) return FIRE_ERR_BAD_ARG;
  uint32_t s = seed;
  auto R = [&s]() { s = s * 1664525u + 1013904223u; return (double)s / 4294967296.0; };   // scene.js:13-16
  double logs[8][8];
  int n = 0;
  auto add = [&](double ax, double ay, double az, double bx, double by, double bz, double r, double burn) {
    double* L = logs[n++];
    L[0] = ax; L[1] = ay; L[2] = az; L[3] = r; L[4] = bx; L[5] = by; L[6] = bz; L[7] = burn;
  };
  add(-0.40, 0.055, -0.17, 0.38, 0.065, -0.13, 0.062, 0.8);
  add(-0.36, 0.060, 0.15, 0.41, 0.050, 0.19, 0.058, 0.8);
  const double PI = 3.141592653589793;
  for (int i = 0; i < 5; ++i) {
    double ang = ((double)i / 5) * PI * 2 + 0.35 + (R() - 0.5) * 0.4;
    double rb = 0.30 + R() * 0.06;
    double bx = std::cos(ang) * rb, by = 0.03, bz = std::sin(ang) * rb;
    double topR = 0.035 + R() * 0.03;
    double ta = ang + PI + (R() - 0.5) * 0.8;
    double tx = std::cos(ta) * topR;
    double ty = 0.36 + R() * 0.1;
    double tz = std::sin(ta) * topR;
    double rr = 0.032 + R() * 0.012;
    add(bx, by, bz, tx, ty, tz, rr, 1.0);
  }
  add(-0.12, 0.035, 0.02, 0.10, 0.03, -0.05, 0.035, 1.0);
  std::memset(out, 0, sizeof(float) * 8 * (size_t)max_logs);
  int keep = n < max_logs ? n : max_logs;
  for (int i = 0; i < keep; ++i)
    for (int c = 0; c < 8; ++c) out[i * 8 + c] = (float)logs[i][c];
  return keep;
}

// Seeded floor spots: uniform on a disc (r = radius * sqrt(u), theta = 2 pi v), flux uniform in [lo, hi].
int fire_make_spots(uint32_t seed, int n, float flux_lo, float flux_hi, float sigma, float radius, float* out) {
  if (!out || n < 0 || n > FIRE_MAX_SPOTS) return FIRE_ERR_BAD_ARG;
  const double PI = 3.141592653589793;
  for (int i = 0; i < n; ++i) {
    double u = rand2(seed, 2u * (uint32_t)i), v = rand2(seed, 2u * (uint32_t)i + 1u);
    double w = rand2(seed ^ 0x9e3779b9u, (uint32_t)i);
    double r = (double)radius * std::sqrt(u), th = 2.0 * PI * v;
    out[5 * i + 0] = (float)(r * std::cos(th));
    out[5 * i + 1] = 0.0f;
    out[5 * i + 2] = (float)(r * std::sin(th));
    out[5 * i + 3] = sigma;
    out[5 * i + 4] = (float)((double)flux_lo + ((double)flux_hi - (double)flux_lo) * w);
  }
  return FIRE_OK;
}

// Sources of the seeded Poisson right-hand side: centre uniform over the grid (cell units), sigma uniform
// in [1, 4] cells, amplitude standard normal (Box-Muller on two uniforms).
int fire_poisson_sources(unsigned seed, int n, const int res[3], float* out) {
  if (!out || !res || n < 0 || n > 4096) return FIRE_ERR_BAD_ARG;
  const double PI = 3.141592653589793;
  for (int i = 0; i < n; ++i) {
    const uint32_t k = 6u * (uint32_t)i;
    const double u1 = std::fmax(rand2(seed, k + 4u), 1e-12), u2 = rand2(seed, k + 5u);
    out[5 * i + 0] = (float)(rand2(seed, k + 0u) * res[0]);
    out[5 * i + 1] = (float)(rand2(seed, k + 1u) * res[1]);
    out[5 * i + 2] = (float)(rand2(seed, k + 2u) * res[2]);
    out[5 * i + 3] = (float)(1.0 + 3.0 * rand2(seed, k + 3u));
    out[5 * i + 4] = (float)(std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * PI * u2));
  }
  return FIRE_OK;
}

}  // extern "C"
