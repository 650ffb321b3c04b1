// CPU oracle for the procedural-fire simulation step.  TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++, the WGSL compute kernels of the reference solver so that the CUDA
// implementation can be checked against it.  Only the test suite, the smoke check and the CPU-baseline
// and reference legs of bench.py load it; the product library never links or calls it.
//
// Every kernel below cites the reference file:line it follows (paths relative to the reference project):
//   src/sim.js          FireSim: advection, curl, forces, divergence, multigrid, projection, geometry
//   src/shaders/lib.js  pcg3d / hash3f / sdCapsule
//   src/noise.js        tileable noise table and its curl table
//   src/scene.js        buildCampfire / packLogs (seeded campfire layout)
//   research/webgpu-bench/poisson.mjs   CPU multigrid convergence study (known-answer test)
//
// The code is templated on the arithmetic type R: R = float restates the FP32 WGSL semantics (the parity
// target of the CUDA kernels), R = double is the FP64 accuracy oracle.  Semantics fixed here (and in the
// CUDA kernels, identically):
//   * textureSampleLevel with a linear sampler is trilinear interpolation in cell units with exact
//     weights (texel i's centre at i + 0.5), clamp-to-edge or repeat addressing;
//   * clamp(x, lo, hi) = min(max(x, lo), hi) with NaN-ignoring min/max (so clamp(NaN, 0, 1) = 0);
//   * mix(a, b, t) = a * (1 - t) + b * t;  smoothstep per the WGSL definition;
//   * normalize(v) = v / sqrt(dot(v, v)); tables are rounded to IEEE half (rgba16float) on store.
// Modes (per simulation): the multigrid's over-relaxation factor; the reference's rgba16float storage of
// every float4 field and the texture unit's ~8-bit filter weights (to state how far the FP32 path sits from
// the reference's own numerics); spot fluxes held in double (finite differences below FP32 resolution).
//
// Pinning.  The multigrid is pinned to the reference's own recorded numbers: the restatement of
// poisson.mjs reproduces results/poisson-128-face.txt digit for digit and results/result-new-mg.json to a
// few per cent.  Advection, the source terms and projection are parity unpinned by the reference: it holds
// no golden vectors for them and its WGSL cannot run here (no WebGPU device, no Node); they are pinned only
// by this line-by-line restatement and by independent numpy restatements of each stage (tests/).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------------------------------------
// Small vector types (component-wise, WGSL-like)
// ------------------------------------------------------------------------------------------------
template <class R> struct V3 {
  R x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
  V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
  V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
  V3 operator*(R s) const { return V3(x * s, y * s, z * s); }
  V3 operator/(R s) const { return V3(x / s, y / s, z / s); }
};
template <class R> struct V4 {
  R x, y, z, w;
  V4() : x(0), y(0), z(0), w(0) {}
  V4(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
  V4 operator+(const V4& o) const { return V4(x + o.x, y + o.y, z + o.z, w + o.w); }
  V4 operator-(const V4& o) const { return V4(x - o.x, y - o.y, z - o.z, w - o.w); }
  V4 operator*(R s) const { return V4(x * s, y * s, z * s, w * s); }
  V3<R> xyz() const { return V3<R>(x, y, z); }
};

template <class R> inline R fmn(R a, R b) { return std::fmin(a, b); }
template <class R> inline R fmx(R a, R b) { return std::fmax(a, b); }
template <class R> inline R clampf(R x, R lo, R hi) { return fmn(fmx(x, lo), hi); }
template <class R> inline R mixf(R a, R b, R t) { return a * (R(1) - t) + b * t; }
// WGSL smoothstep (t = clamp((x - e0) / (e1 - e0), 0, 1); t^2 (3 - 2t)), evaluated as (x - e0) * (1 / (e1 - e0)),
// which is within WGSL's accuracy for smoothstep and is how the CUDA kernels evaluate it.
template <class R> inline R smoothstep(R e0, R e1, R x) {
  const R inv = R(1) / (e1 - e0);
  R t = clampf((x - e0) * inv, R(0), R(1));
  return t * t * (R(3) - R(2) * t);
}
template <class R> inline R dot3(const V3<R>& a, const V3<R>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline R len3(const V3<R>& a) { return std::sqrt(dot3(a, a)); }
template <class R> inline V3<R> min3(const V3<R>& a, const V3<R>& b) { return V3<R>(fmn(a.x, b.x), fmn(a.y, b.y), fmn(a.z, b.z)); }
template <class R> inline V3<R> max3(const V3<R>& a, const V3<R>& b) { return V3<R>(fmx(a.x, b.x), fmx(a.y, b.y), fmx(a.z, b.z)); }
template <class R> inline V4<R> min4(const V4<R>& a, const V4<R>& b) { return V4<R>(fmn(a.x, b.x), fmn(a.y, b.y), fmn(a.z, b.z), fmn(a.w, b.w)); }
template <class R> inline V4<R> max4(const V4<R>& a, const V4<R>& b) { return V4<R>(fmx(a.x, b.x), fmx(a.y, b.y), fmx(a.z, b.z), fmx(a.w, b.w)); }
template <class R> inline V3<R> clamp3(const V3<R>& v, const V3<R>& lo, const V3<R>& hi) { return min3(max3(v, lo), hi); }
template <class R> inline V4<R> clamp4(const V4<R>& v, const V4<R>& lo, const V4<R>& hi) { return min4(max4(v, lo), hi); }
template <class R> inline V3<R> cross3(const V3<R>& a, const V3<R>& b) {
  return V3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ------------------------------------------------------------------------------------------------
// IEEE half rounding (round to nearest even), used where the reference stores rgba16float tables.
// ------------------------------------------------------------------------------------------------
uint16_t f32_to_f16_bits(float f) {
  uint32_t x; std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);          // rounds to >= 65520 -> inf
  if (ax < 0x38800000u) {                                              // result is subnormal or zero
    if (ax < 0x33000000u) return (uint16_t)sign;                       // < 2^-25 rounds to 0
    uint32_t e = ax >> 23;
    uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    uint32_t shift = 126u - e;                                         // 14 + (127 - 1 - e) ... exponent gap
    // value = m * 2^(e-150); half subnormal unit = 2^-24 -> q = m * 2^(e-126)
    uint32_t q = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (q & 1u))) q++;
    return (uint16_t)(sign | q);
  }
  uint32_t e = (ax >> 23) - 127u + 15u;
  uint32_t m = ax & 0x7fffffu;
  uint32_t q = (e << 10) | (m >> 13);
  uint32_t rem = m & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q++;
  return (uint16_t)(sign | q);
}
float f16_bits_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) x = sign;
    else { float v = (float)m * 5.9604644775390625e-08f; std::memcpy(&x, &v, 4); x |= sign; }
  } else if (e == 31) x = sign | 0x7f800000u | (m << 13);
  else x = sign | ((e - 15u + 127u) << 23) | (m << 13);
  float f; std::memcpy(&f, &x, 4); return f;
}
inline float round_half(float f) { return f16_bits_to_f32(f32_to_f16_bits(f)); }

// ------------------------------------------------------------------------------------------------
// Hashes (src/shaders/lib.js:3-18)
// ------------------------------------------------------------------------------------------------
struct U3 { uint32_t x, y, z; };
inline U3 pcg3d(U3 v) {                                           // lib.js:4-10
  v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u; v.z = v.z * 1664525u + 1013904223u;
  v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
  v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16;
  v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
  return v;
}
inline uint32_t pcg1(uint32_t n) {                                // lib.js:11-15
  uint32_t s = n * 747796405u + 2891336453u;
  uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
const float INV_U32 = 2.3283064365386963e-10f;                    // f32(1/4294967295) == 2^-32
inline V3<float> hash3f(int x, int y, int z) {                   // lib.js:16
  U3 h = pcg3d(U3{(uint32_t)x, (uint32_t)y, (uint32_t)z});
  return V3<float>((float)h.x * INV_U32, (float)h.y * INV_U32, (float)h.z * INV_U32);
}
inline float rand2(uint32_t n, uint32_t m) { return (float)pcg1(n ^ pcg1(m)) * INV_U32; }   // lib.js:18

// ------------------------------------------------------------------------------------------------
// Noise tables (src/noise.js:8-54, 69-80).  FP32 arithmetic, stored as half.
// ------------------------------------------------------------------------------------------------
inline int wrapi(int c, int per) { return ((c % per) + per) % per; }     // noise.js:11
inline V3<float> ngrad(int cx, int cy, int cz, int per, int ch, int seed) {   // noise.js:12-15
  V3<float> h = hash3f(wrapi(cx, per) + (ch * 1013 + seed), wrapi(cy, per) + ch * 7919, wrapi(cz, per) + ch * 104729);
  V3<float> v((h.x * 2.0f - 1.0f) + 1e-5f, (h.y * 2.0f - 1.0f) + 1e-5f, (h.z * 2.0f - 1.0f) + 1e-5f);
  float l = std::sqrt(dot3(v, v));
  return V3<float>(v.x / l, v.y / l, v.z / l);
}
inline float fade5(float f) { return f * f * f * (f * (f * 6.0f - 15.0f) + 10.0f); }
float tnoise(V3<float> p, int per, int ch, int seed) {             // noise.js:16-28
  float flx = std::floor(p.x), fly = std::floor(p.y), flz = std::floor(p.z);
  int ix = (int)flx, iy = (int)fly, iz = (int)flz;
  V3<float> f(p.x - flx, p.y - fly, p.z - flz);
  V3<float> u(fade5(f.x), fade5(f.y), fade5(f.z));
  float acc[8];
  for (int k = 0; k < 8; ++k) {
    int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
    V3<float> g = ngrad(ix + ox, iy + oy, iz + oz, per, ch, seed);
    acc[k] = dot3(g, V3<float>(f.x - (float)ox, f.y - (float)oy, f.z - (float)oz));
  }
  float x0 = mixf(acc[0], acc[1], u.x), x1 = mixf(acc[2], acc[3], u.x);
  float x2 = mixf(acc[4], acc[5], u.x), x3 = mixf(acc[6], acc[7], u.x);
  return mixf(mixf(x0, x1, u.y), mixf(x2, x3, u.y), u.z);
}
float tfbm(V3<float> p01, int ch, int seed) {                      // noise.js:29-36
  float s = 0.0f, a = 0.5f; int per = 4;
  for (int o = 0; o < 5; ++o) {
    float fp = (float)per;
    s += a * tnoise(V3<float>(p01.x * fp, p01.y * fp, p01.z * fp), per, ch, seed);
    per *= 2; a *= 0.5f;
  }
  return s * 1.5f;
}
float worley(V3<float> p01, int per, int seed) {                   // noise.js:37-47
  float fp = (float)per;
  V3<float> p(p01.x * fp, p01.y * fp, p01.z * fp);
  float flx = std::floor(p.x), fly = std::floor(p.y), flz = std::floor(p.z);
  int ix = (int)flx, iy = (int)fly, iz = (int)flz;
  V3<float> f(p.x - flx, p.y - fly, p.z - flz);
  float d = 9.0f;
  for (int k = 0; k < 27; ++k) {
    int ox = k % 3 - 1, oy = (k / 3) % 3 - 1, oz = k / 9 - 1;
    V3<float> h = hash3f(wrapi(ix + ox, per) + 77, wrapi(iy + oy, per) + 33, wrapi(iz + oz, per) + seed);
    V3<float> q(((float)ox + h.x) - f.x, ((float)oy + h.y) - f.y, ((float)oz + h.z) - f.z);
    d = fmn(d, len3(q));
  }
  return d;
}

// ------------------------------------------------------------------------------------------------
// Trilinear sampling in cell units (textureSampleLevel, linear filter; src/sim.js:68-69, 129)
// ------------------------------------------------------------------------------------------------
template <class R> struct Grid { int nx, ny, nz; };

inline size_t cidx(int x, int y, int z, int nx, int ny) { return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * (size_t)z); }

template <class R>
inline V4<R> load4(const std::vector<R>& f, int x, int y, int z, int nx, int ny) {
  const R* p = &f[4 * cidx(x, y, z, nx, ny)];
  return V4<R>(p[0], p[1], p[2], p[3]);
}
template <class R>
inline V4<R> ld4(const std::vector<R>& f, int x, int y, int z, int nx, int ny, int nz) {   // sim.js:114
  x = std::min(std::max(x, 0), nx - 1); y = std::min(std::max(y, 0), ny - 1); z = std::min(std::max(z, 0), nz - 1);
  return load4(f, x, y, z, nx, ny);
}
template <class R>
inline void store4(std::vector<R>& f, int x, int y, int z, int nx, int ny, const V4<R>& v) {
  R* p = &f[4 * cidx(x, y, z, nx, ny)];
  p[0] = v.x; p[1] = v.y; p[2] = v.z; p[3] = v.w;
}

// One axis of the clamp-to-edge linear filter: u is the continuous cell coordinate (texel centre at i+.5)
// Texture-unit filter weights: the reference samples its fields through the GPU's linear filter, whose
// interpolation weights are fixed point with about 8 fractional bits, i.e. 1/256 steps (research/webgpu.md,
// "Filter weight precision").  fbits > 0 rounds each axis fraction to the nearest multiple of 2^-fbits;
// fbits = 0 keeps exact weights (the semantics of the CUDA kernels).
template <class R> inline R quant_frac(R f, int fbits) {
  if (fbits <= 0) return f;
  const R sc = R(1 << fbits);
  return std::floor(f * sc + R(0.5)) / sc;
}
template <class R>
inline void axis_clamp(R c, int n, int& i0, int& i1, R& f, int fbits = 0) {
  R u = clampf(c - R(0.5), R(-1), R(n));       // clamping u to [-1, n] does not change a clamp-to-edge sample
  R fl = std::floor(u);
  int i = (int)fl;
  f = quant_frac(u - fl, fbits);
  i0 = std::min(std::max(i, 0), n - 1);
  i1 = std::min(std::max(i + 1, 0), n - 1);
}
template <class R>
inline V4<R> lerp4(const V4<R>& a, const V4<R>& b, R t) {
  R s = R(1) - t;
  return V4<R>(a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t);
}
template <class R>
V4<R> sample_clamp(const std::vector<R>& f, int nx, int ny, int nz, const V3<R>& c, int fbits = 0) {
  int x0, x1, y0, y1, z0, z1; R fx, fy, fz;
  axis_clamp(c.x, nx, x0, x1, fx, fbits); axis_clamp(c.y, ny, y0, y1, fy, fbits); axis_clamp(c.z, nz, z0, z1, fz, fbits);
  V4<R> c00 = lerp4(load4(f, x0, y0, z0, nx, ny), load4(f, x1, y0, z0, nx, ny), fx);
  V4<R> c10 = lerp4(load4(f, x0, y1, z0, nx, ny), load4(f, x1, y1, z0, nx, ny), fx);
  V4<R> c01 = lerp4(load4(f, x0, y0, z1, nx, ny), load4(f, x1, y0, z1, nx, ny), fx);
  V4<R> c11 = lerp4(load4(f, x0, y1, z1, nx, ny), load4(f, x1, y1, z1, nx, ny), fx);
  return lerp4(lerp4(c00, c10, fy), lerp4(c01, c11, fy), fz);
}
// Repeat-addressed sample of a 128^3 table given in normalised coordinates (sim.js:69, 228, 365)
template <class R>
V4<R> sample_repeat(const float* tab, int N, const V3<R>& q, int fbits = 0) {
  R ux = q.x * R(N) - R(0.5), uy = q.y * R(N) - R(0.5), uz = q.z * R(N) - R(0.5);
  R flx = std::floor(ux), fly = std::floor(uy), flz = std::floor(uz);
  R fx = quant_frac(ux - flx, fbits), fy = quant_frac(uy - fly, fbits), fz = quant_frac(uz - flz, fbits);
  // wrap in 64-bit to stay defined for any finite coordinate
  long long ix = (long long)flx, iy = (long long)fly, iz = (long long)flz;
  auto wr = [N](long long i) { long long m = i % N; return (int)(m < 0 ? m + N : m); };
  int x0 = wr(ix), x1 = wr(ix + 1), y0 = wr(iy), y1 = wr(iy + 1), z0 = wr(iz), z1 = wr(iz + 1);
  auto T = [&](int x, int y, int z) {
    const float* p = tab + 4 * ((size_t)x + (size_t)N * ((size_t)y + (size_t)N * z));
    return V4<R>(p[0], p[1], p[2], p[3]);
  };
  V4<R> c00 = lerp4(T(x0, y0, z0), T(x1, y0, z0), fx);
  V4<R> c10 = lerp4(T(x0, y1, z0), T(x1, y1, z0), fx);
  V4<R> c01 = lerp4(T(x0, y0, z1), T(x1, y0, z1), fx);
  V4<R> c11 = lerp4(T(x0, y1, z1), T(x1, y1, z1), fx);
  return lerp4(lerp4(c00, c10, fy), lerp4(c01, c11, fy), fz);
}

// ------------------------------------------------------------------------------------------------
// Parameter block: SIM_FIELDS order (src/sim.js:14-23), 60 floats padded to 64.
// ------------------------------------------------------------------------------------------------
enum {
  P_nx, P_ny, P_nz, P_dx, P_dt, P_time, P_frame, P_seed, P_ox, P_oy, P_oz, P_nLogs,
  P_fuelSrc, P_bedFuel, P_srcTemp, P_bedTemp, P_srcVel, P_srcFreq, P_srcSpeed, P_srcThresh,
  P_ignT, P_kMix, P_rs, P_heatOut, P_expansion, P_sootForm, P_sootOx, P_radCool,
  P_coolRate, P_sootDissip, P_smokeDissip, P_vitDecay, P_fuelDissip, P_buoyancy, P_vortEps, P_turbAmp,
  P_turbFreq, P_turbRise, P_turbEvolve, P_windX, P_windZ, P_gust, P_intensity, P_velDissip,
  P_bedRadius, P_logSrc, P_burstX, P_burstY, P_burstZ, P_burstAmt, P_smolder, P_sponge, P_hotR0, P_hotR1, P_hotY1,
  P_visc, P_lamAge, P_anchorFreq, P_srcFloor, P_anchorGain, P_COUNT
};
static_assert(P_COUNT == 60, "SIM_FIELDS has 60 entries");

// Build-defined extension block (no counterpart in the reference uniform): soot age gate, coal-bed gain
// and Gaussian pyrolysis spots.  Layout: [0] sootAge0 [1] sootAge1 [2] bedGain [3] nSpots
// [4] spotRef (g/s giving unit peak weight), [5..15] constants the CUDA host derives per step (the oracle
// recomputes them where they are used), then from [16] 16 spots x (x, y, z, sigma, flux g/s, 0, 0, 0).
enum { E_sootAge0 = 0, E_sootAge1, E_bedGain, E_nSpots, E_spotRef, E_SPOTS = 16, E_COUNT = 16 + 16 * 8 };

// ------------------------------------------------------------------------------------------------
// The simulation state (src/sim.js:48-101)
// ------------------------------------------------------------------------------------------------
template <class R> struct Level { int nx, ny, nz; R h; std::vector<R> p, b; };

template <class R> struct Sim {
  int nx, ny, nz; size_t N;
  std::vector<R> vel, velX, velY, S, SX, SY, S2, S2X, S2Y, vort, geo;
  std::vector<Level<R>> levels;
  int coarseIters;
  float P[64];
  float E[E_COUNT];
  std::vector<float> logs;          // nLogs * 8
  std::vector<float> noise, curl;   // 128^3 * 4 each (half-rounded values)
  int tabN = 128;
  // Solver and storage modes.  omega: over-relaxation of every multigrid sweep (1 = the reference's
  // Gauss-Seidel update).  store_half: every float4 field (vel, S, S2, their advected copies, vort, geo) is
  // rounded to IEEE half after the stage that writes it, as the reference's rgba16float textures store it
  // (src/sim.js:71-76, 143-145, 163-165, 202); p and b stay FP32 (r32float, src/sim.js:84).  filter_bits:
  // fractional bits of the trilinear weights of every texture sample (0 = exact).
  float omega = 1.0f;
  int store_half = 0;
  int filter_bits = 0;
  // Spot fluxes in double, replacing the FP32 values of the extension block when set (lets finite differences
  // of the FP64 oracle take steps far below the block's FP32 resolution).
  int flux64_set = 0;
  double flux64[16] = {};
};
// rgba16float store: rounds every component of a float4 field to the nearest IEEE half.
template <class R> void round_field_half(std::vector<R>& f) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)f.size(); ++i) f[(size_t)i] = (R)round_half((float)f[(size_t)i]);
}

template <class R> void sim_alloc(Sim<R>& s, int nx, int ny, int nz, double dx) {   // sim.js:71-92
  s.nx = nx; s.ny = ny; s.nz = nz; s.N = (size_t)nx * ny * nz;
  for (auto* f : {&s.vel, &s.velX, &s.velY, &s.S, &s.SX, &s.SY, &s.S2, &s.S2X, &s.S2Y, &s.vort, &s.geo})
    f->assign(4 * s.N, R(0));
  s.levels.clear();
  int x = nx, y = ny, z = nz; double h = dx;
  while (true) {
    Level<R> L; L.nx = x; L.ny = y; L.nz = z; L.h = (R)(float)h;
    L.p.assign((size_t)x * y * z, R(0)); L.b.assign((size_t)x * y * z, R(0));
    s.levels.push_back(std::move(L));
    if (x % 2 || y % 2 || z % 2 || std::min(x, std::min(y, z)) <= 6) break;
    x /= 2; y /= 2; z /= 2; h *= 2;
  }
  const Level<R>& C = s.levels.back();
  double PI = 3.14159265358979323846;
  double mu = (std::cos(PI / C.nx) + std::cos(PI / (2.0 * C.ny)) + std::cos(PI / C.nz)) / 3.0;
  s.coarseIters = (int)std::max(8.0, std::min(64.0, std::ceil(std::log(0.05) / std::log(mu * mu))));
}

// ---------------- geo (src/sim.js:498-523) ----------------
template <class R> R sdCapsule(V3<R> p, V3<R> a, V3<R> b, R r) {     // lib.js:58-62
  V3<R> pa = p - a, ba = b - a;
  R h = clampf(dot3(pa, ba) / dot3(ba, ba), R(0), R(1));
  return len3(pa - ba * h) - r;
}
template <class R> void k_geo(Sim<R>& s) {
  const float* P = s.P;
  const R dx = P[P_dx];
  const int nl = (int)P[P_nLogs];
  const R bedGain = s.E[E_bedGain];
#pragma omp parallel for schedule(static)
  for (int k = 0; k < s.nz; ++k)
    for (int j = 0; j < s.ny; ++j)
      for (int i = 0; i < s.nx; ++i) {
        V3<R> p = V3<R>(P[P_ox], P[P_oy], P[P_oz]) + V3<R>(R(i) + R(0.5), R(j) + R(0.5), R(k) + R(0.5)) * dx;
        R dmin = R(1e9), band = R(0);
        for (int l = 0; l < nl; ++l) {
          const float* A = &s.logs[(size_t)l * 8];
          const float* B = A + 4;
          V3<R> a(A[0], A[1], A[2]), b(B[0], B[1], B[2]);
          R Aw = A[3], Bw = B[3];
          R pxz = std::sqrt(p.x * p.x + p.z * p.z);
          R dd = sdCapsule(p, a, b, Aw);
          dd += Aw * R(0.3) * (R(1) - smoothstep(R(0), R(0.16), pxz)) * Bw;
          dmin = fmn(dmin, dd);
          R bnd = R(1) - smoothstep(R(0), R(1.6) * dx, std::fabs(dd - R(0.6) * dx));
          R hot = Bw * (R(1) - smoothstep((R)P[P_hotR0], (R)P[P_hotR1], pxz)) * (R(1) - smoothstep(R(0.08), (R)P[P_hotY1], p.y));
          band = fmx(band, bnd * hot);
        }
        R r = std::sqrt(p.x * p.x + p.z * p.z);
        R bedH = R(0.05) * (R(1) - smoothstep(R(0), (R)P[P_bedRadius], r)) + R(0.02);
        R bed = (R(1) - smoothstep(R(0), R(2) * dx, p.y - bedH)) *
                (R(1) - smoothstep((R)P[P_bedRadius] * R(0.6), (R)P[P_bedRadius] * R(1.15), r));
        bed = bed * bedGain;
        R solid = dmin < R(-0.5) * dx ? R(1) : R(0);
        store4(s.geo, i, j, k, s.nx, s.ny, V4<R>(band, bed, solid, dmin));
      }
}

// ---------------- advection (src/sim.js:123-197) ----------------
template <class R> struct AdvCtx {
  const Sim<R>* s; R dt, dx; R nxf, nyf, nzf;
  V3<R> sampleVel(const V3<R>& c) const { return sample_clamp(s->vel, s->nx, s->ny, s->nz, c, s->filter_bits).xyz(); }
  V3<R> backtrace(const V3<R>& c) const {                            // sim.js:130-135
    V3<R> v0 = sampleVel(c);
    V3<R> mid = c - v0 * (R(0.5) * dt) / dx;
    V3<R> v1 = sampleVel(mid);
    return c - v1 * dt / dx;
  }
  R outsideFade(const V3<R>& c) const {                              // sim.js:137-140
    R lo = fmn(c.x, c.z);
    R hi = fmx(c.x - nxf, fmx(c.y - nyf, c.z - nzf));
    return clampf(R(1) - fmx(-lo, hi), R(0), R(1));
  }
};
// NOTE on expression order: WGSL `0.5 * dt * v0 / P.dx` is ((0.5*dt)*v0)/dx; `dt * v1 / P.dx` is (dt*v1)/dx.
template <class R> void k_adv1(Sim<R>& s) {                           // sim.js:142-157
  AdvCtx<R> A{&s, (R)s.P[P_dt], (R)s.P[P_dx], R(s.nx), R(s.ny), R(s.nz)};
  const R windX = s.P[P_windX], windZ = s.P[P_windZ];
#pragma omp parallel for schedule(static)
  for (int k = 0; k < s.nz; ++k)
    for (int j = 0; j < s.ny; ++j)
      for (int i = 0; i < s.nx; ++i) {
        V3<R> c(R(i) + R(0.5), R(j) + R(0.5), R(k) + R(0.5));
        V3<R> b = A.backtrace(c);
        R f = A.outsideFade(b);
        R ws = smoothstep(R(0.03), R(0.4), b.y * A.dx);
        V3<R> wind(windX * ws, R(0) * ws, windZ * ws);
        V3<R> sv = sample_clamp(s.vel, s.nx, s.ny, s.nz, b, s.filter_bits).xyz();
        V3<R> vo(mixf(wind.x, sv.x, f), mixf(wind.y, sv.y, f), mixf(wind.z, sv.z, f));
        store4(s.velX, i, j, k, s.nx, s.ny, V4<R>(vo.x, vo.y, vo.z, R(0)));
        store4(s.SX, i, j, k, s.nx, s.ny, sample_clamp(s.S, s.nx, s.ny, s.nz, b, s.filter_bits) * f);
        store4(s.S2X, i, j, k, s.nx, s.ny, sample_clamp(s.S2, s.nx, s.ny, s.nz, b, s.filter_bits) * f);
      }
}
template <class R> void k_adv2(Sim<R>& s) {                           // sim.js:159-197
  AdvCtx<R> A{&s, (R)s.P[P_dt], (R)s.P[P_dx], R(s.nx), R(s.ny), R(s.nz)};
  const int nx = s.nx, ny = s.ny, nz = s.nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        V3<R> c(R(i) + R(0.5), R(j) + R(0.5), R(k) + R(0.5));
        V3<R> v = load4(s.vel, i, j, k, nx, ny).xyz();
        V3<R> fw = c + v * A.dt / A.dx;
        V3<R> vH = load4(s.velX, i, j, k, nx, ny).xyz();
        V4<R> sH = load4(s.SX, i, j, k, nx, ny);
        V4<R> s2H = load4(s.S2X, i, j, k, nx, ny);
        V3<R> vN = vH + (v - sample_clamp(s.velX, nx, ny, nz, fw, s.filter_bits).xyz()) * R(0.5);
        V4<R> sN = sH + (load4(s.S, i, j, k, nx, ny) - sample_clamp(s.SX, nx, ny, nz, fw, s.filter_bits)) * R(0.5);
        V4<R> s2N = s2H + (load4(s.S2, i, j, k, nx, ny) - sample_clamp(s.S2X, nx, ny, nz, fw, s.filter_bits)) * R(0.5);
        V3<R> bt = A.backtrace(c);
        V3<R> b(bt.x - R(0.5), bt.y - R(0.5), bt.z - R(0.5));
        V3<R> bc(clampf(b.x, R(-2), R(nx + 1)), clampf(b.y, R(-2), R(ny + 1)), clampf(b.z, R(-2), R(nz + 1)));
        int b0x = (int)std::floor(bc.x), b0y = (int)std::floor(bc.y), b0z = (int)std::floor(bc.z);
        V3<R> vmn(R(1e9), R(1e9), R(1e9)), vmx(R(-1e9), R(-1e9), R(-1e9));
        V4<R> smn(R(1e9), R(1e9), R(1e9), R(1e9)), smx(R(-1e9), R(-1e9), R(-1e9), R(-1e9));
        V4<R> tmn = smn, tmx = smx;
        for (int q = 0; q < 8; ++q) {
          int qx = b0x + (q & 1), qy = b0y + ((q >> 1) & 1), qz = b0z + ((q >> 2) & 1);
          V3<R> vv = ld4(s.vel, qx, qy, qz, nx, ny, nz).xyz();
          V4<R> ss = ld4(s.S, qx, qy, qz, nx, ny, nz);
          V4<R> tt = ld4(s.S2, qx, qy, qz, nx, ny, nz);
          vmn = min3(vmn, vv); vmx = max3(vmx, vv); smn = min4(smn, ss); smx = max4(smx, ss); tmn = min4(tmn, tt); tmx = max4(tmx, tt);
        }
        if (A.outsideFade(V3<R>(b.x + R(0.5), b.y + R(0.5), b.z + R(0.5))) < R(1)) { vN = vH; sN = sH; s2N = s2H; }
        vN = clamp3(vN, min3(vmn, vH), max3(vmx, vH));
        sN = clamp4(sN, min4(smn, sH), max4(smx, sH));
        s2N = clamp4(s2N, min4(tmn, s2H), max4(tmx, s2H));
        V4<R> z0(R(0), R(0), R(0), R(0));
        store4(s.velY, i, j, k, nx, ny, V4<R>(vN.x, vN.y, vN.z, R(0)));
        store4(s.SY, i, j, k, nx, ny, max4(sN, z0));
        store4(s.S2Y, i, j, k, nx, ny, max4(s2N, z0));
      }
}

// ---------------- curl (src/sim.js:200-211) ----------------
template <class R> void k_curl(Sim<R>& s) {
  const int nx = s.nx, ny = s.ny, nz = s.nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        V3<R> L = ld4(s.velY, i - 1, j, k, nx, ny, nz).xyz(), Rr = ld4(s.velY, i + 1, j, k, nx, ny, nz).xyz();
        V3<R> B = ld4(s.velY, i, j - 1, k, nx, ny, nz).xyz(), T = ld4(s.velY, i, j + 1, k, nx, ny, nz).xyz();
        V3<R> K = ld4(s.velY, i, j, k - 1, nx, ny, nz).xyz(), F = ld4(s.velY, i, j, k + 1, nx, ny, nz).xyz();
        V3<R> w((T.z - B.z) - (F.y - K.y), (F.x - K.x) - (Rr.z - L.z), (Rr.y - L.y) - (T.x - B.x));
        w = w * R(0.5);
        store4(s.vort, i, j, k, nx, ny, V4<R>(w.x, w.y, w.z, len3(w)));
      }
}

// ---------------- forces (src/sim.js:214-396) ----------------
template <class R> inline V4<R> noise4(const Sim<R>& s, const V3<R>& q) {     // sim.js:228
  V4<R> t = sample_repeat(s.noise.data(), s.tabN, q, s.filter_bits);
  return V4<R>(t.x * R(2) - R(1), t.y * R(2) - R(1), t.z * R(2) - R(1), t.w * R(2) - R(1));
}
template <class R> void k_forces(Sim<R>& s) {
  const float* P = s.P;
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  const R dt = P[P_dt], dx = P[P_dx], I = P[P_intensity], seed = P[P_seed], time = P[P_time];
  const R nxf = R(nx), nyf = R(ny), nzf = R(nz);
  const int nSpots = (int)s.E[E_nSpots];
  const R age0 = s.E[E_sootAge0], age1 = s.E[E_sootAge1], spotRef = s.E[E_spotRef];
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        V3<R> p = V3<R>(P[P_ox], P[P_oy], P[P_oz]) + V3<R>(R(i) + R(0.5), R(j) + R(0.5), R(k) + R(0.5)) * dx;
        V4<R> v4 = load4(s.velY, i, j, k, nx, ny);
        V3<R> v = v4.xyz();
        V4<R> sv = load4(s.SY, i, j, k, nx, ny);
        V4<R> s2 = load4(s.S2Y, i, j, k, nx, ny);
        V4<R> geo = load4(s.geo, i, j, k, nx, ny);

        // ---- sources (sim.js:246-284)
        R src = R(0), anchor = R(0);
        if (geo.x > R(0.001)) {
          V3<R> qa = p * (R)P[P_anchorFreq] + V3<R>(seed * R(0.37), R(0), R(0.11));
          anchor = smoothstep(R(-0.05), R(0.25), noise4(s, qa).z);
          V3<R> qn = p * ((R)P[P_srcFreq] * R(0.06)) + V3<R>(seed * R(0.131), R(0), time * (R)P[P_srcSpeed]);
          R pulse = smoothstep((R)P[P_srcThresh] - R(0.25), (R)P[P_srcThresh] + R(0.25), noise4(s, qn).x);
          src = clampf(geo.x * (R)P[P_logSrc] * ((R)P[P_srcFloor] + (R)P[P_anchorGain] * anchor) * mixf(R(0.55), R(1), pulse) * R(1.2), R(0), R(1)) * I;
          src *= R(1) - geo.z;
        }
        // build-defined Gaussian pyrolysis spots (extension; no counterpart in the reference)
        if (nSpots > 0) {
          R acc = R(0);
          for (int q = 0; q < nSpots; ++q) {
            const float* sp = &s.E[E_SPOTS + 8 * q];
            V3<R> d = p - V3<R>(sp[0], sp[1], sp[2]);
            R sg = sp[3];
            R d2 = dot3(d, d);
            const R flux = s.flux64_set ? (R)s.flux64[q] : (R)sp[4];
            if (d2 < R(16) * sg * sg) acc += (flux / spotRef) * std::exp(-d2 / (R(2) * sg * sg));
          }
          src = fmx(src, clampf(acc, R(0), R(1)) * I);
        }
        R srcW = fmn(src, R(1));
        R bedHot = geo.y;
        R bed = geo.y * clampf(I * R(1.4), R(0.3), R(1));
        if (bed > R(0.001)) {
          V3<R> qb = p * R(2.4) + V3<R>(R(0.17), -time * R(0.12), time * R(0.05));
          bed *= smoothstep(R(0), R(0.3), noise4(s, qb).y);
        }
        sv.y = fmx(sv.y, src * (R)P[P_fuelSrc]);
        sv.y = fmx(sv.y, bed * (R)P[P_bedFuel]);
        sv.x = fmx(sv.x, src * (R)P[P_srcTemp]);
        sv.x = fmx(sv.x, bedHot * (R)P[P_bedTemp]);
        R srcAll = fmx(srcW, bed);
        s2.w = mixf(s2.w, R(1), bed * (R(1) - srcW));
        s2.w = mixf(s2.w, R(0), srcW);
        s2.y = s2.y * (R(1) - srcAll);
        s2.x = fmx(s2.x, (R(1) - sv.y) * srcW);
        s2.x = fmx(s2.x, (R(1) - sv.y) * bed * R(0.6));
        R wsrc = R(1) - std::pow(R(1) - clampf(srcW + bed * R(0.4), R(0), R(1)) * R(0.5), dt * R(90));
        v.y = mixf(v.y, fmx(v.y, (R)P[P_srcVel]), wsrc);
        s2.z += geo.x * (R(1) - anchor) * (R)P[P_smolder] * dt * I;

        // ---- burst (sim.js:288-296)
        if (P[P_burstAmt] > 0.0f) {
          R bd = len3(p - V3<R>(P[P_burstX], P[P_burstY], P[P_burstZ]));
          R bw = clampf(std::exp(-bd * bd / R(0.006)) * (R)P[P_burstAmt], R(0), R(1));
          sv.y = fmx(sv.y, R(0.17) * bw);
          sv.x = fmx(sv.x, R(0.9) * bw);
          s2.x *= R(1) - bw;
          s2.w *= R(1) - bw;
          s2.y = fmx(s2.y, R(0.05) * bw * clampf(sv.y + s2.x, R(0), R(1)));
        }
        R ageF = s2.y / fmx(sv.y + s2.x, R(1e-4));

        // ---- combustion (sim.js:299-309)
        R T0 = R(293) + R(1000) * sv.x;
        R o = clampf(R(1) - sv.y - s2.x, R(0), R(1));
        R ign = smoothstep((R)P[P_ignT] - R(50), (R)P[P_ignT] + R(50), T0);
        R b = fmn(sv.y, o / (R)P[P_rs]) * (R(1) - std::exp(-(R)P[P_kMix] * ign * dt));
        sv.y -= b;
        s2.x = fmn(s2.x + (R(1) + (R)P[P_rs]) * b, R(1));
        R dT = fmn((R)P[P_heatOut] * b, fmx(R(2100) - T0, R(0)));
        R T = T0 + dT;
        R q = dT / dt;
        R phi = geo.z > R(0.5) ? R(0) : fmn((R)P[P_expansion] * q / T, R(60));

        // ---- soot (sim.js:312-318); the age gate bounds come from the extension block (reference: 0.015, 0.05)
        ageF = fmn(ageF + dt, R(4));
        sv.z += (R)P[P_sootForm] * b * smoothstep(age0, age1, ageF) * smoothstep(R(1000), R(1400), T) * (R(1) - s2.w);
        sv.z *= std::exp(-(R)P[P_sootOx] * (R(0.25) + o) * smoothstep(R(1100), R(1400), T) * dt);
        sv.z *= std::exp(-(R)P[P_sootOx] * R(0.5) * o * smoothstep(R(850), R(1100), T) * (R(1) - smoothstep(R(1100), R(1300), T)) * dt);
        sv.z *= std::exp(-(R)P[P_sootDissip] * dt);

        // ---- cooling (sim.js:321-330)
        R th = T * R(0.001);
        T -= fmn((R)P[P_radCool] * R(970) * sv.z * th * th * (th * th * th * th - R(0.00737)), R(6000)) * dt;
        R notBurning = R(1) - smoothstep(R(500), R(5000), q);
        T = R(293) + fmx(T - R(293), R(0)) * std::exp(-(R)P[P_coolRate] * notBurning * dt);
        sv.x = (T - R(293)) * R(0.001);
        sv.w = q * R(1e-4);
        sv.y *= std::exp(-(R)P[P_fuelDissip] * dt);
        s2.x *= std::exp(-(R)P[P_vitDecay] * dt);
        s2.z *= std::exp(-(R)P[P_smokeDissip] * dt);
        s2.y = ageF * clampf(sv.y + s2.x, R(0), R(1));

        // ---- buoyancy (sim.js:333)
        v.y += (R)P[P_buoyancy] * sv.x * dt;

        // ---- viscosity (sim.js:339-346)
        if (P[P_visc] > 0.0f) {
          V3<R> lapV = ld4(s.velY, i + 1, j, k, nx, ny, nz).xyz() + ld4(s.velY, i - 1, j, k, nx, ny, nz).xyz()
                     + ld4(s.velY, i, j + 1, k, nx, ny, nz).xyz() + ld4(s.velY, i, j - 1, k, nx, ny, nz).xyz()
                     + ld4(s.velY, i, j, k + 1, nx, ny, nz).xyz() + ld4(s.velY, i, j, k - 1, nx, ny, nz).xyz()
                     - load4(s.velY, i, j, k, nx, ny).xyz() * R(6);
          R nu = (R)P[P_visc] * R(1.5e-5) * std::pow(fmx(T, R(293)) / R(293), R(1.7));
          v = v + lapV * fmn(nu * dt / (dx * dx), R(0.15));
        }
        // ---- laminar base gate (sim.js:350)
        R lamAge = P[P_lamAge];
        R lam = lamAge > R(0) ? smoothstep(R(0.5) * lamAge, fmx(lamAge, R(1e-3)), ageF) : R(1);

        // ---- vorticity confinement (sim.js:353-361)
        V3<R> w = load4(s.vort, i, j, k, nx, ny).xyz();
        V3<R> g(ld4(s.vort, i + 1, j, k, nx, ny, nz).w - ld4(s.vort, i - 1, j, k, nx, ny, nz).w,
                ld4(s.vort, i, j + 1, k, nx, ny, nz).w - ld4(s.vort, i, j - 1, k, nx, ny, nz).w,
                ld4(s.vort, i, j, k + 1, nx, ny, nz).w - ld4(s.vort, i, j, k - 1, nx, ny, nz).w);
        R gl = len3(g);
        if (gl > R(1e-6)) {
          R gate = smoothstep(R(450), R(900), T) * (R(1) - srcAll) * smoothstep(R(0.02), R(0.08), p.y) * lam;
          v = v + cross3(g / gl, w) * ((R)P[P_vortEps] * gate) * dt;
        }

        // ---- curl-noise turbulence (sim.js:364-368)
        V3<R> tq = (p - V3<R>(R(0), time * (R)P[P_turbRise], R(0))) * (R)P[P_turbFreq] + V3<R>(R(0), R(0), time * (R)P[P_turbEvolve]);
        V3<R> cn = sample_repeat(s.curl.data(), s.tabN, tq, s.filter_bits).xyz();
        R tgate = fmx(smoothstep(R(500), R(1100), T), smoothstep(R(0), R(3), sv.w)) * (R(1) - srcAll) *
                  mixf(R(0.6), R(1.8), smoothstep(R(0.2), R(0.75), p.y)) * lam;
        v = v + cn * ((R)P[P_turbAmp] / R(12)) * tgate * dt * R(10);

        // ---- wind (sim.js:372-375)
        R windK = smoothstep(R(0.05), R(0.5), p.y) * (R(1) + (R)P[P_gust]);
        v.x += ((R)P[P_windX] * windK - v.x) * dt * R(0.35) * windK;
        v.z += ((R)P[P_windZ] * windK - v.z) * dt * R(0.35) * windK;
        v = v * std::exp(-(R)P[P_velDissip] * dt);

        // ---- solids & sponges (sim.js:378-388)
        if (geo.z > R(0.5)) { v = V3<R>(R(0), R(0), R(0)); sv.y = R(0); s2.y = R(0); }
        V3<R> fp(R(i) + R(0.5), R(j) + R(0.5), R(k) + R(0.5));
        R side = fmn(fmn(fp.x, nxf - fp.x), fmn(fp.z, nzf - fp.z));
        R sp = (R(1) - smoothstep(R(0), R(5), side)) * (R)P[P_sponge];
        R wsy = smoothstep(R(0.03), R(0.4), p.y);
        R wSx = (R)P[P_windX] * wsy, wSz = (R)P[P_windZ] * wsy;
        R ks = R(1) - std::pow(R(1) - R(0.15) * clampf(sp, R(0), R(1)), dt * R(90));
        v.x = mixf(v.x, wSx, ks); v.z = mixf(v.z, wSz, ks);
        R top = smoothstep(nyf - R(10), nyf, fp.y);
        R kt = std::pow(R(1) - R(0.1) * top, dt * R(90));
        sv.z *= kt; s2.z *= kt;

        R vl = len3(v);
        if (vl > R(15)) v = v * (R(15) / vl);
        bool bad = std::isnan(sv.x) || std::isnan(sv.y) || std::isnan(sv.z) || std::isnan(sv.w) ||
                   std::isnan(s2.x) || std::isnan(s2.y) || std::isnan(s2.z) || std::isnan(s2.w) ||
                   std::isnan(v.x) || std::isnan(v.y) || std::isnan(v.z);
        if (bad) { sv = V4<R>(); s2 = V4<R>(); v = V3<R>(); }
        store4(s.velX, i, j, k, nx, ny, V4<R>(v.x, v.y, v.z, phi));
        store4(s.S, i, j, k, nx, ny, sv);
        store4(s.S2, i, j, k, nx, ny, s2);
      }
}

// ---------------- divergence (src/sim.js:399-413) ----------------
template <class R> void k_div(Sim<R>& s) {
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  const R dx = s.P[P_dx];
  std::vector<R>& b0 = s.levels[0].b;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        V4<R> me = load4(s.velX, i, j, k, nx, ny);
        R L = ld4(s.velX, i - 1, j, k, nx, ny, nz).x, Rr = ld4(s.velX, i + 1, j, k, nx, ny, nz).x;
        R B = ld4(s.velX, i, j - 1, k, nx, ny, nz).y, T = ld4(s.velX, i, j + 1, k, nx, ny, nz).y;
        R K = ld4(s.velX, i, j, k - 1, nx, ny, nz).z, F = ld4(s.velX, i, j, k + 1, nx, ny, nz).z;
        if (j == 0) B = -me.y;
        R div = ((Rr - L) + (T - B) + (F - K)) / (R(2) * dx) - me.w;
        b0[cidx(i, j, k, nx, ny)] = div;
      }
}

// ---------------- multigrid (src/sim.js:415-495, 576-599) ----------------
// omega != 1 over-relaxes the update, p <- fma(omega, p_gs - p, p) (one rounding, as the CUDA sweep computes
// it); omega == 1 is mgSmooth's Gauss-Seidel update.
template <class R> void k_smooth(Level<R>& L, int color, R omega = R(1)) {            // sim.js:417-437
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  const R h2 = L.h * L.h;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = (y + z + color) & 1; x < nx; x += 2) {
        R sum = R(0), diag = R(6);
        if (x > 0) sum += L.p[cidx(x - 1, y, z, nx, ny)]; else diag += R(1);
        if (x < nx - 1) sum += L.p[cidx(x + 1, y, z, nx, ny)]; else diag += R(1);
        if (z > 0) sum += L.p[cidx(x, y, z - 1, nx, ny)]; else diag += R(1);
        if (z < nz - 1) sum += L.p[cidx(x, y, z + 1, nx, ny)]; else diag += R(1);
        if (y > 0) sum += L.p[cidx(x, y - 1, z, nx, ny)]; else diag -= R(1);
        if (y < ny - 1) sum += L.p[cidx(x, y + 1, z, nx, ny)]; else diag += R(1);
        const R gs = (sum - h2 * L.b[cidx(x, y, z, nx, ny)]) / diag;
        R& pc = L.p[cidx(x, y, z, nx, ny)];
        pc = omega == R(1) ? gs : std::fma(omega, gs - pc, pc);
      }
}
template <class R> inline R pghost(const Level<R>& L, int x, int y, int z, R me) {   // sim.js:446-450
  if (x < 0 || z < 0 || x >= L.nx || z >= L.nz || y >= L.ny) return -me;
  if (y < 0) return me;
  return L.p[cidx(x, y, z, L.nx, L.ny)];
}
template <class R> void k_restrict(Level<R>& F, Level<R>& C) {        // sim.js:439-466
  const R ih2 = R(1) / (F.h * F.h);
#pragma omp parallel for schedule(static)
  for (int cz = 0; cz < C.nz; ++cz)
    for (int cy = 0; cy < C.ny; ++cy)
      for (int cx = 0; cx < C.nx; ++cx) {
        R acc = R(0);
        for (int q = 0; q < 8; ++q) {
          int x = 2 * cx + (q & 1), y = 2 * cy + ((q >> 1) & 1), z = 2 * cz + ((q >> 2) & 1);
          R me = F.p[cidx(x, y, z, F.nx, F.ny)];
          R lap = (pghost(F, x - 1, y, z, me) + pghost(F, x + 1, y, z, me) + pghost(F, x, y - 1, z, me) +
                   pghost(F, x, y + 1, z, me) + pghost(F, x, y, z - 1, me) + pghost(F, x, y, z + 1, me) - R(6) * me) * ih2;
          acc += F.b[cidx(x, y, z, F.nx, F.ny)] - lap;
        }
        C.b[cidx(cx, cy, cz, C.nx, C.ny)] = acc * R(0.125);
        C.p[cidx(cx, cy, cz, C.nx, C.ny)] = R(0);
      }
}
template <class R> void k_prolong(Level<R>& F, const Level<R>& C) {   // sim.js:468-495
  const int ncx = F.nx / 2, ncy = F.ny / 2, ncz = F.nz / 2;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < F.nz; ++z)
    for (int y = 0; y < F.ny; ++y)
      for (int x = 0; x < F.nx; ++x) {
        R gx = (R(x) + R(0.5)) * R(0.5) - R(0.5), gy = (R(y) + R(0.5)) * R(0.5) - R(0.5), gz = (R(z) + R(0.5)) * R(0.5) - R(0.5);
        int g0x = (int)std::floor(gx), g0y = (int)std::floor(gy), g0z = (int)std::floor(gz);
        R fx = gx - R(g0x), fy = gy - R(g0y), fz = gz - R(g0z);
        R acc = R(0);
        for (int q = 0; q < 8; ++q) {
          int ox = q & 1, oy = (q >> 1) & 1, oz = (q >> 2) & 1;
          int qx = g0x + ox, qy = g0y + oy, qz = g0z + oz;
          R val = C.p[cidx(std::min(std::max(qx, 0), ncx - 1), std::min(std::max(qy, 0), ncy - 1), std::min(std::max(qz, 0), ncz - 1), C.nx, C.ny)];
          if (qx < 0 || qx >= ncx) val = -val;
          if (qz < 0 || qz >= ncz) val = -val;
          if (qy >= ncy) val = -val;
          R wx = ox ? fx : R(1) - fx, wy = oy ? fy : R(1) - fy, wz = oz ? fz : R(1) - fz;
          acc += val * wx * wy * wz;
        }
        size_t id = cidx(x, y, z, F.nx, F.ny);
        F.p[id] = F.p[id] + acc;
      }
}
template <class R> void smooth_iters(Sim<R>& s, int i, int iters) {   // sim.js:576-586
  const R w = (R)s.omega;
  for (int k = 0; k < iters; ++k) { k_smooth(s.levels[i], 0, w); k_smooth(s.levels[i], 1, w); }
}
template <class R> void vcycle(Sim<R>& s, int pre = 2, int post = 2) {   // sim.js:588-599
  const int n = (int)s.levels.size();
  for (int i = 0; i < n - 1; ++i) { smooth_iters(s, i, pre); k_restrict(s.levels[i], s.levels[i + 1]); }
  smooth_iters(s, n - 1, s.coarseIters);
  for (int i = n - 2; i >= 0; --i) { k_prolong(s.levels[i], s.levels[i + 1]); smooth_iters(s, i, post); }
}
// Relative residual ||b - A p||_2 / ||b||_2 on level 0 (FP64 sums; the operator matches the smoother).
template <class R> void residual_norms(const Sim<R>& s, double* rr, double* bb) {
  const Level<R>& L = s.levels[0];
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  const double ih2 = 1.0 / ((double)L.h * (double)L.h);
  double sr = 0, sb = 0;
#pragma omp parallel for reduction(+ : sr, sb) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        double me = L.p[cidx(x, y, z, nx, ny)];
        double lap = ((double)pghost(L, x - 1, y, z, (R)me) + (double)pghost(L, x + 1, y, z, (R)me) +
                      (double)pghost(L, x, y - 1, z, (R)me) + (double)pghost(L, x, y + 1, z, (R)me) +
                      (double)pghost(L, x, y, z - 1, (R)me) + (double)pghost(L, x, y, z + 1, (R)me) - 6.0 * me) * ih2;
        double bv = L.b[cidx(x, y, z, nx, ny)];
        double r = bv - lap;
        sr += r * r; sb += bv * bv;
      }
  *rr = sr; *bb = sb;
}

// ---------------- projection (src/sim.js:526-550) ----------------
template <class R> void k_project(Sim<R>& s) {
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  const R dx = s.P[P_dx];
  const Level<R>& L = s.levels[0];
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        R me = L.p[cidx(i, j, k, nx, ny)];
        V3<R> g(pghost(L, i + 1, j, k, me) - pghost(L, i - 1, j, k, me),
                pghost(L, i, j + 1, k, me) - pghost(L, i, j - 1, k, me),
                pghost(L, i, j, k + 1, me) - pghost(L, i, j, k - 1, me));
        g = g / (R(2) * dx);
        V3<R> v = load4(s.velX, i, j, k, nx, ny).xyz() - g;
        if (load4(s.geo, i, j, k, nx, ny).z > R(0.5)) v = V3<R>();
        if (j == 0) v.y = fmx(v.y, R(0));
        R vl = len3(v);
        if (vl > R(20) || std::isnan(vl)) v = std::isnan(vl) ? V3<R>() : v * R(20) / vl;
        store4(s.vel, i, j, k, nx, ny, V4<R>(v.x, v.y, v.z, R(0)));
      }
}

// ---------------- full step (src/sim.js:627-648) ----------------
enum { ST_GEO = 0, ST_ADV1, ST_ADV2, ST_CURL, ST_FORCES, ST_DIV, ST_VCYCLE, ST_PROJECT };

// In the rgba16float storage mode, the float4 fields a stage wrote are rounded to half after it.
template <class R> void store_stage_outputs(Sim<R>& s, int st) {
  if (!s.store_half) return;
  switch (st) {
    case ST_GEO: round_field_half(s.geo); break;
    case ST_ADV1: round_field_half(s.velX); round_field_half(s.SX); round_field_half(s.S2X); break;
    case ST_ADV2: round_field_half(s.velY); round_field_half(s.SY); round_field_half(s.S2Y); break;
    case ST_CURL: round_field_half(s.vort); break;
    case ST_FORCES: round_field_half(s.velX); round_field_half(s.S); round_field_half(s.S2); break;
    case ST_PROJECT: round_field_half(s.vel); break;
    default: break;
  }
}
template <class R> void run_stage(Sim<R>& s, int st) {
  switch (st) {
    case ST_GEO: k_geo(s); break;
    case ST_ADV1: k_adv1(s); break;
    case ST_ADV2: k_adv2(s); break;
    case ST_CURL: k_curl(s); break;
    case ST_FORCES: k_forces(s); break;
    case ST_DIV: k_div(s); break;
    case ST_VCYCLE: vcycle(s); break;
    case ST_PROJECT: k_project(s); break;
  }
  store_stage_outputs(s, st);
}

// ---------------- Poisson known-answer study (research/webgpu-bench/poisson.mjs) ----------------
// JS semantics: Float32Array storage, double arithmetic.
struct KLevel { int n; std::vector<float> p, b, r; };
inline size_t KI(int n, int x, int y, int z) { return (size_t)x + (size_t)n * ((size_t)y + (size_t)n * z); }
inline double knb(const KLevel& L, int x, int y, int z, double pc, bool face) {     // poisson.mjs:10-18
  const int n = L.n;
  auto g = [&](int xx, int yy, int zz) -> double {
    if (yy < 0) return pc;
    if (xx < 0 || yy >= n || zz < 0 || xx >= n || zz >= n) return face ? -pc : 0.0;
    return (double)L.p[KI(n, xx, yy, zz)];
  };
  double s = g(x - 1, y, z);
  s += g(x + 1, y, z); s += g(x, y - 1, z); s += g(x, y + 1, z); s += g(x, y, z - 1); s += g(x, y, z + 1);
  return s;
}
void kjacobi(KLevel& L, double h2, double omega, std::vector<float>& tmp, bool face) {   // poisson.mjs:20-27
  const int n = L.n;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        size_t i = KI(n, x, y, z); double pc = L.p[i];
        tmp[i] = (float)(pc + omega * ((knb(L, x, y, z, pc, face) - h2 * (double)L.b[i]) / 6.0 - pc));
      }
  L.p = tmp;
}
void krbgs(KLevel& L, double h2, double omega, bool face) {          // poisson.mjs:28-35
  const int n = L.n;
  for (int color = 0; color < 2; ++color) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = (y + z + color) & 1; x < n; x += 2) {
          size_t i = KI(n, x, y, z); double pc = L.p[i];
          L.p[i] = (float)(pc + omega * ((knb(L, x, y, z, pc, face) - h2 * (double)L.b[i]) / 6.0 - pc));
        }
  }
}
double kresidual(KLevel& L, double h2, bool face) {                   // poisson.mjs:36-43
  const int n = L.n;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        size_t i = KI(n, x, y, z); double pc = L.p[i];
        L.r[i] = (float)((double)L.b[i] - (knb(L, x, y, z, pc, face) - 6.0 * pc) / h2);
      }
  double s = 0;
  for (size_t i = 0; i < L.r.size(); ++i) s += (double)L.r[i] * (double)L.r[i];
  return std::sqrt(s / ((double)n * n * n));
}
void krestrict(const KLevel& F, KLevel& C) {                          // poisson.mjs:44-51
  const int n = C.n;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        double s = 0;
        for (int k = 0; k < 8; ++k) s += (double)F.r[KI(F.n, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + ((k >> 2) & 1))];
        C.b[KI(n, x, y, z)] = (float)(s / 8.0); C.p[KI(n, x, y, z)] = 0.0f;
      }
}
void kprolong(const KLevel& C, KLevel& F) {                           // poisson.mjs:52-65
  const int n = C.n;
  auto cl = [n](int v) { return std::max(0, std::min(n - 1, v)); };
#pragma omp parallel for schedule(static)
  for (int z = 0; z < F.n; ++z)
    for (int y = 0; y < F.n; ++y)
      for (int x = 0; x < F.n; ++x) {
        int cx = x >> 1, cy = y >> 1, cz = z >> 1;
        int ox = (x & 1) ? 1 : -1, oy = (y & 1) ? 1 : -1, oz = (z & 1) ? 1 : -1;
        double v = 0;
        for (int k = 0; k < 8; ++k) {
          int dx = k & 1, dy = (k >> 1) & 1, dz = (k >> 2) & 1;
          double w = (dx ? 0.25 : 0.75) * (dy ? 0.25 : 0.75) * (dz ? 0.25 : 0.75);
          v += w * (double)C.p[KI(n, cl(cx + dx * ox), cl(cy + dy * oy), cl(cz + dz * oz))];
        }
        size_t i = KI(F.n, x, y, z);
        F.p[i] = (float)((double)F.p[i] + v);
      }
}
void kvcycle(std::vector<KLevel>& lv, int l, int pre, int post, int coarse, bool face) {   // poisson.mjs:66-75
  KLevel& L = lv[l];
  double h2 = std::pow(4.0, l);
  if (l == (int)lv.size() - 1) { for (int i = 0; i < coarse; ++i) krbgs(L, h2, 1.0, face); return; }
  for (int i = 0; i < pre; ++i) krbgs(L, h2, 1.0, face);
  kresidual(L, h2, face);
  krestrict(L, lv[l + 1]);
  kvcycle(lv, l + 1, pre, post, coarse, face);
  kprolong(lv[l + 1], L);
  for (int i = 0; i < post; ++i) krbgs(L, h2, 1.0, face);
}
std::vector<float> krhs(int N) {                                      // poisson.mjs:78-92
  std::vector<float> b((size_t)N * N * N);
  auto vel = [N](int x, int y, int z, int comp) -> double {
    double u = (x + 0.5) / N, v = (y + 0.5) / N, w = (z + 0.5) / N;
    double r = std::hypot(u - 0.5, w - 0.5);
    double plume = std::exp(-(r * r) / 0.01) * std::min(1.0, v * 4);
    if (comp == 0) return std::sin(v * 12) * 0.3 + std::sin(w * 31 + u * 7) * 0.2;
    if (comp == 1) return 1.5 * plume + std::cos(u * 9) * 0.2;
    return std::sin(w * 7 + u * 5) * 0.3;
  };
  auto C = [N](int a) { return std::max(0, std::min(N - 1, a)); };
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        double vD = y == 0 ? -vel(x, y, z, 1) : vel(C(x), C(y - 1), C(z), 1);
        b[KI(N, x, y, z)] = (float)(0.5 * ((vel(C(x + 1), C(y), C(z), 0) - vel(C(x - 1), C(y), C(z), 0)) +
                                           (vel(C(x), C(y + 1), C(z), 1) - vD) +
                                           (vel(C(x), C(y), C(z + 1), 2) - vel(C(x), C(y), C(z - 1), 2))));
      }
  return b;
}

}  // namespace

// ================================================================================================
// C interface for the test harness (ctypes)
// ================================================================================================
struct OracleSim {
  int dbl;
  Sim<float> f;
  Sim<double> d;
};

template <class R> static std::vector<R>* field_ptr(Sim<R>& s, int which) {
  switch (which) {
    case 0: return &s.vel; case 1: return &s.velX; case 2: return &s.velY;
    case 3: return &s.S; case 4: return &s.SX; case 5: return &s.SY;
    case 6: return &s.S2; case 7: return &s.S2X; case 8: return &s.S2Y;
    case 9: return &s.vort; case 10: return &s.geo;
    default: return nullptr;
  }
}

template <class R, class T> static void copy_out(const std::vector<R>& v, T* out) { for (size_t i = 0; i < v.size(); ++i) out[i] = (T)v[i]; }
template <class R, class T> static void copy_in(std::vector<R>& v, const T* in) { for (size_t i = 0; i < v.size(); ++i) v[i] = (R)in[i]; }

extern "C" {

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// Noise table (noise.js:8-54): out = N^3 * 4 floats holding the half-rounded texel values.
void orc_noise_table(int N, int seed, float* out) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        float Nf = (float)N;
        V3<float> p(((float)x + 0.5f) / Nf, ((float)y + 0.5f) / Nf, ((float)z + 0.5f) / Nf);
        float a = tfbm(p, 0, seed), b = tfbm(p, 1, seed), c = tfbm(p, 2, seed);
        float w = 0.65f * worley(p, 8, seed) + 0.35f * worley(p, 16, seed);
        float* o = out + 4 * ((size_t)x + (size_t)N * ((size_t)y + (size_t)N * z));
        o[0] = round_half(a * 0.5f + 0.5f); o[1] = round_half(b * 0.5f + 0.5f); o[2] = round_half(c * 0.5f + 0.5f);
        o[3] = round_half(clampf(w, 0.0f, 1.0f));
      }
}
// Curl table (noise.js:69-80) from a (half-valued) noise table.
void orc_curl_table(int N, const float* noise, float* out) {
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        auto L = [&](int cx, int cy, int cz) {
          cx = (cx + N) % N; cy = (cy + N) % N; cz = (cz + N) % N;
          const float* t = noise + 4 * ((size_t)cx + (size_t)N * ((size_t)cy + (size_t)N * cz));
          return V3<float>(t[0] * 2.0f - 1.0f, t[1] * 2.0f - 1.0f, t[2] * 2.0f - 1.0f);
        };
        V3<float> dx = L(x + 1, y, z) - L(x - 1, y, z);
        V3<float> dy = L(x, y + 1, z) - L(x, y - 1, z);
        V3<float> dz = L(x, y, z + 1) - L(x, y, z - 1);
        float sc = (float)N / 2.0f;
        V3<float> c((dy.z - dz.y) * sc, (dz.x - dx.z) * sc, (dx.y - dy.x) * sc);
        float* o = out + 4 * ((size_t)x + (size_t)N * ((size_t)y + (size_t)N * z));
        o[0] = round_half(c.x); o[1] = round_half(c.y); o[2] = round_half(c.z); o[3] = round_half(len3(c));
      }
}
uint16_t orc_f32_to_f16(float f) { return f32_to_f16_bits(f); }
float orc_f16_to_f32(uint16_t h) { return f16_bits_to_f32(h); }
void orc_hash3f(int x, int y, int z, float* out3) { V3<float> h = hash3f(x, y, z); out3[0] = h.x; out3[1] = h.y; out3[2] = h.z; }
uint32_t orc_pcg(uint32_t n) { return pcg1(n); }
float orc_rand2(uint32_t n, uint32_t m) { return rand2(n, m); }

// buildCampfire(seed) + packLogs(max=16) (src/scene.js:13-42, 92-98): returns 16*8 floats.
void orc_build_campfire(uint32_t seed, float* out128) {
  uint32_t s = seed;
  auto R = [&s]() { s = s * 1664525u + 1013904223u; return (double)s / 4294967296.0; };
  std::vector<std::vector<double>> logs;
  auto add = [&](double ax, double ay, double az, double bx, double by, double bz, double r, double burn) {
    logs.push_back({ax, ay, az, r, bx, by, bz, burn});
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
  for (int i = 0; i < 128; ++i) out128[i] = 0.0f;
  for (size_t i = 0; i < logs.size() && i < 16; ++i)
    for (int c = 0; c < 8; ++c) out128[i * 8 + c] = (float)logs[i][c];
}

// SIM_DEFAULTS (src/sim.js:25-44) as the 64-float uniform block in SIM_FIELDS order (src/sim.js:14-23).
// The entries the simulation fills itself (dims, dx, dt, time, frame, seed, origin, nLogs) and the padding
// to 64 floats are 0.
void orc_sim_defaults(float* out64) {
  for (int i = 0; i < 64; ++i) out64[i] = 0.0f;
  const struct { int k; float v; } d[] = {
    {P_fuelSrc, 0.13f}, {P_bedFuel, 0.16f}, {P_srcTemp, 0.75f}, {P_bedTemp, 0.82f}, {P_srcVel, 0.25f},
    {P_srcFreq, 35.0f}, {P_srcSpeed, 0.06f}, {P_srcThresh, 0.0f},
    {P_ignT, 550.0f}, {P_kMix, 30.0f}, {P_rs, 4.7f}, {P_heatOut, 7700.0f}, {P_expansion, 0.7f},
    {P_sootForm, 25.0f}, {P_sootOx, 30.0f}, {P_radCool, 0.25f},
    {P_coolRate, 3.0f}, {P_sootDissip, 0.4f}, {P_smokeDissip, 0.3f}, {P_vitDecay, 1.5f}, {P_fuelDissip, 0.3f},
    {P_buoyancy, 26.8f},
    {P_vortEps, 8.0f}, {P_turbAmp, 0.8f}, {P_turbFreq, 1.5f}, {P_turbRise, 1.5f}, {P_turbEvolve, 0.6f},
    {P_windX, 0.0f}, {P_windZ, 0.0f}, {P_gust, 0.0f}, {P_intensity, 1.0f}, {P_velDissip, 0.05f},
    {P_bedRadius, 0.22f}, {P_hotR0, 0.12f}, {P_hotR1, 0.45f}, {P_hotY1, 0.5f}, {P_logSrc, 1.0f},
    {P_burstX, 0.0f}, {P_burstY, 0.0f}, {P_burstZ, 0.0f}, {P_burstAmt, 0.0f}, {P_smolder, 0.02f}, {P_sponge, 1.0f},
    {P_visc, 0.0f}, {P_lamAge, 0.0f}, {P_anchorFreq, 1.6f}, {P_srcFloor, 0.25f}, {P_anchorGain, 0.95f},
  };
  for (const auto& e : d) out64[e.k] = e.v;
}
// Seeded pyrolysis spots of the synthetic workloads (a build-defined emitter; the reference has none):
// spot i sits at radius r sqrt(u), angle 2 pi v on the floor, with u = rand2(seed, 2i), v = rand2(seed, 2i+1)
// and flux lo + (hi - lo) rand2(seed ^ 0x9e3779b9, i), where rand2(n, m) = pcg(n ^ pcg(m)) / (2^32 - 1) is the
// hash of src/shaders/lib.js:18 divided in double on the host; 5 floats per spot (x, y, z, sigma, flux g/s),
// evaluated in double and stored as float.
void orc_make_spots(uint32_t seed, int n, float lo, float hi, float sigma, float radius, float* out) {
  const double PI = 3.141592653589793;
  auto r2 = [](uint32_t a, uint32_t b) { return (double)pcg1(a ^ pcg1(b)) / 4294967295.0; };
  for (int i = 0; i < n; ++i) {
    const double u = r2(seed, 2u * (uint32_t)i), v = r2(seed, 2u * (uint32_t)i + 1u), w = r2(seed ^ 0x9e3779b9u, (uint32_t)i);
    const double r = (double)radius * std::sqrt(u), th = 2.0 * PI * v;
    out[5 * i + 0] = (float)(r * std::cos(th));
    out[5 * i + 1] = 0.0f;
    out[5 * i + 2] = (float)(r * std::sin(th));
    out[5 * i + 3] = sigma;
    out[5 * i + 4] = (float)((double)lo + ((double)hi - (double)lo) * w);
  }
}

void* orc_create(int nx, int ny, int nz, double dx, int dbl) {
  OracleSim* o = new OracleSim();
  o->dbl = dbl;
  if (dbl) sim_alloc(o->d, nx, ny, nz, dx); else sim_alloc(o->f, nx, ny, nz, dx);
  for (int i = 0; i < 64; ++i) { o->f.P[i] = 0; o->d.P[i] = 0; }
  for (int i = 0; i < E_COUNT; ++i) { o->f.E[i] = 0; o->d.E[i] = 0; }
  return o;
}
void orc_destroy(void* h) { delete (OracleSim*)h; }
int orc_num_levels(void* h) { OracleSim* o = (OracleSim*)h; return o->dbl ? (int)o->d.levels.size() : (int)o->f.levels.size(); }
void orc_level_info(void* h, int l, int* dims3, double* hh) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) { auto& L = o->d.levels[l]; dims3[0] = L.nx; dims3[1] = L.ny; dims3[2] = L.nz; *hh = L.h; }
  else { auto& L = o->f.levels[l]; dims3[0] = L.nx; dims3[1] = L.ny; dims3[2] = L.nz; *hh = L.h; }
}
int orc_coarse_iters(void* h) { OracleSim* o = (OracleSim*)h; return o->dbl ? o->d.coarseIters : o->f.coarseIters; }
void orc_set_params(void* h, const float* p64) { OracleSim* o = (OracleSim*)h; std::memcpy(o->f.P, p64, 64 * 4); std::memcpy(o->d.P, p64, 64 * 4); }
void orc_set_ext(void* h, const float* e) { OracleSim* o = (OracleSim*)h; std::memcpy(o->f.E, e, E_COUNT * 4); std::memcpy(o->d.E, e, E_COUNT * 4); }
int orc_ext_count() { return E_COUNT; }
void orc_set_logs(void* h, const float* logs, int nlogs) {
  OracleSim* o = (OracleSim*)h;
  o->f.logs.assign(logs, logs + (size_t)nlogs * 8); o->d.logs = o->f.logs;
}
void orc_set_tables(void* h, int N, const float* noise, const float* curl) {
  OracleSim* o = (OracleSim*)h;
  size_t n = (size_t)N * N * N * 4;
  o->f.tabN = o->d.tabN = N;
  o->f.noise.assign(noise, noise + n); o->f.curl.assign(curl, curl + n);
  o->d.noise = o->f.noise; o->d.curl = o->f.curl;
}
// Fields are exchanged as float or double arrays (4 * cells) depending on `as_double`.
int orc_get_field(void* h, int which, void* out, int as_double) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) { auto* f = field_ptr(o->d, which); if (!f) return -1; if (as_double) copy_out(*f, (double*)out); else copy_out(*f, (float*)out); }
  else { auto* f = field_ptr(o->f, which); if (!f) return -1; if (as_double) copy_out(*f, (double*)out); else copy_out(*f, (float*)out); }
  return 0;
}
int orc_set_field(void* h, int which, const void* in, int as_double) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) { auto* f = field_ptr(o->d, which); if (!f) return -1; if (as_double) copy_in(*f, (const double*)in); else copy_in(*f, (const float*)in); }
  else { auto* f = field_ptr(o->f, which); if (!f) return -1; if (as_double) copy_in(*f, (const double*)in); else copy_in(*f, (const float*)in); }
  return 0;
}
// Level arrays: which = 0 -> p, 1 -> b
int orc_get_level(void* h, int l, int which, void* out, int as_double) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) { auto& L = o->d.levels[l]; auto& v = which ? L.b : L.p; if (as_double) copy_out(v, (double*)out); else copy_out(v, (float*)out); }
  else { auto& L = o->f.levels[l]; auto& v = which ? L.b : L.p; if (as_double) copy_out(v, (double*)out); else copy_out(v, (float*)out); }
  return 0;
}
int orc_set_level(void* h, int l, int which, const void* in, int as_double) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) { auto& L = o->d.levels[l]; auto& v = which ? L.b : L.p; if (as_double) copy_in(v, (const double*)in); else copy_in(v, (const float*)in); }
  else { auto& L = o->f.levels[l]; auto& v = which ? L.b : L.p; if (as_double) copy_in(v, (const double*)in); else copy_in(v, (const float*)in); }
  return 0;
}
void orc_stage(void* h, int st) { OracleSim* o = (OracleSim*)h; if (o->dbl) run_stage(o->d, st); else run_stage(o->f, st); }
// MG pieces on explicit levels, for kernel-level parity.
void orc_mg_smooth(void* h, int l, int color) {
  OracleSim* o = (OracleSim*)h;
  if (o->dbl) k_smooth(o->d.levels[l], color, (double)o->d.omega); else k_smooth(o->f.levels[l], color, o->f.omega);
}
void orc_mg_restrict(void* h, int l) { OracleSim* o = (OracleSim*)h; if (o->dbl) k_restrict(o->d.levels[l], o->d.levels[l + 1]); else k_restrict(o->f.levels[l], o->f.levels[l + 1]); }
void orc_mg_prolong(void* h, int l) { OracleSim* o = (OracleSim*)h; if (o->dbl) k_prolong(o->d.levels[l], o->d.levels[l + 1]); else k_prolong(o->f.levels[l], o->f.levels[l + 1]); }
void orc_mg_vcycle(void* h, int pre, int post) { OracleSim* o = (OracleSim*)h; if (o->dbl) vcycle(o->d, pre, post); else vcycle(o->f, pre, post); }
void orc_residual(void* h, double* rr, double* bb) { OracleSim* o = (OracleSim*)h; if (o->dbl) residual_norms(o->d, rr, bb); else residual_norms(o->f, rr, bb); }

// One full step (sim.js:627-648) with the caller-provided parameter block; geo is rebuilt when
// `rebuild_geo` is set.  The caller owns time/frame bookkeeping (it writes them into the block).
// vcycles < 0 means: run V-cycles until the relative residual is <= tol, at most -vcycles cycles;
// the number of cycles run is returned.
int orc_step(void* h, int rebuild_geo, int vcycles, double tol) {
  OracleSim* o = (OracleSim*)h;
  auto go = [&](auto& s) {
    if (rebuild_geo) run_stage(s, ST_GEO);
    for (int st : {ST_ADV1, ST_ADV2, ST_CURL, ST_FORCES, ST_DIV}) run_stage(s, st);
    int done = 0;
    if (vcycles >= 0) { for (int i = 0; i < vcycles; ++i) vcycle(s); done = vcycles; }
    else {
      for (int i = 0; i < -vcycles; ++i) {
        vcycle(s); ++done;
        double rr, bb; residual_norms(s, &rr, &bb);
        if (std::sqrt(rr) <= tol * std::sqrt(bb)) break;
      }
    }
    run_stage(s, ST_PROJECT);
    return done;
  };
  return o->dbl ? go(o->d) : go(o->f);
}
// Solver / storage modes (see Sim): omega, rgba16float storage of the float4 fields, filter weight bits.
void orc_set_modes(void* h, double omega, int store_half, int filter_bits) {
  OracleSim* o = (OracleSim*)h;
  o->f.omega = o->d.omega = (float)omega;
  o->f.store_half = o->d.store_half = store_half;
  o->f.filter_bits = o->d.filter_bits = filter_bits;
}
// Spot fluxes (g/s) in double for the next steps, overriding the extension block's FP32 values; n = 0 clears.
void orc_set_flux64(void* h, const double* flux, int n) {
  OracleSim* o = (OracleSim*)h;
  o->f.flux64_set = o->d.flux64_set = n > 0;
  for (int i = 0; i < 16; ++i) o->f.flux64[i] = o->d.flux64[i] = i < n ? flux[i] : 0.0;
}
// Sweeps on the coarsest level (the constructor's coarseIters rule, src/sim.js:88-92, unless set here).
void orc_set_coarse_iters(void* h, int iters) { OracleSim* o = (OracleSim*)h; o->f.coarseIters = o->d.coarseIters = iters; }
// Reset (sim.js:606-618): zero every velocity / scalar / vorticity field and every pressure level.
void orc_reset(void* h) {
  OracleSim* o = (OracleSim*)h;
  auto go = [&](auto& s) {
    for (int w = 0; w < 10; ++w) { auto* f = field_ptr(s, w); std::fill(f->begin(), f->end(), 0); }
    for (auto& L : s.levels) std::fill(L.p.begin(), L.p.end(), 0);
  };
  if (o->dbl) go(o->d); else go(o->f);
}

// poisson.mjs study: mode 0 = Jacobi(omega), 1 = RB-SOR(omega) with the study's checkpoints
// (5,10,20,40,80,160), 2 = MG V(pre,post) with `coarse` sweeps for `cycles` cycles.
// hist receives residual / initial residual.  Returns the initial RMS residual.
double orc_poisson_study(int N, int face, int mode, double omega, int pre, int post, int coarse, int cycles, double* hist) {
  std::vector<float> B = krhs(N);
  auto fresh = [&](int n) { KLevel L; L.n = n; size_t c = (size_t)n * n * n; L.p.assign(c, 0.f); L.b.assign(c, 0.f); L.r.assign(c, 0.f); return L; };
  KLevel L0 = fresh(N); L0.b = B;
  double r0 = kresidual(L0, 1.0, face);
  if (mode == 0 || mode == 1) {
    const int cps[6] = {5, 10, 20, 40, 80, 160};
    std::vector<float> tmp((size_t)N * N * N);
    int c = 0;
    for (int k = 1; k <= 160; ++k) {
      if (mode == 0) kjacobi(L0, 1.0, omega, tmp, face); else krbgs(L0, 1.0, omega, face);
      if (c < 6 && k == cps[c]) { hist[c] = kresidual(L0, 1.0, face) / r0; ++c; }
    }
  } else {
    std::vector<KLevel> lv;
    for (int n = N; n >= 4; n >>= 1) lv.push_back(fresh(n));
    lv[0].b = B;
    for (int k = 0; k < cycles; ++k) { kvcycle(lv, 0, pre, post, coarse, face); hist[k] = kresidual(lv[0], 1.0, face) / r0; }
  }
  return r0;
}
void orc_poisson_rhs(int N, float* out) { std::vector<float> b = krhs(N); std::memcpy(out, b.data(), b.size() * 4); }

// ---- one spark update (src/sparks.js:55-142) over `count` sparks of 16 floats, FP32.  U: the 27 uniforms in
// SPARK_FIELDS order.  Spawn slots go to dead sparks in index order (one of the orders the reference's
// atomic counter can produce).  vel: the simulation's velocity field (float4 per cell); curl: the 128^3
// curl table as float4. ----
void orc_sparks_step(float* sp, int count, const float* U, const float* vel, int nx, int ny, int nz, const float* curl, int N) {
  enum { dt_, time_, frame_, count_, nBase_, nBurst_, bX_, bY_, bZ_, bSpeed_, bRad_, ox_, oy_, oz_, sx_, sy_, sz_, turb_, lifeK_,
         bedR_, seed_, sizeK_, upK_, bFan_, bSize_, aimX_, aimZ_ };
  const std::vector<float> vf(vel, vel + 4 * (size_t)nx * ny * nz);
  const uint32_t seed = (uint32_t)U[seed_], frame = (uint32_t)U[frame_];
  auto r = [&](uint32_t slot, uint32_t k) { return rand2(slot * 7919u + k * 104729u + seed, frame); };
  auto gauss = [&](uint32_t slot, uint32_t k) {
    const float u1 = std::fmax(r(slot, k), 1e-6f), u2 = r(slot, k + 1u);
    return std::sqrt(-2.0f * std::log(u1)) * std::cos(6.2831853f * u2);
  };
  auto normalize = [](V3<float> v) { return v / std::sqrt(dot3(v, v)); };
  auto fluidVel = [&](V3<float> p) {   // sparks.js:70-78
    const V3<float> g((p.x - U[ox_]) / U[sx_], (p.y - U[oy_]) / U[sy_], (p.z - U[oz_]) / U[sz_]);
    if (g.x < 0.0f || g.y < 0.0f || g.z < 0.0f || g.x > 1.0f || g.y > 1.0f || g.z > 1.0f) {
      if (g.y > 1.0f && std::sqrt(p.x * p.x + p.z * p.z) < 0.5f) return V3<float>(0.0f, 1.6f / (1.0f + (g.y - 1.0f) * 1.5f), 0.0f);
      return V3<float>();
    }
    return sample_clamp(vf, nx, ny, nz, V3<float>(g.x * (float)nx, g.y * (float)ny, g.z * (float)nz)).xyz();
  };
  const uint32_t want = (uint32_t)(U[nBase_] + U[nBurst_]);
  uint32_t deadSeen = 0;
  for (int i = 0; i < count; ++i) {
    float* s = sp + 16 * (size_t)i;
    if (s[14] < 0.5f) {   // dead: spawn (sparks.js:82-111)
      const uint32_t slot = deadSeen++;
      if (want == 0u || slot >= want) continue;
      const bool burst = slot >= (uint32_t)U[nBase_];
      V3<float> p, v;
      if (burst) {
        p = V3<float>(U[bX_], U[bY_], U[bZ_]) + (V3<float>(r(slot, 7u), r(slot, 8u), r(slot, 9u)) - V3<float>(0.5f, 0.5f, 0.5f)) * U[bRad_] * 2.0f;
        V3<float> radial(p.x, 0.0f, p.z);
        radial = len3(radial) > 1e-3f ? normalize(radial) : V3<float>();
        const V3<float> aim(U[aimX_], 0.0f, U[aimZ_]);
        const V3<float> dir = normalize(V3<float>(gauss(slot, 1u), std::fabs(gauss(slot, 3u)) * 1.2f + 0.7f, gauss(slot, 5u)) + (radial + aim) * U[bFan_]);
        v = dir * U[bSpeed_] * (0.5f + 0.8f * r(slot, 10u));
      } else {
        const float a = r(slot, 1u) * 6.2831853f, rr = std::sqrt(r(slot, 2u)) * U[bedR_];
        p = V3<float>(std::cos(a) * rr, 0.05f + r(slot, 3u) * 0.12f, std::sin(a) * rr);
        v = V3<float>(gauss(slot, 4u) * 0.4f, 0.6f + r(slot, 6u) * 1.8f, gauss(slot, 11u) * 0.4f);
      }
      const float dmm = clampf(0.5f * std::exp(0.55f * gauss(slot, 13u)) * U[sizeK_] * (burst ? U[bSize_] : 1.0f), 0.15f, 2.5f);
      const float tb = (0.25f + 2.0f * dmm * dmm) * (0.6f + 0.8f * r(slot, 15u)) * U[lifeK_];
      const float T0 = 1230.0f + 70.0f * gauss(slot, 16u) + (burst ? 80.0f : 0.0f);
      const float fl = r(slot, 20u) < 0.45f ? 5.0f + 15.0f * r(slot, 18u) : 0.0f;
      const float o[16] = {p.x, p.y, p.z, 0.0f, v.x, v.y, v.z, tb, p.x, p.y, p.z, T0, dmm, r(slot, 19u), 1.0f, fl};
      std::memcpy(s, o, sizeof o);
      continue;
    }
    // alive: integrate (sparks.js:113-141)
    const float dt = U[dt_], dmm = s[12];
    V3<float> p(s[0], s[1], s[2]), v(s[4], s[5], s[6]);
    const float tau = std::fmax(0.4f * dmm * dmm, 0.01f);
    V3<float> u = fluidVel(p) * U[upK_];
    const V3<float> tq = p * 0.9f + V3<float>(0.0f, -U[time_] * 0.5f, U[time_] * 0.13f + s[13] * 3.0f);
    const float turbAmp = U[turb_] * (0.3f + 3.0f * smoothstep(0.4f, 1.2f, p.y)) / 12.0f;
    u = u + sample_repeat(curl, N, tq).xyz() * turbAmp;
    const float k = 1.0f - std::exp(-dt / tau);
    v = V3<float>(mixf(v.x, u.x, k), mixf(v.y, u.y, k), mixf(v.z, u.z, k));
    v.y -= 9.81f * (1.0f - 0.004f) * dt * (dmm < 0.3f ? 0.2f : 1.0f);
    const float qx = p.x, qy = p.y, qz = p.z;
    p = p + v * dt;
    float T = s[11];
    const float tb = s[7] - dt;
    if (tb > 0.0f) {
      const float rel = len3(u - v);
      T = mixf(T, 1180.0f + 60.0f * std::fmin(rel, 3.0f) + 60.0f * (s[13] - 0.5f), 1.0f - std::exp(-dt / 0.3f));
    } else {
      T = 293.0f + (T - 293.0f) * std::exp(-dt / (0.06f + 0.08f * dmm));
    }
    const float age = s[3] + dt;
    const float alive = (T < 760.0f || p.y < 0.0f || p.y > 4.5f || std::sqrt(p.x * p.x + p.z * p.z) > 3.0f || age > 12.0f) ? 0.0f : 1.0f;
    const float o[16] = {p.x, p.y, p.z, age, v.x, v.y, v.z, tb, qx, qy, qz, T, s[12], s[13], alive, s[15]};
    std::memcpy(s, o, sizeof o);
  }
}

// ---- the renderer's fire passes (src/renderer.js:104-165 pLights, 194-326 pVolume), FP32.  U: the 60
// uniforms in the library's order (fire_volume_uniforms); S, S2: float4 fields; lut: 2 x n x 4 blackbody
// LUT; lights: 8 x (pos+power, colour+spread) as 16 float4. ----
enum VolIdx {
  V_width, V_height, V_vw, V_vh, V_time, V_frame, V_camX, V_camY, V_camZ, V_tanFov, V_fwdX, V_fwdY, V_fwdZ, V_aspect, V_rgtX, V_rgtY,
  V_rgtZ, V_jitX, V_upX, V_upY, V_upZ, V_jitY, V_ox, V_oy, V_oz, V_dx, V_sx, V_sy, V_sz, V_tempScale, V_nx, V_ny, V_nz, V_nLights,
  V_stepMul, V_sootAbs, V_sootEmit, V_emitK, V_blueK, V_smokeScat, V_smokeG, V_detailAmt, V_detailFreq, V_detailSpeed, V_lightK,
  V_bbTmin, V_bbTmax, V_bbN, V_emitTempLo, V_sootScat, V_sootEdge, V_cubic, V_flameSharp, V_lightDt, V_flickerK, V_lensX, V_lensY,
  V_focus, V_depthW, V_depthH, V_COUNT
};
static V3<float> bb_row(const float* U, const float* lut, float T, int row) {   // renderer.js:74-80
  const float x = clampf((T - U[V_bbTmin]) / (U[V_bbTmax] - U[V_bbTmin]), 0.0f, 1.0f) * (U[V_bbN] - 1.0f);
  const unsigned i = (unsigned)std::floor(x), n = (unsigned)U[V_bbN];
  const float f = x - std::floor(x);
  const float* a = lut + 4 * ((size_t)row * n + i);
  const float* b = lut + 4 * ((size_t)row * n + std::min(i + 1u, n - 1u));
  return V3<float>(mixf(a[0], b[0], f), mixf(a[1], b[1], f), mixf(a[2], b[2], f));
}
static float lumf(const V3<float>& c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

void orc_volume_lights(const float* U, const float* S, int nx_, int ny_, int nz_, const float* lut, float* lstate, float* lights) {
  const unsigned nx = nx_, ny = ny_, nz = nz_, NL = 8, bandH = ny / NL, hx = nx / 2, hb = bandH / 2, total = hx * hb * (nz / 2);
  for (unsigned wg = 0; wg < NL; ++wg) {
    const unsigned y0 = wg * bandH;
    float P[256][4] = {}, C[256][4] = {};
    for (unsigned li = 0; li < 256; ++li)   // the 256 lanes of the band's workgroup, each in its own order
      for (unsigned i = li; i < total; i += 256) {
        const unsigned ix = (i % hx) * 2, iy = ((i / hx) % hb) * 2 + y0, iz = (i / (hx * hb)) * 2;
        const float* s = S + 4 * ((size_t)ix + (size_t)nx * (iy + (size_t)ny * iz));
        const float T = 293.0f + s[0] * U[V_tempScale];
        if (T < 700.0f) continue;
        const V3<float> e = bb_row(U, lut, T, 1) * (s[2] * U[V_sootEmit]) * U[V_emitK];
        const float w = lumf(e);
        const V3<float> pos = V3<float>(U[V_ox], U[V_oy], U[V_oz]) + (V3<float>((float)ix, (float)iy, (float)iz) + V3<float>(1, 1, 1)) * U[V_dx];
        P[li][0] += pos.x * w; P[li][1] += pos.y * w; P[li][2] += pos.z * w; P[li][3] += w;
        C[li][0] += e.x; C[li][1] += e.y; C[li][2] += e.z; C[li][3] += dot3(pos, pos) * w;
      }
    for (unsigned s = 128; s > 0; s >>= 1)   // the workgroup's tree
      for (unsigned li = 0; li < s; ++li)
        for (int k = 0; k < 4; ++k) { P[li][k] += P[li + s][k]; C[li][k] += C[li + s][k]; }
    const float w = P[0][3];
    const V3<float> cen = w > 1e-6f ? V3<float>(P[0][0], P[0][1], P[0][2]) / w : V3<float>(0.0f, ((float)y0 + (float)bandH * 0.5f) * U[V_dx], 0.0f);
    const float spread = w > 1e-6f ? std::fmax(C[0][3] / w - dot3(cen, cen), 0.0f) : 0.04f;
    const V3<float> J = V3<float>(C[0][0], C[0][1], C[0][2]) * ((float)(nx * bandH * nz) / (float)total) * U[V_dx] * U[V_dx] * U[V_dx];
    float* sp = lstate + 4 * wg;
    float* sc = lstate + 4 * (NL + wg);
    float* sm = lstate + 4 * (2 * NL + wg);
    if (U[V_lightDt] < 0.0f || sm[3] <= 0.0f) {
      const float a[4] = {cen.x, cen.y, cen.z, spread}, b[4] = {J.x, J.y, J.z, 0.0f}, c[4] = {J.x, J.y, J.z, 1.0f};
      std::memcpy(sp, a, 16); std::memcpy(sc, b, 16); std::memcpy(sm, c, 16);
    } else {
      const float dtl = U[V_lightDt];
      const float a = 1.0f - std::exp(-dtl / 0.08f), ap = 1.0f - std::exp(-dtl / 0.15f), am = 1.0f - std::exp(-dtl / 1.5f);
      const float tgt[4] = {cen.x, cen.y, cen.z, spread};
      for (int k = 0; k < 4; ++k) sp[k] = mixf(sp[k], tgt[k], ap);
      const float Jv[3] = {J.x, J.y, J.z};
      for (int k = 0; k < 3; ++k) { sc[k] = mixf(sc[k], Jv[k], a); sm[k] = mixf(sm[k], Jv[k], am); }
      sc[3] = 0.0f; sm[3] = 1.0f;
    }
    const float ratio = lumf(V3<float>(sc[0], sc[1], sc[2])) / std::fmax(lumf(V3<float>(sm[0], sm[1], sm[2])), 1e-9f);
    const V3<float> Jc = V3<float>(sc[0], sc[1], sc[2]) * std::pow(std::fmax(ratio, 1e-4f), U[V_flickerK] - 1.0f);
    const float wl = lumf(Jc);
    const bool on = wl > 1e-3f * lumf(V3<float>(sm[0], sm[1], sm[2])) && wl > 0.0f;
    const float L[8] = {sp[0], sp[1], sp[2], on ? wl : 0.0f, on ? Jc.x : 0.0f, on ? Jc.y : 0.0f, on ? Jc.z : 0.0f, sp[3]};
    std::memcpy(lights + 8 * wg, L, sizeof L);
  }
}

void orc_volume_render(const float* U, const float* S, const float* S2, int nx, int ny, int nz, const float* curl, int N, const float* lut,
                       const float* lights, float* vol, float* aux) {
  const std::vector<float> sv(S, S + 4 * (size_t)nx * ny * nz), s2v(S2, S2 + 4 * (size_t)nx * ny * nz);
  const int vw = (int)U[V_vw], vh = (int)U[V_vh];
  auto smooth = [](float e0, float e1, float x) { return smoothstep(e0, e1, x); };
  auto fract = [](float x) { return x - std::floor(x); };
#pragma omp parallel for schedule(dynamic, 4)
  for (int iy = 0; iy < vh; ++iy)
    for (int ix = 0; ix < vw; ++ix) {
      const float pxx = (float)ix + 0.5f + U[V_jitX] * (U[V_vw] / U[V_width]), pxy = (float)iy + 0.5f + U[V_jitY] * (U[V_vw] / U[V_width]);
      const float ndx = pxx / U[V_vw] * 2.0f - 1.0f, ndy = 1.0f - pxy / U[V_vh] * 2.0f;
      const V3<float> fwd(U[V_fwdX], U[V_fwdY], U[V_fwdZ]), rgt(U[V_rgtX], U[V_rgtY], U[V_rgtZ]), up(U[V_upX], U[V_upY], U[V_upZ]);
      V3<float> dPin = fwd + rgt * ndx * U[V_tanFov] * U[V_aspect] + up * ndy * U[V_tanFov];
      dPin = dPin / std::sqrt(dot3(dPin, dPin));
      V3<float> ro(U[V_camX], U[V_camY], U[V_camZ]), rd = dPin;
      if (U[V_focus] > 0.0f) {
        const V3<float> o = ro + rgt * U[V_lensX] + up * U[V_lensY];
        const V3<float> q = ro + dPin * (U[V_focus] / dot3(dPin, fwd));
        const V3<float> dq = q - o;
        ro = o;
        rd = dq / std::sqrt(dot3(dq, dq));
      }
      const float sd = 1e9f;
      const V3<float> bmin(U[V_ox], U[V_oy], U[V_oz]), bmax = bmin + V3<float>(U[V_sx], U[V_sy], U[V_sz]);
      const V3<float> inv(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
      const V3<float> t0 = (bmin - ro) * inv, t1 = (bmax - ro) * inv;
      const float tn = std::fmax(std::fmax(std::fmax(std::fmin(t0.x, t1.x), std::fmin(t0.y, t1.y)), std::fmin(t0.z, t1.z)), 0.0f);
      const float tf = std::fmin(std::fmin(std::fmin(std::fmax(t0.x, t1.x), std::fmax(t0.y, t1.y)), std::fmax(t0.z, t1.z)), sd);
      V3<float> L;
      float Tr = 1.0f, haze = 0.0f;
      if (tf > tn) {
        const float ds = U[V_dx] * U[V_stepMul];
        const float fm = std::fmod(U[V_frame], 64.0f);
        const float ipx = (float)ix + 5.588238f * fm, ipy = (float)iy + 5.588238f * fm;
        const float jit = fract(52.9829189f * fract(ipx * 0.06711056f + ipy * 0.00583715f));
        float t = tn + ds * jit;
        const V3<float> dims(U[V_nx], U[V_ny], U[V_nz]);
        for (int it = 0; it < 1200; ++it) {
          if (t > tf || Tr < 0.003f) break;
          const V3<float> p = ro + rd * t;
          V3<float> g = (p - bmin) / U[V_dx];
          float mottle = 0.0f;
          if (U[V_detailAmt] > 0.0f) {
            const float rise = U[V_detailSpeed] * (0.5f + 1.5f * smooth(0.0f, 1.0f, p.y));
            const float ph = U[V_time] / 0.7f;
            const float f0 = fract(ph), f1 = fract(ph + 0.5f);
            const float w0 = 1.0f - std::fabs(2.0f * f0 - 1.0f);
            const V3<float> o0 = V3<float>(0.37f, 0.0f, 0.61f) * std::floor(ph), o1 = V3<float>(0.71f, 0.0f, 0.29f) * std::floor(ph + 0.5f);
            const V3<float> q0 = (p - V3<float>(0.0f, rise * f0 * 0.7f, 0.0f)) * U[V_detailFreq] * 0.25f + o0;
            const V3<float> q1 = (p - V3<float>(0.0f, rise * f1 * 0.7f, 0.0f)) * U[V_detailFreq] * 0.25f + o1;
            const V4<float> c0 = sample_repeat(curl, N, q0), c1 = sample_repeat(curl, N, q1);
            const V4<float> cw = c0 * w0 + c1 * (1.0f - w0);
            g = g + (cw.xyz() * (U[V_detailAmt] * 0.12f)) * V3<float>(1.0f, 0.6f, 1.0f);
            mottle = cw.w * 0.08f - 0.6f;
          }
          V4<float> s = sample_clamp(sv, nx, ny, nz, g);   // the cubic option is not restated
          const float edge = std::fmin(std::fmin(g.x, dims.x - g.x), std::fmin(g.z, dims.z - g.z));
          const float fade = smooth(0.02f, 0.15f, edge * U[V_dx]) * smooth(0.0f, 0.4f, (dims.y - g.y) * U[V_dx]);
          s = s * fade;
          const float T = 293.0f + s.x * U[V_tempScale] + mottle * 60.0f * U[V_detailAmt] * (s.x >= 0.3f ? 1.0f : 0.0f);
          float soot = s.z;
          if (U[V_sootEdge] > 0.0f) soot *= smooth(0.6f * U[V_sootEdge], 1.4f * U[V_sootEdge], soot);
          float smoke = 0.0f;
          if (U[V_smokeScat] > 0.0f) smoke = sample_clamp(s2v, nx, ny, nz, g).z * fade;
          if (soot > 1e-4f || s.w > 1e-3f || smoke > 1e-4f) {
            const float sigSoot = soot * U[V_sootAbs];
            const float sigS = sigSoot * U[V_sootScat] + smoke * U[V_smokeScat];
            const float sigT = sigSoot + smoke * U[V_smokeScat] * 1.1f + 1e-6f;
            V3<float> e;
            if (T > U[V_emitTempLo]) e = bb_row(U, lut, T, 1) * (soot * U[V_sootEmit]) * U[V_emitK];
            e = e + V3<float>(0.15f, 0.3f, 1.0f) * std::pow(s.w, 1.6f) * (U[V_blueK] / 3.0f) * std::exp(-soot * 2.0f);
            V3<float> ins;
            if (sigS * Tr > 1e-6f) {
              for (int k = 0; k < (int)U[V_nLights]; ++k) {
                const float* Lk = lights + 8 * k;
                const V3<float> toL = V3<float>(Lk[0], Lk[1], Lk[2]) - p;
                const float r2 = dot3(toL, toL) + Lk[7] * 0.6f + 0.004f;
                const float c = dot3(rd, toL * (1.0f / std::sqrt(r2)));
                const float g2 = U[V_smokeG] * U[V_smokeG];
                const float hgv = (1.0f - g2) / (4.0f * 3.14159265f * std::pow(1.0f + g2 - 2.0f * U[V_smokeG] * c, 1.5f));
                ins = ins + V3<float>(Lk[4], Lk[5], Lk[6]) * hgv / r2;
              }
              ins = ins * (sigS * U[V_lightK]);
            }
            const float a = std::exp(-sigT * ds);
            const float w = sigT * ds < 1e-4f ? ds : (1.0f - a) / sigT;
            L = L + (e + ins) * Tr * w;
            Tr *= a;
          }
          haze += std::fmax(s.x - 0.05f, 0.0f) * ds;
          t += ds;
        }
      }
      float* o = vol + 4 * ((size_t)ix + (size_t)vw * iy);
      o[0] = L.x; o[1] = L.y; o[2] = L.z; o[3] = Tr;
      aux[2 * ((size_t)ix + (size_t)vw * iy)] = haze;
      aux[2 * ((size_t)ix + (size_t)vw * iy) + 1] = sd;
    }
}

// ---- FP64 reference solution of the step's pressure equation (the operator of k_smooth / k_restrict:
// sum of the six ghost-ruled neighbours minus 6 p, over h^2; p = 0 on sides and top, zero gradient at the
// floor, src/sim.js:417-466).  -A is symmetric positive definite, so conjugate gradients apply. ----
static void op_apply(int nx, int ny, int nz, double ih2, const double* x, double* out) {
#pragma omp parallel for schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int i = 0; i < nx; ++i) {
        const size_t c = cidx(i, y, z, nx, ny);
        const double me = x[c];
        const double xm = i > 0 ? x[c - 1] : -me, xp = i < nx - 1 ? x[c + 1] : -me;
        const double ym = y > 0 ? x[c - nx] : me, yp = y < ny - 1 ? x[c + nx] : -me;
        const double zm = z > 0 ? x[c - (size_t)nx * ny] : -me, zp = z < nz - 1 ? x[c + (size_t)nx * ny] : -me;
        out[c] = (xm + xp + ym + yp + zm + zp - 6.0 * me) * ih2;
      }
}
static double dotp(const double* a, const double* b, size_t n) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long long i = 0; i < (long long)n; ++i) s += a[i] * b[i];
  return s;
}
// A x (FP64) for the tests.
void orc_pressure_apply(int nx, int ny, int nz, double h, const double* x, double* out) { op_apply(nx, ny, nz, 1.0 / (h * h), x, out); }
// ||b - A x|| / ||b|| in FP64 of FP32 arrays.
double orc_pressure_rel_residual(int nx, int ny, int nz, double h, const float* b, const float* x) {
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> xd(x, x + n), ax(n);
  op_apply(nx, ny, nz, 1.0 / (h * h), xd.data(), ax.data());
  double rr = 0, bb = 0;
#pragma omp parallel for reduction(+ : rr, bb) schedule(static)
  for (long long i = 0; i < (long long)n; ++i) {
    const double r = (double)b[i] - ax[i];
    rr += r * r;
    bb += (double)b[i] * (double)b[i];
  }
  return bb > 0 ? std::sqrt(rr / bb) : 0.0;
}
// Conjugate gradients on -A x = -b in FP64 from x = 0 until ||b - A x|| <= tol ||b||; returns iterations.
int orc_pressure_cg(int nx, int ny, int nz, double h, const double* b, double* x, double tol, int maxit, double* rel_out) {
  const size_t n = (size_t)nx * ny * nz;
  const double ih2 = 1.0 / (h * h);
  std::vector<double> r(n), p(n), q(n);
  for (size_t i = 0; i < n; ++i) { x[i] = 0.0; r[i] = -b[i]; p[i] = r[i]; }   // residual of -A x = -b at x = 0
  const double bb = dotp(b, b, n);
  double rr = dotp(r.data(), r.data(), n);
  int it = 0;
  while (it < maxit && rr > tol * tol * bb) {
    op_apply(nx, ny, nz, ih2, p.data(), q.data());
    for (size_t i = 0; i < n; ++i) q[i] = -q[i];
    const double alpha = rr / dotp(p.data(), q.data(), n);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    const double rr2 = dotp(r.data(), r.data(), n);
    const double beta = rr2 / rr;
    rr = rr2;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) p[i] = r[i] + beta * p[i];
    ++it;
  }
  if (rel_out) *rel_out = bb > 0 ? std::sqrt(rr / bb) : 0.0;
  return it;
}

}  // extern "C"
