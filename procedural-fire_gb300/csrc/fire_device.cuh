// Device helpers for the fire simulation kernels: WGSL builtin semantics, hashing and trilinear sampling.
//
// The semantics match the CPU oracle exactly (same expression order):
//   clamp(x, lo, hi) = fminf(fmaxf(x, lo), hi)   (NaN -> lo)
//   mix(a, b, t)     = a * (1 - t) + b * t
//   smoothstep       = t * t * (3 - 2 t), t = clamp((x - e0) / (e1 - e0), 0, 1)
//   textureSampleLevel(linear) = trilinear in cell units (texel i's centre at i + 0.5), exact weights.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>
#include "fire_internal.h"

namespace fire {

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
// smoothstep with t = (x - e0) * (1 / (e1 - e0)): the reciprocal folds to a constant for literal edges, so
// the ~15 smoothsteps per cell cost no division (well inside WGSL's smoothstep accuracy; the oracle uses
// the same formula).
// sstep_inv takes the reciprocal precomputed: for edges that are per-step parameters the host evaluates
// 1 / (e1 - e0) once, in the same FP32 operations, so the result is the same bit for bit.
__device__ __forceinline__ float sstep_inv(float e0, float inv, float x) {
  float t = clampf((x - e0) * inv, 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float sstep(float e0, float e1, float x) { return sstep_inv(e0, 1.0f / (e1 - e0), x); }

// ---- double-float ("df64") accumulation: value = hi + lo with |lo| <= ulp(hi)/2 ----
// GB300 executes FP64 on a slow path, so every cross-thread reduction accumulates in pairs of FP32 with
// error-free TwoSum (~48-bit significand) instead of double; trees run in a fixed order, so results are
// deterministic.
struct df64 { float hi, lo; };
__device__ __forceinline__ df64 df_make(float a) { df64 r; r.hi = a; r.lo = 0.0f; return r; }
__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);   // TwoSum error of a.hi + b.hi
  const float lo = err + (a.lo + b.lo);
  df64 r;
  r.hi = s + lo;
  r.lo = lo - (r.hi - s);
  return r;
}
__device__ __forceinline__ df64 df_shfl_down(df64 v, int o) {
  df64 r;
  r.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
  r.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
  return r;
}
__device__ __forceinline__ df64 df_warp_sum(df64 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = df_add(v, df_shfl_down(v, o));
  return v;
}
__device__ __forceinline__ double df_to_double(df64 v) { return (double)v.hi + (double)v.lo; }

// Sums `count` float4 partial pairs (x + y, z + w as df64) in a fixed order with NT threads standing in for
// SUMV virtual threads: virtual thread v takes partials v, v+SUMV, ...; each virtual warp is reduced by a
// warp tree, and the SUMV/32 warp sums by a final warp tree.  The result depends only on `count` and the
// partials, never on which CTA or how many real threads run it.  Thread 0 receives (A, B); all NT threads
// of the CTA must call it (one __syncthreads inside); sa, sb: shared arrays of SUMV/32 entries.
constexpr int SUMV = 1024;
constexpr int SUM_BATCH = 4;   // partials per virtual thread loaded together
template <int NT>
__device__ __forceinline__ void sum_pairs_fixed(const float4* partials, int count, int tid, df64* sa, df64* sb, df64& A, df64& B) {
  static_assert(SUMV % NT == 0 && NT % 32 == 0, "virtual threads map onto whole warps");
  constexpr int J = SUMV / NT;
  df64 a[J], b[J];
#pragma unroll
  for (int j = 0; j < J; ++j) { a[j] = df_make(0.0f); b[j] = df_make(0.0f); }
  for (int i0 = 0; i0 < count; i0 += SUM_BATCH * SUMV) {
    // all loads of the batch first (they are independent), then the adds in each virtual thread's order
    float4 q[J][SUM_BATCH];
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
      for (int u = 0; u < SUM_BATCH; ++u) {
        const int i = i0 + u * SUMV + tid + NT * j;
        q[j][u] = i < count ? __ldcg(partials + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
      for (int u = 0; u < SUM_BATCH; ++u) {
        if (i0 + u * SUMV + tid + NT * j < count) {
          a[j] = df_add(a[j], df64{q[j][u].x, q[j][u].y});
          b[j] = df_add(b[j], df64{q[j][u].z, q[j][u].w});
        }
      }
  }
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int v = tid + NT * j;
    const df64 wa = df_warp_sum(a[j]);
    const df64 wb = df_warp_sum(b[j]);
    if ((tid & 31) == 0) { sa[v >> 5] = wa; sb[v >> 5] = wb; }
  }
  __syncthreads();
  if (tid < 32) {
    A = df_warp_sum(sa[tid]);
    B = df_warp_sum(sb[tid]);
  }
}

// The simulation of this CTA of a batched launch and the CTA's position in that simulation's grid
// (binary search of the flat block index in the map's prefix sums).
__device__ __forceinline__ void batch_locate(const BatchMap& m, uint3& blk, int& inst) {
  const int b = (int)blockIdx.x;
  int lo = 0, hi = m.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (m.prefix[mid] <= b) lo = mid; else hi = mid - 1;
  }
  const int lb = b - m.prefix[lo], gx = m.gx[lo], gy = m.gy[lo];
  blk = make_uint3((unsigned)(lb % gx), (unsigned)((lb / gx) % gy), (unsigned)(lb / (gx * gy)));
  inst = m.inst[lo];
}

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 xyz(const float4& v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ f3 fmin3(f3 a, f3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ f3 fmax3(f3 a, f3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float4 fmin4(float4 a, float4 b) { return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w)); }
__device__ __forceinline__ float4 fmax4(float4 a, float4 b) { return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w)); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 sub4(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ float4 mul4(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

__device__ __forceinline__ size_t cell(int x, int y, int z, int nx, int ny) {
  return (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * (size_t)z);
}
__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }
// textureLoad with clamped coordinates (`ld`, src/sim.js:114)
__device__ __forceinline__ float4 ldc(const float4* __restrict__ f, int x, int y, int z, Dims d) {
  x = min(max(x, 0), d.nx - 1); y = min(max(y, 0), d.ny - 1); z = min(max(z, 0), d.nz - 1);
  return __ldg(f + (x + d.nx * (y + d.ny * z)));   // 32-bit offset, as in sample()
}

// ---- hashes (src/shaders/lib.js:3-18) ----
__device__ __forceinline__ uint3 pcg3d(uint3 v) {
  v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u; v.z = v.z * 1664525u + 1013904223u;
  v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
  v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16;
  v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
  return v;
}
constexpr float kInvU32 = 2.3283064365386963e-10f;   // f32(1 / 4294967295) == 2^-32
__device__ __forceinline__ f3 hash3f(int x, int y, int z) {
  uint3 h = pcg3d(make_uint3((unsigned)x, (unsigned)y, (unsigned)z));
  return mk3(__uint2float_rn(h.x) * kInvU32, __uint2float_rn(h.y) * kInvU32, __uint2float_rn(h.z) * kInvU32);
}

// ---- trilinear sampling, clamp-to-edge, in cell units ----
struct Tap {
  int x0, x1, y0, y1, z0, z1;
  float fx, fy, fz;
};
__device__ __forceinline__ void axis_clamp(float c, int n, int& i0, int& i1, float& f) {
  float u = clampf(c - 0.5f, -1.0f, (float)n);   // clamping u to [-1, n] does not change a clamp-to-edge sample
  float fl = floorf(u);
  int i = (int)fl;
  f = u - fl;
  i0 = min(max(i, 0), n - 1);
  i1 = min(max(i + 1, 0), n - 1);
}
__device__ __forceinline__ Tap make_tap(f3 c, Dims d) {
  Tap t;
  axis_clamp(c.x, d.nx, t.x0, t.x1, t.fx);
  axis_clamp(c.y, d.ny, t.y0, t.y1, t.fy);
  axis_clamp(c.z, d.nz, t.z0, t.z1, t.fz);
  return t;
}
__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  float s = 1.0f - t;
  return make_float4(a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t);
}
// Cell offsets of the gathers are 32-bit (a simulation has fewer than 2^31 cells, checked at creation): half the
// registers of 64-bit offsets, which keeps the MacCormack kernels' eight-texel stencils out of local memory.
__device__ __forceinline__ float4 sample(const float4* __restrict__ f, const Tap& t, Dims d) {
  const int sy = d.nx, sz = d.nx * d.ny;
  const int r00 = t.y0 * sy + t.z0 * sz, r10 = t.y1 * sy + t.z0 * sz;
  const int r01 = t.y0 * sy + t.z1 * sz, r11 = t.y1 * sy + t.z1 * sz;
  float4 c00 = lerp4(__ldg(f + r00 + t.x0), __ldg(f + r00 + t.x1), t.fx);
  float4 c10 = lerp4(__ldg(f + r10 + t.x0), __ldg(f + r10 + t.x1), t.fx);
  float4 c01 = lerp4(__ldg(f + r01 + t.x0), __ldg(f + r01 + t.x1), t.fx);
  float4 c11 = lerp4(__ldg(f + r11 + t.x0), __ldg(f + r11 + t.x1), t.fx);
  return lerp4(lerp4(c00, c10, t.fy), lerp4(c01, c11, t.fy), t.fz);
}

// ---- repeat-addressed sampling of a 128^3 half4 table in normalised coordinates ----
__device__ __forceinline__ float4 h4(uint2 v) {
  __half2 a = *reinterpret_cast<__half2*>(&v.x);
  __half2 b = *reinterpret_cast<__half2*>(&v.y);
  float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ int wrapN(long long i) { long long m = i % TABLE_N; return (int)(m < 0 ? m + TABLE_N : m); }
__device__ __forceinline__ float4 sample_table(const uint2* __restrict__ tab, f3 q) {
  const float N = (float)TABLE_N;
  float ux = q.x * N - 0.5f, uy = q.y * N - 0.5f, uz = q.z * N - 0.5f;
  float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
  float fx = ux - flx, fy = uy - fly, fz = uz - flz;
  long long ix = (long long)flx, iy = (long long)fly, iz = (long long)flz;
  int x0 = wrapN(ix), x1 = wrapN(ix + 1), y0 = wrapN(iy), y1 = wrapN(iy + 1), z0 = wrapN(iz), z1 = wrapN(iz + 1);
  auto T = [&](int x, int y, int z) { return h4(__ldg(tab + x + TABLE_N * (y + TABLE_N * z))); };
  float4 c00 = lerp4(T(x0, y0, z0), T(x1, y0, z0), fx);
  float4 c10 = lerp4(T(x0, y1, z0), T(x1, y1, z0), fx);
  float4 c01 = lerp4(T(x0, y0, z1), T(x1, y0, z1), fx);
  float4 c11 = lerp4(T(x0, y1, z1), T(x1, y1, z1), fx);
  return lerp4(lerp4(c00, c10, fy), lerp4(c01, c11, fy), fz);
}


// ---- shared by the step kernels (fire_step.cu) and their adjoints (fire_adjoint.cu) ----
// Scalars entering from outside the domain are ambient (src/sim.js:137-140)
__device__ __forceinline__ float outside_fade(f3 c, Dims d) {
  float lo = fminf(c.x, c.z);
  float hi = fmaxf(c.x - (float)d.nx, fmaxf(c.y - (float)d.ny, c.z - (float)d.nz));
  return clampf(1.0f - fmaxf(-lo, hi), 0.0f, 1.0f);
}
// RK2 midpoint back-trace in cells (src/sim.js:129-135).  The first velocity sample sits exactly on the
// cell centre, where the trilinear weights are (1, 0) on every axis, so it equals the cell's own value.
__device__ __forceinline__ f3 backtrace(const float4* __restrict__ vel, f3 c, f3 v0, float dt, float dx, Dims d) {
  f3 mid = c - v0 * (0.5f * dt) / dx;
  f3 v1 = xyz(sample(vel, make_tap(mid, d), d));
  return c - v1 * dt / dx;
}

// Vorticity at cell (x, y, z) (already inside the domain), from clamped velY neighbours.
__device__ __forceinline__ float4 curl_at(const float4* __restrict__ v, int x, int y, int z, Dims d) {
  f3 L = xyz(ldc(v, x - 1, y, z, d)), R = xyz(ldc(v, x + 1, y, z, d));
  f3 B = xyz(ldc(v, x, y - 1, z, d)), T = xyz(ldc(v, x, y + 1, z, d));
  f3 K = xyz(ldc(v, x, y, z - 1, d)), F = xyz(ldc(v, x, y, z + 1, d));
  f3 w = mk3((T.z - B.z) - (F.y - K.y), (F.x - K.x) - (R.z - L.z), (R.y - L.y) - (T.x - B.x)) * 0.5f;
  return make_float4(w.x, w.y, w.z, len3(w));
}

__device__ __forceinline__ float4 noise4(const uint2* __restrict__ tab, f3 q) {    // src/sim.js:228
  float4 t = sample_table(tab, q);
  return make_float4(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f, t.w * 2.0f - 1.0f);
}

}  // namespace fire
