// Diagnostics reductions: FIRE.stats (per-channel min / max / mean / non-finite count) and FIRE.profile's
// heat release rate (src/main.js:268-294, 347-352), as deterministic device reductions.  Per-cell work is
// FP32 (min and max are exact); sums accumulate in double-float (df64) through fixed-order trees, so the
// results are identical from run to run and use no FP64 instructions (a slow path on GB300).
#include "fire_device.cuh"

namespace fire {

constexpr int SB = 256;
constexpr int STATS_MAX_CTAS = 1216;   // 8 per SM on 152 SMs

__device__ __forceinline__ float wminf(float v) { for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o)); return v; }
__device__ __forceinline__ float wmaxf(float v) { for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o)); return v; }
__device__ __forceinline__ int wsumi(int v) { for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o); return v; }

// Per-channel partial of one CTA.
struct ChanPart { float mn, mx; df64 sum; int bad; };
__device__ __forceinline__ ChanPart cp_merge(ChanPart a, const ChanPart& b) {
  a.mn = fminf(a.mn, b.mn);
  a.mx = fmaxf(a.mx, b.mx);
  a.sum = df_add(a.sum, b.sum);
  a.bad += b.bad;
  return a;
}
__device__ __forceinline__ ChanPart cp_warp(ChanPart v) {
  v.mn = wminf(v.mn);
  v.mx = wmaxf(v.mx);
  v.sum = df_warp_sum(v.sum);
  v.bad = wsumi(v.bad);
  return v;
}
// Block-wide merge (fixed order); the result is valid in thread 0.
__device__ __forceinline__ ChanPart cp_block(ChanPart v, ChanPart* sh) {
  v = cp_warp(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    ChanPart e;
    e.mn = INFINITY; e.mx = -INFINITY; e.sum = df_make(0.0f); e.bad = 0;
    v = l < SB / 32 ? sh[l] : e;
    v = cp_warp(v);
  }
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(SB) k_stats(const float4* __restrict__ f, long long n, ChanPart* __restrict__ partials) {
  __shared__ ChanPart sh[SB / 32];
  ChanPart c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) { c[k].mn = INFINITY; c[k].mx = -INFINITY; c[k].sum = df_make(0.0f); c[k].bad = 0; }
  float sm[4] = {0.0f, 0.0f, 0.0f, 0.0f};   // a thread's FP32 running sums (a dozen cells), widened at the end
  for (long long t = (long long)blockIdx.x * SB + threadIdx.x; t < n; t += (long long)gridDim.x * SB) {
    const float4 v = __ldg(f + t);
    const float a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!isfinite(a[k])) { c[k].bad += 1; continue; }
      c[k].mn = fminf(c[k].mn, a[k]);
      c[k].mx = fmaxf(c[k].mx, a[k]);
      sm[k] += a[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    c[k].sum = df_make(sm[k]);
    ChanPart r = cp_block(c[k], sh);
    if (threadIdx.x == 0) partials[4 * (size_t)blockIdx.x + k] = r;
  }
}
// out16 = 4 x (min, max, mean, bad); mean divides by all cells, as FIRE.stats does.
__global__ void __launch_bounds__(SB) k_stats_final(const ChanPart* __restrict__ partials, int count, long long n, double* __restrict__ out16) {
  __shared__ ChanPart sh[SB / 32];
  for (int k = 0; k < 4; ++k) {
    ChanPart v;
    v.mn = INFINITY; v.mx = -INFINITY; v.sum = df_make(0.0f); v.bad = 0;
    for (int i = threadIdx.x; i < count; i += SB) v = cp_merge(v, partials[4 * (size_t)i + k]);
    v = cp_block(v, sh);
    if (threadIdx.x == 0) {
      out16[4 * k + 0] = v.mn;
      out16[4 * k + 1] = v.mx;
      out16[4 * k + 2] = df_to_double(v.sum) / (double)n;
      out16[4 * k + 3] = (double)v.bad;
    }
  }
}

// Heat release rate: Q = sum over cells with q > 0 of 354800 q / T * dx^3 (W), q = S.w * 1e4, T = 293 + 1000 S.x.
__global__ void __launch_bounds__(SB) k_hrr(const float4* __restrict__ S, long long n, df64* __restrict__ partials) {
  __shared__ df64 sh[SB / 32];
  float acc = 0.0f;   // this thread's sum of q / T over a dozen cells
  for (long long t = (long long)blockIdx.x * SB + threadIdx.x; t < n; t += (long long)gridDim.x * SB) {
    const float4 s = __ldg(S + t);
    const float q = s.w * 1e4f;
    if (q > 0.0f) acc += q / (293.0f + 1000.0f * s.x);
  }
  df64 v = df_warp_sum(df_make(acc));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = df_warp_sum(threadIdx.x < SB / 32 ? sh[threadIdx.x] : df_make(0.0f));
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}
__global__ void __launch_bounds__(SB) k_hrr_final(const df64* __restrict__ partials, int count, double scale, double* __restrict__ out) {
  __shared__ df64 sh[SB / 32];
  df64 v = df_make(0.0f);
  for (int i = threadIdx.x; i < count; i += SB) v = df_add(v, partials[i]);
  v = df_warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = df_warp_sum(threadIdx.x < SB / 32 ? sh[threadIdx.x] : df_make(0.0f));
    if (threadIdx.x == 0) out[0] = df_to_double(v) * scale;
  }
}

// fire_sim_stats_async's diagnostics in one pass over S: the stats of S (as k_stats) and the heat release
// (as k_hrr) from the same loads.  Per thread, per CTA and in the final merge every sum runs in the order of
// k_stats / k_stats_final and k_hrr / k_hrr_final, so the results are those kernels' bit for bit.
__global__ void __launch_bounds__(SB) k_diag(const float4* __restrict__ S, long long n, ChanPart* __restrict__ cparts,
                                             df64* __restrict__ hparts) {
  __shared__ ChanPart sh[SB / 32];
  __shared__ df64 shh[SB / 32];
  ChanPart c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) { c[k].mn = INFINITY; c[k].mx = -INFINITY; c[k].sum = df_make(0.0f); c[k].bad = 0; }
  float sm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  float acc = 0.0f;
  for (long long t = (long long)blockIdx.x * SB + threadIdx.x; t < n; t += (long long)gridDim.x * SB) {
    const float4 v = __ldg(S + t);
    const float a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!isfinite(a[k])) { c[k].bad += 1; continue; }
      c[k].mn = fminf(c[k].mn, a[k]);
      c[k].mx = fmaxf(c[k].mx, a[k]);
      sm[k] += a[k];
    }
    const float q = v.w * 1e4f;
    if (q > 0.0f) acc += q / (293.0f + 1000.0f * v.x);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    c[k].sum = df_make(sm[k]);
    ChanPart r = cp_block(c[k], sh);
    if (threadIdx.x == 0) cparts[4 * (size_t)blockIdx.x + k] = r;
  }
  df64 h = df_warp_sum(df_make(acc));
  if ((threadIdx.x & 31) == 0) shh[threadIdx.x >> 5] = h;
  __syncthreads();
  if (threadIdx.x < 32) {
    h = df_warp_sum(threadIdx.x < SB / 32 ? shh[threadIdx.x] : df_make(0.0f));
    if (threadIdx.x == 0) hparts[blockIdx.x] = h;
  }
}
// out17 = 4 x (min, max, mean, bad) of S, then the heat release (kW).
__global__ void __launch_bounds__(SB) k_diag_final(const ChanPart* __restrict__ cparts, const df64* __restrict__ hparts, int count,
                                                   long long n, double scale, double* __restrict__ out17) {
  __shared__ ChanPart sh[SB / 32];
  __shared__ df64 shh[SB / 32];
  ChanPart v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) { v[k].mn = INFINITY; v[k].mx = -INFINITY; v[k].sum = df_make(0.0f); v[k].bad = 0; }
  df64 h = df_make(0.0f);
  for (int i = threadIdx.x; i < count; i += SB) {   // each channel's merge runs in k_stats_final's order
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = cp_merge(v[k], cparts[4 * (size_t)i + k]);
    h = df_add(h, hparts[i]);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const ChanPart r = cp_block(v[k], sh);
    if (threadIdx.x == 0) {
      out17[4 * k + 0] = r.mn;
      out17[4 * k + 1] = r.mx;
      out17[4 * k + 2] = df_to_double(r.sum) / (double)n;
      out17[4 * k + 3] = (double)r.bad;
    }
  }
  h = df_warp_sum(h);
  if ((threadIdx.x & 31) == 0) shh[threadIdx.x >> 5] = h;
  __syncthreads();
  if (threadIdx.x < 32) {
    h = df_warp_sum(threadIdx.x < SB / 32 ? shh[threadIdx.x] : df_make(0.0f));
    if (threadIdx.x == 0) out17[16] = df_to_double(h) * scale;
  }
}

// FIRE.profile's rows (src/main.js:322-340): one CTA per profile row j = 4 * blockIdx.x.  Threads stride over
// the x-z plane of that row (x fastest, coalesced); T in FP64 as the reference's JS computes it; maxima are
// exact; the centreline sum runs per thread in cell order and then through a fixed warp/block tree.
__global__ void __launch_bounds__(SB) k_height_profile(const float4* __restrict__ S, int nx, int ny, int nz, double dx,
                                                       double* __restrict__ rows6) {
  __shared__ double s_tmax[SB / 32], s_tc[SB / 32];
  __shared__ float s_soot[SB / 32], s_fuel[SB / 32];
  __shared__ int s_hot[SB / 32], s_nc[SB / 32];
  const int j = 4 * blockIdx.x;
  double tmax = 0.0, tc = 0.0;
  float soot = 0.0f, fuel = 0.0f;
  int hot = 0, nc = 0;
  const double cx = nx / 2.0, cz = nz / 2.0;
  const long long plane = (long long)nx * nz;
  for (long long t = threadIdx.x; t < plane; t += SB) {
    const int i = (int)(t % nx), k = (int)(t / nx);
    const float4 s = __ldg(S + i + (size_t)nx * ((size_t)j + (size_t)ny * k));
    const double T = 293.0 + 1000.0 * (double)s.x;
    tmax = fmax(tmax, T);
    soot = fmaxf(soot, s.z);
    fuel = fmaxf(fuel, s.y);
    if (T > 1000.0) hot += 1;
    if (fabs(i - cx) < 3.0 && fabs(k - cz) < 3.0) { tc += T; nc += 1; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    tmax = fmax(tmax, __shfl_down_sync(0xffffffffu, tmax, o));
    tc += __shfl_down_sync(0xffffffffu, tc, o);
    soot = fmaxf(soot, __shfl_down_sync(0xffffffffu, soot, o));
    fuel = fmaxf(fuel, __shfl_down_sync(0xffffffffu, fuel, o));
    hot += __shfl_down_sync(0xffffffffu, hot, o);
    nc += __shfl_down_sync(0xffffffffu, nc, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { s_tmax[w] = tmax; s_tc[w] = tc; s_soot[w] = soot; s_fuel[w] = fuel; s_hot[w] = hot; s_nc[w] = nc; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < SB / 32; ++q) {
      tmax = fmax(tmax, s_tmax[q]); tc += s_tc[q]; soot = fmaxf(soot, s_soot[q]); fuel = fmaxf(fuel, s_fuel[q]);
      hot += s_hot[q]; nc += s_nc[q];
    }
    double* r = rows6 + 6 * (size_t)blockIdx.x;
    r[0] = (j + 0.5) * dx;
    r[1] = tc / nc;   // nc > 0: the centreline window always holds a cell
    r[2] = tmax;
    r[3] = soot;
    r[4] = fuel;
    r[5] = hot;
  }
}

int stats_partials_count(Dims d) {
  long long n = (long long)d.nx * d.ny * d.nz;
  long long b = (n + SB - 1) / SB;
  return (int)(b < STATS_MAX_CTAS ? b : STATS_MAX_CTAS);
}
// `partials` is the shared scratch (>= 128 bytes per CTA); a ChanPart is 20 bytes, 4 per CTA.
void launch_stats(const float4* f, Dims d, double* partials, double* out16, cudaStream_t st) {
  static_assert(sizeof(ChanPart) * 4 <= 128, "stats partials exceed the scratch stride");
  long long n = (long long)d.nx * d.ny * d.nz;
  int nb = stats_partials_count(d);
  ChanPart* part = reinterpret_cast<ChanPart*>(partials);
  k_stats<<<nb, SB, 0, st>>>(f, n, part);
  k_stats_final<<<1, SB, 0, st>>>(part, nb, n, out16);
}
int height_profile_rows(Dims d) { return (d.ny + 3) / 4; }
void launch_height_profile(const float4* S, Dims d, double dx, double* rows6, cudaStream_t st) {
  k_height_profile<<<height_profile_rows(d), SB, 0, st>>>(S, d.nx, d.ny, d.nz, dx, rows6);
}
// `partials`: the stats partials (80 bytes per CTA) followed by the heat-release partials (8 bytes per CTA).
void launch_diag(const float4* S, Dims d, float dx, double* partials, double* out17, cudaStream_t st) {
  long long n = (long long)d.nx * d.ny * d.nz;
  int nb = stats_partials_count(d);
  double vol = (double)dx * (double)dx * (double)dx;
  ChanPart* cpart = reinterpret_cast<ChanPart*>(partials);
  df64* hpart = reinterpret_cast<df64*>(cpart + 4 * (size_t)nb);
  static_assert(sizeof(ChanPart) * 4 + sizeof(df64) <= 128 && sizeof(ChanPart) * 4 % alignof(df64) == 0,
                "diagnostics partials fit the scratch stride");
  k_diag<<<nb, SB, 0, st>>>(S, n, cpart, hpart);
  k_diag_final<<<1, SB, 0, st>>>(cpart, hpart, nb, n, 354800.0 * vol * 1e-3, out17);   // W -> kW
}
void launch_hrr(const float4* S, Dims d, float dx, double* partials, double* out1, cudaStream_t st) {
  long long n = (long long)d.nx * d.ny * d.nz;
  int nb = stats_partials_count(d);
  double vol = (double)dx * (double)dx * (double)dx;
  df64* part = reinterpret_cast<df64*>(partials);
  k_hrr<<<nb, SB, 0, st>>>(S, n, part);
  k_hrr_final<<<1, SB, 0, st>>>(part, nb, 354800.0 * vol * 1e-3, out1);   // W -> kW
}

}  // namespace fire
