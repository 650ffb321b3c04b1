// Diagnostics reductions: FIRE.stats (per-channel min / max / mean / non-finite count) and FIRE.profile's
// heat release rate (src/main.js:268-294, 347-352), as deterministic device reductions.  Each CTA writes
// its partials; one CTA combines them in a fixed order, so results are identical from run to run.
#include "fire_device.cuh"

namespace fire {

constexpr int SB = 256;
constexpr int STATS_MAX_CTAS = 1216;   // 8 per SM on 152 SMs

__device__ __forceinline__ double wmin(double v) { for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o)); return v; }
__device__ __forceinline__ double wmax(double v) { for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o)); return v; }
__device__ __forceinline__ double wsum(double v) { for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o); return v; }

// partial layout per CTA: 4 channels x (min, max, sum, bad)
__global__ void __launch_bounds__(SB) k_stats(const float4* __restrict__ f, long long n, double* __restrict__ partials) {
  // Per-cell work is FP32 (min/max are exact in FP32; a thread sums ~a dozen cells), everything above the
  // thread is FP64 in a fixed order: GB300's FP64 rate is a small fraction of its FP32 rate.
  __shared__ double sh[SB / 32][16];
  float mn[4], mx[4], sm[4];
  int bd[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) { mn[c] = INFINITY; mx[c] = -INFINITY; sm[c] = 0.0f; bd[c] = 0; }
  for (long long t = (long long)blockIdx.x * SB + threadIdx.x; t < n; t += (long long)gridDim.x * SB) {
    float4 v = __ldg(f + t);
    float a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (!isfinite(a[c])) { bd[c] += 1; continue; }
      mn[c] = fminf(mn[c], a[c]);
      mx[c] = fmaxf(mx[c], a[c]);
      sm[c] += a[c];
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    double a = wmin((double)mn[c]), b = wmax((double)mx[c]), s = wsum((double)sm[c]), z = wsum((double)bd[c]);
    if (l == 0) { sh[w][4 * c] = a; sh[w][4 * c + 1] = b; sh[w][4 * c + 2] = s; sh[w][4 * c + 3] = z; }
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    const int k = threadIdx.x, kind = k & 3;
    double acc = sh[0][k];
    for (int i = 1; i < SB / 32; ++i) {
      double v = sh[i][k];
      acc = kind == 0 ? fmin(acc, v) : kind == 1 ? fmax(acc, v) : acc + v;
    }
    partials[16 * (size_t)blockIdx.x + k] = acc;
  }
}
// out16 = 4 x (min, max, mean, bad); mean divides by all cells, as FIRE.stats does.
__global__ void k_stats_final(const double* __restrict__ partials, int count, long long n, double* __restrict__ out16) {
  const int k = threadIdx.x;
  if (k >= 16) return;
  const int kind = k & 3;
  double acc = kind == 0 ? INFINITY : kind == 1 ? -INFINITY : 0.0;
  for (int i = 0; i < count; ++i) {
    double v = partials[16 * (size_t)i + k];
    acc = kind == 0 ? fmin(acc, v) : kind == 1 ? fmax(acc, v) : acc + v;
  }
  out16[k] = kind == 2 ? acc / (double)n : acc;
}

// Heat release rate: Q = sum over cells with q > 0 of 354800 q / T * dx^3 (W), q = S.w * 1e4, T = 293 + 1000 S.x.
__global__ void __launch_bounds__(SB) k_hrr(const float4* __restrict__ S, long long n, double vol, double* __restrict__ partials) {
  __shared__ double sh[SB / 32];
  float accf = 0.0f;   // sum of q / T over this thread's cells (FP32); scaled and widened below
  for (long long t = (long long)blockIdx.x * SB + threadIdx.x; t < n; t += (long long)gridDim.x * SB) {
    float4 s = __ldg(S + t);
    float q = s.w * 1e4f;
    if (q > 0.0f) accf += q / (293.0f + 1000.0f * s.x);
  }
  double acc = wsum((double)accf * 354800.0 * vol);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < SB / 32; ++i) a += sh[i];
    partials[blockIdx.x] = a;
  }
}
__global__ void k_sum1(const double* __restrict__ partials, int count, double scale, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double a = 0.0;
  for (int i = 0; i < count; ++i) a += partials[i];
  out[0] = a * scale;
}

int stats_partials_count(Dims d) {
  long long n = (long long)d.nx * d.ny * d.nz;
  long long b = (n + SB - 1) / SB;
  return (int)(b < STATS_MAX_CTAS ? b : STATS_MAX_CTAS);
}
void launch_stats(const float4* f, Dims d, double* partials, double* out16, cudaStream_t st) {
  long long n = (long long)d.nx * d.ny * d.nz;
  int nb = stats_partials_count(d);
  k_stats<<<nb, SB, 0, st>>>(f, n, partials);
  k_stats_final<<<1, 32, 0, st>>>(partials, nb, n, out16);
}
void launch_hrr(const float4* S, Dims d, float dx, double* partials, double* out1, cudaStream_t st) {
  long long n = (long long)d.nx * d.ny * d.nz;
  int nb = stats_partials_count(d);
  double vol = (double)dx * (double)dx * (double)dx;
  k_hrr<<<nb, SB, 0, st>>>(S, n, vol, partials);
  k_sum1<<<1, 32, 0, st>>>(partials, nb, 1e-3, out1);   // W -> kW
}

}  // namespace fire
