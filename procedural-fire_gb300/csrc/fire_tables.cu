// One-shot kernels: the tileable noise table, its curl table, and the static emitter geometry.
//
// This translation unit is compiled with -fmad=false so that every multiply and add is rounded on its
// own, in the order the WGSL writes it; with IEEE division and square root (nvcc's defaults) the tables
// and the geometry come out bit-identical to the CPU oracle.
#include "fire_device.cuh"

namespace fire {

// ---- noise table (src/noise.js:8-54) ----
__device__ __forceinline__ int wrapi(int c, int per) { return ((c % per) + per) % per; }
__device__ __forceinline__ f3 ngrad(int cx, int cy, int cz, int per, int ch, int seed) {
  f3 h = hash3f(wrapi(cx, per) + (ch * 1013 + seed), wrapi(cy, per) + ch * 7919, wrapi(cz, per) + ch * 104729);
  f3 v = mk3((h.x * 2.0f - 1.0f) + 1e-5f, (h.y * 2.0f - 1.0f) + 1e-5f, (h.z * 2.0f - 1.0f) + 1e-5f);
  float l = sqrtf(dot3(v, v));
  return mk3(v.x / l, v.y / l, v.z / l);
}
__device__ __forceinline__ float fade5(float f) { return f * f * f * (f * (f * 6.0f - 15.0f) + 10.0f); }
__device__ float tnoise(f3 p, int per, int ch, int seed) {
  float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
  int ix = (int)flx, iy = (int)fly, iz = (int)flz;
  f3 f = mk3(p.x - flx, p.y - fly, p.z - flz);
  f3 u = mk3(fade5(f.x), fade5(f.y), fade5(f.z));
  float acc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
    f3 g = ngrad(ix + ox, iy + oy, iz + oz, per, ch, seed);
    acc[k] = dot3(g, mk3(f.x - (float)ox, f.y - (float)oy, f.z - (float)oz));
  }
  float x0 = mixf(acc[0], acc[1], u.x), x1 = mixf(acc[2], acc[3], u.x);
  float x2 = mixf(acc[4], acc[5], u.x), x3 = mixf(acc[6], acc[7], u.x);
  return mixf(mixf(x0, x1, u.y), mixf(x2, x3, u.y), u.z);
}
__device__ float tfbm(f3 p01, int ch, int seed) {
  float s = 0.0f, a = 0.5f;
  int per = 4;
  for (int o = 0; o < 5; ++o) {
    float fp = (float)per;
    s += a * tnoise(mk3(p01.x * fp, p01.y * fp, p01.z * fp), per, ch, seed);
    per *= 2; a *= 0.5f;
  }
  return s * 1.5f;
}
__device__ float worley(f3 p01, int per, int seed) {
  float fp = (float)per;
  f3 p = mk3(p01.x * fp, p01.y * fp, p01.z * fp);
  float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
  int ix = (int)flx, iy = (int)fly, iz = (int)flz;
  f3 f = mk3(p.x - flx, p.y - fly, p.z - flz);
  float d = 9.0f;
  for (int k = 0; k < 27; ++k) {
    int ox = k % 3 - 1, oy = (k / 3) % 3 - 1, oz = k / 9 - 1;
    f3 h = hash3f(wrapi(ix + ox, per) + 77, wrapi(iy + oy, per) + 33, wrapi(iz + oz, per) + seed);
    f3 q = mk3(((float)ox + h.x) - f.x, ((float)oy + h.y) - f.y, ((float)oz + h.z) - f.z);
    d = fminf(d, len3(q));
  }
  return d;
}
__device__ __forceinline__ uint2 pack_h4(float a, float b, float c, float d) {
  __half2 lo = __halves2half2(__float2half_rn(a), __float2half_rn(b));
  __half2 hi = __halves2half2(__float2half_rn(c), __float2half_rn(d));
  uint2 r;
  r.x = *reinterpret_cast<unsigned*>(&lo);
  r.y = *reinterpret_cast<unsigned*>(&hi);
  return r;
}
__global__ void __launch_bounds__(256) k_noise(uint2* __restrict__ out, int N, int seed) {
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= N) return;
  float Nf = (float)N;
  f3 p = mk3(((float)x + 0.5f) / Nf, ((float)y + 0.5f) / Nf, ((float)z + 0.5f) / Nf);
  float a = tfbm(p, 0, seed), b = tfbm(p, 1, seed), c = tfbm(p, 2, seed);
  float w = 0.65f * worley(p, 8, seed) + 0.35f * worley(p, 16, seed);
  out[(size_t)x + (size_t)N * ((size_t)y + (size_t)N * z)] =
      pack_h4(a * 0.5f + 0.5f, b * 0.5f + 0.5f, c * 0.5f + 0.5f, clampf(w, 0.0f, 1.0f));
}

// ---- curl table (src/noise.js:69-80) ----
__global__ void __launch_bounds__(256) k_curltab(const uint2* __restrict__ noise, uint2* __restrict__ out, int N) {
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= N) return;
  auto L = [&](int cx, int cy, int cz) {
    cx = (cx + N) % N; cy = (cy + N) % N; cz = (cz + N) % N;
    float4 t = h4(noise[(size_t)cx + (size_t)N * ((size_t)cy + (size_t)N * cz)]);
    return mk3(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f);
  };
  f3 dx = L(x + 1, y, z) - L(x - 1, y, z);
  f3 dy = L(x, y + 1, z) - L(x, y - 1, z);
  f3 dz = L(x, y, z + 1) - L(x, y, z - 1);
  float sc = (float)N / 2.0f;
  f3 c = mk3((dy.z - dz.y) * sc, (dz.x - dx.z) * sc, (dx.y - dy.x) * sc);
  out[(size_t)x + (size_t)N * ((size_t)y + (size_t)N * z)] = pack_h4(c.x, c.y, c.z, len3(c));
}

// ---- static emitter geometry (src/sim.js:498-523) ----
__device__ __forceinline__ float sdCapsule(f3 p, f3 a, f3 b, float r) {   // src/shaders/lib.js:58-62
  f3 pa = p - a, ba = b - a;
  float h = clampf(dot3(pa, ba) / dot3(ba, ba), 0.0f, 1.0f);
  return len3(pa - ba * h) - r;
}
__global__ void __launch_bounds__(256) k_geo(const float* __restrict__ P, const float* __restrict__ logs,
                                             float4* __restrict__ geo, unsigned char* __restrict__ solidMask, Dims d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  const float dx = P[P_dx];
  const int nl = (int)P[P_nLogs];
  const float bedGain = P[P_STRIDE + E_bedGain];
  f3 p = mk3(P[P_ox], P[P_oy], P[P_oz]) + mk3((float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f) * dx;
  float dmin = 1e9f, band = 0.0f;
  for (int l = 0; l < nl; ++l) {
    const float* A = logs + 8 * l;
    const float* B = A + 4;
    f3 a = mk3(A[0], A[1], A[2]), b = mk3(B[0], B[1], B[2]);
    float Aw = A[3], Bw = B[3];
    float pxz = sqrtf(p.x * p.x + p.z * p.z);
    float dd = sdCapsule(p, a, b, Aw);
    dd += Aw * 0.3f * (1.0f - sstep(0.0f, 0.16f, pxz)) * Bw;
    dmin = fminf(dmin, dd);
    float bnd = 1.0f - sstep(0.0f, 1.6f * dx, fabsf(dd - 0.6f * dx));
    float hot = Bw * (1.0f - sstep(P[P_hotR0], P[P_hotR1], pxz)) * (1.0f - sstep(0.08f, P[P_hotY1], p.y));
    band = fmaxf(band, bnd * hot);
  }
  float r = sqrtf(p.x * p.x + p.z * p.z);
  float bedH = 0.05f * (1.0f - sstep(0.0f, P[P_bedRadius], r)) + 0.02f;
  float bed = (1.0f - sstep(0.0f, 2.0f * dx, p.y - bedH)) *
              (1.0f - sstep(P[P_bedRadius] * 0.6f, P[P_bedRadius] * 1.15f, r));
  bed = bed * bedGain;
  float solid = dmin < -0.5f * dx ? 1.0f : 0.0f;
  geo[cell(i, j, k, d.nx, d.ny)] = make_float4(band, bed, solid, dmin);
  solidMask[cell(i, j, k, d.nx, d.ny)] = solid > 0.5f ? 1 : 0;
}
__global__ void __launch_bounds__(256) k_solid_mask(const float4* __restrict__ geo, unsigned char* __restrict__ solid, long long n) {
  long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t < n) solid[t] = geo[t].z > 0.5f ? 1 : 0;
}

void launch_noise_table(uint2* noise, int N, int seed, cudaStream_t st) {
  dim3 b(128), g((N + 127) / 128, N, N);
  k_noise<<<g, b, 0, st>>>(noise, N, seed);
}
void launch_curl_table(const uint2* noise, uint2* curl, int N, cudaStream_t st) {
  dim3 b(128), g((N + 127) / 128, N, N);
  k_curltab<<<g, b, 0, st>>>(noise, curl, N);
}
void launch_geo(const float* P, const float* logs, float4* geo, unsigned char* solid, Dims d, cudaStream_t st) {
  dim3 b(32, 8), g((d.nx + 31) / 32, (d.ny + 7) / 8, d.nz);
  k_geo<<<g, b, 0, st>>>(P, logs, geo, solid, d);
}
void launch_solid_mask(const float4* geo, unsigned char* solid, Dims d, cudaStream_t st) {
  long long n = (long long)d.nx * d.ny * d.nz;
  k_solid_mask<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(geo, solid, n);
}

}  // namespace fire
