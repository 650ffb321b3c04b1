// Standalone pressure Poisson solver: the step's multigrid (src/sim.js:415-495, 576-599) iterated to a
// relative-residual tolerance, in the plain FP32 form or as mixed-precision iterative refinement.
//
// Mixed-precision form (FIRE_POISSON_FP16 / FIRE_POISSON_BF16):
//   x, b and every residual are FP32; the correction equation A e = r is solved approximately by V(2,2)
//   cycles whose level arrays (p and b of every level above the shared-memory tail) are stored in IEEE half
//   or bfloat16, with all arithmetic in FP32 registers.  Halving the bytes of the fine levels is the point:
//   at 256x512x256 the level-0 arrays of the FP32 form (268 MB) do not fit the 129 MB L2 and every sweep is
//   HBM-bound.  The residual handed to the correction solve is scaled by 1/RMS of the previous residual, so
//   it stays O(1) inside half's range; the scale is undone when the correction is added.  The coarsest
//   level is solved in FP64 (64 red-black sweeps on a double copy in shared memory).
// Loop on the device:
//   pre:   ||b||^2  -> scale 1/RMS(b);  r0 = b - A x0 (written scaled into the level-0 RHS);  test
//   WHILE: V-cycle(s) on (e, r~);  x += e * unscale;  r = b - A x (written scaled);  test
// where each test is one small kernel that sums the residual partials in a fixed order (double-float),
// updates the scales and sets the conditional node's value.  The FP32 form runs the step's own V-cycle on
// (x, b) with the same pre-pass and test.
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/fire_sim.h"
#include "fire_internal.h"
#include "fire_device.cuh"
#include "fire_launch.cuh"
#include "fire_nvtx.h"

namespace fire {
namespace {

constexpr int GX = 32, GY = 4, GZ = 2, NT = GX * GY * GZ;
constexpr int SMZ = 2;   // cells of one colour per smoother thread (as the step's smoother)
constexpr int RZ = 8;    // z-planes per residual thread
constexpr int SUMSQ_CTAS = 1024;
constexpr int COARSE64_SWEEPS = 64;

// ---- storage types: loads widen to FP32, stores round to nearest ----
template <typename T> struct Sto;
template <> struct Sto<float> {
  static __device__ __forceinline__ float ld(const float* p) { return *p; }
  static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
};
template <> struct Sto<__half> {
  static __device__ __forceinline__ float ld(const __half* p) { return __half2float(*p); }
  static __device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
};
template <> struct Sto<__nv_bfloat16> {
  static __device__ __forceinline__ float ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
  static __device__ __forceinline__ void st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
};

// A level's array in one of two layouts.  Plain: x fastest, then y, then z.  Red-black split (even nx): the
// cells of colour (x + y + z) & 1 == c are stored contiguously in half c (nx/2 * ny * nz elements each) at
// (x >> 1) + (nx/2) * (y + ny * z), so a colour sweep reads one half, writes the other with unit stride and
// touches each byte once (the interleaved layout moves whole cache lines of both colours every sweep).
template <typename T>
struct LV {
  T* a;
  int nx, ny, nz, split;
  __device__ __forceinline__ T* at(int x, int y, int z) const {
    if (!split) return a + (x + nx * (y + ny * z));
    const int hx = nx >> 1;
    return a + (((x + y + z) & 1) ? hx * ny * nz : 0) + (x >> 1) + hx * (y + ny * z);
  }
};

// Red-black sweep of one colour (mgSmooth, src/sim.js:417-437) on T storage in the plain layout.  zero_nbrs:
// the level's current values are taken as zero (the first half-sweep of a correction solve from e = 0: the
// colour being updated never reads its own old value, so the other colour's stale contents are not read).
template <typename T>
__global__ void __launch_bounds__(NT) k_psmooth(T* __restrict__ p, const T* __restrict__ b, int nx, int ny, int nz, float h, int color,
                                                int zero_nbrs) {
  pdl_wait();
  pdl_trigger();
  const int gx = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int zb = (blockIdx.z * GZ + threadIdx.z) * SMZ;
  if (y >= ny) return;
  const float h2 = h * h;
  const int sy = nx, sz = nx * ny;
  float v[SMZ];
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) {
      const int c = x + y * sy + z * sz;
      float sum = 0.0f, diag = 6.0f;
      const bool rd = !zero_nbrs;
      if (x > 0) { if (rd) sum += Sto<T>::ld(p + c - 1); } else diag += 1.0f;
      if (x < nx - 1) { if (rd) sum += Sto<T>::ld(p + c + 1); } else diag += 1.0f;
      if (z > 0) { if (rd) sum += Sto<T>::ld(p + c - sz); } else diag += 1.0f;
      if (z < nz - 1) { if (rd) sum += Sto<T>::ld(p + c + sz); } else diag += 1.0f;
      if (y > 0) { if (rd) sum += Sto<T>::ld(p + c - sy); } else diag -= 1.0f;
      if (y < ny - 1) { if (rd) sum += Sto<T>::ld(p + c + sy); } else diag += 1.0f;
      v[k] = __fdividef(sum - h2 * Sto<T>::ld(b + c), diag);
    }
  }
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) Sto<T>::st(p + x + sy * y + sz * z, v[k]);
  }
}
// The same sweep on the red-black split layout: a thread updates the colour cell at half-index gx of SMZ
// rows; its x neighbours are the other colour's entries gx - 1 + s and gx + s (s = the cell's x parity),
// its y and z neighbours the other colour's entry gx of the adjacent rows.
template <typename T, bool kZero>
__global__ void __launch_bounds__(NT) k_psmooth_rb(T* __restrict__ p, const T* __restrict__ b, int nx, int ny, int nz, float h, int color) {
  pdl_wait();
  pdl_trigger();
  const int hx = nx >> 1, half = hx * ny * nz, ry = hx, rz = hx * ny;
  const int gx = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int zb = (blockIdx.z * GZ + threadIdx.z) * SMZ;
  if (gx >= hx || y >= ny) return;
  T* __restrict__ pc = p + color * half;
  const T* __restrict__ po = p + (1 - color) * half;
  const T* __restrict__ bc = b + color * half;
  const float h2 = h * h;
  float v[SMZ];
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    if (z < nz) {
      const int s = (y + z + color) & 1;
      const int r = gx + ry * y + rz * z;
      float sum = 0.0f, diag = 6.0f;
      if (gx > 0 || s) { if (!kZero) sum += Sto<T>::ld(po + r - 1 + s); } else diag += 1.0f;
      if (gx < hx - 1 || !s) { if (!kZero) sum += Sto<T>::ld(po + r + s); } else diag += 1.0f;
      if (z > 0) { if (!kZero) sum += Sto<T>::ld(po + r - rz); } else diag += 1.0f;
      if (z < nz - 1) { if (!kZero) sum += Sto<T>::ld(po + r + rz); } else diag += 1.0f;
      if (y > 0) { if (!kZero) sum += Sto<T>::ld(po + r - ry); } else diag -= 1.0f;
      if (y < ny - 1) { if (!kZero) sum += Sto<T>::ld(po + r + ry); } else diag += 1.0f;
      v[k] = __fdividef(sum - h2 * Sto<T>::ld(bc + r), diag);
    }
  }
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    if (z < nz) Sto<T>::st(pc + gx + ry * y + rz * z, v[k]);
  }
}

// Two adjacent entries (2 g, 2 g + 1) as one 4- or 8-byte load / store.
template <typename T> struct Pair;
template <> struct Pair<float> {
  static __device__ __forceinline__ float2 ld(const float* p) { return *reinterpret_cast<const float2*>(p); }
  static __device__ __forceinline__ void st(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
};
template <> struct Pair<__half> {
  static __device__ __forceinline__ float2 ld(const __half* p) { return __half22float2(*reinterpret_cast<const __half2*>(p)); }
  static __device__ __forceinline__ void st(__half* p, float a, float b) { *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b); }
};
template <> struct Pair<__nv_bfloat16> {
  static __device__ __forceinline__ float2 ld(const __nv_bfloat16* p) { return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p)); }
  static __device__ __forceinline__ void st(__nv_bfloat16* p, float a, float b) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
  }
};
// k_psmooth_rb with a pair of same-colour cells (half-indices 2 g, 2 g + 1 of one row) per thread and SMZ
// rows: b, the y and z neighbours and the result move as pairs; the three x neighbours of the pair are one
// pair plus one scalar of the other colour (which side depends on the row's x parity s).  Needs nx % 4 == 0
// so every colour half and row starts at an even entry.  Same arithmetic and order as k_psmooth_rb.
template <typename T, bool kZero>
__global__ void __launch_bounds__(NT) k_psmooth_rb2(T* __restrict__ p, const T* __restrict__ b, int nx, int ny, int nz, float h, int color) {
  pdl_wait();
  pdl_trigger();
  const int hx = nx >> 1, half = hx * ny * nz, ry = hx, rz = hx * ny;
  const int g = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int zb = (blockIdx.z * GZ + threadIdx.z) * SMZ;
  const int gx = 2 * g;
  if (gx >= hx || y >= ny) return;
  T* __restrict__ pc = p + color * half;
  const T* __restrict__ po = p + (1 - color) * half;
  const T* __restrict__ bc = b + color * half;
  const float h2 = h * h;
  float v0[SMZ], v1[SMZ];
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    if (z < nz) {
      const int s = (y + z + color) & 1;
      const int r = gx + ry * y + rz * z;
      float2 o = make_float2(0.0f, 0.0f), ym = o, yp = o, zm = o, zp = o;
      float side = 0.0f;
      // x neighbours: s = 0 -> entries 2g-1 (cell 0's x-), 2g, 2g+1; s = 1 -> 2g, 2g+1, 2g+2 (cell 1's x+)
      const bool cell0_xm = gx > 0 || s, cell1_xp = gx + 1 < hx - 1 || !s;
      if (!kZero) {
        o = Pair<T>::ld(po + r);
        if (!s && cell0_xm) side = Sto<T>::ld(po + r - 1);
        if (s && cell1_xp) side = Sto<T>::ld(po + r + 2);
        if (z > 0) zm = Pair<T>::ld(po + r - rz);
        if (z < nz - 1) zp = Pair<T>::ld(po + r + rz);
        if (y > 0) ym = Pair<T>::ld(po + r - ry);
        if (y < ny - 1) yp = Pair<T>::ld(po + r + ry);
      }
      const float2 bv = Pair<T>::ld(bc + r);
      // cell 0 (half-index 2g): x- = s ? o.x : side, x+ = s ? o.y : o.x
      {
        float sum = 0.0f, diag = 6.0f;
        if (cell0_xm) { if (!kZero) sum += s ? o.x : side; } else diag += 1.0f;
        if (!kZero) sum += s ? o.y : o.x;   // x+ of cell 0 always exists (cell 1 follows it)
        if (z > 0) { if (!kZero) sum += zm.x; } else diag += 1.0f;
        if (z < nz - 1) { if (!kZero) sum += zp.x; } else diag += 1.0f;
        if (y > 0) { if (!kZero) sum += ym.x; } else diag -= 1.0f;
        if (y < ny - 1) { if (!kZero) sum += yp.x; } else diag += 1.0f;
        v0[k] = __fdividef(sum - h2 * bv.x, diag);
      }
      // cell 1 (half-index 2g+1): x- = s ? o.y : o.x, x+ = s ? side : o.y
      {
        float sum = 0.0f, diag = 6.0f;
        if (!kZero) sum += s ? o.y : o.x;   // x- of cell 1 always exists
        if (cell1_xp) { if (!kZero) sum += s ? side : o.y; } else diag += 1.0f;
        if (z > 0) { if (!kZero) sum += zm.y; } else diag += 1.0f;
        if (z < nz - 1) { if (!kZero) sum += zp.y; } else diag += 1.0f;
        if (y > 0) { if (!kZero) sum += ym.y; } else diag -= 1.0f;
        if (y < ny - 1) { if (!kZero) sum += yp.y; } else diag += 1.0f;
        v1[k] = __fdividef(sum - h2 * bv.y, diag);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {
    const int z = zb + k;
    if (z < nz) Pair<T>::st(pc + gx + ry * y + rz * z, v0[k], v1[k]);
  }
}

template <typename T>
__device__ __forceinline__ float pgv(const LV<T>& L, int x, int y, int z, float me) {
  if (x < 0 || z < 0 || x >= L.nx || z >= L.nz || y >= L.ny) return -me;
  if (y < 0) return me;
  return Sto<T>::ld(L.at(x, y, z));
}
// Fused residual + 8-child restriction (src/sim.js:439-466); coarse p set to 0.  Either level in either layout.
template <typename TF, typename TC>
__global__ void __launch_bounds__(NT) k_prestrict(const TF* __restrict__ p, const TF* __restrict__ b, int fsplit, int nx, int ny, int nz,
                                                  float h, TC* __restrict__ bc, TC* __restrict__ pc, int csplit) {
  pdl_wait();
  pdl_trigger();
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
  if (cx >= cnx || cy >= cny || cz >= cnz) return;
  const LV<TF> P{const_cast<TF*>(p), nx, ny, nz, fsplit}, B{const_cast<TF*>(b), nx, ny, nz, fsplit};
  const float ih2 = 1.0f / (h * h);
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int x = 2 * cx + (q & 1), y = 2 * cy + ((q >> 1) & 1), z = 2 * cz + ((q >> 2) & 1);
    const float me = Sto<TF>::ld(P.at(x, y, z));
    const float lap = (pgv(P, x - 1, y, z, me) + pgv(P, x + 1, y, z, me) + pgv(P, x, y - 1, z, me) + pgv(P, x, y + 1, z, me) +
                       pgv(P, x, y, z - 1, me) + pgv(P, x, y, z + 1, me) - 6.0f * me) * ih2;
    acc += Sto<TF>::ld(B.at(x, y, z)) - lap;
  }
  const LV<TC> PC{pc, cnx, cny, cnz, csplit}, BC{bc, cnx, cny, cnz, csplit};
  Sto<TC>::st(BC.at(cx, cy, cz), acc * 0.125f);
  Sto<TC>::st(PC.at(cx, cy, cz), 0.0f);
}
// Trilinear prolongation with mirror ghosts (src/sim.js:468-495), coarse-cell centric as the step's k_prolong.
template <typename TF, typename TC>
__global__ void __launch_bounds__(NT) k_pprolong(TF* __restrict__ p, int fsplit, const TC* __restrict__ pc, int csplit, int nx, int ny, int nz) {
  pdl_wait();
  pdl_trigger();
  const int ncx = nx / 2, ncy = ny / 2, ncz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
  if (cx >= ncx || cy >= ncy || cz >= ncz) return;
  const LV<TC> C{const_cast<TC*>(pc), ncx, ncy, ncz, csplit};
  const LV<TF> F{p, nx, ny, nz, fsplit};
  float v[3][3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int qx = cx + c - 1, qy = cy + bb - 1, qz = cz + a - 1;
        float val = Sto<TC>::ld(C.at(min(max(qx, 0), ncx - 1), min(max(qy, 0), ncy - 1), min(max(qz, 0), ncz - 1)));
        if (qx < 0 || qx >= ncx) val = -val;
        if (qz < 0 || qz >= ncz) val = -val;
        if (qy >= ncy) val = -val;
        v[a][bb][c] = val;
      }
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const float fx = dx ? 0.25f : 0.75f, fy = dy ? 0.25f : 0.75f, fz = dz ? 0.25f : 0.75f;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int ox = q & 1, oy = (q >> 1) & 1, oz = (q >> 2) & 1;
          const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy, wz = oz ? fz : 1.0f - fz;
          acc += v[dz + oz][dy + oy][dx + ox] * wx * wy * wz;
        }
        TF* pf = F.at(2 * cx + dx, 2 * cy + dy, 2 * cz + dz);
        Sto<TF>::st(pf, Sto<TF>::ld(pf) + acc);
      }
}

// Value of cell (x, y, z) of a red-black split level (half = nx/2 * ny * nz, hx = nx/2).
template <typename T>
__device__ __forceinline__ float ld_rb(const T* p, int half, int hx, int ny, int x, int y, int z) {
  return Sto<T>::ld(p + (((x + y + z) & 1) ? half : 0) + (x >> 1) + hx * (y + ny * z));
}
// Fused residual + 8-child restriction (src/sim.js:439-466) from a red-black split fine level into a plain
// coarse level.  The 32 distinct fine values the 8 children and their faces need (a 4x4x4 block without
// its edges and corners) are loaded once into v[z][y][x] (offsets -1..2 around the children); the
// arithmetic and its order are k_prestrict's, so the results are identical.
template <typename TF, typename TC>
__global__ void __launch_bounds__(NT) k_prestrict_rb(const TF* __restrict__ p, const TF* __restrict__ b, int nx, int ny, int nz, float h,
                                                     TC* __restrict__ bc, TC* __restrict__ pc) {
  pdl_wait();
  pdl_trigger();
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
  if (cx >= cnx || cy >= cny || cz >= cnz) return;
  const int hx = nx >> 1, half = hx * ny * nz;
  const int x0 = 2 * cx - 1, y0 = 2 * cy - 1, z0 = 2 * cz - 1;
  float v[4][4][4];
#pragma unroll
  for (int iz = 0; iz < 4; ++iz)
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 4; ++ix) {
        const bool cz_ = iz == 1 || iz == 2, cy_ = iy == 1 || iy == 2, cx_ = ix == 1 || ix == 2;
        const int inner = (cz_ ? 1 : 0) + (cy_ ? 1 : 0) + (cx_ ? 1 : 0);
        v[iz][iy][ix] = 0.0f;
        if (inner >= 2) {   // children (inner == 3) and their face neighbours (inner == 2)
          const int x = x0 + ix, y = y0 + iy, z = z0 + iz;
          if (x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz) v[iz][iy][ix] = ld_rb(p, half, hx, ny, x, y, z);
        }
      }
  const float ih2 = 1.0f / (h * h);
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int dx = q & 1, dy = (q >> 1) & 1, dz = (q >> 2) & 1;
    const int ix = 1 + dx, iy = 1 + dy, iz = 1 + dz;
    const int x = 2 * cx + dx, y = 2 * cy + dy, z = 2 * cz + dz;
    const float me = v[iz][iy][ix];
    const float gxm = x > 0 ? v[iz][iy][ix - 1] : -me, gxp = x < nx - 1 ? v[iz][iy][ix + 1] : -me;
    const float gym = y > 0 ? v[iz][iy - 1][ix] : me, gyp = y < ny - 1 ? v[iz][iy + 1][ix] : -me;
    const float gzm = z > 0 ? v[iz - 1][iy][ix] : -me, gzp = z < nz - 1 ? v[iz + 1][iy][ix] : -me;
    const float lap = (gxm + gxp + gym + gyp + gzm + gzp - 6.0f * me) * ih2;
    acc += ld_rb(b, half, hx, ny, x, y, z) - lap;
  }
  const int t = cx + cnx * (cy + cny * cz);
  Sto<TC>::st(bc + t, acc * 0.125f);
  Sto<TC>::st(pc + t, 0.0f);
}
// k_pprolong from a plain coarse level into a red-black split fine level: child (2cx+dx, 2cy+dy, 2cz+dz)
// is entry cx of colour half (dx + dy + dz) & 1 in its row.
template <typename TF, typename TC>
__global__ void __launch_bounds__(NT) k_pprolong_rb(TF* __restrict__ p, const TC* __restrict__ pc, int nx, int ny, int nz) {
  pdl_wait();
  pdl_trigger();
  const int ncx = nx / 2, ncy = ny / 2, ncz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
  if (cx >= ncx || cy >= ncy || cz >= ncz) return;
  const int hx = nx >> 1, half = hx * ny * nz;
  float v[3][3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int qx = cx + c - 1, qy = cy + bb - 1, qz = cz + a - 1;
        float val = Sto<TC>::ld(pc + min(max(qx, 0), ncx - 1) + ncx * (min(max(qy, 0), ncy - 1) + ncy * min(max(qz, 0), ncz - 1)));
        if (qx < 0 || qx >= ncx) val = -val;
        if (qz < 0 || qz >= ncz) val = -val;
        if (qy >= ncy) val = -val;
        v[a][bb][c] = val;
      }
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const float fx = dx ? 0.25f : 0.75f, fy = dy ? 0.25f : 0.75f, fz = dz ? 0.25f : 0.75f;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int ox = q & 1, oy = (q >> 1) & 1, oz = (q >> 2) & 1;
          const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy, wz = oz ? fz : 1.0f - fz;
          acc += v[dz + oz][dy + oy][dx + ox] * wx * wy * wz;
        }
        TF* pf = p + (((dx + dy + dz) & 1) ? half : 0) + cx + hx * ((2 * cy + dy) + ny * (2 * cz + dz));
        Sto<TF>::st(pf, Sto<TF>::ld(pf) + acc);
      }
}

// Solver state on the device.
struct PState {
  double bb;        // ||b||^2
  double rel;       // last relative residual
  double rel0;      // relative residual before the first cycle
  int iters;        // cycles / refinement steps of this solve
  int pad;
  float sc[2];      // sc[0]: unscale of the correction being solved for; sc[1]: scale of the next residual
};

// Writes the CTA's (x, y, z, w) partial (df64 pairs (rr, bb)) into slot `slot`.
__device__ __forceinline__ void cta_partial(float rrf, float bbf, float4* partials, int slot) {
  __shared__ df64 sr[NT / 32], sb[NT / 32];
  const int tid = threadIdx.x + GX * (threadIdx.y + GY * threadIdx.z);
  df64 rr = df_warp_sum(df_make(rrf));
  df64 bb = df_warp_sum(df_make(bbf));
  if ((tid & 31) == 0) { sr[tid >> 5] = rr; sb[tid >> 5] = bb; }
  __syncthreads();
  if (tid < 32) {
    rr = tid < NT / 32 ? sr[tid] : df_make(0.0f);
    bb = tid < NT / 32 ? sb[tid] : df_make(0.0f);
    rr = df_warp_sum(rr);
    bb = df_warp_sum(bb);
    if (tid == 0) partials[slot] = make_float4(rr.hi, rr.lo, bb.hi, bb.lo);
  }
}

// ||b||^2 partials over a fixed grid of SUMSQ_CTAS CTAs (grid-stride), deterministic.
__global__ void __launch_bounds__(NT) k_sumsq(const float* __restrict__ b, long long n, float4* __restrict__ partials) {
  pdl_wait();
  pdl_trigger();
  const int tid = threadIdx.x + GX * (threadIdx.y + GY * threadIdx.z);
  float s = 0.0f;
  for (long long i = (long long)blockIdx.x * NT + tid; i < n; i += (long long)gridDim.x * NT) {
    const float v = __ldg(b + i);
    s += v * v;
  }
  cta_partial(0.0f, s, partials, blockIdx.x);
}

// Laplacian numerator of one cell written as a sum of neighbour differences, (nb - me) per face with the
// ghost rules (p = 0 faces: ghost - me = -2 me; floor: 0).  Each difference is correctly rounded relative to
// itself, so the sum carries no cancellation of the 6|p| scale against 6 p: the residual of a converged
// solution is computed to its own precision, not to eps |p| / h^2.
__device__ __forceinline__ float lap_diff(float me, float xm, float xp, float ym, float yp, float zm, float zp, bool hxm, bool hxp,
                                          bool hym, bool hyp, bool hzm, bool hzp) {
  const float d2 = -2.0f * me;
  return ((hxm ? xm - me : d2) + (hxp ? xp - me : d2)) + ((hym ? ym - me : 0.0f) + (hyp ? yp - me : d2)) +
         ((hzm ? zm - me : d2) + (hzp ? zp - me : d2));
}
// r = b - A (xh + xl) over RZ planes of column (x, y) (xl may be null); the residual scaled by sc[1] is stored
// into rT (if given).  Partials: (||r||^2, ||b||^2).
template <typename TR>
__global__ void __launch_bounds__(NT) k_pres(const float* __restrict__ xh, const float* __restrict__ xl, const float* __restrict__ b,
                                             TR* __restrict__ rT, int rsplit, const PState* __restrict__ ps, int nx, int ny, int nz, float ih2,
                                             float4* __restrict__ partials) {
  pdl_wait();
  pdl_trigger();
  const int x = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int z0 = (blockIdx.z * GZ + threadIdx.z) * RZ;
  float rr = 0.0f, bb = 0.0f;
  if (x < nx && y < ny && z0 < nz) {
    const float s = rT ? ps->sc[1] : 1.0f;
    const int sy = nx, sz = nx * ny;
    const bool hxm = x > 0, hxp = x < nx - 1, hym = y > 0, hyp = y < ny - 1;
    int t = x + sy * y + sz * z0;
    float prev = z0 > 0 ? __ldg(xh + t - sz) : 0.0f, cur = __ldg(xh + t);
    float lprev = 0.0f, lcur = 0.0f;
    if (xl) { lprev = z0 > 0 ? __ldg(xl + t - sz) : 0.0f; lcur = __ldg(xl + t); }
#pragma unroll
    for (int k = 0; k < RZ; ++k) {
      const int z = z0 + k;
      if (z < nz) {
        const bool hzm = z > 0, hzp = z + 1 < nz;
        const float next = hzp ? __ldg(xh + t + sz) : 0.0f;
        float d = lap_diff(cur, hxm ? __ldg(xh + t - 1) : 0.0f, hxp ? __ldg(xh + t + 1) : 0.0f, hym ? __ldg(xh + t - sy) : 0.0f,
                           hyp ? __ldg(xh + t + sy) : 0.0f, prev, next, hxm, hxp, hym, hyp, hzm, hzp);
        float lnext = 0.0f, dl = 0.0f;
        if (xl) {
          lnext = hzp ? __ldg(xl + t + sz) : 0.0f;
          dl = lap_diff(lcur, hxm ? __ldg(xl + t - 1) : 0.0f, hxp ? __ldg(xl + t + 1) : 0.0f, hym ? __ldg(xl + t - sy) : 0.0f,
                        hyp ? __ldg(xl + t + sy) : 0.0f, lprev, lnext, hxm, hxp, hym, hyp, hzm, hzp);
        }
        const float bv = __ldg(b + t);
        const float r = (bv - d * ih2) - dl * ih2;
        if (rT) Sto<TR>::st(LV<TR>{rT, nx, ny, nz, rsplit}.at(x, y, z), r * s);
        rr += r * r;
        bb += bv * bv;
        prev = cur; cur = next;
        lprev = lcur; lcur = lnext;
        t += sz;
      }
    }
  }
  cta_partial(rr, bb, partials, blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

// k_pres for even nx with one thread per x pair (2 gx, 2 gx + 1) and RZ planes: every load of xh, xl and b
// is a float2 (plus one scalar on each side for the x neighbours), and the two residuals land at entry gx
// of the two colour halves when rT is red-black split.
// kFull: nz is a multiple of the planes a CTA covers, so no plane test is needed inside the march.
template <typename TR, bool kFull>
__global__ void __launch_bounds__(NT) k_pres2(const float* __restrict__ xh, const float* __restrict__ xl, const float* __restrict__ b,
                                              TR* __restrict__ rT, int rsplit, const PState* __restrict__ ps, int nx, int ny, int nz, float ih2,
                                              float4* __restrict__ partials) {
  pdl_wait();
  pdl_trigger();
  const int hx = nx >> 1;
  const int gx = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int z0 = (blockIdx.z * GZ + threadIdx.z) * RZ;
  float rr = 0.0f, bb = 0.0f;
  if (gx < hx && y < ny && z0 < nz) {
    const float s = rT ? ps->sc[1] : 1.0f;
    const int sy = nx, sz = nx * ny, halfn = hx * ny * nz;
    const bool hxm = gx > 0, hxp = gx < hx - 1, hym = y > 0, hyp = y < ny - 1;
    const float2 zero2 = make_float2(0.0f, 0.0f);
    auto ld2 = [](const float* q) { return __ldg(reinterpret_cast<const float2*>(q)); };
    int t = 2 * gx + sy * y + sz * z0;
    float2 hp = z0 > 0 ? ld2(xh + t - sz) : zero2, hc = ld2(xh + t);
    float2 lp = zero2, lc = zero2;
    if (xl) { lp = z0 > 0 ? ld2(xl + t - sz) : zero2; lc = ld2(xl + t); }
#pragma unroll
    for (int k = 0; k < RZ; ++k) {
      const int z = z0 + k;
      if (kFull || z < nz) {
        const bool hzm = z > 0, hzp = z + 1 < nz;
        const float2 hn = hzp ? ld2(xh + t + sz) : zero2;
        const float hl = hxm ? __ldg(xh + t - 1) : 0.0f, hr = hxp ? __ldg(xh + t + 2) : 0.0f;
        const float2 hym2 = hym ? ld2(xh + t - sy) : zero2, hyp2 = hyp ? ld2(xh + t + sy) : zero2;
        const float d0 = lap_diff(hc.x, hl, hc.y, hym2.x, hyp2.x, hp.x, hn.x, hxm, true, hym, hyp, hzm, hzp);
        const float d1 = lap_diff(hc.y, hc.x, hr, hym2.y, hyp2.y, hp.y, hn.y, true, hxp, hym, hyp, hzm, hzp);
        float dl0 = 0.0f, dl1 = 0.0f;
        float2 ln = zero2;
        if (xl) {
          ln = hzp ? ld2(xl + t + sz) : zero2;
          const float ll = hxm ? __ldg(xl + t - 1) : 0.0f, lr = hxp ? __ldg(xl + t + 2) : 0.0f;
          const float2 lym2 = hym ? ld2(xl + t - sy) : zero2, lyp2 = hyp ? ld2(xl + t + sy) : zero2;
          dl0 = lap_diff(lc.x, ll, lc.y, lym2.x, lyp2.x, lp.x, ln.x, hxm, true, hym, hyp, hzm, hzp);
          dl1 = lap_diff(lc.y, lc.x, lr, lym2.y, lyp2.y, lp.y, ln.y, true, hxp, hym, hyp, hzm, hzp);
        }
        const float2 bv = ld2(b + t);
        const float r0 = (bv.x - d0 * ih2) - dl0 * ih2, r1 = (bv.y - d1 * ih2) - dl1 * ih2;
        if (rT) {
          if (rsplit) {
            const int c0 = (y + z) & 1, idx = gx + hx * (y + ny * z);
            Sto<TR>::st(rT + c0 * halfn + idx, r0 * s);
            Sto<TR>::st(rT + (1 - c0) * halfn + idx, r1 * s);
          } else {
            Sto<TR>::st(rT + t, r0 * s);
            Sto<TR>::st(rT + t + 1, r1 * s);
          }
        }
        rr += r0 * r0;
        rr += r1 * r1;
        bb += bv.x * bv.x;
        bb += bv.y * bv.y;
        hp = hc; hc = hn;
        lp = lc; lc = ln;
        t += sz;
      }
    }
  }
  cta_partial(rr, bb, partials, blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

// (xh, xl) += e * sc[0] as a double-float (FP32 pair) update: Knuth's TwoSum then renormalisation, so the
// pair keeps ~44 bits of the solution while every stored array stays FP32.  4 cells per thread.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float d) {
  const float s = __fadd_rn(hi, d);
  const float bp = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(d, bp));
  const float l2 = __fadd_rn(lo, err);
  hi = __fadd_rn(s, l2);
  lo = __fsub_rn(l2, __fsub_rn(hi, s));
}
// One thread per x pair (2 gx, 2 gx + 1) of a row: the pair is one float2 of xh and xl, and in the split
// layout its two e values sit at the same half-index of the two colour halves.
template <typename TE>
__global__ void __launch_bounds__(NT) k_pupdate(float* __restrict__ xh, float* __restrict__ xl, const TE* __restrict__ e, int esplit,
                                                const PState* __restrict__ ps, int nx, int ny, int nz) {
  pdl_wait();
  pdl_trigger();
  const int gx = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y, z = blockIdx.z * GZ + threadIdx.z;
  const int x = 2 * gx;
  if (x >= nx || y >= ny || z >= nz) return;
  const float u = ps->sc[0];
  const LV<TE> E{const_cast<TE*>(e), nx, ny, nz, esplit};
  const int t = x + nx * (y + ny * z);
  if (x + 1 < nx && (nx & 1) == 0) {
    float2 hv = *reinterpret_cast<const float2*>(xh + t);
    float2 lv = *reinterpret_cast<const float2*>(xl + t);
    pair_add(hv.x, lv.x, __fmul_rn(Sto<TE>::ld(E.at(x, y, z)), u));
    pair_add(hv.y, lv.y, __fmul_rn(Sto<TE>::ld(E.at(x + 1, y, z)), u));
    *reinterpret_cast<float2*>(xh + t) = hv;
    *reinterpret_cast<float2*>(xl + t) = lv;
  } else {
    pair_add(xh[t], xl[t], __fmul_rn(Sto<TE>::ld(E.at(x, y, z)), u));
    if (x + 1 < nx) pair_add(xh[t + 1], xl[t + 1], __fmul_rn(Sto<TE>::ld(E.at(x + 1, y, z)), u));
  }
}

// mode 0: ||b||^2 from the sumsq partials; sets the first scale.  mode 1: the residual test (first = 1
// before the loop).  Sets the WHILE condition: continue while rel > tol and iters < max_iters.
__global__ void __launch_bounds__(NT) k_ptest(const float4* __restrict__ partials, int count, PState* __restrict__ ps, int mode, int first,
                                              double tol, int max_iters, double ncells, cudaGraphConditionalHandle h, int set_cond) {
  __shared__ df64 sa[SUMV / 32], sb[SUMV / 32];
  pdl_wait();
  pdl_trigger();
  df64 A, B;
  sum_pairs_fixed<NT>(partials, count, threadIdx.x, sa, sb, A, B);
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    const double bb = df_to_double(B);
    ps->bb = bb;
    ps->sc[0] = 1.0f;
    ps->sc[1] = bb > 0.0 ? (float)(1.0 / sqrt(bb / ncells)) : 1.0f;
    return;
  }
  const double rr = df_to_double(A), bb = ps->bb;
  const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  ps->rel = rel;
  if (first) { ps->rel0 = rel; ps->iters = 0; } else { ps->iters += 1; }
  ps->sc[0] = 1.0f / ps->sc[1];
  ps->sc[1] = rr > 0.0 ? (float)(1.0 / sqrt(rr / ncells)) : 1.0f;
  if (set_cond) cudaGraphSetConditional(h, (rel > tol && ps->iters < max_iters) ? 1u : 0u);
}

// ---- RHS: sum of Gaussian sources + per-cell normal noise, then the mean removed ----
constexpr int MAX_SOURCES = 256;
__global__ void __launch_bounds__(NT) k_rhs(float* __restrict__ b, int nx, int ny, int nz, const float* __restrict__ src, int ns, float noise,
                                            unsigned seed, float4* __restrict__ partials) {
  __shared__ float s[MAX_SOURCES * 5];
  const int tid = threadIdx.x + GX * (threadIdx.y + GY * threadIdx.z);
  for (int i = tid; i < ns * 5; i += NT) s[i] = src[i];
  __syncthreads();
  const int x = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y, z = blockIdx.z * GZ + threadIdx.z;
  float v = 0.0f;
  if (x < nx && y < ny && z < nz) {
    const float px = (float)x + 0.5f, py = (float)y + 0.5f, pz = (float)z + 0.5f;
    for (int i = 0; i < ns; ++i) {
      const float dx = px - s[5 * i], dy = py - s[5 * i + 1], dz = pz - s[5 * i + 2], sg = s[5 * i + 3];
      v += s[5 * i + 4] * expf(-(dx * dx + dy * dy + dz * dz) / (2.0f * sg * sg));
    }
    const uint3 hv = pcg3d(make_uint3((unsigned)x, (unsigned)y, (unsigned)z ^ (seed * 0x9E3779B9u)));
    const float u1 = ((float)(hv.x >> 8) + 1.0f) * (1.0f / 16777216.0f);   // (0, 1]
    const float u2 = (float)(hv.y >> 8) * (1.0f / 16777216.0f);            // [0, 1)
    v += noise * sqrtf(-2.0f * logf(u1)) * cosf(6.283185307179586f * u2);
    b[x + nx * (y + ny * z)] = v;
  }
  cta_partial(0.0f, v, partials, blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}
__global__ void __launch_bounds__(NT) k_mean(const float4* __restrict__ partials, int count, double ncells, double* __restrict__ mean) {
  __shared__ df64 sa[SUMV / 32], sb[SUMV / 32];
  df64 A, B;
  sum_pairs_fixed<NT>(partials, count, threadIdx.x, sa, sb, A, B);
  if (threadIdx.x == 0) mean[0] = df_to_double(B) / ncells;
}
__global__ void k_sub_mean(float* __restrict__ b, long long n, const double* __restrict__ mean) {
  const float m = (float)mean[0];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) b[i] -= m;
}

dim3 grid3(int x, int y, int z) { return dim3((x + GX - 1) / GX, (y + GY - 1) / GY, (z + GZ - 1) / GZ); }
const dim3 kBlock(GX, GY, GZ);

}  // namespace
}  // namespace fire

using namespace fire;

// Storage type of a level's arrays.
enum { STO_F32 = 0, STO_F16 = 1, STO_BF16 = 2 };
// One level of the solver: storage type, layout (red-black split or plain) and device arrays.
struct PLevel {
  int nx, ny, nz;
  float h;
  int sto;
  int split;
  void* p;
  void* b;
};

struct FirePoisson {
  int device = 0;
  int res[3] = {0, 0, 0};
  float h = 0;
  int prec = FIRE_POISSON_FP32;
  bool ir = false;              // iterative refinement (every form but FIRE_POISSON_FP32)
  long long cells = 0;
  std::vector<PLevel> levels;
  std::vector<MGLevel> mg;      // float view (levels >= tailFirst are FP32; all levels in the FP32 form)
  int tailFirst = 0;
  int coarseIters = 8;
  void* arena = nullptr;
  float4* partials = nullptr;
  int partialsCount = 0;
  PState* state = nullptr;      // the solve's
  PState* state2 = nullptr;     // fire_poisson_residual's (so it never disturbs a solve's result)
  double* mean = nullptr;
  int* err = nullptr;
  float* src = nullptr;
  float* xlo = nullptr;         // low half of the solution pair when the caller passes none
  double* cinv = nullptr;       // inverse of the coarsest operator (transposed), FP64, or null
  cudaStream_t capStream = nullptr;
  cudaGraphExec_t exec = nullptr;
  // the captured graph's arguments
  const float* gb = nullptr;
  float* gx = nullptr;
  float* gxl = nullptr;
  double gtol = -1;
  int gmax = -1, ginner = -1;
};

namespace {

size_t align_up(size_t v) { return (v + 255) / 256 * 256; }
size_t elem_bytes(int sto) { return sto == STO_F32 ? 4 : 2; }
int storage_of(int prec) { return prec == FIRE_POISSON_FP16 ? STO_F16 : prec == FIRE_POISSON_BF16 ? STO_BF16 : STO_F32; }

template <typename T>
void psmooth_t(const PLevel& L, int color, int zero, cudaStream_t st) {
  if (L.split && L.nx % 4 == 0) {
    const dim3 g = grid3(L.nx >> 2, L.ny, (L.nz + SMZ - 1) / SMZ);
    if (zero) launch_pdl(k_psmooth_rb2<T, true>, g, kBlock, 0, st, (T*)L.p, (const T*)L.b, L.nx, L.ny, L.nz, L.h, color);
    else launch_pdl(k_psmooth_rb2<T, false>, g, kBlock, 0, st, (T*)L.p, (const T*)L.b, L.nx, L.ny, L.nz, L.h, color);
  } else if (L.split) {
    const dim3 g = grid3(L.nx >> 1, L.ny, (L.nz + SMZ - 1) / SMZ);
    if (zero) launch_pdl(k_psmooth_rb<T, true>, g, kBlock, 0, st, (T*)L.p, (const T*)L.b, L.nx, L.ny, L.nz, L.h, color);
    else launch_pdl(k_psmooth_rb<T, false>, g, kBlock, 0, st, (T*)L.p, (const T*)L.b, L.nx, L.ny, L.nz, L.h, color);
  } else {
    const dim3 g = grid3((L.nx + 1) >> 1, L.ny, (L.nz + SMZ - 1) / SMZ);
    launch_pdl(k_psmooth<T>, g, kBlock, 0, st, (T*)L.p, (const T*)L.b, L.nx, L.ny, L.nz, L.h, color, zero);
  }
}
void psmooth(const PLevel& L, int color, int zero, cudaStream_t st) {
  switch (L.sto) {
    case STO_F16: psmooth_t<__half>(L, color, zero, st); break;
    case STO_BF16: psmooth_t<__nv_bfloat16>(L, color, zero, st); break;
    default: psmooth_t<float>(L, color, zero, st);
  }
}
template <typename TF, typename TC>
void prestrict_tt(const PLevel& F, const PLevel& C, cudaStream_t st) {
  if (F.split && !C.split)
    launch_pdl(k_prestrict_rb<TF, TC>, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (const TF*)F.p, (const TF*)F.b, F.nx, F.ny, F.nz, F.h,
               (TC*)C.b, (TC*)C.p);
  else
    launch_pdl(k_prestrict<TF, TC>, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (const TF*)F.p, (const TF*)F.b, F.split, F.nx, F.ny, F.nz,
               F.h, (TC*)C.b, (TC*)C.p, C.split);
}
template <typename TF>
void prestrict_to(const PLevel& F, const PLevel& C, cudaStream_t st) {
  switch (C.sto) {
    case STO_F16: prestrict_tt<TF, __half>(F, C, st); break;
    case STO_BF16: prestrict_tt<TF, __nv_bfloat16>(F, C, st); break;
    default: prestrict_tt<TF, float>(F, C, st);
  }
}
void prestrict(const PLevel& F, const PLevel& C, cudaStream_t st) {
  switch (F.sto) {
    case STO_F16: prestrict_to<__half>(F, C, st); break;
    case STO_BF16: prestrict_to<__nv_bfloat16>(F, C, st); break;
    default: prestrict_to<float>(F, C, st);
  }
}
template <typename TF, typename TC>
void pprolong_tt(const PLevel& F, const PLevel& C, cudaStream_t st) {
  if (F.split && !C.split)
    launch_pdl(k_pprolong_rb<TF, TC>, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (TF*)F.p, (const TC*)C.p, F.nx, F.ny, F.nz);
  else
    launch_pdl(k_pprolong<TF, TC>, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (TF*)F.p, F.split, (const TC*)C.p, C.split, F.nx, F.ny, F.nz);
}
template <typename TF>
void pprolong_from(const PLevel& F, const PLevel& C, cudaStream_t st) {
  switch (C.sto) {
    case STO_F16: pprolong_tt<TF, __half>(F, C, st); break;
    case STO_BF16: pprolong_tt<TF, __nv_bfloat16>(F, C, st); break;
    default: pprolong_tt<TF, float>(F, C, st);
  }
}
void pprolong(const PLevel& F, const PLevel& C, cudaStream_t st) {
  switch (F.sto) {
    case STO_F16: pprolong_from<__half>(F, C, st); break;
    case STO_BF16: pprolong_from<__nv_bfloat16>(F, C, st); break;
    default: pprolong_from<float>(F, C, st);
  }
}

// The residual kernel's grid: x pairs for even nx (k_pres2), single cells otherwise (k_pres).
dim3 pres_grid(const PLevel& L) {
  const int cols = (L.nx % 2 == 0) ? L.nx / 2 : L.nx;
  return dim3((cols + GX - 1) / GX, (L.ny + GY - 1) / GY, (L.nz + GZ * RZ - 1) / (GZ * RZ));
}

// r = b - A (xh + xl); written scaled into level 0's RHS when `write` (refinement forms); partials for the test.
template <typename TR>
void pres_t(FirePoisson* ps, const PState* state, const float* b, const float* xh, const float* xl, TR* rT, int rsplit, cudaStream_t st) {
  const PLevel& L = ps->levels[0];
  if (L.nx % 2 == 0 && L.nz % (GZ * RZ) == 0)
    launch_pdl(k_pres2<TR, true>, pres_grid(L), kBlock, 0, st, xh, xl, b, rT, rsplit, state, L.nx, L.ny, L.nz, 1.0f / (L.h * L.h),
               ps->partials);
  else if (L.nx % 2 == 0)
    launch_pdl(k_pres2<TR, false>, pres_grid(L), kBlock, 0, st, xh, xl, b, rT, rsplit, state, L.nx, L.ny, L.nz, 1.0f / (L.h * L.h),
               ps->partials);
  else
    launch_pdl(k_pres<TR>, pres_grid(L), kBlock, 0, st, xh, xl, b, rT, rsplit, state, L.nx, L.ny, L.nz, 1.0f / (L.h * L.h), ps->partials);
}
void pres(FirePoisson* ps, const PState* state, const float* b, const float* xh, const float* xl, bool write, cudaStream_t st) {
  const PLevel& L = ps->levels[0];
  if (!write) { pres_t<float>(ps, state, b, xh, xl, nullptr, 0, st); return; }
  switch (L.sto) {
    case STO_F16: pres_t<__half>(ps, state, b, xh, xl, (__half*)L.b, L.split, st); break;
    case STO_BF16: pres_t<__nv_bfloat16>(ps, state, b, xh, xl, (__nv_bfloat16*)L.b, L.split, st); break;
    default: pres_t<float>(ps, state, b, xh, xl, (float*)L.b, L.split, st);
  }
}
template <typename TE>
void pupdate_t(FirePoisson* ps, float* xh, float* xl, cudaStream_t st) {
  const PLevel& L = ps->levels[0];
  launch_pdl(k_pupdate<TE>, grid3((L.nx + 1) >> 1, L.ny, L.nz), kBlock, 0, st, xh, xl, (const TE*)L.p, L.split, (const PState*)ps->state,
             L.nx, L.ny, L.nz);
}
void pupdate(FirePoisson* ps, float* xh, float* xl, cudaStream_t st) {
  switch (ps->levels[0].sto) {
    case STO_F16: pupdate_t<__half>(ps, xh, xl, st); break;
    case STO_BF16: pupdate_t<__nv_bfloat16>(ps, xh, xl, st); break;
    default: pupdate_t<float>(ps, xh, xl, st);
  }
}
void ptest(FirePoisson* ps, PState* state, int mode, int first, int count, double tol, int max_iters, cudaGraphConditionalHandle h,
           int set_cond, cudaStream_t st) {
  launch_pdl(k_ptest, dim3(1), dim3(NT), 0, st, (const float4*)ps->partials, count, state, mode, first, tol, max_iters,
             (double)ps->cells, h, set_cond);
}
int pres_count(const FirePoisson* ps) {
  const dim3 g = pres_grid(ps->levels[0]);
  return (int)(g.x * g.y * g.z);
}

// One V(2,2) cycle of the correction solve on (levels[0].p, levels[0].b); zero_first: e starts at zero.  The
// coarsest level is solved exactly in FP64 (dense inverse) or, when too large for that, by FP64 sweeps.
void ir_vcycle(FirePoisson* ps, bool zero_first, cudaStream_t st) {
  const int n = (int)ps->levels.size(), T = ps->tailFirst, top = std::min(T, n - 1);
  std::vector<PLevel>& L = ps->levels;
  for (int i = 0; i < top; ++i) {
    for (int k = 0; k < 2; ++k) {
      psmooth(L[i], 0, (i == 0 && zero_first && k == 0) ? 1 : 0, st);
      psmooth(L[i], 1, 0, st);
    }
    prestrict(L[i], L[i + 1], st);
  }
  if (T < n) {
    launch_tail(ps->mg.data(), T, n, 2, 2, COARSE64_SWEEPS, ps->err, st, true, ps->cinv);
  } else {
    for (int k = 0; k < ps->coarseIters; ++k) {
      psmooth(L[n - 1], 0, (n == 1 && zero_first && k == 0) ? 1 : 0, st);
      psmooth(L[n - 1], 1, 0, st);
    }
  }
  for (int i = top - 1; i >= 0; --i) {
    pprolong(L[i], L[i + 1], st);
    for (int k = 0; k < 2; ++k) { psmooth(L[i], 0, 0, st); psmooth(L[i], 1, 0, st); }
  }
}
// The step's V(2,2) cycle (src/sim.js:588-599) on (x, b).
void fp32_vcycle(FirePoisson* ps, cudaStream_t st) {
  const int n = (int)ps->mg.size(), T = ps->tailFirst, top = std::min(T, n - 1);
  for (int i = 0; i < top; ++i) {
    for (int k = 0; k < 2; ++k) { launch_smooth(ps->mg[i], 0, st); launch_smooth(ps->mg[i], 1, st); }
    launch_restrict(ps->mg[i], ps->mg[i + 1], st);
  }
  if (T < n) launch_tail(ps->mg.data(), T, n, 2, 2, ps->coarseIters, ps->err, st);
  else for (int k = 0; k < ps->coarseIters; ++k) { launch_smooth(ps->mg[n - 1], 0, st); launch_smooth(ps->mg[n - 1], 1, st); }
  for (int i = top - 1; i >= 0; --i) {
    launch_prolong(ps->mg[i], ps->mg[i + 1], st);
    for (int k = 0; k < 2; ++k) { launch_smooth(ps->mg[i], 0, st); launch_smooth(ps->mg[i], 1, st); }
  }
}

// Dense inverse of the coarsest operator A (A p = (sum of ghost-ruled neighbours - diag p) / h^2, as the
// smoother's fixed point), by Gauss-Jordan elimination with partial pivoting in FP64; stored transposed
// (column i of the inverse is row i) so a warp's lanes read consecutive addresses.
bool coarse_inverse(const MGLevel& C, std::vector<double>& out) {
  const int nx = C.nx, ny = C.ny, nz = C.nz, n = nx * ny * nz;
  const double ih2 = 1.0 / ((double)C.h * (double)C.h);
  std::vector<double> a((size_t)n * n, 0.0), inv((size_t)n * n, 0.0);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int c = x + nx * (y + ny * z);
        double diag = 6.0;
        auto nb = [&](bool inside, int o, double ghost) {
          if (inside) a[(size_t)c * n + o] += ih2; else diag += ghost;
        };
        nb(x > 0, c - 1, 1.0);
        nb(x < nx - 1, c + 1, 1.0);
        nb(z > 0, c - nx * ny, 1.0);
        nb(z < nz - 1, c + nx * ny, 1.0);
        nb(y > 0, c - nx, -1.0);
        nb(y < ny - 1, c + nx, 1.0);
        a[(size_t)c * n + c] -= diag * ih2;
        inv[(size_t)c * n + c] = 1.0;
      }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(a[(size_t)r * n + col]) > std::fabs(a[(size_t)piv * n + col])) piv = r;
    if (a[(size_t)piv * n + col] == 0.0) return false;
    if (piv != col)
      for (int k = 0; k < n; ++k) {
        std::swap(a[(size_t)piv * n + k], a[(size_t)col * n + k]);
        std::swap(inv[(size_t)piv * n + k], inv[(size_t)col * n + k]);
      }
    const double d = 1.0 / a[(size_t)col * n + col];
    for (int k = 0; k < n; ++k) { a[(size_t)col * n + k] *= d; inv[(size_t)col * n + k] *= d; }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = a[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) { a[(size_t)r * n + k] -= f * a[(size_t)col * n + k]; inv[(size_t)r * n + k] -= f * inv[(size_t)col * n + k]; }
    }
  }
  out.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) out[(size_t)j * n + i] = inv[(size_t)i * n + j];
  return true;
}

#define PCK(call)                                     \
  do {                                                \
    if ((call) != cudaSuccess) return FIRE_ERR_CUDA;  \
  } while (0)

// Captures the whole solve (pre-pass, conditional WHILE loop) for (b, x, x_lo, tol, max_iters, inner).
int build_graph(FirePoisson* ps, const float* b, float* x, float* xl, double tol, int max_iters, int inner) {
  if (ps->exec) { cudaGraphExecDestroy(ps->exec); ps->exec = nullptr; }
  const bool ir = ps->ir;
  if (!ir) { ps->mg[0].p = x; ps->mg[0].b = const_cast<float*>(b); }
  float* lo = ir ? (xl ? xl : ps->xlo) : nullptr;
  cudaStream_t st = ps->capStream;
  cudaGraph_t g = nullptr;
  PCK(cudaGraphCreate(&g, 0));
  PCK(cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  // tol = 0 asks for exactly max_iters iterations: they are unrolled into the graph (no conditional node,
  // so every kernel node can also be profiled); otherwise the iterations run in a WHILE node
  const bool unroll = tol == 0.0 && max_iters <= 64;
  cudaGraphConditionalHandle h = 0;
  if (!unroll && cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGraph_t tmp;
    cudaStreamEndCapture(st, &tmp);
    cudaGraphDestroy(g);
    return FIRE_ERR_CUDA;
  }
  if (ir && !xl) cudaMemsetAsync(ps->xlo, 0, sizeof(float) * (size_t)ps->cells, st);   // the pair starts at (x, 0)
  launch_pdl(k_sumsq, dim3(SUMSQ_CTAS), dim3(NT), 0, st, b, ps->cells, ps->partials);
  ptest(ps, ps->state, 0, 1, SUMSQ_CTAS, tol, max_iters, h, 0, st);
  pres(ps, ps->state, b, x, lo, ir, st);
  ptest(ps, ps->state, 1, 1, pres_count(ps), tol, max_iters, h, unroll ? 0 : 1, st);
  // one iteration: correction cycle(s), update, residual, test
  auto body = [&](cudaStream_t s, int set_cond) {
    if (ir) {
      // the correction solve starts from e = 0: the first half-sweep ignores e's old contents, except when
      // level 0 itself is inside the shared-memory tail, which loads e
      if (ps->tailFirst == 0) cudaMemsetAsync(ps->levels[0].p, 0, sizeof(float) * (size_t)ps->cells, s);
      for (int c = 0; c < inner; ++c) ir_vcycle(ps, c == 0, s);
      pupdate(ps, x, lo, s);
      pres(ps, ps->state, b, x, lo, true, s);
    } else {
      fp32_vcycle(ps, s);
      pres(ps, ps->state, b, x, nullptr, false, s);
    }
    ptest(ps, ps->state, 1, 0, pres_count(ps), tol, max_iters, h, set_cond, s);
  };
  bool bodyOk = true;
  if (unroll) {
    for (int it = 0; it < max_iters; ++it) body(st, 0);
  } else {
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg;
    const cudaGraphNode_t* deps;
    size_t ndeps;
    PCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    PCK(cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &cp));
    PCK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaStream_t bs = nullptr;
    PCK(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    if (cudaStreamBeginCaptureToGraph(bs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
      cudaStreamDestroy(bs);
      return FIRE_ERR_CUDA;
    }
    body(bs, 1);
    cudaGraph_t bodyOut;
    bodyOk = cudaStreamEndCapture(bs, &bodyOut) == cudaSuccess;
    cudaStreamDestroy(bs);
  }
  cudaGraph_t outg;
  const bool ok = cudaStreamEndCapture(st, &outg) == cudaSuccess && bodyOk;
  if (!ok || cudaGetLastError() != cudaSuccess) { cudaGraphDestroy(g); return FIRE_ERR_CUDA; }
  const cudaError_t e = cudaGraphInstantiate(&ps->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { ps->exec = nullptr; return FIRE_ERR_CUDA; }
  ps->gb = b; ps->gx = x; ps->gxl = xl; ps->gtol = tol; ps->gmax = max_iters; ps->ginner = inner;
  return FIRE_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(dev);
  }
  ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

constexpr int COARSE_DIRECT_MAX = 512;   // coarsest levels up to this many cells get the dense FP64 inverse

}  // namespace

extern "C" {

int fire_poisson_create(const int res[3], float h, int precision, int device, FirePoisson** out) {
  FIRE_RANGE("fire_poisson_create");
  if (!out) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  if (!res || res[0] < 2 || res[1] < 2 || res[2] < 2 || !(h > 0.0f)) return FIRE_ERR_BAD_ARG;
  if (precision < FIRE_POISSON_FP32 || precision > FIRE_POISSON_IR32) return FIRE_ERR_BAD_ARG;
  if ((long long)res[0] * res[1] * res[2] >= (1LL << 31)) return FIRE_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return FIRE_ERR_NO_DEVICE;
  DeviceGuard dg(device);
  FirePoisson* ps = new FirePoisson();
  ps->device = device;
  for (int i = 0; i < 3; ++i) ps->res[i] = res[i];
  ps->h = h;
  ps->prec = precision;
  ps->ir = precision != FIRE_POISSON_FP32;
  ps->cells = (long long)res[0] * res[1] * res[2];
  // level hierarchy and coarse sweeps as FireSim builds them (src/sim.js:79-92)
  {
    int x = res[0], y = res[1], z = res[2];
    double hh = h;
    while (true) {
      ps->mg.push_back(MGLevel{x, y, z, (float)hh, nullptr, nullptr});
      if (x % 2 || y % 2 || z % 2 || std::min(x, std::min(y, z)) <= 6) break;
      x /= 2; y /= 2; z /= 2; hh *= 2;
    }
    const MGLevel& C = ps->mg.back();
    const double PI = 3.14159265358979323846;
    const double mu = (std::cos(PI / C.nx) + std::cos(PI / (2.0 * C.ny)) + std::cos(PI / C.nz)) / 3.0;
    ps->coarseIters = (int)std::max(8.0, std::min(64.0, std::ceil(std::log(0.05) / std::log(mu * mu))));
  }
  const int n = (int)ps->mg.size();
  ps->tailFirst = tail_first(ps->mg.data(), n, ps->ir);
  std::vector<double> cinv;
  const MGLevel& C = ps->mg.back();
  const int ccells = C.nx * C.ny * C.nz;
  const bool direct = ps->ir && ps->tailFirst < n && ccells <= COARSE_DIRECT_MAX && coarse_inverse(C, cinv);
  // arena: level arrays (level 0 of the FP32 form is the caller's x and b), partials, state
  size_t off = 0;
  std::vector<size_t> pOff(n), bOff(n);
  ps->levels.resize(n);
  const int sto = storage_of(precision);
  for (int l = 0; l < n; ++l) {
    const MGLevel& M = ps->mg[l];
    PLevel& L = ps->levels[l];
    L.nx = M.nx; L.ny = M.ny; L.nz = M.nz; L.h = M.h;
    L.sto = (ps->ir && l < ps->tailFirst) ? sto : STO_F32;
    // level 0 (the only level whose arrays outgrow L2) in the red-black split layout; the rest plain
    L.split = (ps->ir && l == 0 && l < ps->tailFirst && M.nx % 2 == 0) ? 1 : 0;
    const size_t bytes = align_up((size_t)M.nx * M.ny * M.nz * elem_bytes(L.sto));
    if (l == 0 && !ps->ir) { pOff[l] = bOff[l] = (size_t)-1; continue; }
    pOff[l] = off; off += bytes;
    bOff[l] = off; off += bytes;
  }
  {
    const dim3 g = pres_grid(ps->levels[0]);
    const dim3 gr = grid3(res[0], res[1], res[2]);
    ps->partialsCount = std::max<int>(SUMSQ_CTAS, std::max<int>((int)(g.x * g.y * g.z), (int)(gr.x * gr.y * gr.z)));
  }
  const size_t partOff = off; off = align_up(off + sizeof(float4) * (size_t)ps->partialsCount);
  const size_t stateOff = off; off = align_up(off + 2 * sizeof(PState));
  const size_t meanOff = off; off = align_up(off + sizeof(double));
  const size_t errOff = off; off = align_up(off + sizeof(int));
  const size_t srcOff = off; off = align_up(off + sizeof(float) * MAX_SOURCES * 5);
  const size_t loOff = off; if (ps->ir) off = align_up(off + sizeof(float) * (size_t)ps->cells);
  const size_t cinvOff = off; if (direct) off = align_up(off + sizeof(double) * cinv.size());
  if (cudaMalloc(&ps->arena, off) != cudaSuccess) { delete ps; return FIRE_ERR_OOM; }
  char* A = (char*)ps->arena;
  for (int l = 0; l < n; ++l) {
    if (pOff[l] == (size_t)-1) continue;
    ps->levels[l].p = A + pOff[l];
    ps->levels[l].b = A + bOff[l];
    if (ps->levels[l].sto == STO_F32) { ps->mg[l].p = (float*)(A + pOff[l]); ps->mg[l].b = (float*)(A + bOff[l]); }
  }
  ps->partials = (float4*)(A + partOff);
  ps->state = (PState*)(A + stateOff);
  ps->state2 = ps->state + 1;
  ps->mean = (double*)(A + meanOff);
  ps->err = (int*)(A + errOff);
  ps->src = (float*)(A + srcOff);
  if (ps->ir) ps->xlo = (float*)(A + loOff);
  if (direct) ps->cinv = (double*)(A + cinvOff);
  if (cudaMemset(ps->arena, 0, off) != cudaSuccess || mg_configure(TAIL_SMEM_BUDGET) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ps->capStream, cudaStreamNonBlocking) != cudaSuccess ||
      (direct && cudaMemcpy(ps->cinv, cinv.data(), sizeof(double) * cinv.size(), cudaMemcpyHostToDevice) != cudaSuccess)) {
    fire_poisson_destroy(ps);
    return FIRE_ERR_CUDA;
  }
  *out = ps;
  return FIRE_OK;
}

int fire_poisson_destroy(FirePoisson* ps) {
  if (!ps) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  cudaDeviceSynchronize();
  if (ps->exec) cudaGraphExecDestroy(ps->exec);
  if (ps->capStream) cudaStreamDestroy(ps->capStream);
  if (ps->arena) cudaFree(ps->arena);
  delete ps;
  return FIRE_OK;
}

int fire_poisson_solve(FirePoisson* ps, const float* b, float* x, float* x_lo, double tol, int max_iters, int inner_cycles, void* stream) {
  FIRE_RANGE("fire_poisson_solve");
  if (!ps || !b || !x || !(tol >= 0.0) || max_iters < 0 || (const void*)b == (const void*)x) return FIRE_ERR_BAD_ARG;
  if (x_lo && ((const void*)x_lo == (const void*)x || (const void*)x_lo == (const void*)b)) return FIRE_ERR_BAD_ARG;
  if (ps->ir && (inner_cycles < 1 || inner_cycles > 16)) return FIRE_ERR_BAD_ARG;
  if (!ps->ir) { inner_cycles = 1; x_lo = nullptr; }
  // the update and the residual read x, x_lo and b as float2 pairs
  if (((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(x_lo) | reinterpret_cast<uintptr_t>(b)) & 15u) != 0) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  if (!ps->exec || ps->gb != b || ps->gx != x || ps->gxl != x_lo || ps->gtol != tol || ps->gmax != max_iters || ps->ginner != inner_cycles) {
    const int rc = build_graph(ps, b, x, x_lo, tol, max_iters, inner_cycles);
    if (rc) return rc;
  }
  return cudaGraphLaunch(ps->exec, reinterpret_cast<cudaStream_t>(stream)) == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

int fire_poisson_result(FirePoisson* ps, FirePoissonResult* out) {
  if (!ps || !out) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  if (cudaDeviceSynchronize() != cudaSuccess) return FIRE_ERR_CUDA;
  PState s;
  int err = 0;
  if (cudaMemcpy(&s, ps->state, sizeof s, cudaMemcpyDeviceToHost) != cudaSuccess) return FIRE_ERR_CUDA;
  if (cudaMemcpy(&err, ps->err, sizeof err, cudaMemcpyDeviceToHost) != cudaSuccess) return FIRE_ERR_CUDA;
  if (err) {
    cudaMemset(ps->err, 0, sizeof(int));
    return FIRE_ERR_CUDA;
  }
  out->iterations = s.iters;
  out->rel_residual = s.rel;
  out->rel_residual_initial = s.rel0;
  out->b_norm = std::sqrt(s.bb);
  return FIRE_OK;
}

int fire_poisson_residual(FirePoisson* ps, const float* b, const float* x, const float* x_lo, double* rel) {
  if (!ps || !b || !x || !rel) return FIRE_ERR_BAD_ARG;
  if (((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(x_lo) | reinterpret_cast<uintptr_t>(b)) & 15u) != 0) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  cudaStream_t st = ps->capStream;
  launch_pdl(k_sumsq, dim3(SUMSQ_CTAS), dim3(NT), 0, st, b, ps->cells, ps->partials);
  ptest(ps, ps->state2, 0, 1, SUMSQ_CTAS, 0.0, 0, 0, 0, st);
  pres(ps, ps->state2, b, x, x_lo, false, st);
  ptest(ps, ps->state2, 1, 1, pres_count(ps), 0.0, 0, 0, 0, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return FIRE_ERR_CUDA;
  PState s;
  if (cudaMemcpy(&s, ps->state2, sizeof s, cudaMemcpyDeviceToHost) != cudaSuccess) return FIRE_ERR_CUDA;
  *rel = s.rel;
  return FIRE_OK;
}

int fire_poisson_set_study(FirePoisson* ps, int coarse_sweeps) {
  if (!ps || ps->ir || coarse_sweeps < 1 || coarse_sweeps > 4096) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  if (cudaDeviceSynchronize() != cudaSuccess) return FIRE_ERR_CUDA;
  for (MGLevel& L : ps->mg) L.study = 1;
  ps->coarseIters = coarse_sweeps;
  ps->tailFirst = tail_first(ps->mg.data(), (int)ps->mg.size(), false);   // single-CTA tails in this variant
  if (ps->exec) { cudaGraphExecDestroy(ps->exec); ps->exec = nullptr; }
  return FIRE_OK;
}

int fire_poisson_make_rhs(FirePoisson* ps, float* b, unsigned seed, int n_sources, float noise, void* stream) {
  FIRE_RANGE("fire_poisson_make_rhs");
  if (!ps || !b || n_sources < 0 || n_sources > MAX_SOURCES) return FIRE_ERR_BAD_ARG;
  DeviceGuard dg(ps->device);
  std::vector<float> src((size_t)std::max(1, n_sources) * 5, 0.0f);
  if (n_sources > 0 && fire_poisson_sources(seed, n_sources, ps->res, src.data()) != FIRE_OK) return FIRE_ERR_BAD_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the source table travels by a synchronous copy (it is a few KB, once per right-hand side)
  if (cudaStreamSynchronize(st) != cudaSuccess) return FIRE_ERR_CUDA;
  if (cudaMemcpy(ps->src, src.data(), sizeof(float) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess) return FIRE_ERR_CUDA;
  const dim3 g = grid3(ps->res[0], ps->res[1], ps->res[2]);
  k_rhs<<<g, kBlock, 0, st>>>(b, ps->res[0], ps->res[1], ps->res[2], ps->src, n_sources, noise, seed, ps->partials);
  k_mean<<<1, NT, 0, st>>>(ps->partials, (int)(g.x * g.y * g.z), (double)ps->cells, ps->mean);
  k_sub_mean<<<1024, 256, 0, st>>>(b, ps->cells, ps->mean);
  return cudaGetLastError() == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

}  // extern "C"
