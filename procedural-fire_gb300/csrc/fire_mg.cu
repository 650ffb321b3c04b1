// Geometric multigrid for the pressure Poisson equation (src/sim.js:415-495, 576-599).
//
// Cell-centred 7-point Laplacian, open sides and top (p = 0 on the boundary face: ghost = -p),
// solid floor (Neumann: ghost = p).  Level l has spacing h = dx * 2^l; the equation per level is
// sum_nb(p) - 6 p = h^2 b with the ghost rules folded into the diagonal of the red-black Gauss-Seidel
// update, exactly as mgSmooth does.
//
// GB300 mapping:
//  * the fine levels run one launch per colour sweep, restriction and prolongation on 3D grids of
//    32 x 4 x 2 CTAs (32-bit index arithmetic, no integer division); at 128x256x128 the level-0 arrays
//    (p and b, 33.5 MB) stay resident in the 129 MB L2 across the cycle;
//  * every level small enough to fit, with all coarser ones, in one CTA's shared memory is solved by a
//    single-CTA kernel that runs the rest of the V-cycle out of shared memory; levels of <= 256 cells
//    inside it run on one warp with __syncwarp, so the coarsest sweeps cost no CTA-wide barriers;
//  * every kernel uses programmatic dependent launch (fire_launch.cuh) so consecutive launches overlap.
#include <algorithm>
#include <cstring>
#include <cooperative_groups.h>

#include "fire_device.cuh"
#include "fire_launch.cuh"

namespace fire {

constexpr int GX = 32, GY = 4, GZ = 2;   // CTA shape of the level kernels (256 threads)

// ---------------- red-black Gauss-Seidel update of one cell (src/sim.js:417-437) ----------------
// Neighbours in the order mgSmooth sums them: x-, x+, z-, z+, y-, y+.
__device__ __forceinline__ float rb_update(const float* p, const float* b, int x, int y, int z, int nx, int ny, int nz, float h2) {
  const int sy = nx, sz = nx * ny;
  const int c = x + y * sy + z * sz;
  float sum = 0.0f, diag = 6.0f;
  if (x > 0) sum += p[c - 1]; else diag += 1.0f;
  if (x < nx - 1) sum += p[c + 1]; else diag += 1.0f;
  if (z > 0) sum += p[c - sz]; else diag += 1.0f;
  if (z < nz - 1) sum += p[c + sz]; else diag += 1.0f;
  if (y > 0) sum += p[c - sy]; else diag -= 1.0f;
  if (y < ny - 1) sum += p[c + sy]; else diag += 1.0f;
  // WGSL's `/` is specified to 2.5 ULP; the fast reciprocal-multiply quotient (<= 2 ULP) keeps the
  // smoother at a handful of instructions per cell instead of an IEEE division sequence.  sum - h2 b is one
  // explicit FMA in every form of the sweep (launch per colour, shared-memory tails), so they give the same bits.
  return __fdividef(__fmaf_rn(-h2, b[c], sum), diag);
}
// The convergence studies' red-black update (research/webgpu-bench/wgsl/mg.wgsl smoothRB, poisson.mjs:28-35):
// ghosts take the cell's old value (floor +p, open faces -p), summed x-, x+, y-, y+, z-, z+;
// pg = (sum - h^2 b) / 6 and p <- mix(p, pg, omega) (pg itself when omega = 1).
__device__ __forceinline__ float study_update(const float* p, const float* b, int x, int y, int z, int nx, int ny, int nz, float h2,
                                              float omega) {
  const int sy = nx, sz = nx * ny;
  const int c = x + y * sy + z * sz;
  const float pc = p[c];
  const float s = (x > 0 ? p[c - 1] : -pc) + (x < nx - 1 ? p[c + 1] : -pc) + (y > 0 ? p[c - sy] : pc) +
                  (y < ny - 1 ? p[c + sy] : -pc) + (z > 0 ? p[c - sz] : -pc) + (z < nz - 1 ? p[c + sz] : -pc);
  const float pg = (s - h2 * b[c]) / 6.0f;
  return omega == 1.0f ? pg : fmaf(omega, pg - pc, pc);
}
// Each thread updates SMZ cells of one colour, SMZ planes apart in z (unrolled and independent, so their
// loads are in flight together): the sweep is latency-bound on L2 hits, and fewer, longer CTAs also cut the
// CTA turnover that leaves warp slots idle.
#ifndef FIRE_SMOOTH_Z
#define FIRE_SMOOTH_Z 2
#endif
constexpr int SMZ = FIRE_SMOOTH_Z;
// omega != 1 over-relaxes the update (p + omega (p_gs - p)); omega == 1 is the reference's Gauss-Seidel
// update bit for bit.
template <bool kRelax, bool kStudy = false, int kZ = SMZ>
__device__ __forceinline__ void smooth_body_t(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz, float h, int color,
                                              uint3 blk, float omega) {
  pdl_wait();
  pdl_trigger();
  const int gx = blk.x * GX + threadIdx.x, y = blk.y * GY + threadIdx.y;
  const int zb = (blk.z * GZ + threadIdx.z) * kZ;
  if (y >= ny) return;
  const float h2 = h * h;
  float v[kZ];
#pragma unroll
  for (int k = 0; k < kZ; ++k) {   // all reads first (a colour's cells never read each other) ...
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) {
      if (kStudy) {
        v[k] = study_update(p, b, x, y, z, nx, ny, nz, h2, omega);
        continue;
      }
      v[k] = rb_update(p, b, x, y, z, nx, ny, nz, h2);
      if (kRelax) {
        const float old = p[x + nx * (y + ny * z)];
        v[k] = fmaf(omega, v[k] - old, old);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kZ; ++k) {   // ... then the writes
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) p[x + nx * (y + ny * z)] = v[k];
  }
}
__device__ __forceinline__ void smooth_body(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz, float h, int color,
                                            uint3 blk, float omega = 1.0f) {
  if (omega == 1.0f) smooth_body_t<false>(p, b, nx, ny, nz, h, color, blk, omega);
  else smooth_body_t<true>(p, b, nx, ny, nz, h, color, blk, omega);
}

// ---------------- fused residual + restriction (src/sim.js:439-466) ----------------
__device__ __forceinline__ float pghost(const float* p, int x, int y, int z, int nx, int ny, int nz, float me) {
  if (x < 0 || z < 0 || x >= nx || z >= nz || y >= ny) return -me;
  if (y < 0) return me;
  return p[x + nx * (y + ny * z)];
}
__device__ __forceinline__ float restrict_cell(const float* p, const float* b, int cx, int cy, int cz, int nx, int ny, int nz, float ih2) {
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int x = 2 * cx + (q & 1), y = 2 * cy + ((q >> 1) & 1), z = 2 * cz + ((q >> 2) & 1);
    const int c = x + nx * (y + ny * z);
    const float me = p[c];
    const float lap = (pghost(p, x - 1, y, z, nx, ny, nz, me) + pghost(p, x + 1, y, z, nx, ny, nz, me) +
                       pghost(p, x, y - 1, z, nx, ny, nz, me) + pghost(p, x, y + 1, z, nx, ny, nz, me) +
                       pghost(p, x, y, z - 1, nx, ny, nz, me) + pghost(p, x, y, z + 1, nx, ny, nz, me) - 6.0f * me) * ih2;
    acc += b[c] - lap;
  }
  return acc * 0.125f;
}
__device__ __forceinline__ void restrict_body(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz, float h,
                                              float* __restrict__ bc, float* __restrict__ pc, uint3 blk) {
  pdl_wait();
  pdl_trigger();
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const int cx = blk.x * GX + threadIdx.x, cy = blk.y * GY + threadIdx.y, cz = blk.z * GZ + threadIdx.z;
  if (cx >= cnx || cy >= cny || cz >= cnz) return;
  const float ih2 = 1.0f / (h * h);
  const int t = cx + cnx * (cy + cny * cz);
  bc[t] = restrict_cell(p, b, cx, cy, cz, nx, ny, nz, ih2);
  pc[t] = 0.0f;
}
// Restriction fused with the coarse level's first colour-0 sweep.  The coarse pressure starts at zero, so that
// sweep's update of a colour-0 cell reads only the cell's own right-hand side: it is formed here from the value
// just restricted with the smoother's arithmetic (rb_update over zero neighbours: the same diagonal, the same
// explicit FMA and quotient, the same relaxation from an old value of zero), so the result is bit-identical
// to restricting and then sweeping.  Colour-1 cells keep zero.
template <bool kRelax>
__device__ __forceinline__ void restrict_smooth_body(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                     float h, float* __restrict__ bc, float* __restrict__ pc, float hc, float omega,
                                                     uint3 blk) {
  pdl_wait();
  pdl_trigger();
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const int cx = blk.x * GX + threadIdx.x, cy = blk.y * GY + threadIdx.y, cz = blk.z * GZ + threadIdx.z;
  if (cx >= cnx || cy >= cny || cz >= cnz) return;
  const int t = cx + cnx * (cy + cny * cz);
  const float r = restrict_cell(p, b, cx, cy, cz, nx, ny, nz, 1.0f / (h * h));
  bc[t] = r;
  float v = 0.0f;
  if (((cx + cy + cz) & 1) == 0) {
    float diag = 6.0f;   // rb_update's ghost rules: open sides and top add 1, the floor subtracts 1
    if (cx == 0) diag += 1.0f;
    if (cx == cnx - 1) diag += 1.0f;
    if (cz == 0) diag += 1.0f;
    if (cz == cnz - 1) diag += 1.0f;
    if (cy == 0) diag -= 1.0f;
    if (cy == cny - 1) diag += 1.0f;
    v = __fdividef(__fmaf_rn(-(hc * hc), r, 0.0f), diag);
    if (kRelax) v = fmaf(omega, v - 0.0f, 0.0f);
  }
  pc[t] = v;
}

// ---------------- prolongation with mirror ghosts (src/sim.js:468-495) ----------------
template <bool kClamp = false>
__device__ __forceinline__ float prolong_cell(const float* pc, int x, int y, int z, int ncx, int ncy, int ncz) {
  const float gx = ((float)x + 0.5f) * 0.5f - 0.5f, gy = ((float)y + 0.5f) * 0.5f - 0.5f, gz = ((float)z + 0.5f) * 0.5f - 0.5f;
  const int g0x = (int)floorf(gx), g0y = (int)floorf(gy), g0z = (int)floorf(gz);
  const float fx = gx - (float)g0x, fy = gy - (float)g0y, fz = gz - (float)g0z;
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int ox = q & 1, oy = (q >> 1) & 1, oz = (q >> 2) & 1;
    const int qx = g0x + ox, qy = g0y + oy, qz = g0z + oz;
    float val = pc[min(max(qx, 0), ncx - 1) + ncx * (min(max(qy, 0), ncy - 1) + ncy * min(max(qz, 0), ncz - 1))];
    // odd mirror (Dirichlet) on sides/top, even (Neumann) at the floor; one flip per axis outside (the
    // studies' prolongation clamps to the edge without flips)
    if (!kClamp) {
      if (qx < 0 || qx >= ncx) val = -val;
      if (qz < 0 || qz >= ncz) val = -val;
      if (qy >= ncy) val = -val;
    }
    const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy, wz = oz ? fz : 1.0f - fz;
    acc += val * wx * wy * wz;
  }
  return acc;
}
// One thread per coarse cell: the 3x3x3 coarse neighbourhood (with the mirror signs of prolong_cell) is
// loaded once and the 8 fine children are formed from it.  For fine index c = 2 cc + d the trilinear base is
// g0 = cc - 1 + d with fraction 0.75 (d = 0) or 0.25 (d = 1), so child d reads coarse offsets d-1 and d;
// each child's sum runs in prolong_cell's order, so the result is identical.
template <bool kClamp = false>
__device__ __forceinline__ void prolong_body(float* __restrict__ p, const float* __restrict__ pc, int nx, int ny, int nz, uint3 blk) {
  pdl_wait();
  pdl_trigger();
  const int ncx = nx / 2, ncy = ny / 2, ncz = nz / 2;
  const int cx = blk.x * GX + threadIdx.x, cy = blk.y * GY + threadIdx.y, cz = blk.z * GZ + threadIdx.z;
  if (cx >= ncx || cy >= ncy || cz >= ncz) return;
  float v[3][3][3];   // [dz][dy][dx] for offsets -1..1
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int qx = cx + c - 1, qy = cy + bb - 1, qz = cz + a - 1;
        float val = __ldg(pc + min(max(qx, 0), ncx - 1) + ncx * (min(max(qy, 0), ncy - 1) + ncy * min(max(qz, 0), ncz - 1)));
        if (!kClamp) {
          if (qx < 0 || qx >= ncx) val = -val;
          if (qz < 0 || qz >= ncz) val = -val;
          if (qy >= ncy) val = -val;
        }
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
        const int t = (2 * cx + dx) + nx * ((2 * cy + dy) + ny * (2 * cz + dz));
        p[t] = p[t] + acc;
      }
}

// Per-level kernels of one simulation, and their batched forms over many simulations (one grid; each CTA
// finds its simulation's level from the BatchMap and runs the same body).
__global__ void __launch_bounds__(GX * GY * GZ) k_smooth(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz, float h,
                                                         int color, float omega) {
  smooth_body(p, b, nx, ny, nz, h, color, blockIdx, omega);
}
// One cell per thread, for levels too small to fill the GPU with SMZ cells per thread.
__global__ void __launch_bounds__(GX * GY * GZ) k_smooth1(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz, float h,
                                                          int color, float omega) {
  if (omega == 1.0f) smooth_body_t<false, false, 1>(p, b, nx, ny, nz, h, color, blockIdx, omega);
  else smooth_body_t<true, false, 1>(p, b, nx, ny, nz, h, color, blockIdx, omega);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_restrict(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                           float h, float* __restrict__ bc, float* __restrict__ pc) {
  restrict_body(p, b, nx, ny, nz, h, bc, pc, blockIdx);
}
template <bool kRelax>
__global__ void __launch_bounds__(GX * GY * GZ) k_restrict_smooth(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny,
                                                                  int nz, float h, float* __restrict__ bc, float* __restrict__ pc, float hc,
                                                                  float omega) {
  restrict_smooth_body<kRelax>(p, b, nx, ny, nz, h, bc, pc, hc, omega, blockIdx);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_prolong(float* __restrict__ p, const float* __restrict__ pc, int nx, int ny, int nz) {
  prolong_body(p, pc, nx, ny, nz, blockIdx);
}
// The convergence studies' smoother and prolongation (MGLevel::study).
__global__ void __launch_bounds__(GX * GY * GZ) k_smooth_study(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                               float h, int color, float omega) {
  smooth_body_t<false, true>(p, b, nx, ny, nz, h, color, blockIdx, omega);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_prolong_clamp(float* __restrict__ p, const float* __restrict__ pc, int nx, int ny, int nz) {
  prolong_body<true>(p, pc, nx, ny, nz, blockIdx);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_smooth_b(const __grid_constant__ BatchMap m, const __grid_constant__ LevelBatch L, int color) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  const MGLevel& v = L.l[i];
  smooth_body(v.p, v.b, v.nx, v.ny, v.nz, v.h, color, blk, v.omega);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_restrict_b(const __grid_constant__ BatchMap m, const __grid_constant__ LevelBatch F,
                                                             const __grid_constant__ LevelBatch C) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  restrict_body(F.l[i].p, F.l[i].b, F.l[i].nx, F.l[i].ny, F.l[i].nz, F.l[i].h, C.l[i].b, C.l[i].p, blk);
}
__global__ void __launch_bounds__(GX * GY * GZ) k_prolong_b(const __grid_constant__ BatchMap m, const __grid_constant__ LevelBatch F,
                                                            const __grid_constant__ LevelBatch C) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  prolong_body(F.l[i].p, C.l[i].p, F.l[i].nx, F.l[i].ny, F.l[i].nz, blk);
}

// ---------------- single-CTA tail V-cycle out of shared memory ----------------
// Cells are visited as a flat index split into (x, y, z) with a float-reciprocal quotient and a one-step
// correction (exact for indices below 2^24), several times cheaper than integer division.  Levels with
// at most TAIL_WARP_CELLS cells run on warp 0 alone, synchronised with __syncwarp.
constexpr int TAIL_THREADS = 1024;
constexpr int TAIL_WARP_CELLS = 256;
constexpr int TAIL_MAX_LEVELS = 12;
struct TailLevels {
  int n;                       // number of levels in the tail
  int small;                   // first tail level with <= TAIL_WARP_CELLS cells (n if none)
  int nx[TAIL_MAX_LEVELS], ny[TAIL_MAX_LEVELS], nz[TAIL_MAX_LEVELS];
  float h[TAIL_MAX_LEVELS];
  int off[TAIL_MAX_LEVELS];    // float offset of level l's p in shared memory (b follows p)
  float* gp[TAIL_MAX_LEVELS];  // global copies (written back at the end)
  float* gb[TAIL_MAX_LEVELS];
  int coarse;                  // coarsest-level sweeps (used by the batched tails; per-simulation launches pass it)
  float omega;                 // over-relaxation of the sweeps (1: Gauss-Seidel)
  int coarse64;                // 1: the coarsest level is solved in FP64: p = cinv b with the dense inverse
  int doff;                    //    (transposed, global memory) if cinv is set, else `coarse` FP64 sweeps on a
  const double* cinv;          //    double copy at float offset doff
  int study;                   // 1: the convergence studies' smoother and prolongation (MGLevel::study)
  int wait_polls;              // poll limit of the wait for the staging copies (TAIL_WAIT_POLLS; a test lowers it)
};
struct FastDiv {
  int d;
  float r;
  __device__ FastDiv(int dd) : d(dd), r(1.0f / (float)dd) {}
  __device__ __forceinline__ int div(int t) const {
    int q = __float2int_rz((float)t * r);
    const int rem = t - q * d;
    if (rem < 0) --q;
    else if (rem >= d) ++q;
    return q;
  }
};
// A group of threads working on one level: the whole CTA (barrier = __syncthreads) or warp 0 (__syncwarp).
template <bool kWarp>
struct Team {
  int rank;
  static constexpr int size = kWarp ? 32 : TAIL_THREADS;
  __device__ __forceinline__ void sync() const { if (kWarp) __syncwarp(); else __syncthreads(); }
};
// Spreads a team over a box of ax x ay x az items: thread extents (tx, ty, tz) and this thread's start.
// Each thread then strides through the box in 3D, so no index division happens per item.
struct Box3 {
  int tx, ty, tz, x0, y0, z0;
  __device__ Box3(int size, int rank, int ax, int ay, int az) {
    tx = min(ax, size);
    ty = min(ay, size / tx);
    tz = min(az, size / (tx * ty));
    x0 = rank % tx;
    const int r = rank / tx;
    y0 = r % ty;
    z0 = r / ty;
    if (z0 >= tz) z0 = 1 << 30;   // surplus thread: its loops never run (prolongation is read-modify-write)
  }
};
template <bool kWarp, bool kRelax, bool kStudy = false>
__device__ void tail_smooth_t(const Team<kWarp>& tm, float* p, const float* b, int nx, int ny, int nz, float h, int iters, float omega) {
  const int hx = (nx + 1) >> 1;
  const float h2 = h * h;
  const Box3 bx(tm.size, tm.rank, hx, ny, nz);
  for (int it = 0; it < iters; ++it)
    for (int color = 0; color < 2; ++color) {
      for (int z = bx.z0; z < nz; z += bx.tz)
        for (int y = bx.y0; y < ny; y += bx.ty)
          for (int gx = bx.x0; gx < hx; gx += bx.tx) {
            const int x = gx * 2 + ((y + z + color) & 1);
            if (x < nx) {
              const int c = x + nx * (y + ny * z);
              if (kStudy) {
                p[c] = study_update(p, b, x, y, z, nx, ny, nz, h2, omega);
                continue;
              }
              const float v = rb_update(p, b, x, y, z, nx, ny, nz, h2);
              p[c] = kRelax ? fmaf(omega, v - p[c], p[c]) : v;
            }
          }
      tm.sync();
    }
}
// `iters` red-black sweeps of one level (over-relaxed by omega when omega != 1).
template <bool kWarp>
__device__ void tail_smooth(const Team<kWarp>& tm, float* p, const float* b, int nx, int ny, int nz, float h, int iters, float omega,
                            int study = 0) {
  if (study) tail_smooth_t<kWarp, false, true>(tm, p, b, nx, ny, nz, h, iters, omega);
  else if (omega == 1.0f) tail_smooth_t<kWarp, false>(tm, p, b, nx, ny, nz, h, iters, omega);
  else tail_smooth_t<kWarp, true>(tm, p, b, nx, ny, nz, h, iters, omega);
}
// `iters` red-black sweeps in FP64 on a double copy (dp: p then b) of one level; p is written back in FP32.
// The update is mgSmooth's (src/sim.js:417-437) with IEEE double division.
template <bool kWarp>
__device__ void tail_smooth_fp64(const Team<kWarp>& tm, float* p, const float* b, int nx, int ny, int nz, float h, int iters, double* dp) {
  const int n = nx * ny * nz;
  double* db = dp + n;
  for (int t = tm.rank; t < n; t += tm.size) { dp[t] = (double)p[t]; db[t] = (double)b[t]; }
  tm.sync();
  const int hx = (nx + 1) >> 1, sy = nx, sz = nx * ny;
  const double h2 = (double)h * (double)h;
  const Box3 bx(tm.size, tm.rank, hx, ny, nz);
  for (int it = 0; it < iters; ++it)
    for (int color = 0; color < 2; ++color) {
      for (int z = bx.z0; z < nz; z += bx.tz)
        for (int y = bx.y0; y < ny; y += bx.ty)
          for (int gx = bx.x0; gx < hx; gx += bx.tx) {
            const int x = gx * 2 + ((y + z + color) & 1);
            if (x >= nx) continue;
            const int c = x + y * sy + z * sz;
            double sum = 0.0, diag = 6.0;
            if (x > 0) sum += dp[c - 1]; else diag += 1.0;
            if (x < nx - 1) sum += dp[c + 1]; else diag += 1.0;
            if (z > 0) sum += dp[c - sz]; else diag += 1.0;
            if (z < nz - 1) sum += dp[c + sz]; else diag += 1.0;
            if (y > 0) sum += dp[c - sy]; else diag -= 1.0;
            if (y < ny - 1) sum += dp[c + sy]; else diag += 1.0;
            dp[c] = (sum - h2 * db[c]) / diag;
          }
      tm.sync();
    }
  for (int t = tm.rank; t < n; t += tm.size) p[t] = (float)dp[t];
  tm.sync();
}
// Exact coarsest solve in FP64: p = A^-1 b with the dense inverse stored transposed (mt[j * n + i] = inv[i][j]),
// so the team's lanes read consecutive rows; four accumulators break the FMA dependency chain.
template <bool kWarp>
__device__ void tail_direct_fp64(const Team<kWarp>& tm, float* p, const float* b, int n, const double* __restrict__ mt) {
  for (int i = tm.rank; i < n; i += tm.size) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int j = 0;
    for (; j + 3 < n; j += 4) {
      a0 = fma(__ldg(mt + (size_t)j * n + i), (double)b[j], a0);
      a1 = fma(__ldg(mt + (size_t)(j + 1) * n + i), (double)b[j + 1], a1);
      a2 = fma(__ldg(mt + (size_t)(j + 2) * n + i), (double)b[j + 2], a2);
      a3 = fma(__ldg(mt + (size_t)(j + 3) * n + i), (double)b[j + 3], a3);
    }
    for (; j < n; ++j) a0 = fma(__ldg(mt + (size_t)j * n + i), (double)b[j], a0);
    p[i] = (float)((a0 + a1) + (a2 + a3));
  }
  tm.sync();
}
template <bool kWarp>
__device__ void tail_restrict(const Team<kWarp>& tm, const TailLevels& T, float* sm, int l) {
  const int nx = T.nx[l], ny = T.ny[l], nz = T.nz[l];
  const float* p = sm + T.off[l];
  const float* b = p + nx * ny * nz;
  const int cnx = T.nx[l + 1], cny = T.ny[l + 1], cnz = T.nz[l + 1];
  float* pc = sm + T.off[l + 1];
  float* bc = pc + cnx * cny * cnz;
  const float ih2 = 1.0f / (T.h[l] * T.h[l]);
  const Box3 bx(tm.size, tm.rank, cnx, cny, cnz);
  for (int cz = bx.z0; cz < cnz; cz += bx.tz)
    for (int cy = bx.y0; cy < cny; cy += bx.ty)
      for (int cx = bx.x0; cx < cnx; cx += bx.tx) {
        const int t = cx + cnx * (cy + cny * cz);
        bc[t] = restrict_cell(p, b, cx, cy, cz, nx, ny, nz, ih2);
        pc[t] = 0.0f;
      }
  tm.sync();
}
template <bool kWarp>
__device__ void tail_prolong(const Team<kWarp>& tm, const TailLevels& T, float* sm, int l) {
  const int nx = T.nx[l], ny = T.ny[l], nz = T.nz[l];
  float* p = sm + T.off[l];
  const float* pc = sm + T.off[l + 1];
  const Box3 bx(tm.size, tm.rank, nx, ny, nz);
  for (int z = bx.z0; z < nz; z += bx.tz)
    for (int y = bx.y0; y < ny; y += bx.ty)
      for (int x = bx.x0; x < nx; x += bx.tx) {
        const int t = x + nx * (y + ny * z);
        p[t] = p[t] + (T.study ? prolong_cell<true>(pc, x, y, z, nx / 2, ny / 2, nz / 2) : prolong_cell(pc, x, y, z, nx / 2, ny / 2, nz / 2));
      }
  tm.sync();
}
// V-cycle over tail levels [from, n) with one team (src/sim.js:588-599 restricted to these levels).
template <bool kWarp>
__device__ void tail_vcycle(const Team<kWarp>& tm, const TailLevels& T, float* sm, int from, int pre, int post, int coarse) {
  const int n = T.n;
  for (int l = from; l < n - 1; ++l) {
    float* p = sm + T.off[l];
    tail_smooth(tm, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre, T.omega, T.study);
    tail_restrict(tm, T, sm, l);
  }
  {
    float* p = sm + T.off[n - 1];
    if (T.coarse64 && T.cinv)
      tail_direct_fp64(tm, p, p + T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1], T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1], T.cinv);
    else if (T.coarse64)
      tail_smooth_fp64(tm, p, p + T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1], T.nx[n - 1], T.ny[n - 1], T.nz[n - 1], T.h[n - 1], coarse,
                       reinterpret_cast<double*>(sm + T.doff));
    else
      tail_smooth(tm, p, p + T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1], T.nx[n - 1], T.ny[n - 1], T.nz[n - 1], T.h[n - 1], coarse, T.omega, T.study);
  }
  for (int l = n - 2; l >= from; --l) {
    tail_prolong(tm, T, sm, l);
    float* p = sm + T.off[l];
    tail_smooth(tm, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post, T.omega, T.study);
  }
}
// The V-cycle over all levels of T with one CTA of TAIL_THREADS threads: levels above T.small with the
// whole CTA, the rest on warp 0.
// Exact coarsest solve with the whole CTA: thread t forms a partial of row t % n over the columns
// j = t / n, t / n + K, ... (K = TAIL_THREADS / n chunks, consecutive threads read consecutive rows), the
// partials go to shared memory (dp) and each row is summed over its K partials in a fixed order.
__device__ void tail_direct_fp64_cta(int tid, float* p, const float* b, int n, const double* __restrict__ mt, double* dp) {
  const int K = TAIL_THREADS / n;
  if (tid < n * K) {
    const int i = tid % n, k = tid / n;
    double a0 = 0.0, a1 = 0.0;
    int j = k;
    for (; j + K < n; j += 2 * K) {
      a0 = fma(__ldg(mt + (size_t)j * n + i), (double)b[j], a0);
      a1 = fma(__ldg(mt + (size_t)(j + K) * n + i), (double)b[j + K], a1);
    }
    if (j < n) a0 = fma(__ldg(mt + (size_t)j * n + i), (double)b[j], a0);
    dp[k * n + i] = a0 + a1;
  }
  __syncthreads();
  if (tid < n) {
    double s = 0.0;
    for (int k = 0; k < K; ++k) s += dp[k * n + tid];
    p[tid] = (float)s;
  }
  __syncthreads();
}
__device__ void tail_cta_vcycle(const TailLevels& T, float* sm, int tid, int pre, int post, int coarse) {
  const Team<false> cta{tid};
  const int S = T.small;
  if (T.coarse64 && T.cinv) {
    // levels [0, S) with the CTA, [S, n-1) on warp 0, the exact coarsest solve with the whole CTA
    const int n = T.n, top = min(S, n - 1);
    for (int l = 0; l < top; ++l) {
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre, T.omega, T.study);
      tail_restrict(cta, T, sm, l);
    }
    if (tid < 32) {
      const Team<true> wp{tid};
      for (int l = top; l < n - 1; ++l) {
        float* p = sm + T.off[l];
        tail_smooth(wp, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre, T.omega, T.study);
        tail_restrict(wp, T, sm, l);
      }
    }
    __syncthreads();
    {
      float* p = sm + T.off[n - 1];
      const int nc = T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1];
      tail_direct_fp64_cta(tid, p, p + nc, nc, T.cinv, reinterpret_cast<double*>(sm + T.doff));
    }
    if (tid < 32) {
      const Team<true> wp{tid};
      for (int l = n - 2; l >= top; --l) {
        tail_prolong(wp, T, sm, l);
        float* p = sm + T.off[l];
        tail_smooth(wp, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post, T.omega, T.study);
      }
    }
    __syncthreads();
    for (int l = top - 1; l >= 0; --l) {
      tail_prolong(cta, T, sm, l);
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post, T.omega, T.study);
    }
    return;
  }
  if (S == 0) {
    if (tid < 32) tail_vcycle(Team<true>{tid}, T, sm, 0, pre, post, coarse);
    __syncthreads();
  } else if (S >= T.n) {
    tail_vcycle(cta, T, sm, 0, pre, post, coarse);
  } else {
    // large levels [0, S) with the whole CTA; the V-cycle below S (levels S..n-1) on warp 0
    for (int l = 0; l < S; ++l) {
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre, T.omega, T.study);
      tail_restrict(cta, T, sm, l);
    }
    if (tid < 32) tail_vcycle(Team<true>{tid}, T, sm, S, pre, post, coarse);
    __syncthreads();
    for (int l = S - 1; l >= 0; --l) {
      tail_prolong(cta, T, sm, l);
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post, T.omega, T.study);
    }
  }
}
// ---- TMA bulk copies between global and shared memory (cp.async.bulk, mbarrier completion) ----
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for phase 0 of the barrier for at most about a second and at most max_polls polls; returns false if
// a limit was reached.
__device__ __forceinline__ bool mbar_wait0(uint64_t* bar, int max_polls = TAIL_WAIT_POLLS) {
  const unsigned long long t0 = global_ns();
  for (int it = 0; it < max_polls; ++it) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(smem_addr(bar)), "r"(0u) : "memory");
    if (done) return true;
    if ((it & 63) == 63 && global_ns() - t0 > 1000000000ull) return false;
  }
  return false;
}
// Makes this thread's generic-proxy shared-memory writes visible to the async proxy (TMA); every writing
// thread runs it before the CTA barrier that precedes a bulk store.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ bool bulk_ok(const void* g, const void* s, unsigned bytes) {
  return ((reinterpret_cast<uintptr_t>(g) | reinterpret_cast<uintptr_t>(s) | bytes) & 15u) == 0;
}

__device__ __forceinline__ void tail_body(const TailLevels& T, int pre, int post, int coarse, int* err) {
  extern __shared__ float sm[];
  __shared__ alignas(8) uint64_t bar;
  pdl_wait();
  pdl_trigger();
  const int tid = threadIdx.x;
  {  // stage the first tail level's p and b (restriction already wrote them) with two TMA bulk copies
    const int n0 = T.nx[0] * T.ny[0] * T.nz[0];
    float* p = sm + T.off[0];
    float* b = p + n0;
    const unsigned bytes = (unsigned)n0 * 4u;
    const bool bulk = bulk_ok(T.gp[0], p, bytes) && bulk_ok(T.gb[0], b, bytes);
    if (bulk) {
      if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, 2u * bytes);
        bulk_g2s(p, T.gp[0], bytes, &bar);
        bulk_g2s(b, T.gb[0], bytes, &bar);
      }
      __syncthreads();                        // the barrier is initialised before anyone polls it
      if (!mbar_wait0(&bar, T.wait_polls)) {  // bounded wait: report and leave instead of hanging
        if (tid == 0) atomicExch(err, 1);
        // copies may still be landing in this CTA's shared memory: a second wait, at the full bound, for them
        // before the CTA exits and its shared memory can be handed to another CTA
        mbar_wait0(&bar, TAIL_WAIT_POLLS);
        return;
      }
    } else {
      for (int t = tid; t < n0; t += TAIL_THREADS) { p[t] = T.gp[0][t]; b[t] = T.gb[0][t]; }
    }
    __syncthreads();
  }
  tail_cta_vcycle(T, sm, tid, pre, post, coarse);
  // write the first tail level's p back (it feeds the next prolongation) with one bulk store; the coarser
  // tail levels are scratch and stay in shared memory
  {
    const int n0 = T.nx[0] * T.ny[0] * T.nz[0];
    const float* p = sm + T.off[0];
    const unsigned bytes = (unsigned)n0 * 4u;
    if (bulk_ok(T.gp[0], p, bytes)) {
      fence_proxy_async();
      __syncthreads();
      if (tid == 0) bulk_s2g(T.gp[0], p, bytes);
    } else {
      for (int t = tid; t < n0; t += TAIL_THREADS) T.gp[0][t] = p[t];
    }
  }
}

// ---------------- cluster tail: the finer tail levels spread over a thread-block cluster ----------------
// CTA r of a CTAIL_CLUSTER-CTA cluster holds z-planes [r P, (r+1) P) of p and b of every distributed level
// (P = nz / CTAIL_CLUSTER, even), at the same shared-memory offset in every CTA.  A plane just outside the
// slab is read from the neighbouring CTA's shared memory through the cluster's distributed shared-memory
// window, so each colour sweep, restriction and prolongation is one phase closed by a cluster barrier
// (release/acquire at cluster scope) instead of a kernel launch.  The coarsest levels are gathered on CTA 0:
// the last distributed restriction writes straight into CTA 0's shared memory, CTA 0 runs them as k_tail
// does while the other CTAs wait at the barrier, and the prolongation reads them back from CTA 0.
// Every arithmetic expression is the one of the launch-per-phase kernels above, in the same order.
#ifndef FIRE_TAIL_CLUSTER
#define FIRE_TAIL_CLUSTER 8
#endif
constexpr int CTAIL_CLUSTER = FIRE_TAIL_CLUSTER;
constexpr int CTAIL_MIN_CELLS = 512;   // a distributed level gives every CTA at least this many cells
struct CTailLevels {
  int nd;                              // the first nd tail levels are distributed
  int nx[TAIL_MAX_LEVELS], ny[TAIL_MAX_LEVELS], nz[TAIL_MAX_LEVELS], P[TAIL_MAX_LEVELS];
  float h[TAIL_MAX_LEVELS];
  int off[TAIL_MAX_LEVELS];            // float offset of the level's p slab in every CTA (its b slab follows)
  float* gp;                           // global p and b of the first tail level
  float* gb;
  TailLevels G;                        // the gathered levels; offsets into CTA 0's shared memory
};
namespace cg = cooperative_groups;
// This CTA's view of one distributed level.
struct DSlab {
  int nx, ny, nz, P, z0, plane;
  float h;
  float* p;                            // planes z0 .. z0+P-1 of p; b follows at p + P * plane
};
__device__ __forceinline__ DSlab make_slab(const CTailLevels& T, int l, unsigned r, float* sm) {
  DSlab s;
  s.nx = T.nx[l]; s.ny = T.ny[l]; s.nz = T.nz[l]; s.P = T.P[l];
  s.z0 = (int)r * s.P;
  s.plane = s.nx * s.ny;
  s.h = T.h[l];
  s.p = sm + T.off[l];
  return s;
}
// Plane z (z0-1 <= z <= z0+P) of p: local, a neighbour CTA's edge plane, or nullptr outside the domain.
__device__ __forceinline__ const float* dplane(const cg::cluster_group& cl, const DSlab& s, int z, unsigned r) {
  if (z < 0 || z >= s.nz) return nullptr;
  if (z < s.z0) return cl.map_shared_rank(s.p + (s.P - 1) * s.plane, (int)r - 1);
  if (z >= s.z0 + s.P) return cl.map_shared_rank(s.p, (int)r + 1);
  return s.p + (z - s.z0) * s.plane;
}
// rb_update with the z neighbours given as plane pointers (nullptr = domain face).
__device__ __forceinline__ float rb_update_planes(const float* pl, const float* pm, const float* pu, const float* bm, int x, int y,
                                                  int nx, int ny, float h2) {
  const int c = x + y * nx;
  float sum = 0.0f, diag = 6.0f;
  if (x > 0) sum += pm[c - 1]; else diag += 1.0f;
  if (x < nx - 1) sum += pm[c + 1]; else diag += 1.0f;
  if (pl) sum += pl[c]; else diag += 1.0f;
  if (pu) sum += pu[c]; else diag += 1.0f;
  if (y > 0) sum += pm[c - nx]; else diag -= 1.0f;
  if (y < ny - 1) sum += pm[c + nx]; else diag += 1.0f;
  return __fdividef(__fmaf_rn(-h2, bm[c], sum), diag);
}
template <bool kRelax>
__device__ void ct_smooth_t(const cg::cluster_group& cl, const DSlab& s, unsigned r, int tid, int iters, float omega) {
  const int hx = (s.nx + 1) >> 1;
  const float h2 = s.h * s.h;
  const float* b = s.p + s.P * s.plane;
  const Box3 bx(TAIL_THREADS, tid, hx, s.ny, s.P);
  for (int it = 0; it < iters; ++it)
    for (int color = 0; color < 2; ++color) {
      for (int zl = bx.z0; zl < s.P; zl += bx.tz) {
        const int z = s.z0 + zl;
        float* pm = s.p + zl * s.plane;
        const float* pl = dplane(cl, s, z - 1, r);
        const float* pu = dplane(cl, s, z + 1, r);
        const float* bm = b + zl * s.plane;
        for (int y = bx.y0; y < s.ny; y += bx.ty)
          for (int gx = bx.x0; gx < hx; gx += bx.tx) {
            const int x = gx * 2 + ((y + z + color) & 1);
            if (x < s.nx) {
              const float v = rb_update_planes(pl, pm, pu, bm, x, y, s.nx, s.ny, h2);
              pm[x + s.nx * y] = kRelax ? fmaf(omega, v - pm[x + s.nx * y], pm[x + s.nx * y]) : v;
            }
          }
      }
      cl.sync();
    }
}
__device__ void ct_smooth(const cg::cluster_group& cl, const DSlab& s, unsigned r, int tid, int iters, float omega) {
  if (omega == 1.0f) ct_smooth_t<false>(cl, s, r, tid, iters, omega);
  else ct_smooth_t<true>(cl, s, r, tid, iters, omega);
}
// Fused residual + 8-child restriction of this CTA's slab into coarse planes z0/2 .. z0/2 + P/2 - 1.
// cp points at coarse plane z0/2 of p (local, or in CTA 0 for a gathered level); b is cb_off floats after p.
__device__ void ct_restrict(const cg::cluster_group& cl, const DSlab& s, unsigned r, int tid, float* cp, int cb_off) {
  const int cnx = s.nx / 2, cny = s.ny / 2, cP = s.P / 2, nx = s.nx, ny = s.ny;
  const float ih2 = 1.0f / (s.h * s.h);
  const float* b = s.p + s.P * s.plane;
  const Box3 bx(TAIL_THREADS, tid, cnx, cny, cP);
  for (int czl = bx.z0; czl < cP; czl += bx.tz) {
    const int fz = s.z0 + 2 * czl;   // first child plane
    const float* q[4] = {dplane(cl, s, fz - 1, r), s.p + 2 * czl * s.plane, s.p + (2 * czl + 1) * s.plane, dplane(cl, s, fz + 2, r)};
    const float* bq[2] = {b + 2 * czl * s.plane, b + (2 * czl + 1) * s.plane};
    for (int cy = bx.y0; cy < cny; cy += bx.ty)
      for (int cx = bx.x0; cx < cnx; cx += bx.tx) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int x = 2 * cx + (k & 1), y = 2 * cy + ((k >> 1) & 1), dz = (k >> 2) & 1;
          const float* pl = q[dz];
          const float* pm = q[1 + dz];
          const float* pu = q[2 + dz];
          const int c = x + nx * y;
          const float me = pm[c];
          const float gxm = x > 0 ? pm[c - 1] : -me, gxp = x < nx - 1 ? pm[c + 1] : -me;
          const float gym = y > 0 ? pm[c - nx] : me, gyp = y < ny - 1 ? pm[c + nx] : -me;
          const float gzm = pl ? pl[c] : -me, gzp = pu ? pu[c] : -me;
          const float lap = (gxm + gxp + gym + gyp + gzm + gzp - 6.0f * me) * ih2;
          acc += bq[dz][c] - lap;
        }
        const int t = cx + cnx * (cy + cny * czl);
        cp[cb_off + t] = acc * 0.125f;
        cp[t] = 0.0f;
      }
  }
  cl.sync();
}
// Coarse source of a prolongation: a distributed level (slab of this CTA) or the gathered level in CTA 0.
struct CSrc {
  const float* base;   // distributed: this CTA's slab; gathered: plane 0 in CTA 0 (already mapped)
  int z0, P, plane;
  bool dist;
};
__device__ __forceinline__ const float* csrc_plane(const cg::cluster_group& cl, const CSrc& c, int cz, unsigned r) {
  if (!c.dist) return c.base + cz * c.plane;
  if (cz < c.z0) return cl.map_shared_rank(c.base + (c.P - 1) * c.plane, (int)r - 1);
  if (cz >= c.z0 + c.P) return cl.map_shared_rank(c.base, (int)r + 1);
  return c.base + (cz - c.z0) * c.plane;
}
// k_prolong's coarse-cell-centric prolongation for the coarse planes over this CTA's fine slab.
__device__ void ct_prolong(const cg::cluster_group& cl, const DSlab& s, const CSrc& src, unsigned r, int tid) {
  const int ncx = s.nx / 2, ncy = s.ny / 2, ncz = s.nz / 2, cP = s.P / 2, cz0 = s.z0 / 2, nx = s.nx;
  const Box3 bx(TAIL_THREADS, tid, ncx, ncy, cP);
  for (int czl = bx.z0; czl < cP; czl += bx.tz) {
    const int cz = cz0 + czl;
    const float* pq[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) pq[a] = csrc_plane(cl, src, min(max(cz + a - 1, 0), ncz - 1), r);
    for (int cy = bx.y0; cy < ncy; cy += bx.ty)
      for (int cx = bx.x0; cx < ncx; cx += bx.tx) {
        float v[3][3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const int qx = cx + c - 1, qy = cy + bb - 1, qz = cz + a - 1;
              float val = pq[a][min(max(qx, 0), ncx - 1) + ncx * min(max(qy, 0), ncy - 1)];
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
              float* pf = s.p + (2 * czl + dz) * s.plane + (2 * cx + dx) + nx * (2 * cy + dy);
              *pf = *pf + acc;
            }
      }
  }
  cl.sync();
}
__device__ __forceinline__ void ctail_body(const CTailLevels& T, int pre, int post, int coarse) {
  extern __shared__ float4 sm4[];
  float* sm = reinterpret_cast<float*>(sm4);
  const cg::cluster_group cl = cg::this_cluster();
  const unsigned r = cl.block_rank();
  const int tid = threadIdx.x;
  pdl_wait();
  pdl_trigger();
  const bool vec = ((reinterpret_cast<uintptr_t>(T.gp) | reinterpret_cast<uintptr_t>(T.gb)) & 15u) == 0;
  {  // this CTA's slab of the first tail level: one contiguous z-range of p and of b in global memory
    const DSlab s = make_slab(T, 0, r, sm);
    const int n = s.P * s.plane;   // a multiple of 4: distributed levels have even nx and ny
    const size_t g0 = (size_t)s.z0 * s.plane;
    float* lb = s.p + n;
    if (vec) {
      const float4* gp = reinterpret_cast<const float4*>(T.gp + g0);
      const float4* gb = reinterpret_cast<const float4*>(T.gb + g0);
      for (int t = tid; t < n / 4; t += TAIL_THREADS) {
        reinterpret_cast<float4*>(s.p)[t] = gp[t];
        reinterpret_cast<float4*>(lb)[t] = gb[t];
      }
    } else {
      for (int t = tid; t < n; t += TAIL_THREADS) { s.p[t] = T.gp[g0 + t]; lb[t] = T.gb[g0 + t]; }
    }
  }
  cl.sync();
  float* g0p = sm + T.G.off[0];
  float* g0r = r == 0 ? g0p : cl.map_shared_rank(g0p, 0);
  const int gplane = T.G.nx[0] * T.G.ny[0];
  const int gcells = gplane * T.G.nz[0];
  for (int l = 0; l < T.nd; ++l) {
    const DSlab s = make_slab(T, l, r, sm);
    ct_smooth(cl, s, r, tid, pre, T.G.omega);
    if (l + 1 < T.nd) {
      const DSlab c = make_slab(T, l + 1, r, sm);
      ct_restrict(cl, s, r, tid, c.p, c.P * c.plane);
    } else {
      ct_restrict(cl, s, r, tid, g0r + (s.z0 / 2) * gplane, gcells);
    }
  }
  if (r == 0) tail_cta_vcycle(T.G, sm, tid, pre, post, coarse);
  cl.sync();
  for (int l = T.nd - 1; l >= 0; --l) {
    const DSlab s = make_slab(T, l, r, sm);
    CSrc src;
    if (l + 1 < T.nd) {
      const DSlab c = make_slab(T, l + 1, r, sm);
      src = CSrc{c.p, c.z0, c.P, c.plane, true};
    } else {
      src = CSrc{g0r, 0, T.G.nz[0], gplane, false};
    }
    ct_prolong(cl, s, src, r, tid);
    ct_smooth(cl, s, r, tid, post, T.G.omega);
  }
  {  // the first tail level's p back to global memory (the next prolongation reads it)
    const DSlab s = make_slab(T, 0, r, sm);
    const int n = s.P * s.plane;
    const size_t g0 = (size_t)s.z0 * s.plane;
    if (vec) {
      float4* gp = reinterpret_cast<float4*>(T.gp + g0);
      for (int t = tid; t < n / 4; t += TAIL_THREADS) gp[t] = reinterpret_cast<const float4*>(s.p)[t];
    } else {
      for (int t = tid; t < n; t += TAIL_THREADS) T.gp[g0 + t] = s.p[t];
    }
  }
}

__global__ void __launch_bounds__(TAIL_THREADS, 1) k_tail(TailLevels T, int pre, int post, int coarse, int* err) {
  tail_body(T, pre, post, coarse, err);
}
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_ctail(CTailLevels T, int pre, int post, int coarse) { ctail_body(T, pre, post, coarse); }
// Batched tails: CTA b (single-CTA form) or cluster b (cluster form) runs the tail of simulation b.
// Each simulation's coarsest sweeps come from its descriptor.
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_tail_b(const TailLevels* __restrict__ T, int pre, int post, int* err) {
  tail_body(T[blockIdx.x], pre, post, T[blockIdx.x].coarse, err);
}
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_ctail_b(const CTailLevels* __restrict__ T, int pre, int post) {
  const CTailLevels& t = T[blockIdx.x / CTAIL_CLUSTER];
  ctail_body(t, pre, post, t.G.coarse);
}

// ---------------- residual norms ||b - A p||^2 and ||b||^2 (FP64 above the thread, fixed order) ----------------
constexpr int RB = GX * GY * GZ;
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// One partial pair per CTA (3D grid over the level, RZ planes per thread); the CTA index is its slot.
// The per-cell residual and its square are FP32; each thread's RZ-cell sum and every reduction above the
// thread accumulate in double-float (df64, fire_device.cuh) in a fixed order, so the result is
// deterministic and carries ~48 bits without FP64 instructions.  Partials: float4 (rr.hi, rr.lo, bb.hi, bb.lo).
constexpr int RZ = 8;
// The residual-driven loop's prediction of the first cycle a step tests, kept in counter slot 3 (the solve's
// only state between steps, so checkpoints and the adjoint's recomputation carry it): bits 0-7 the cycle,
// bits 8-15 the steps left until the next probe (a step that tests one cycle earlier than the last step
// needed, to find a falling need), bits 16-23 the probe interval, bit 24 set while a probe step runs.  After
// a probe that succeeds (the need fell) the next step probes again, and so does every step until one fails;
// a failed probe doubles the interval, up to MG_PROBE_MAX steps.  The next step also probes at once after a step whose need rose (a burst or a moved
// log often raises it for a single step) or whose final residual lies MG_PREDICT_RHO below the tolerance
// (one cycle fewer would have reached it if a cycle reduces the residual at least that much).
constexpr double MG_PREDICT_RHO = 0.3;
constexpr int MG_PROBE_MAX = 8;
__device__ __forceinline__ int mg_first_test(int slot3) { return slot3 & 0xff; }
// Sums of r^2 and b^2 over planes z0 .. z0+RZ-1 of column (x, y), r = b - A p with the ghost rules of
// pghost.  The column is marched in z with the z neighbours carried in registers; the x/y face tests are
// per column, so a cell costs 6 loads and a handful of selects.
__device__ __forceinline__ void residual_column(const float* __restrict__ p, const float* __restrict__ b, int x, int y, int z0, int nx,
                                                int ny, int nz, float ih2, float& rr, float& bb) {
  const int sy = nx, sz = nx * ny;
  const bool hxm = x > 0, hxp = x < nx - 1, hym = y > 0, hyp = y < ny - 1;
  int t = x + sy * y + sz * z0;
  float prev = z0 > 0 ? __ldg(p + t - sz) : 0.0f;
  float cur = __ldg(p + t);
#pragma unroll
  for (int k = 0; k < RZ; ++k) {
    const int z = z0 + k;
    if (z < nz) {
      const bool hzp = z + 1 < nz;
      const float next = hzp ? __ldg(p + t + sz) : 0.0f;
      const float me = cur;
      const float xm = hxm ? __ldg(p + t - 1) : -me, xp = hxp ? __ldg(p + t + 1) : -me;
      const float ym = hym ? __ldg(p + t - sy) : me, yp = hyp ? __ldg(p + t + sy) : -me;
      const float zm = z > 0 ? prev : -me, zp = hzp ? next : -me;
      const float lap = (xm + xp + ym + yp + zm + zp - 6.0f * me) * ih2;
      const float bv = __ldg(b + t);
      const float res = bv - lap;
      rr += res * res;
      bb += bv * bv;
      prev = cur;
      cur = next;
      t += sz;
    }
  }
}
// gate (residual-driven loop only, else null): the loop's counters; the norm is skipped while the cycle
// about to complete (gate[0] + 1) is below the first cycle at which this step tests convergence (gate[3]).
__global__ void __launch_bounds__(RB) k_residual(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                 float ih2, float4* __restrict__ partials, const int* __restrict__ gate) {
  __shared__ df64 sr[RB / 32], sb[RB / 32];
  pdl_wait();
  pdl_trigger();
  if (gate && gate[0] + 1 < mg_first_test(gate[3])) return;   // uniform over the grid
  const int x = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int z0 = (blockIdx.z * GZ + threadIdx.z) * RZ;
  const int tid = threadIdx.x + GX * (threadIdx.y + GY * threadIdx.z);
  float rrf = 0.0f, bbf = 0.0f;   // this thread's RZ cells in FP32, widened to df64 once below
  if (x < nx && y < ny && z0 < nz) residual_column(p, b, x, y, z0, nx, ny, nz, ih2, rrf, bbf);
  df64 rr = df_warp_sum(df_make(rrf));
  df64 bb = df_warp_sum(df_make(bbf));
  if ((tid & 31) == 0) { sr[tid >> 5] = rr; sb[tid >> 5] = bb; }
  __syncthreads();
  if (tid < 32) {
    rr = tid < RB / 32 ? sr[tid] : df_make(0.0f);
    bb = tid < RB / 32 ? sb[tid] : df_make(0.0f);
    rr = df_warp_sum(rr);
    bb = df_warp_sum(bb);
    if (tid == 0) partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = make_float4(rr.hi, rr.lo, bb.hi, bb.lo);
  }
}
// out2 = (||r||^2, ||b||^2) as doubles.
__global__ void __launch_bounds__(RB) k_sum_pairs(const float4* __restrict__ partials, int count, double* __restrict__ out2) {
  __shared__ df64 sa[SUMV / 32], sb[SUMV / 32];
  pdl_wait();
  pdl_trigger();
  df64 a, b;
  sum_pairs_fixed<RB>(partials, count, threadIdx.x, sa, sb, a, b);
  if (threadIdx.x == 0) { out2[0] = df_to_double(a); out2[1] = df_to_double(b); }
}
// The residual-driven loop's test after k_residual: sums the partials with sum_pairs_fixed (so the norm
// equals k_residual + k_sum_pairs bit for bit), counts the cycle and sets the WHILE node's condition: loop
// again while the relative residual is above `tol` and fewer than `max_cycles` cycles have run.
__global__ void __launch_bounds__(RB) k_sum_decide(const float4* __restrict__ partials, int count, double* __restrict__ sums2,
                                                   double tol, int max_cycles, int* __restrict__ counter,
                                                   double* __restrict__ rel_out, cudaGraphConditionalHandle h) {
  __shared__ df64 sa[SUMV / 32], sb[SUMV / 32];
  __shared__ int skip;
  pdl_wait();
  pdl_trigger();
  // Cycles before the predicted first test run without a convergence test (each skipped test saves the norm's
  // pass over level 0 and the sum); the solve still stops only on a tested residual <= tol (or at max_cycles).
  // The prediction is set when a step stops (below) from the cycle count it needed and its final residual.
  if (threadIdx.x == 0) {
    const int c = counter[0] + 1;
    skip = c < mg_first_test(counter[3]);
    if (skip) {
      counter[0] = c;
      counter[1] += 1;   // cumulative cycles since creation
      cudaGraphSetConditional(h, 1u);
    }
  }
  __syncthreads();
  if (skip) return;
  df64 A, B;
  sum_pairs_fixed<RB>(partials, count, threadIdx.x, sa, sb, A, B);
  if (threadIdx.x == 0) {
    const double s0 = df_to_double(A), s1 = df_to_double(B);
    sums2[0] = s0;
    sums2[1] = s1;
    const int c = counter[0] + 1;
    counter[0] = c;
    counter[1] += 1;
    const double rel = s1 > 0.0 ? sqrt(s0 / s1) : 0.0;
    rel_out[0] = rel;
    const bool more = rel > tol && c < max_cycles;
    // The next step tests first at this step's count c, or at c - 1 (a probe) when one cycle fewer could
    // have reached the tolerance (rel <= MG_PREDICT_RHO * tol) or the probe interval has run out.  A step
    // whose need fell runs at most one cycle more than it needs until the next probe.
    if (!more) {
      const int slot = counter[3], first = mg_first_test(slot);
      const bool probed = (slot & (1 << 24)) != 0;
      const bool fell = probed && c == first;   // the probe's earlier test passed
      int left = (slot >> 8) & 0xff, every = (slot >> 16) & 0xff;
      if (probed) every = fell ? 1 : min(max(2 * every, 1), MG_PROBE_MAX);
      const bool rose = c > first + (probed ? 1 : 0);
      const bool probe = fell || rose || rel <= MG_PREDICT_RHO * tol || left <= 0;
      left = probe ? max(every, 1) - 1 : left - 1;
      counter[3] = min(max(1, probe ? c - 1 : c), max_cycles - 1) | (left << 8) | (every << 16) | (probe ? 1 << 24 : 0);
    }
    cudaGraphSetConditional(h, more ? 1u : 0u);
  }
}

// ---------------- launchers ----------------
static dim3 grid3(int x, int y, int z) { return dim3((x + GX - 1) / GX, (y + GY - 1) / GY, (z + GZ - 1) / GZ); }
static const dim3 kBlock(GX, GY, GZ);

// A level whose SMZ-cell grid fits in one wave (8 resident CTAs of 256 threads on each of the 152 SMs) runs
// one cell per thread instead: twice the CTAs, the same bits (a colour's cells never read each other).
// Measured at 128x256x128 (levels 1 and 2 switch): 10 us less solve per step.
constexpr unsigned SMOOTH1_CTAS = 1216;
cudaError_t launch_smooth(const MGLevel& L, int color, cudaStream_t st) {
  const dim3 g = grid3((L.nx + 1) >> 1, L.ny, (L.nz + SMZ - 1) / SMZ);
  if (!L.study && g.x * g.y * g.z < SMOOTH1_CTAS)
    return launch_pdl(k_smooth1, grid3((L.nx + 1) >> 1, L.ny, L.nz), kBlock, 0, st, L.p, (const float*)L.b, L.nx, L.ny, L.nz, L.h, color,
                      L.omega);
  return launch_pdl(L.study ? k_smooth_study : k_smooth, g, kBlock, 0, st, L.p, (const float*)L.b, L.nx, L.ny, L.nz, L.h, color, L.omega);
}
cudaError_t launch_restrict(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  return launch_pdl(k_restrict, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (const float*)F.p, (const float*)F.b, F.nx, F.ny, F.nz, F.h, C.b, C.p);
}
cudaError_t launch_restrict_smooth(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  if (C.study) return cudaErrorInvalidValue;   // the studies' smoother has its own update; not fused
  return launch_pdl(C.omega == 1.0f ? k_restrict_smooth<false> : k_restrict_smooth<true>, grid3(C.nx, C.ny, C.nz), kBlock, 0, st,
                    (const float*)F.p, (const float*)F.b, F.nx, F.ny, F.nz, F.h, C.b, C.p, C.h, C.omega);
}
cudaError_t launch_prolong(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  return launch_pdl(F.study ? k_prolong_clamp : k_prolong, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, F.p, (const float*)C.p, F.nx, F.ny, F.nz);
}
// Number of leading levels of [first, n) that the cluster tail distributes: each has z-planes for an even
// number per CTA, at least CTAIL_MIN_CELLS cells per CTA, and a coarser level below it.
static int tail_dist_levels(const MGLevel* levels, int first, int n) {
  if (CTAIL_CLUSTER < 2 || (first < n && levels[first].study)) return 0;   // the studies' variant runs single-CTA tails only
  int d = 0;
  for (int l = first; l < n - 1 && d < TAIL_MAX_LEVELS; ++l) {
    const MGLevel& L = levels[l];
    const long cells = (long)L.nx * L.ny * L.nz;
    if (L.nz % (2 * CTAIL_CLUSTER) != 0 || cells < (long)CTAIL_CLUSTER * CTAIL_MIN_CELLS) break;
    ++d;
  }
  return d;
}
// Floats after the tail levels' p/b arrays where the FP64 copy of the coarsest level starts (8-byte aligned).
static size_t tail_fp64_offset(size_t floats) { return (floats + 1) & ~(size_t)1; }
size_t tail_smem_bytes(const MGLevel* levels, int first, int n, bool coarse64) {
  const int nd = tail_dist_levels(levels, first, n);
  size_t floats = 0;
  for (int l = first; l < n; ++l) {
    const size_t cells = (size_t)levels[l].nx * levels[l].ny * levels[l].nz;
    floats += 2 * (l < first + nd ? cells / CTAIL_CLUSTER : cells);
  }
  if (coarse64)   // the FP64 copy of the coarsest level (sweeps) or the direct solve's row partials
    floats = tail_fp64_offset(floats) +
             std::max<size_t>(4 * (size_t)levels[n - 1].nx * levels[n - 1].ny * levels[n - 1].nz, 2 * (size_t)TAIL_THREADS);
  return floats * sizeof(float);
}
bool tail_fits(const MGLevel* levels, int first, int n, bool coarse64) {
  return first >= 0 && first < n && n - first - tail_dist_levels(levels, first, n) <= TAIL_MAX_LEVELS &&
         tail_smem_bytes(levels, first, n, coarse64) <= TAIL_SMEM_BUDGET;
}
// Where the tail starts, from measurements in CUDA graphs on GB300 (us per V-cycle for the coarse end):
//   128x256x128: tail from 32x64x32 (cluster) 57.4 | 32x64x32 as 10 launches + tail from 16x32x16 (cluster)
//   20.6 + 30.8 = 51.4 | two levels as launches + tail from 8x16x8 (single CTA) 20.6 + 20.6 + 16.5 = 57.7;
//   the same ordering at 64x128x64 and 256x512x256.  A level of more than TAIL_FIRST_CELLS (8192) cells is cheaper
//   as its own launches than inside the tail, so a simulation's tail starts at the finest level that fits and
//   is no larger than that.  An ensemble runs its members' tails side by side in one launch, which hides a
//   larger tail's latency, so it lets the tail start at the finest level that fits.
int tail_first(const MGLevel* levels, int n, bool coarse64, long max_cells) {
  int first = n;
  for (int l = n - 1; l >= 0 && tail_fits(levels, l, n, coarse64) && (long)levels[l].nx * levels[l].ny * levels[l].nz <= max_cells; --l)
    first = l;
  return first;
}
// Levels [first, n) as a TailLevels block whose first level's p starts `off` floats into shared memory.
static TailLevels make_tail_levels(const MGLevel* levels, int first, int n, int off, bool coarse64, const double* cinv) {
  TailLevels T;
  T.n = n - first;
  T.small = T.n;
  for (int l = 0; l < T.n; ++l) {
    const MGLevel& L = levels[first + l];
    T.nx[l] = L.nx; T.ny[l] = L.ny; T.nz[l] = L.nz; T.h[l] = L.h;
    T.off[l] = off;
    off += 2 * L.nx * L.ny * L.nz;
    T.gp[l] = L.p; T.gb[l] = L.b;
    if (T.small == T.n && L.nx * L.ny * L.nz <= TAIL_WARP_CELLS) T.small = l;
  }
  T.coarse = 0;
  T.omega = T.n > 0 ? levels[first].omega : 1.0f;
  T.study = T.n > 0 ? levels[first].study : 0;
  T.wait_polls = TAIL_WAIT_POLLS;
  T.coarse64 = coarse64 ? 1 : 0;
  T.doff = (int)tail_fp64_offset((size_t)off);
  T.cinv = coarse64 ? cinv : nullptr;
  return T;
}
// The cluster tail's descriptor: the first nd levels distributed, the rest gathered on CTA 0.
static CTailLevels make_ctail_levels(const MGLevel* levels, int first, int n, int nd, bool coarse64, const double* cinv) {
  CTailLevels T;
  T.nd = nd;
  int off = 0;
  for (int l = 0; l < nd; ++l) {
    const MGLevel& L = levels[first + l];
    T.nx[l] = L.nx; T.ny[l] = L.ny; T.nz[l] = L.nz; T.h[l] = L.h;
    T.P[l] = L.nz / CTAIL_CLUSTER;
    T.off[l] = off;
    off += 2 * L.nx * L.ny * T.P[l];
  }
  T.gp = levels[first].p;
  T.gb = levels[first].b;
  T.G = make_tail_levels(levels, first + nd, n, off, coarse64, cinv);
  return T;
}
cudaError_t launch_tail(const MGLevel* levels, int first, int n, int pre, int post, int coarse, int* err, cudaStream_t st, bool coarse64,
                        const double* cinv, int wait_polls) {
  const size_t smem = tail_smem_bytes(levels, first, n, coarse64);
  const int nd = tail_dist_levels(levels, first, n);
  if (nd == 0) {
    TailLevels T = make_tail_levels(levels, first, n, 0, coarse64, cinv);
    T.wait_polls = wait_polls;
    return launch_pdl(k_tail, dim3(1), dim3(TAIL_THREADS), smem, st, T, pre, post, coarse, err);
  }
  const CTailLevels T = make_ctail_levels(levels, first, n, nd, coarse64, cinv);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CTAIL_CLUSTER);
  cfg.blockDim = dim3(TAIL_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CTAIL_CLUSTER;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_ctail, T, pre, post, coarse);
}
cudaError_t mg_configure(size_t max_tail_smem) {
  for (const void* k : {(const void*)k_tail, (const void*)k_ctail, (const void*)k_tail_b, (const void*)k_ctail_b}) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_tail_smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
dim3 smooth_grid(const MGLevel& L) { return grid3((L.nx + 1) >> 1, L.ny, (L.nz + SMZ - 1) / SMZ); }
dim3 coarse_grid(const MGLevel& C) { return grid3(C.nx, C.ny, C.nz); }
void launch_smooth_batch(const BatchMap& m, const LevelBatch& L, int color, cudaStream_t st) {
  launch_pdl(k_smooth_b, dim3(m.prefix[m.n]), kBlock, 0, st, m, L, color);
}
void launch_restrict_batch(const BatchMap& m, const LevelBatch& F, const LevelBatch& C, cudaStream_t st) {
  launch_pdl(k_restrict_b, dim3(m.prefix[m.n]), kBlock, 0, st, m, F, C);
}
void launch_prolong_batch(const BatchMap& m, const LevelBatch& F, const LevelBatch& C, cudaStream_t st) {
  launch_pdl(k_prolong_b, dim3(m.prefix[m.n]), kBlock, 0, st, m, F, C);
}
int tail_kind(const MGLevel* levels, int first, int n) { return tail_dist_levels(levels, first, n) > 0 ? 1 : 0; }
size_t tail_desc_size(int kind) { return kind ? sizeof(CTailLevels) : sizeof(TailLevels); }
void tail_desc_fill(const MGLevel* levels, int first, int n, int coarse, void* out) {
  const int nd = tail_dist_levels(levels, first, n);
  if (nd == 0) {
    TailLevels T = make_tail_levels(levels, first, n, 0, false, nullptr);
    T.coarse = coarse;
    std::memcpy(out, &T, sizeof T);
  } else {
    CTailLevels T = make_ctail_levels(levels, first, n, nd, false, nullptr);
    T.G.coarse = coarse;
    std::memcpy(out, &T, sizeof T);
  }
}
void launch_tail_batch(int kind, const void* dev_descs, int count, size_t smem, int pre, int post, int* err, cudaStream_t st) {
  if (count <= 0) return;
  if (kind == 0) {
    launch_pdl(k_tail_b, dim3(count), dim3(TAIL_THREADS), smem, st, (const TailLevels*)dev_descs, pre, post, err);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CTAIL_CLUSTER * count);
  cfg.blockDim = dim3(TAIL_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CTAIL_CLUSTER;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k_ctail_b, (const CTailLevels*)dev_descs, pre, post);
}
static dim3 residual_grid(const MGLevel& L) { return grid3(L.nx, L.ny, (L.nz + RZ - 1) / RZ); }
int residual_partials_count(const MGLevel& L) {
  dim3 g = residual_grid(L);
  return (int)(g.x * g.y * g.z);
}
void launch_residual(const MGLevel& L, double* partials, double* out2, cudaStream_t st) {
  float4* part4 = reinterpret_cast<float4*>(partials);   // 16 bytes per CTA (the buffer holds 128 per CTA)
  launch_pdl(k_residual, residual_grid(L), kBlock, 0, st, (const float*)L.p, (const float*)L.b, L.nx, L.ny, L.nz,
             1.0f / (L.h * L.h), part4, (const int*)nullptr);
  launch_pdl(k_sum_pairs, dim3(1), dim3(RB), 0, st, (const float4*)part4, residual_partials_count(L), out2);
}
void launch_residual_decide(const MGLevel& L, double* partials, double* sums2, double tol, int max_cycles, int* counter,
                            double* rel_out, cudaGraphConditionalHandle h, cudaStream_t st) {
  float4* part4 = reinterpret_cast<float4*>(partials);
  launch_pdl(k_residual, residual_grid(L), kBlock, 0, st, (const float*)L.p, (const float*)L.b, L.nx, L.ny, L.nz,
             1.0f / (L.h * L.h), part4, (const int*)counter);
  launch_pdl(k_sum_decide, dim3(1), dim3(RB), 0, st, (const float4*)part4, residual_partials_count(L), sums2, tol, max_cycles,
             counter, rel_out, h);
}
// Clears the per-step cycle count before a residual-driven solve that no clearing divergence kernel precedes.
__global__ void k_mg_counter_reset(int* counter) { if (threadIdx.x == 0) counter[0] = 0; }
void launch_mg_counter_reset(int* counter, cudaStream_t st) { k_mg_counter_reset<<<1, 32, 0, st>>>(counter); }

}  // namespace fire

