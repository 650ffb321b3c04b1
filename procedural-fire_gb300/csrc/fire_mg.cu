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
  // smoother at a handful of instructions per cell instead of an IEEE division sequence
  return __fdividef(sum - h2 * b[c], diag);
}
// Each thread updates SMZ cells of one colour, SMZ planes apart in z (unrolled and independent, so their
// loads are in flight together): the sweep is latency-bound on L2 hits, and fewer, longer CTAs also cut the
// CTA turnover that leaves warp slots idle.
#ifndef FIRE_SMOOTH_Z
#define FIRE_SMOOTH_Z 2
#endif
constexpr int SMZ = FIRE_SMOOTH_Z;
__global__ void __launch_bounds__(GX * GY * GZ) k_smooth(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                         float h, int color) {
  pdl_wait();
  pdl_trigger();
  const int gx = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int zb = (blockIdx.z * GZ + threadIdx.z) * SMZ;
  if (y >= ny) return;
  const float h2 = h * h;
  float v[SMZ];
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {   // all reads first (a colour's cells never read each other) ...
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) v[k] = rb_update(p, b, x, y, z, nx, ny, nz, h2);
  }
#pragma unroll
  for (int k = 0; k < SMZ; ++k) {   // ... then the writes
    const int z = zb + k;
    const int x = gx * 2 + ((y + z + color) & 1);
    if (z < nz && x < nx) p[x + nx * (y + ny * z)] = v[k];
  }
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
__global__ void __launch_bounds__(GX * GY * GZ) k_restrict(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                           float h, float* __restrict__ bc, float* __restrict__ pc) {
  pdl_wait();
  pdl_trigger();
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
  if (cx >= cnx || cy >= cny || cz >= cnz) return;
  const float ih2 = 1.0f / (h * h);
  const int t = cx + cnx * (cy + cny * cz);
  bc[t] = restrict_cell(p, b, cx, cy, cz, nx, ny, nz, ih2);
  pc[t] = 0.0f;
}

// ---------------- prolongation with mirror ghosts (src/sim.js:468-495) ----------------
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
    // odd mirror (Dirichlet) on sides/top, even (Neumann) at the floor; one flip per axis outside
    if (qx < 0 || qx >= ncx) val = -val;
    if (qz < 0 || qz >= ncz) val = -val;
    if (qy >= ncy) val = -val;
    const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy, wz = oz ? fz : 1.0f - fz;
    acc += val * wx * wy * wz;
  }
  return acc;
}
// One thread per coarse cell: the 3x3x3 coarse neighbourhood (with the mirror signs of prolong_cell) is
// loaded once and the 8 fine children are formed from it.  For fine index c = 2 cc + d the trilinear base is
// g0 = cc - 1 + d with fraction 0.75 (d = 0) or 0.25 (d = 1), so child d reads coarse offsets d-1 and d;
// each child's sum runs in prolong_cell's order, so the result is identical.
__global__ void __launch_bounds__(GX * GY * GZ) k_prolong(float* __restrict__ p, const float* __restrict__ pc, int nx, int ny, int nz) {
  pdl_wait();
  pdl_trigger();
  const int ncx = nx / 2, ncy = ny / 2, ncz = nz / 2;
  const int cx = blockIdx.x * GX + threadIdx.x, cy = blockIdx.y * GY + threadIdx.y, cz = blockIdx.z * GZ + threadIdx.z;
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
        const int t = (2 * cx + dx) + nx * ((2 * cy + dy) + ny * (2 * cz + dz));
        p[t] = p[t] + acc;
      }
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
template <bool kWarp>
__device__ void tail_smooth(const Team<kWarp>& tm, float* p, const float* b, int nx, int ny, int nz, float h, int iters) {
  const int hx = (nx + 1) >> 1;
  const float h2 = h * h;
  const Box3 bx(tm.size, tm.rank, hx, ny, nz);
  for (int it = 0; it < iters; ++it)
    for (int color = 0; color < 2; ++color) {
      for (int z = bx.z0; z < nz; z += bx.tz)
        for (int y = bx.y0; y < ny; y += bx.ty)
          for (int gx = bx.x0; gx < hx; gx += bx.tx) {
            const int x = gx * 2 + ((y + z + color) & 1);
            if (x < nx) p[x + nx * (y + ny * z)] = rb_update(p, b, x, y, z, nx, ny, nz, h2);
          }
      tm.sync();
    }
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
        p[t] = p[t] + prolong_cell(pc, x, y, z, nx / 2, ny / 2, nz / 2);
      }
  tm.sync();
}
// V-cycle over tail levels [from, n) with one team (src/sim.js:588-599 restricted to these levels).
template <bool kWarp>
__device__ void tail_vcycle(const Team<kWarp>& tm, const TailLevels& T, float* sm, int from, int pre, int post, int coarse) {
  const int n = T.n;
  for (int l = from; l < n - 1; ++l) {
    float* p = sm + T.off[l];
    tail_smooth(tm, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre);
    tail_restrict(tm, T, sm, l);
  }
  {
    float* p = sm + T.off[n - 1];
    tail_smooth(tm, p, p + T.nx[n - 1] * T.ny[n - 1] * T.nz[n - 1], T.nx[n - 1], T.ny[n - 1], T.nz[n - 1], T.h[n - 1], coarse);
  }
  for (int l = n - 2; l >= from; --l) {
    tail_prolong(tm, T, sm, l);
    float* p = sm + T.off[l];
    tail_smooth(tm, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post);
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
// Waits for phase 0 of the barrier with an iteration limit; returns false if the limit was reached.
__device__ __forceinline__ bool mbar_wait0(uint64_t* bar) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(smem_addr(bar)), "r"(0u) : "memory");
    if (done) return true;
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

__global__ void __launch_bounds__(TAIL_THREADS, 1) k_tail(TailLevels T, int pre, int post, int coarse, int* err) {
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
      if (!mbar_wait0(&bar)) {                // bounded wait: report and leave instead of hanging
        if (tid == 0) atomicExch(err, 1);
        return;
      }
    } else {
      for (int t = tid; t < n0; t += TAIL_THREADS) { p[t] = T.gp[0][t]; b[t] = T.gb[0][t]; }
    }
    __syncthreads();
  }
  const Team<false> cta{tid};
  const int S = T.small;
  if (S == 0) {
    if (tid < 32) tail_vcycle(Team<true>{tid}, T, sm, 0, pre, post, coarse);
    __syncthreads();
  } else if (S >= T.n) {
    tail_vcycle(cta, T, sm, 0, pre, post, coarse);
  } else {
    // large levels [0, S) with the whole CTA; the V-cycle below S (levels S..n-1) on warp 0
    for (int l = 0; l < S; ++l) {
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], pre);
      tail_restrict(cta, T, sm, l);
    }
    if (tid < 32) tail_vcycle(Team<true>{tid}, T, sm, S, pre, post, coarse);
    __syncthreads();
    for (int l = S - 1; l >= 0; --l) {
      tail_prolong(cta, T, sm, l);
      float* p = sm + T.off[l];
      tail_smooth(cta, p, p + T.nx[l] * T.ny[l] * T.nz[l], T.nx[l], T.ny[l], T.nz[l], T.h[l], post);
    }
  }
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
constexpr int RZ = 4;
__global__ void __launch_bounds__(RB) k_residual(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                 float ih2, float4* __restrict__ partials) {
  __shared__ df64 sr[RB / 32], sb[RB / 32];
  pdl_wait();
  pdl_trigger();
  const int x = blockIdx.x * GX + threadIdx.x, y = blockIdx.y * GY + threadIdx.y;
  const int tid = threadIdx.x + GX * (threadIdx.y + GY * threadIdx.z);
  float rrf = 0.0f, bbf = 0.0f;   // this thread's RZ cells in FP32, widened to df64 once below
  if (x < nx && y < ny) {
#pragma unroll
    for (int k = 0; k < RZ; ++k) {   // unrolled without early exit: all RZ cells' loads are in flight together
      const int z = (blockIdx.z * GZ + threadIdx.z) * RZ + k;
      if (z >= nz) continue;
      const int t = x + nx * (y + ny * z);
      const float me = __ldg(p + t);
      const float lap = (pghost(p, x - 1, y, z, nx, ny, nz, me) + pghost(p, x + 1, y, z, nx, ny, nz, me) +
                         pghost(p, x, y - 1, z, nx, ny, nz, me) + pghost(p, x, y + 1, z, nx, ny, nz, me) +
                         pghost(p, x, y, z - 1, nx, ny, nz, me) + pghost(p, x, y, z + 1, nx, ny, nz, me) - 6.0f * me) * ih2;
      const float bv = __ldg(b + t);
      const float res = bv - lap;
      rrf += res * res;
      bbf += bv * bv;
    }
  }
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
// Sums `count` partial pairs in a fixed order (thread t takes t, t+1024, ...; then a fixed tree), in df64;
// out2 = (||r||^2, ||b||^2) as doubles.
constexpr int SUMT = 1024;
__global__ void __launch_bounds__(SUMT) k_sum_pairs(const float4* __restrict__ partials, int count, double* __restrict__ out2) {
  __shared__ df64 sa[SUMT / 32], sb[SUMT / 32];
  pdl_wait();
  pdl_trigger();
  df64 a = df_make(0.0f), b = df_make(0.0f);
  for (int i = threadIdx.x; i < count; i += SUMT) {
    const float4 q = partials[i];
    a = df_add(a, df64{q.x, q.y});
    b = df_add(b, df64{q.z, q.w});
  }
  a = df_warp_sum(a);
  b = df_warp_sum(b);
  if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
  __syncthreads();
  if (threadIdx.x < 32) {
    a = df_warp_sum(sa[threadIdx.x]);
    b = df_warp_sum(sb[threadIdx.x]);
    if (threadIdx.x == 0) { out2[0] = df_to_double(a); out2[1] = df_to_double(b); }
  }
}

// ---------------- launchers ----------------
static dim3 grid3(int x, int y, int z) { return dim3((x + GX - 1) / GX, (y + GY - 1) / GY, (z + GZ - 1) / GZ); }
static const dim3 kBlock(GX, GY, GZ);

void launch_smooth(const MGLevel& L, int color, cudaStream_t st) {
  launch_pdl(k_smooth, grid3((L.nx + 1) >> 1, L.ny, (L.nz + SMZ - 1) / SMZ), kBlock, 0, st, L.p, (const float*)L.b, L.nx, L.ny,
             L.nz, L.h, color);
}
void launch_restrict(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  launch_pdl(k_restrict, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, (const float*)F.p, (const float*)F.b, F.nx, F.ny, F.nz, F.h, C.b, C.p);
}
void launch_prolong(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  launch_pdl(k_prolong, grid3(C.nx, C.ny, C.nz), kBlock, 0, st, F.p, (const float*)C.p, F.nx, F.ny, F.nz);
}
size_t tail_smem_bytes(const MGLevel* levels, int first, int n) {
  size_t cells = 0;
  for (int l = first; l < n; ++l) cells += (size_t)levels[l].nx * levels[l].ny * levels[l].nz;
  return cells * 2 * sizeof(float);
}
void launch_tail(const MGLevel* levels, int first, int n, int pre, int post, int coarse, int* err, cudaStream_t st) {
  TailLevels T;
  T.n = n - first;
  T.small = T.n;
  int off = 0;
  for (int l = 0; l < T.n; ++l) {
    const MGLevel& L = levels[first + l];
    T.nx[l] = L.nx; T.ny[l] = L.ny; T.nz[l] = L.nz; T.h[l] = L.h;
    T.off[l] = off;
    off += 2 * L.nx * L.ny * L.nz;
    T.gp[l] = L.p; T.gb[l] = L.b;
    if (T.small == T.n && L.nx * L.ny * L.nz <= TAIL_WARP_CELLS) T.small = l;
  }
  launch_pdl(k_tail, dim3(1), dim3(TAIL_THREADS), (size_t)off * sizeof(float), st, T, pre, post, coarse, err);
}
cudaError_t mg_configure(size_t max_tail_smem) {
  return cudaFuncSetAttribute(k_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_tail_smem);
}
static dim3 residual_grid(const MGLevel& L) { return grid3(L.nx, L.ny, (L.nz + RZ - 1) / RZ); }
int residual_partials_count(const MGLevel& L) {
  dim3 g = residual_grid(L);
  return (int)(g.x * g.y * g.z);
}
void launch_residual(const MGLevel& L, double* partials, double* out2, cudaStream_t st) {
  float4* part4 = reinterpret_cast<float4*>(partials);   // 16 bytes per CTA (the buffer holds 128 per CTA)
  launch_pdl(k_residual, residual_grid(L), kBlock, 0, st, (const float*)L.p, (const float*)L.b, L.nx, L.ny, L.nz,
             1.0f / (L.h * L.h), part4);
  launch_pdl(k_sum_pairs, dim3(1), dim3(SUMT), 0, st, (const float4*)part4, residual_partials_count(L), out2);
}

}  // namespace fire

// ---------------- residual-driven loop control (conditional WHILE node body tail) ----------------
namespace fire {
// sums2 = (||r||^2, ||b||^2) of level 0 after the cycle just run.  Keeps looping while the relative
// residual is above `tol` and fewer than `max_cycles` cycles have run.
__global__ void k_mg_decide(const double* __restrict__ sums2, double tol, int max_cycles, int* __restrict__ counter,
                            double* __restrict__ rel_out, cudaGraphConditionalHandle h) {
  pdl_wait();
  if (threadIdx.x != 0) return;
  const int c = counter[0] + 1;
  counter[0] = c;
  counter[1] += 1;   // cumulative cycles since creation
  const double rel = sums2[1] > 0.0 ? sqrt(sums2[0] / sums2[1]) : 0.0;
  rel_out[0] = rel;
  cudaGraphSetConditional(h, (rel > tol && c < max_cycles) ? 1u : 0u);
}
__global__ void k_mg_counter_reset(int* counter) { if (threadIdx.x == 0) counter[0] = 0; }
void launch_mg_decide(const double* sums2, double tol, int max_cycles, int* counter, double* rel_out,
                      cudaGraphConditionalHandle h, cudaStream_t st) {
  launch_pdl(k_mg_decide, dim3(1), dim3(32), 0, st, sums2, tol, max_cycles, counter, rel_out, h);
}
void launch_mg_counter_reset(int* counter, cudaStream_t st) { k_mg_counter_reset<<<1, 32, 0, st>>>(counter); }
}  // namespace fire
