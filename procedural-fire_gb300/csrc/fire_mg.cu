// Geometric multigrid for the pressure Poisson equation (src/sim.js:415-495, 576-599).
//
// Cell-centred 7-point Laplacian, open sides and top (p = 0 on the boundary face: ghost = -p),
// solid floor (Neumann: ghost = p).  Level l has spacing h = dx * 2^l; the equation per level is
// sum_nb(p) - 6 p = h^2 b with the ghost rules folded into the diagonal of the red-black Gauss-Seidel
// update, exactly as mgSmooth does.
//
// GB300 mapping: the fine levels run as one launch per colour sweep (the grid is large enough to fill
// 152 SMs); every level small enough to fit, with all coarser ones, in one CTA's shared memory is
// solved by a single-CTA kernel that runs the rest of the V-cycle (smoothing, restriction, the coarse
// sweeps and prolongation) out of shared memory with __syncthreads between colours.  At 128x256x128
// this replaces the 3 coarsest levels' ~40 launches per cycle with one.
#include "fire_device.cuh"

namespace fire {

constexpr int MB = 256;

// ---------------- red-black Gauss-Seidel sweep, one colour (src/sim.js:417-437) ----------------
__device__ __forceinline__ float rb_update(const float* p, const float* b, int x, int y, int z, int nx, int ny, int nz, float h2) {
  const size_t c = (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z);
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  float sum = 0.0f, diag = 6.0f;
  if (x > 0) sum += p[c - 1]; else diag += 1.0f;
  if (x < nx - 1) sum += p[c + 1]; else diag += 1.0f;
  if (z > 0) sum += p[c - sz]; else diag += 1.0f;
  if (z < nz - 1) sum += p[c + sz]; else diag += 1.0f;
  if (y > 0) sum += p[c - sy]; else diag -= 1.0f;
  if (y < ny - 1) sum += p[c + sy]; else diag += 1.0f;
  return (sum - h2 * b[c]) / diag;
}
__global__ void __launch_bounds__(MB) k_smooth(float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                               float h, int color) {
  const int hx = (nx + 1) >> 1;
  const long long t = (long long)blockIdx.x * MB + threadIdx.x;
  const long long total = (long long)hx * ny * nz;
  if (t >= total) return;
  const int gx = (int)(t % hx);
  const long long r = t / hx;
  const int y = (int)(r % ny), z = (int)(r / ny);
  const int x = gx * 2 + ((y + z + color) & 1);
  if (x >= nx) return;
  p[(size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z)] = rb_update(p, b, x, y, z, nx, ny, nz, h * h);
}

// ---------------- fused residual + restriction (src/sim.js:439-466) ----------------
__device__ __forceinline__ float pghost(const float* p, int x, int y, int z, int nx, int ny, int nz, float me) {
  if (x < 0 || z < 0 || x >= nx || z >= nz || y >= ny) return -me;
  if (y < 0) return me;
  return p[(size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z)];
}
__device__ __forceinline__ float restrict_cell(const float* p, const float* b, int cx, int cy, int cz, int nx, int ny, int nz, float ih2) {
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int x = 2 * cx + (q & 1), y = 2 * cy + ((q >> 1) & 1), z = 2 * cz + ((q >> 2) & 1);
    const float me = p[(size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z)];
    const float lap = (pghost(p, x - 1, y, z, nx, ny, nz, me) + pghost(p, x + 1, y, z, nx, ny, nz, me) +
                       pghost(p, x, y - 1, z, nx, ny, nz, me) + pghost(p, x, y + 1, z, nx, ny, nz, me) +
                       pghost(p, x, y, z - 1, nx, ny, nz, me) + pghost(p, x, y, z + 1, nx, ny, nz, me) - 6.0f * me) * ih2;
    acc += b[(size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z)] - lap;
  }
  return acc * 0.125f;
}
__global__ void __launch_bounds__(MB) k_restrict(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                 float h, float* __restrict__ bc, float* __restrict__ pc) {
  const int cnx = nx / 2, cny = ny / 2, cnz = nz / 2;
  const long long t = (long long)blockIdx.x * MB + threadIdx.x;
  if (t >= (long long)cnx * cny * cnz) return;
  const int cx = (int)(t % cnx);
  const long long r = t / cnx;
  const int cy = (int)(r % cny), cz = (int)(r / cny);
  const float ih2 = 1.0f / (h * h);
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
    float val = pc[(size_t)min(max(qx, 0), ncx - 1) + (size_t)ncx * ((size_t)min(max(qy, 0), ncy - 1) + (size_t)ncy * min(max(qz, 0), ncz - 1))];
    // odd mirror (Dirichlet) on sides/top, even (Neumann) at the floor; one flip per axis outside
    if (qx < 0 || qx >= ncx) val = -val;
    if (qz < 0 || qz >= ncz) val = -val;
    if (qy >= ncy) val = -val;
    const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy, wz = oz ? fz : 1.0f - fz;
    acc += val * wx * wy * wz;
  }
  return acc;
}
__global__ void __launch_bounds__(MB) k_prolong(float* __restrict__ p, const float* __restrict__ pc, int nx, int ny, int nz) {
  const long long t = (long long)blockIdx.x * MB + threadIdx.x;
  if (t >= (long long)nx * ny * nz) return;
  const int x = (int)(t % nx);
  const long long r = t / nx;
  const int y = (int)(r % ny), z = (int)(r / ny);
  p[t] = p[t] + prolong_cell(pc, x, y, z, nx / 2, ny / 2, nz / 2);
}

// ---------------- single-CTA tail V-cycle out of shared memory ----------------
constexpr int TAIL_THREADS = 1024;
constexpr int TAIL_MAX_LEVELS = 12;
struct TailLevels {
  int n;                       // number of levels in the tail
  int nx[TAIL_MAX_LEVELS], ny[TAIL_MAX_LEVELS], nz[TAIL_MAX_LEVELS];
  float h[TAIL_MAX_LEVELS];
  int off[TAIL_MAX_LEVELS];    // float offset of level l's p in shared memory (b follows p)
  float* gp[TAIL_MAX_LEVELS];  // global copies (written back at the end)
  float* gb[TAIL_MAX_LEVELS];
};
__device__ void tail_smooth(float* p, const float* b, int nx, int ny, int nz, float h, int iters) {
  const int hx = (nx + 1) >> 1;
  const int total = hx * ny * nz;
  const float h2 = h * h;
  for (int it = 0; it < iters; ++it)
    for (int color = 0; color < 2; ++color) {
      for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int gx = t % hx, r = t / hx, y = r % ny, z = r / ny;
        const int x = gx * 2 + ((y + z + color) & 1);
        if (x < nx) p[x + nx * (y + ny * z)] = rb_update(p, b, x, y, z, nx, ny, nz, h2);
      }
      __syncthreads();
    }
}
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_tail(TailLevels T, int pre, int post, int coarse) {
  extern __shared__ float sm[];
  // stage the first tail level's p and b (restriction already wrote them)
  {
    const int n0 = T.nx[0] * T.ny[0] * T.nz[0];
    float* p = sm + T.off[0];
    float* b = p + n0;
    for (int t = threadIdx.x; t < n0; t += blockDim.x) { p[t] = T.gp[0][t]; b[t] = T.gb[0][t]; }
    __syncthreads();
  }
  const int n = T.n;
  for (int l = 0; l < n - 1; ++l) {
    const int nl = T.nx[l] * T.ny[l] * T.nz[l];
    float* p = sm + T.off[l];
    float* b = p + nl;
    tail_smooth(p, b, T.nx[l], T.ny[l], T.nz[l], T.h[l], pre);
    const int cnx = T.nx[l + 1], cny = T.ny[l + 1], cnz = T.nz[l + 1];
    const int nc = cnx * cny * cnz;
    float* pc = sm + T.off[l + 1];
    float* bc = pc + nc;
    const float ih2 = 1.0f / (T.h[l] * T.h[l]);
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
      const int cx = t % cnx, r = t / cnx, cy = r % cny, cz = r / cny;
      bc[t] = restrict_cell(p, b, cx, cy, cz, T.nx[l], T.ny[l], T.nz[l], ih2);
      pc[t] = 0.0f;
    }
    __syncthreads();
  }
  {
    const int l = n - 1;
    const int nl = T.nx[l] * T.ny[l] * T.nz[l];
    float* p = sm + T.off[l];
    tail_smooth(p, p + nl, T.nx[l], T.ny[l], T.nz[l], T.h[l], coarse);
  }
  for (int l = n - 2; l >= 0; --l) {
    const int nl = T.nx[l] * T.ny[l] * T.nz[l];
    float* p = sm + T.off[l];
    float* b = p + nl;
    const float* pc = sm + T.off[l + 1];
    const int nx = T.nx[l], ny = T.ny[l], nz = T.nz[l];
    for (int t = threadIdx.x; t < nl; t += blockDim.x) {
      const int x = t % nx, r = t / nx, y = r % ny, z = r / ny;
      p[t] = p[t] + prolong_cell(pc, x, y, z, nx / 2, ny / 2, nz / 2);
    }
    __syncthreads();
    tail_smooth(p, b, nx, ny, nz, T.h[l], post);
  }
  // write every tail level back (level 0 of the tail feeds the next prolongation)
  for (int l = 0; l < n; ++l) {
    const int nl = T.nx[l] * T.ny[l] * T.nz[l];
    const float* p = sm + T.off[l];
    for (int t = threadIdx.x; t < nl; t += blockDim.x) { T.gp[l][t] = p[t]; T.gb[l][t] = p[nl + t]; }
  }
}

// ---------------- residual norms ||b - A p||^2 and ||b||^2 (FP64, fixed order) ----------------
constexpr int RB = 256;
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__global__ void __launch_bounds__(RB) k_residual(const float* __restrict__ p, const float* __restrict__ b, int nx, int ny, int nz,
                                                 float h, double* __restrict__ partials) {
  __shared__ double sr[RB / 32], sb[RB / 32];
  const long long total = (long long)nx * ny * nz;
  const double ih2 = 1.0 / ((double)h * (double)h);
  double rr = 0.0, bb = 0.0;
  for (long long t = (long long)blockIdx.x * RB + threadIdx.x; t < total; t += (long long)gridDim.x * RB) {
    const int x = (int)(t % nx);
    const long long r = t / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const float me = __ldg(p + t);
    const double lap = ((double)pghost(p, x - 1, y, z, nx, ny, nz, me) + (double)pghost(p, x + 1, y, z, nx, ny, nz, me) +
                        (double)pghost(p, x, y - 1, z, nx, ny, nz, me) + (double)pghost(p, x, y + 1, z, nx, ny, nz, me) +
                        (double)pghost(p, x, y, z - 1, nx, ny, nz, me) + (double)pghost(p, x, y, z + 1, nx, ny, nz, me) -
                        6.0 * (double)me) * ih2;
    const double bv = (double)__ldg(b + t);
    const double res = bv - lap;
    rr += res * res;
    bb += bv * bv;
  }
  rr = warp_sum(rr);
  bb = warp_sum(bb);
  if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = rr; sb[threadIdx.x >> 5] = bb; }
  __syncthreads();
  if (threadIdx.x < 32) {
    rr = threadIdx.x < RB / 32 ? sr[threadIdx.x] : 0.0;
    bb = threadIdx.x < RB / 32 ? sb[threadIdx.x] : 0.0;
    rr = warp_sum(rr);
    bb = warp_sum(bb);
    if (threadIdx.x == 0) { partials[2 * blockIdx.x] = rr; partials[2 * blockIdx.x + 1] = bb; }
  }
}
// Sums `count` pairs of partials in a fixed order: thread t takes pairs t, t+256, ...; then a tree.
__global__ void __launch_bounds__(RB) k_sum_pairs(const double* __restrict__ partials, int count, double* __restrict__ out2) {
  __shared__ double sa[RB / 32], sb[RB / 32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < count; i += RB) { a += partials[2 * i]; b += partials[2 * i + 1]; }
  a = warp_sum(a);
  b = warp_sum(b);
  if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
  __syncthreads();
  if (threadIdx.x < 32) {
    a = threadIdx.x < RB / 32 ? sa[threadIdx.x] : 0.0;
    b = threadIdx.x < RB / 32 ? sb[threadIdx.x] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
    if (threadIdx.x == 0) { out2[0] = a; out2[1] = b; }
  }
}

// ---------------- launchers ----------------
static inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_smooth(const MGLevel& L, int color, cudaStream_t st) {
  long long n = (long long)((L.nx + 1) >> 1) * L.ny * L.nz;
  k_smooth<<<blocks_for(n, MB), MB, 0, st>>>(L.p, L.b, L.nx, L.ny, L.nz, L.h, color);
}
void launch_restrict(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  long long n = (long long)C.nx * C.ny * C.nz;
  k_restrict<<<blocks_for(n, MB), MB, 0, st>>>(F.p, F.b, F.nx, F.ny, F.nz, F.h, C.b, C.p);
}
void launch_prolong(const MGLevel& F, const MGLevel& C, cudaStream_t st) {
  long long n = (long long)F.nx * F.ny * F.nz;
  k_prolong<<<blocks_for(n, MB), MB, 0, st>>>(F.p, C.p, F.nx, F.ny, F.nz);
}
size_t tail_smem_bytes(const MGLevel* levels, int first, int n) {
  size_t cells = 0;
  for (int l = first; l < n; ++l) cells += (size_t)levels[l].nx * levels[l].ny * levels[l].nz;
  return cells * 2 * sizeof(float);
}
void launch_tail(const MGLevel* levels, int first, int n, int pre, int post, int coarse, cudaStream_t st) {
  TailLevels T;
  T.n = n - first;
  int off = 0;
  for (int l = 0; l < T.n; ++l) {
    const MGLevel& L = levels[first + l];
    T.nx[l] = L.nx; T.ny[l] = L.ny; T.nz[l] = L.nz; T.h[l] = L.h;
    T.off[l] = off;
    off += 2 * L.nx * L.ny * L.nz;
    T.gp[l] = L.p; T.gb[l] = L.b;
  }
  size_t smem = (size_t)off * sizeof(float);
  k_tail<<<1, TAIL_THREADS, smem, st>>>(T, pre, post, coarse);
}
cudaError_t mg_configure(size_t max_tail_smem) {
  return cudaFuncSetAttribute(k_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_tail_smem);
}
int residual_partials_count(const MGLevel& L) {
  long long n = (long long)L.nx * L.ny * L.nz;
  long long b = (n + RB - 1) / RB;
  return (int)(b < 1216 ? b : 1216);   // 8 CTAs per SM on 152 SMs
}
void launch_residual(const MGLevel& L, double* partials, double* out2, cudaStream_t st) {
  int nb = residual_partials_count(L);
  k_residual<<<nb, RB, 0, st>>>(L.p, L.b, L.nx, L.ny, L.nz, L.h, partials);
  k_sum_pairs<<<1, RB, 0, st>>>(partials, nb, out2);
}

}  // namespace fire

// ---------------- residual-driven loop control (conditional WHILE node body tail) ----------------
namespace fire {
// sums2 = (||r||^2, ||b||^2) of level 0 after the cycle just run.  Keeps looping while the relative
// residual is above `tol` and fewer than `max_cycles` cycles have run.
__global__ void k_mg_decide(const double* __restrict__ sums2, double tol, int max_cycles, int* __restrict__ counter,
                            double* __restrict__ rel_out, cudaGraphConditionalHandle h) {
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
  k_mg_decide<<<1, 32, 0, st>>>(sums2, tol, max_cycles, counter, rel_out, h);
}
void launch_mg_counter_reset(int* counter, cudaStream_t st) { k_mg_counter_reset<<<1, 32, 0, st>>>(counter); }
}  // namespace fire
