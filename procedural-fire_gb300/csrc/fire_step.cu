// Per-step stencil kernels of the fire simulation: MacCormack advection, curl + forces (fused),
// divergence and projection.  Each kernel restates one WGSL compute shader of src/sim.js; the line
// ranges are given per kernel.  One thread per cell; CTAs cover 32 x 4 x 2 bricks so the gathers of
// the semi-Lagrangian back-trace and the 7-point stencils hit L1 (the forces stage instead marches 32 x 8
// column tiles up z, one wave of resident CTAs).  Fields are dense float4 arrays, x fastest, so every warp
// reads and writes 512 contiguous bytes per field.
#include <type_traits>
#include "fire_device.cuh"
#include "fire_launch.cuh"

namespace fire {

constexpr int BX = 32, BY = 4, BZ = 2;
// Minimum resident CTAs per SM requested from the register allocator for the gather-heavy kernels
// (latency-bound: more resident warps hide more of the dependent back-trace loads).
#ifndef FIRE_ADV_MIN_CTAS
#define FIRE_ADV_MIN_CTAS 4
#endif
#ifndef FIRE_FORCES_MIN_CTAS
#define FIRE_FORCES_MIN_CTAS 4
#endif

struct CellId { int i, j, k; bool ok; };
// Every stencil kernel starts here: wait for the predecessor grid (programmatic dependent launch), let the
// successor's launch begin, and locate this thread's cell.
// `blk` is the CTA's position in the simulation's grid: blockIdx for a per-simulation launch, or the
// position a batched launch derived from its flat block index (BatchMap).
// Cell tiles a stage can run with: the per-simulation kernels use Tile0; the batched (ensemble) kernels are
// instantiated for every CELL_TILES entry and the ensemble's autotuner picks one per stage.
template <int TX, int TY, int TZ> struct Tile { static constexpr int X = TX, Y = TY, Z = TZ; };
using Tile0 = Tile<BX, BY, BZ>;
template <class T = Tile0>
__device__ __forceinline__ CellId cell_id(Dims d, uint3 blk) {
  pdl_wait();
  pdl_trigger();
  CellId c;
  c.i = blk.x * T::X + threadIdx.x;
  c.j = blk.y * T::Y + threadIdx.y;
  c.k = blk.z * T::Z + threadIdx.z;
  c.ok = c.i < d.nx && c.j < d.ny && c.k < d.nz;
  return c;
}
__device__ __forceinline__ CellId cell_id(Dims d) { return cell_id<Tile0>(d, blockIdx); }
static dim3 grid_for(Dims d) { return dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ); }
static dim3 block_shape() { return dim3(BX, BY, BZ); }


// ---------------- adv1 (src/sim.js:142-157) ----------------
template <class TileT = Tile0>
__device__ __forceinline__ void adv1_body(const float* __restrict__ P, const Fields& f, Dims d, uint3 blk) {
  CellId id = cell_id<TileT>(d, blk);
  if (!id.ok) return;
  const float dt = __ldg(P + P_dt), dx = __ldg(P + P_dx);
  const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
  f3 c = mk3((float)id.i + 0.5f, (float)id.j + 0.5f, (float)id.k + 0.5f);
  f3 b = backtrace(f.vel, c, xyz(__ldg(f.vel + ci)), dt, dx, d);
  float fade = outside_fade(b, d);
  float ws = sstep(0.03f, 0.4f, b.y * dx);
  f3 wind = mk3(__ldg(P + P_windX) * ws, 0.0f * ws, __ldg(P + P_windZ) * ws);
  Tap t = make_tap(b, d);
  f3 sv = xyz(sample(f.vel, t, d));
  f.velX[ci] = make_float4(mixf(wind.x, sv.x, fade), mixf(wind.y, sv.y, fade), mixf(wind.z, sv.z, fade), 0.0f);
  f.SX[ci] = mul4(sample(f.S, t, d), fade);
  f.S2X[ci] = mul4(sample(f.S2, t, d), fade);
}

// ---------------- adv2 (src/sim.js:159-197) ----------------
template <class TileT = Tile0>
__device__ __forceinline__ void adv2_body(const float* __restrict__ P, const Fields& f, Dims d, uint3 blk) {
  CellId id = cell_id<TileT>(d, blk);
  if (!id.ok) return;
  const float dt = __ldg(P + P_dt), dx = __ldg(P + P_dx);
  const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
  f3 c = mk3((float)id.i + 0.5f, (float)id.j + 0.5f, (float)id.k + 0.5f);
  f3 v = xyz(__ldg(f.vel + ci));
  // reverse advection of the forward result
  f3 fw = c + v * dt / dx;
  f3 vH = xyz(__ldg(f.velX + ci));
  float4 sH = __ldg(f.SX + ci);
  float4 s2H = __ldg(f.S2X + ci);
  Tap tf = make_tap(fw, d);
  f3 vN = vH + (v - xyz(sample(f.velX, tf, d))) * 0.5f;
  float4 sN = add4(sH, mul4(sub4(__ldg(f.S + ci), sample(f.SX, tf, d)), 0.5f));
  float4 s2N = add4(s2H, mul4(sub4(__ldg(f.S2 + ci), sample(f.S2X, tf, d)), 0.5f));
  // clamp to the range of the source stencil at the back-traced point (Selle et al. 2008)
  f3 bt = backtrace(f.vel, c, v, dt, dx, d);
  f3 b = mk3(bt.x - 0.5f, bt.y - 0.5f, bt.z - 0.5f);
  int b0x = (int)floorf(clampf(b.x, -2.0f, (float)(d.nx + 1)));
  int b0y = (int)floorf(clampf(b.y, -2.0f, (float)(d.ny + 1)));
  int b0z = (int)floorf(clampf(b.z, -2.0f, (float)(d.nz + 1)));
  f3 vmn = mk3(1e9f, 1e9f, 1e9f), vmx = mk3(-1e9f, -1e9f, -1e9f);
  float4 smn = make_float4(1e9f, 1e9f, 1e9f, 1e9f), smx = make_float4(-1e9f, -1e9f, -1e9f, -1e9f);
  float4 tmn = smn, tmx = smx;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    int qx = b0x + (q & 1), qy = b0y + ((q >> 1) & 1), qz = b0z + ((q >> 2) & 1);
    f3 vv = xyz(ldc(f.vel, qx, qy, qz, d));
    float4 ss = ldc(f.S, qx, qy, qz, d);
    float4 tt = ldc(f.S2, qx, qy, qz, d);
    vmn = fmin3(vmn, vv); vmx = fmax3(vmx, vv);
    smn = fmin4(smn, ss); smx = fmax4(smx, ss);
    tmn = fmin4(tmn, tt); tmx = fmax4(tmx, tt);
  }
  if (outside_fade(mk3(b.x + 0.5f, b.y + 0.5f, b.z + 0.5f), d) < 1.0f) { vN = vH; sN = sH; s2N = s2H; }
  vN = fmin3(fmax3(vN, fmin3(vmn, vH)), fmax3(vmx, vH));
  sN = fmin4(fmax4(sN, fmin4(smn, sH)), fmax4(smx, sH));
  s2N = fmin4(fmax4(s2N, fmin4(tmn, s2H)), fmax4(tmx, s2H));
  const float4 z0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  f.velY[ci] = make_float4(vN.x, vN.y, vN.z, 0.0f);
  f.SY[ci] = fmax4(sN, z0);
  f.S2Y[ci] = fmax4(s2N, z0);
}

// ---------------- curl (src/sim.js:200-211) ----------------
__global__ void __launch_bounds__(256) k_curl(Fields f, Dims d) {
  CellId id = cell_id(d);
  if (!id.ok) return;
  f.vort[cell(id.i, id.j, id.k, d.nx, d.ny)] = curl_at(f.velY, id.i, id.j, id.k, d);
}

// ---------------- forces (src/sim.js:214-396), with the curl recomputed in place ----------------
// The reference runs a separate curl dispatch into a vorticity texture and reads 7 taps of it here.
// This kernel computes those 7 vorticity values from velY directly (the taps are clamped to the
// domain exactly as `ld` clamps them), so the vorticity field never round-trips through HBM.
// Per-cell physics of the forces kernel.  `nb` supplies the velY/vorticity neighbourhood: the centre
// velY value, the centre vorticity, the gradient of |w| from the 6 clamped vorticity taps, and the
// velY Laplacian (only evaluated when visc > 0).
// The cell's own SY, S2Y and geometry values are passed in (the z-marching kernel prefetches them a plane
// ahead).
// Readers of the per-step parameter block for the forces physics: from global memory (batched, eager and
// adjoint launches), or from the kernel's own parameter space (the step graph's launch, whose block is set on
// the instantiated graph before every step), where each read is a constant-bank operand instead of a load.
struct ParamsGlobal {
  const float* __restrict__ P;
  __device__ __forceinline__ float operator[](int i) const { return __ldg(P + i); }
};
struct ParamsByValue {
  const ParamBlock& b;
  __device__ __forceinline__ float operator[](int i) const { return b.v[i]; }
};
template <class PA, class Nb>
__device__ __forceinline__ void forces_cell(const PA& pa, const Fields& f, const uint2* __restrict__ noiseT,
                                            const uint2* __restrict__ curlT, Dims d, int i, int j, int k, unsigned ci,
                                            const Nb& nb, float4 s, float4 s2, const float4 geo) {
  const float dt = pa[P_dt], dx = pa[P_dx], I = pa[P_intensity];
  const float seed = pa[P_seed], time = pa[P_time];
  f3 p = mk3(pa[P_ox], pa[P_oy], pa[P_oz]) + mk3((float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f) * dx;
  float4 v4 = nb.vel_center();
  f3 v = xyz(v4);

  // ---- sources: pyrolysis on the hot log surfaces + the coal bed (src/sim.js:246-284)
  float src = 0.0f, anchor = 0.0f;
  if (geo.x > 0.001f) {
    f3 qa = p * pa[P_anchorFreq] + mk3(seed * 0.37f, 0.0f, 0.11f);
    anchor = sstep(-0.05f, 0.25f, noise4(noiseT, qa).z);
    f3 qn = p * (pa[P_srcFreq] * 0.06f) + mk3(seed * 0.131f, 0.0f, time * pa[P_srcSpeed]);
    const float th = pa[P_srcThresh];
    float pulse = sstep_inv(th - 0.25f, pa[P_STRIDE + E_invPulse], noise4(noiseT, qn).x);
    src = clampf(geo.x * pa[P_logSrc] * (pa[P_srcFloor] + pa[P_anchorGain] * anchor) * mixf(0.55f, 1.0f, pulse) * 1.2f,
                 0.0f, 1.0f) * I;
    src *= 1.0f - geo.z;
  }
  // Gaussian pyrolysis spots (build-defined extension; none by default)
  const int nSpots = (int)pa[P_STRIDE + E_nSpots];
  if (nSpots > 0 && p.y < pa[P_STRIDE + E_spotTop]) {   // above every spot's 4-sigma reach the sum is exactly 0
    const float spotRef = pa[P_STRIDE + E_spotRef];
    float acc = 0.0f;
    for (int q = 0; q < nSpots; ++q) {
      const int sp = P_STRIDE + E_SPOTS + SPOT_STRIDE * q;
      f3 dd = p - mk3(pa[sp + 0], pa[sp + 1], pa[sp + 2]);
      float sg = pa[sp + 3];
      float d2 = dot3(dd, dd);
      if (d2 < 16.0f * sg * sg) acc += (pa[sp + 4] / spotRef) * expf(-d2 / (2.0f * sg * sg));
    }
    src = fmaxf(src, clampf(acc, 0.0f, 1.0f) * I);
  }
  const float srcW = fminf(src, 1.0f);
  const float bedHot = geo.y;
  float bed = geo.y * clampf(I * 1.4f, 0.3f, 1.0f);
  if (bed > 0.001f) {
    f3 qb = p * 2.4f + mk3(0.17f, -time * 0.12f, time * 0.05f);
    bed *= sstep(0.0f, 0.3f, noise4(noiseT, qb).y);
  }
  s.y = fmaxf(s.y, src * pa[P_fuelSrc]);
  s.y = fmaxf(s.y, bed * pa[P_bedFuel]);
  s.x = fmaxf(s.x, src * pa[P_srcTemp]);
  s.x = fmaxf(s.x, bedHot * pa[P_bedTemp]);
  const float srcAll = fmaxf(srcW, bed);
  s2.w = mixf(s2.w, 1.0f, bed * (1.0f - srcW));
  s2.w = mixf(s2.w, 0.0f, srcW);
  s2.y = s2.y * (1.0f - srcAll);
  s2.x = fmaxf(s2.x, (1.0f - s.y) * srcW);
  s2.x = fmaxf(s2.x, (1.0f - s.y) * bed * 0.6f);
  // pow(1, y) = 1 exactly, so cells without a source skip the pow (here and for the sponge/top factors below)
  const float wsa = clampf(srcW + bed * 0.4f, 0.0f, 1.0f);
  float wsrc = wsa > 0.0f ? 1.0f - powf(1.0f - wsa * 0.5f, dt * 90.0f) : 0.0f;
  v.y = mixf(v.y, fmaxf(v.y, pa[P_srcVel]), wsrc);
  s2.z += geo.x * (1.0f - anchor) * pa[P_smolder] * dt * I;

  // ---- burst (src/sim.js:288-296)
  const float burstAmt = pa[P_burstAmt];
  if (burstAmt > 0.0f) {
    float bd = len3(p - mk3(pa[P_burstX], pa[P_burstY], pa[P_burstZ]));
    float bw = clampf(expf(-bd * bd / 0.006f) * burstAmt, 0.0f, 1.0f);
    s.y = fmaxf(s.y, 0.17f * bw);
    s.x = fmaxf(s.x, 0.9f * bw);
    s2.x *= 1.0f - bw;
    s2.w *= 1.0f - bw;
    s2.y = fmaxf(s2.y, 0.05f * bw * clampf(s.y + s2.x, 0.0f, 1.0f));
  }
  float ageF = s2.y / fmaxf(s.y + s2.x, 1e-4f);

  // ---- mixing-limited combustion (src/sim.js:299-309)
  const float T0 = 293.0f + 1000.0f * s.x;
  const float o = clampf(1.0f - s.y - s2.x, 0.0f, 1.0f);
  const float ignT = pa[P_ignT], rs = pa[P_rs];
  const float ign = sstep_inv(ignT - 50.0f, pa[P_STRIDE + E_invIgn], T0);
  const float b = fminf(s.y, o / rs) * (1.0f - expf(-pa[P_kMix] * ign * dt));
  s.y -= b;
  s2.x = fminf(s2.x + (1.0f + rs) * b, 1.0f);
  const float dT = fminf(pa[P_heatOut] * b, fmaxf(2100.0f - T0, 0.0f));
  float T = T0 + dT;
  const float q = dT / dt;
  const float phi = geo.z > 0.5f ? 0.0f : fminf(pa[P_expansion] * q / T, 60.0f);

  // ---- soot (src/sim.js:312-318); the age gate bounds come from the extension block
  const float sootOx = pa[P_sootOx];
  ageF = fminf(ageF + dt, 4.0f);
  s.z += pa[P_sootForm] * b * sstep_inv(pa[P_STRIDE + E_sootAge0], pa[P_STRIDE + E_invSootAge], ageF) * sstep(1000.0f, 1400.0f, T) * (1.0f - s2.w);
  s.z *= expf(-sootOx * (0.25f + o) * sstep(1100.0f, 1400.0f, T) * dt);
  s.z *= expf(-sootOx * 0.5f * o * sstep(850.0f, 1100.0f, T) * (1.0f - sstep(1100.0f, 1300.0f, T)) * dt);
  s.z *= pa[P_STRIDE + E_decaySoot];   // exp(-sootDissip dt), the same for every cell (host-evaluated)

  // ---- cooling (src/sim.js:321-330)
  const float th = T * 0.001f;
  T -= fminf(pa[P_radCool] * 970.0f * s.z * th * th * (th * th * th * th - 0.00737f), 6000.0f) * dt;
  const float notBurning = 1.0f - sstep(500.0f, 5000.0f, q);
  T = 293.0f + fmaxf(T - 293.0f, 0.0f) * expf(-pa[P_coolRate] * notBurning * dt);
  s.x = (T - 293.0f) * 0.001f;
  s.w = q * 1e-4f;
  s.y *= pa[P_STRIDE + E_decayFuel];    // exp(-fuelDissip dt)
  s2.x *= pa[P_STRIDE + E_decayVit];    // exp(-vitDecay dt)
  s2.z *= pa[P_STRIDE + E_decaySmoke];  // exp(-smokeDissip dt)
  s2.y = ageF * clampf(s.y + s2.x, 0.0f, 1.0f);

  // ---- buoyancy (src/sim.js:333)
  v.y += pa[P_buoyancy] * s.x * dt;

  // ---- hot-gas viscosity (src/sim.js:339-346)
  const float visc = pa[P_visc];
  if (visc > 0.0f) {
    f3 lapV = nb.lap_v();
    float nu = visc * 1.5e-5f * powf(fmaxf(T, 293.0f) / 293.0f, 1.7f);
    v = v + lapV * fminf(nu * dt / (dx * dx), 0.15f);
  }
  // ---- laminar flame base (src/sim.js:350)
  const float lamAge = pa[P_lamAge];
  const float lam = lamAge > 0.0f ? sstep(0.5f * lamAge, fmaxf(lamAge, 1e-3f), ageF) : 1.0f;

  // ---- vorticity confinement (src/sim.js:353-361).  Where the gate is exactly 0 (gas below 450 K, the
  // sources, the floor layer) the increment is a signed zero, so it is skipped; only the sign of a zero
  // velocity component can differ.
  const float gate = sstep(450.0f, 900.0f, T) * (1.0f - srcAll) * sstep(0.02f, 0.08f, p.y) * lam;
  if (gate != 0.0f) {
    const f3 g = nb.grad_w();
    const float gl = len3(g);
    if (gl > 1e-6f) v = v + cross3(g / gl, xyz(nb.vort_center())) * (pa[P_vortEps] * gate) * dt;
  }

  // ---- sub-grid turbulence: rising, evolving curl noise (src/sim.js:364-368); skipped the same way where
  // its gate is exactly 0 (below 500 K with no heat release: most of the domain), which saves the table sample
  const float tgate = fmaxf(sstep(500.0f, 1100.0f, T), sstep(0.0f, 3.0f, s.w)) * (1.0f - srcAll) *
                      mixf(0.6f, 1.8f, sstep(0.2f, 0.75f, p.y)) * lam;
  if (tgate != 0.0f) {
    f3 tq = (p - mk3(0.0f, time * pa[P_turbRise], 0.0f)) * pa[P_turbFreq] + mk3(0.0f, 0.0f, time * pa[P_turbEvolve]);
    f3 cn = xyz(sample_table(curlT, tq));
    v = v + cn * pa[P_STRIDE + E_turbK] * tgate * dt * 10.0f;   // E_turbK = turbAmp / 12
  }

  // ---- wind above the logs (src/sim.js:372-375)
  const float windX = pa[P_windX], windZ = pa[P_windZ];
  const float windK = sstep(0.05f, 0.5f, p.y) * (1.0f + pa[P_gust]);
  v.x += (windX * windK - v.x) * dt * 0.35f * windK;
  v.z += (windZ * windK - v.z) * dt * 0.35f * windK;
  v = v * pa[P_STRIDE + E_decayVel];    // exp(-velDissip dt)

  // ---- solids & sponge layers (src/sim.js:378-388)
  if (geo.z > 0.5f) { v = mk3(0.0f, 0.0f, 0.0f); s.y = 0.0f; s2.y = 0.0f; }
  f3 fp = mk3((float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f);
  float side = fminf(fminf(fp.x, (float)d.nx - fp.x), fminf(fp.z, (float)d.nz - fp.z));
  float sp = (1.0f - sstep(0.0f, 5.0f, side)) * pa[P_sponge];
  float wsy = sstep(0.03f, 0.4f, p.y);
  float wSx = windX * wsy, wSz = windZ * wsy;
  const float spc = clampf(sp, 0.0f, 1.0f);
  float ks = spc > 0.0f ? 1.0f - powf(1.0f - 0.15f * spc, dt * 90.0f) : 0.0f;
  v.x = mixf(v.x, wSx, ks);
  v.z = mixf(v.z, wSz, ks);
  float top = sstep((float)d.ny - 10.0f, (float)d.ny, fp.y);
  float kt = top > 0.0f ? powf(1.0f - 0.1f * top, dt * 90.0f) : 1.0f;
  s.z *= kt;
  s2.z *= kt;

  float vl = len3(v);
  if (vl > 15.0f) v = v * (15.0f / vl);
  bool bad = isnan(s.x) || isnan(s.y) || isnan(s.z) || isnan(s.w) || isnan(s2.x) || isnan(s2.y) || isnan(s2.z) ||
             isnan(s2.w) || isnan(v.x) || isnan(v.y) || isnan(v.z);
  if (bad) {
    s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    s2 = s;
    v = mk3(0.0f, 0.0f, 0.0f);
  }
  f.velX[ci] = make_float4(v.x, v.y, v.z, phi);
  f.S[ci] = s;
  f.S2[ci] = s2;
}

// Neighbourhood from global memory: either the vorticity field written by the curl stage, or (fused)
// the 7 vorticity taps recomputed from clamped velY loads.
template <bool kFusedCurl>
struct GlobalNb {
  const Fields& f;
  Dims d;
  int i, j, k;
  __device__ float4 vel_center() const { return __ldg(f.velY + cell(i, j, k, d.nx, d.ny)); }
  __device__ float4 vort_center() const {
    return kFusedCurl ? curl_at(f.velY, i, j, k, d) : __ldg(f.vort + cell(i, j, k, d.nx, d.ny));
  }
  __device__ f3 grad_w() const {
    if (kFusedCurl)
      return mk3(curl_at(f.velY, min(i + 1, d.nx - 1), j, k, d).w - curl_at(f.velY, max(i - 1, 0), j, k, d).w,
                 curl_at(f.velY, i, min(j + 1, d.ny - 1), k, d).w - curl_at(f.velY, i, max(j - 1, 0), k, d).w,
                 curl_at(f.velY, i, j, min(k + 1, d.nz - 1), d).w - curl_at(f.velY, i, j, max(k - 1, 0), d).w);
    return mk3(ldc(f.vort, i + 1, j, k, d).w - ldc(f.vort, i - 1, j, k, d).w,
               ldc(f.vort, i, j + 1, k, d).w - ldc(f.vort, i, j - 1, k, d).w,
               ldc(f.vort, i, j, k + 1, d).w - ldc(f.vort, i, j, k - 1, d).w);
  }
  __device__ f3 lap_v() const {   // src/sim.js:340-343, same summation order
    f3 l = xyz(ldc(f.velY, i + 1, j, k, d)) + xyz(ldc(f.velY, i - 1, j, k, d));
    l = l + xyz(ldc(f.velY, i, j + 1, k, d));
    l = l + xyz(ldc(f.velY, i, j - 1, k, d));
    l = l + xyz(ldc(f.velY, i, j, k + 1, d));
    l = l + xyz(ldc(f.velY, i, j, k - 1, d));
    return l - xyz(vel_center()) * 6.0f;
  }
};
template <bool kFusedCurl>
__global__ void __launch_bounds__(256) k_forces(const float* __restrict__ P, Fields f, const uint2* __restrict__ noiseT,
                                                const uint2* __restrict__ curlT, Dims d) {
  CellId id = cell_id(d);
  if (!id.ok) return;
  GlobalNb<kFusedCurl> nb{f, d, id.i, id.j, id.k};
  const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
  forces_cell(ParamsGlobal{P}, f, noiseT, curlT, d, id.i, id.j, id.k, (unsigned)ci, nb, __ldg(f.SY + ci), __ldg(f.S2Y + ci),
              __ldg(f.geo + ci));
}

// ---- z-marching shared-memory variant of curl + forces ----
// A CTA of 32 x 8 threads owns a 32 x 8 column tile and marches through a run of planes (FZ planes per CTA
// in the batched kernel; an equal share of all (column, plane) units in the one-wave kernel).  Shared memory holds a
// ring of 5 velY planes (tile + 2-cell halo, clamped to the domain like `ld`) and a ring of 3 planes of the
// vorticity magnitude |w| (tile + 1-cell halo), which is all the confinement gradient reads; the vorticity
// vector itself is needed only at the cell, where confinement acts, and is formed there from the velY ring
// with the same arithmetic.  |w| at a halo position outside the domain is that of the clamped position,
// which is what `ld(vortT, c +- e)` returns.  Each velY value is loaded ~2x per cell (halo overhead) instead
// of the 42 gathers of the per-cell recompute.
constexpr int FT_X = 32, FT_Y = 8, FZ = 16;
constexpr int VX = FT_X + 4, VY = FT_Y + 4;      // velY plane with 2-cell halo
constexpr int WX = FT_X + 2, WY = FT_Y + 2;      // vorticity plane with 1-cell halo
// Ring slots are addressed by logical z (z >= -2): velY plane z lives in slot (z + 10) % 5, vorticity
// plane z in slot (z + 9) % 3.
__device__ __forceinline__ float4* vslot(float4* vbuf, int z) { return vbuf + ((z + 10) % 5) * (VX * VY); }
__device__ __forceinline__ float* wslot(float* wbuf, int z) { return wbuf + ((z + 9) % 3) * (WX * WY); }
// The curl of velY at tile position c (a VX*VY offset) from planes K (z-1), P0 (z), F (z+1), given the
// positions of its x and y neighbours (clamped to the domain by the caller); the arithmetic of curl_at.
__device__ __forceinline__ f3 curl_tile(const float4* K, const float4* P0, const float4* F, int c, int cxm, int cxp, int cym,
                                        int cyp) {
  f3 L = xyz(P0[cxm]), R = xyz(P0[cxp]);
  f3 B = xyz(P0[cym]), T = xyz(P0[cyp]);
  f3 Kv = xyz(K[c]), Fv = xyz(F[c]);
  return mk3((T.z - B.z) - (Fv.y - Kv.y), (Fv.x - Kv.x) - (R.z - L.z), (R.y - L.y) - (T.x - B.x)) * 0.5f;
}
struct TileNb {
  const float4 *vm, *v0, *vp;   // velY planes z-1, z, z+1 (VX*VY each)
  const float *wm, *w0, *wp;    // |w| planes z-1, z, z+1 (WX*WY each)
  int tx, ty;                   // thread position in the tile
  __device__ float4 vel_center() const { return v0[(ty + 2) * VX + tx + 2]; }
  // The cell is inside the domain and the ring's halo holds clamped positions, so its four in-plane
  // neighbours in the ring are the clamped neighbours; vm / vp are the clamped planes z -+ 1.
  __device__ float4 vort_center() const {
    const int c = (ty + 2) * VX + tx + 2;
    const f3 w = curl_tile(vm, v0, vp, c, c - 1, c + 1, c - VX, c + VX);
    return make_float4(w.x, w.y, w.z, 0.0f);
  }
  __device__ f3 grad_w() const {
    const int c = (ty + 1) * WX + tx + 1;
    return mk3(w0[c + 1] - w0[c - 1], w0[c + WX] - w0[c - WX], wp[c] - wm[c]);
  }
  __device__ f3 lap_v() const {   // src/sim.js:340-343, same summation order
    const int c = (ty + 2) * VX + tx + 2;
    f3 l = xyz(v0[c + 1]) + xyz(v0[c - 1]);
    l = l + xyz(v0[c + VX]);
    l = l + xyz(v0[c - VX]);
    l = l + xyz(vp[c]);
    l = l + xyz(vm[c]);
    return l - xyz(v0[c]) * 6.0f;
  }
};
__device__ __forceinline__ int clampi(int v, int n) { return min(max(v, 0), n - 1); }
// 16-byte asynchronous global -> shared copy (cached in L2 only), and its group commit / wait.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// The plane-independent part of a thread's share of the ring traffic for one column tile, worked out once
// per march: each thread copies velY elements t = tid and tid + 256 of a plane and forms vorticity elements
// t = tid and tid + 256.
//  * vsrc[k]: x + nx * y of velY element k's source, clamped to the domain as `ld` does (-1: no element);
//  * wtap[k]: vorticity element k's velY ring offset (bits 0-9) and which of its x-, x+, y-, y+ neighbours lie
//    inside the domain (bits 10-13; a clamped neighbour is the centre itself) (-1: no element).
constexpr int FT_N = FT_X * FT_Y;
static_assert(VX * VY <= 2 * FT_N && WX * WY <= 2 * FT_N && VX * VY < 1024, "two ring elements per thread, 10-bit offsets");
struct MarchPlan {
  int vsrc[2], wtap[2];
};
__device__ __forceinline__ MarchPlan march_plan(int x0, int y0, Dims d) {
  MarchPlan m;
  const int tid = threadIdx.y * FT_X + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int t = tid + k * FT_N;
    m.vsrc[k] = -1;
    m.wtap[k] = -1;
    if (t < VX * VY) {
      const int lx = t % VX, ly = t / VX;
      m.vsrc[k] = clampi(x0 + lx - 2, d.nx) + d.nx * clampi(y0 + ly - 2, d.ny);
    }
    if (t < WX * WY) {
      const int lx = t % WX, ly = t / WX;
      // clamp the position to the domain, then express it in tile coordinates (velY tile origin at -2)
      const int gx = clampi(x0 + lx - 1, d.nx), gy = clampi(y0 + ly - 1, d.ny);
      const int c = (gy - y0 + 2) * VX + (gx - x0 + 2);
      m.wtap[k] = c | (gx > 0) << 10 | (gx < d.nx - 1) << 11 | (gy > 0) << 12 | (gy < d.ny - 1) << 13;
    }
  }
  return m;
}
// Starts the copy of logical plane z (clamped) of velY for the march's tile into `dst`; the caller commits and
// waits.
__device__ __forceinline__ void load_vplane(float4* dst, const float4* __restrict__ velY, const MarchPlan& m, int z, Dims d) {
  const unsigned zo = (unsigned)clampi(z, d.nz) * (unsigned)(d.nx * d.ny);
  const int tid = threadIdx.y * FT_X + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 2; ++k)
    if (m.vsrc[k] >= 0) cp_async16(dst + tid + k * FT_N, velY + (zo + (unsigned)m.vsrc[k]));
}
// |w| of logical plane zlog into `dst` (positions clamped to the domain), from the velY ring.  The planes it
// reads (clamp(zlog) and its clamped z neighbours) are resident in the ring when this is called.
__device__ __forceinline__ void curl_plane(float* dst, float4* vbuf, const MarchPlan& m, int zlog, Dims d) {
  const int zc = clampi(zlog, d.nz);
  const float4* PK = vslot(vbuf, clampi(zc - 1, d.nz));
  const float4* P0 = vslot(vbuf, zc);
  const float4* PF = vslot(vbuf, clampi(zc + 1, d.nz));
  const int tid = threadIdx.y * FT_X + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int tap = m.wtap[k];
    if (tap < 0) continue;
    const int c = tap & 1023;
    const f3 w = curl_tile(PK, P0, PF, c, c - ((tap >> 10) & 1), c + ((tap >> 11) & 1), c - ((tap >> 12) & 1) * VX,
                           c + ((tap >> 13) & 1) * VX);
    dst[tid + k * FT_N] = len3(w);
  }
}
// Marches the column tile at (x0, y0) through planes [z0, z1), z1 > z0.  The copy of the next velY plane is
// started before the current plane's source terms and completes behind them: it goes to the slot of plane
// z - 2, which nothing reads any more (the vorticity of z - 1 was formed three planes ago, and the previous
// plane's Laplacian finished before the last barrier).
template <class PA>
__device__ __forceinline__ void forces_march(const PA& pa, const Fields& f, const uint2* __restrict__ noiseT,
                                             const uint2* __restrict__ curlT, Dims d, int x0, int y0, int z0, int z1,
                                             float4* fsm) {
  float4* vbuf = fsm;                                        // 5 * VX * VY
  float* wbuf = reinterpret_cast<float*>(fsm + 5 * VX * VY);  // 3 * WX * WY
  const MarchPlan m = march_plan(x0, y0, d);
  for (int z = z0 - 2; z <= z0 + 2; ++z) load_vplane(vslot(vbuf, z), f.velY, m, z, d);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  for (int z = z0 - 1; z <= z0 + 1; ++z) curl_plane(wslot(wbuf, z), vbuf, m, z, d);
  __syncthreads();
  const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
  const bool mine = i < d.nx && j < d.ny;
  const unsigned plane = (unsigned)(d.nx * d.ny);
  unsigned ci = mine ? (unsigned)i + (unsigned)d.nx * ((unsigned)j + (unsigned)d.ny * (unsigned)z0) : 0u;
  // this thread's SY, S2Y, geo for the current plane, loaded one plane ahead
  float4 s_n = make_float4(0.0f, 0.0f, 0.0f, 0.0f), s2_n = s_n, g_n = s_n;
  if (mine) { s_n = __ldg(f.SY + ci); s2_n = __ldg(f.S2Y + ci); g_n = __ldg(f.geo + ci); }
  for (int z = z0; z < z1; ++z, ci += plane) {
    const float4 s = s_n, s2 = s2_n, g = g_n;
    const bool more = z + 1 < z1;
    if (more) {
      load_vplane(vslot(vbuf, z + 3), f.velY, m, z + 3, d);   // into the slot of plane z - 2
      cp_async_commit();
    }
    if (mine && more) { s_n = __ldg(f.SY + ci + plane); s2_n = __ldg(f.S2Y + ci + plane); g_n = __ldg(f.geo + ci + plane); }
    if (mine) {
      TileNb nb;
      nb.vm = vslot(vbuf, z - 1); nb.v0 = vslot(vbuf, z); nb.vp = vslot(vbuf, z + 1);
      nb.wm = wslot(wbuf, z - 1); nb.w0 = wslot(wbuf, z); nb.wp = wslot(wbuf, z + 1);
      nb.tx = threadIdx.x;
      nb.ty = threadIdx.y;
      forces_cell(pa, f, noiseT, curlT, d, i, j, z, ci, nb, s, s2, g);
    }
    if (more) {
      cp_async_wait_all();
      __syncthreads();          // plane z + 3 is visible; everyone is done with vorticity plane z - 1
      curl_plane(wslot(wbuf, z + 2), vbuf, m, z + 2, d);       // replaces vorticity plane z - 1
      __syncthreads();
    }
  }
}
// The batched kernel's CTA: column tile (blk.x, blk.y), planes [blk.z * ZD, blk.z * ZD + ZD).
template <int ZD = FZ>   // planes one CTA marches through
__device__ __forceinline__ void forces_tiled_body(const float* __restrict__ P, const Fields& f, const uint2* __restrict__ noiseT,
                                                  const uint2* __restrict__ curlT, Dims d, uint3 blk, float4* fsm) {
  pdl_wait();
  pdl_trigger();
  const int z0 = blk.z * ZD;
  forces_march(ParamsGlobal{P}, f, noiseT, curlT, d, blk.x * FT_X, blk.y * FT_Y, z0, min(z0 + ZD, d.nz), fsm);
}
constexpr size_t FORCES_TILED_SMEM = sizeof(float4) * 5 * VX * VY + sizeof(float) * 3 * WX * WY;

// ---------------- divergence minus the expansion target (src/sim.js:399-413) ----------------
template <class TileT = Tile0>
__device__ __forceinline__ void div_body(const float* __restrict__ P, const float4* __restrict__ velX, float* __restrict__ b0, Dims d,
                                         uint3 blk) {
  CellId id = cell_id<TileT>(d, blk);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float dx = __ldg(P + P_dx);
  float4 me = __ldg(velX + ci);
  float L = ldc(velX, i - 1, j, k, d).x, R = ldc(velX, i + 1, j, k, d).x;
  float B = ldc(velX, i, j - 1, k, d).y, T = ldc(velX, i, j + 1, k, d).y;
  float K = ldc(velX, i, j, k - 1, d).z, F = ldc(velX, i, j, k + 1, d).z;
  if (j == 0) B = -me.y;   // solid floor
  b0[ci] = ((R - L) + (T - B) + (F - K)) / (2.0f * dx) - me.w;
}

// ---------------- projection (src/sim.js:526-550) ----------------
__device__ __forceinline__ float pr(const float* __restrict__ p, int x, int y, int z, Dims d, float me) {
  if (x < 0 || z < 0 || x >= d.nx || z >= d.nz || y >= d.ny) return -me;   // open sides/top: p = 0 on the face
  if (y < 0) return me;                                                    // floor: Neumann
  return __ldg(p + cell(x, y, z, d.nx, d.ny));
}
template <class TileT = Tile0>
__device__ __forceinline__ void project_body(const float* __restrict__ P, const float4* __restrict__ velX, const float* __restrict__ p0,
                                             const unsigned char* __restrict__ solid, float4* __restrict__ vel, Dims d, uint3 blk) {
  CellId id = cell_id<TileT>(d, blk);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float dx = __ldg(P + P_dx);
  float me = __ldg(p0 + ci);
  f3 g = mk3(pr(p0, i + 1, j, k, d, me) - pr(p0, i - 1, j, k, d, me),
             pr(p0, i, j + 1, k, d, me) - pr(p0, i, j - 1, k, d, me),
             pr(p0, i, j, k + 1, d, me) - pr(p0, i, j, k - 1, d, me)) / (2.0f * dx);
  f3 v = xyz(__ldg(velX + ci)) - g;
  if (__ldg(solid + ci)) v = mk3(0.0f, 0.0f, 0.0f);   // geo.b > 0.5
  if (j == 0) v.y = fmaxf(v.y, 0.0f);
  float vl = len3(v);
  if (vl > 20.0f || isnan(vl)) v = isnan(vl) ? mk3(0.0f, 0.0f, 0.0f) : v * 20.0f / vl;
  vel[ci] = make_float4(v.x, v.y, v.z, 0.0f);
}

// ---------------- per-simulation kernels ----------------
__global__ void __launch_bounds__(256, FIRE_ADV_MIN_CTAS) k_adv1(const float* __restrict__ P, Fields f, Dims d) { adv1_body(P, f, d, blockIdx); }
__global__ void __launch_bounds__(256, FIRE_ADV_MIN_CTAS) k_adv2(const float* __restrict__ P, Fields f, Dims d) { adv2_body(P, f, d, blockIdx); }
// One wave of resident CTAs.  The (column tile, plane) units, planes fastest, are split into gridDim.x equal
// contiguous ranges, so every SM marches the same number of planes (a grid of fixed-depth chunks leaves its
// last wave partly idle); a range that runs into the next column restarts the march there.
template <class PA>
__device__ __forceinline__ void forces_persistent(const PA& pa, const Fields& f, const uint2* __restrict__ noiseT,
                                                  const uint2* __restrict__ curlT, Dims d, float4* fsm) {
  pdl_wait();
  pdl_trigger();
  const int gx = (d.nx + FT_X - 1) / FT_X, gy = (d.ny + FT_Y - 1) / FT_Y;
  const long long units = (long long)gx * gy * d.nz;
  long long u = units * blockIdx.x / gridDim.x;
  const long long end = units * (blockIdx.x + 1) / gridDim.x;
  while (u < end) {
    const int col = (int)(u / d.nz), z0 = (int)(u % d.nz);
    const int z1 = (int)min((long long)d.nz, z0 + (end - u));
    forces_march(pa, f, noiseT, curlT, d, (col % gx) * FT_X, (col / gx) * FT_Y, z0, z1, fsm);
    u += z1 - z0;
    if (u < end) __syncthreads();   // the next march refills the rings
  }
}
__global__ void __launch_bounds__(FT_X * FT_Y, FIRE_FORCES_MIN_CTAS) k_forces_tiled(const float* __restrict__ P, Fields f,
                                                                                     const uint2* __restrict__ noiseT,
                                                                                     const uint2* __restrict__ curlT, Dims d) {
  extern __shared__ float4 fsm[];
  forces_persistent(ParamsGlobal{P}, f, noiseT, curlT, d, fsm);
}
__global__ void __launch_bounds__(FT_X * FT_Y, FIRE_FORCES_MIN_CTAS) k_forces_tiled_pb(const __grid_constant__ ParamBlock pb, Fields f,
                                                                                        const uint2* __restrict__ noiseT,
                                                                                        const uint2* __restrict__ curlT, Dims d) {
  extern __shared__ float4 fsm[];
  forces_persistent(ParamsByValue{pb}, f, noiseT, curlT, d, fsm);
}
// mg_counter (the residual-driven step graph only, else null): the solve that follows counts its V-cycles
// from zero, so this kernel clears the count instead of a separate launch.
__global__ void __launch_bounds__(256) k_div(const float* __restrict__ P, const float4* __restrict__ velX, float* __restrict__ b0, Dims d,
                                             int* __restrict__ mg_counter) {
  div_body(P, velX, b0, d, blockIdx);
  if (mg_counter && (blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y | threadIdx.z) == 0) *mg_counter = 0;
}
__global__ void __launch_bounds__(256) k_project(const float* __restrict__ P, const float4* __restrict__ velX, const float* __restrict__ p0,
                                                 const unsigned char* __restrict__ solid, float4* __restrict__ vel, Dims d) {
  project_body(P, velX, p0, solid, vel, d, blockIdx);
}

// ---------------- batched kernels: one grid over many independent simulations ----------------
// Each CTA finds its simulation and its position in that simulation's grid from the flat block index
// (BatchMap), then runs the same body as the per-simulation kernel: the arithmetic, and so the results,
// are those of stepping each simulation alone.
template <class T>
__global__ void __launch_bounds__(256, FIRE_ADV_MIN_CTAS) k_adv1_b(const __grid_constant__ BatchMap m, const __grid_constant__ StepBatch I) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  adv1_body<T>(I.s[i].P, I.s[i].f, I.s[i].d, blk);
}
template <class T>
__global__ void __launch_bounds__(256, FIRE_ADV_MIN_CTAS) k_adv2_b(const __grid_constant__ BatchMap m, const __grid_constant__ StepBatch I) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  adv2_body<T>(I.s[i].P, I.s[i].f, I.s[i].d, blk);
}
template <int ZD>
__global__ void __launch_bounds__(FT_X * FT_Y, FIRE_FORCES_MIN_CTAS) k_forces_b(const __grid_constant__ BatchMap m, const __grid_constant__ StepBatch I,
                                                                                 const uint2* __restrict__ noiseT, const uint2* __restrict__ curlT) {
  extern __shared__ float4 fsm[];
  uint3 blk; int i;
  batch_locate(m, blk, i);
  forces_tiled_body<ZD>(I.s[i].P, I.s[i].f, noiseT, curlT, I.s[i].d, blk, fsm);
}
template <class T>
__global__ void __launch_bounds__(256) k_div_b(const __grid_constant__ BatchMap m, const __grid_constant__ StepBatch I) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  div_body<T>(I.s[i].P, I.s[i].f.velX, I.s[i].b0, I.s[i].d, blk);
}
template <class T>
__global__ void __launch_bounds__(256) k_project_b(const __grid_constant__ BatchMap m, const __grid_constant__ StepBatch I) {
  uint3 blk; int i;
  batch_locate(m, blk, i);
  project_body<T>(I.s[i].P, I.s[i].f.velX, I.s[i].p0, I.s[i].f.solid, I.s[i].f.vel, I.s[i].d, blk);
}

// The tile candidates of the batched stages: CELL_TILES cell tiles (256 threads each; x stays 32 or 64 wide
// for coalescing) and FORCES_TILES z-march depths of the forces tile.
template <class F> void with_cell_tile(int v, F&& f) {
  switch (v) {
    case 1: f(Tile<32, 8, 1>{}); break;
    case 2: f(Tile<32, 2, 4>{}); break;
    case 3: f(Tile<64, 4, 1>{}); break;
    default: f(Tile0{}); break;
  }
}
static_assert(CELL_TILES == 4, "with_cell_tile lists every cell tile");
constexpr int kForcesDepth[FORCES_TILES] = {FZ, 8, 32};
template <class F> void with_forces_depth(int v, F&& f) {
  switch (v) {
    case 1: f(std::integral_constant<int, 8>{}); break;
    case 2: f(std::integral_constant<int, 32>{}); break;
    default: f(std::integral_constant<int, FZ>{}); break;
  }
}

// ---------------- launchers ----------------
void launch_adv1(const float* P, Fields f, Dims d, cudaStream_t st) { launch_pdl(k_adv1, grid_for(d), block_shape(), 0, st, P, f, d); }
void launch_adv2(const float* P, Fields f, Dims d, cudaStream_t st) { launch_pdl(k_adv2, grid_for(d), block_shape(), 0, st, P, f, d); }
void launch_curl(Fields f, Dims d, cudaStream_t st) { launch_pdl(k_curl, grid_for(d), block_shape(), 0, st, f, d); }
// Resident k_forces_tiled CTAs of each device (CTAs per SM x SMs), set by step_configure.
constexpr int kMaxDevices = 64;
static int g_forces_wave[kMaxDevices];
static dim3 forces_wave_grid(Dims d) {
  const long long units = (long long)((d.nx + FT_X - 1) / FT_X) * ((d.ny + FT_Y - 1) / FT_Y) * d.nz;
  int dev = 0;
  cudaGetDevice(&dev);
  const int wave = dev >= 0 && dev < kMaxDevices && g_forces_wave[dev] > 0 ? g_forces_wave[dev] : 4 * 152;
  return dim3((unsigned)(units < wave ? units : wave));
}
void launch_forces(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st) {
  launch_pdl(k_forces_tiled, forces_wave_grid(d), dim3(FT_X, FT_Y), FORCES_TILED_SMEM, st, P, f, noise, curl, d);
}
void launch_forces_pb(const ParamBlock& pb, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st) {
  launch_pdl(k_forces_tiled_pb, forces_wave_grid(d), dim3(FT_X, FT_Y), FORCES_TILED_SMEM, st, pb, f, noise, curl, d);
}
cudaError_t forces_pb_set(cudaGraphExec_t exec, cudaGraphNode_t node, const ParamBlock& pb, Fields f, const uint2* noise,
                          const uint2* curl, Dims d) {
  void* args[] = {(void*)&pb, (void*)&f, (void*)&noise, (void*)&curl, (void*)&d};
  cudaKernelNodeParams kp = {};
  kp.func = (void*)k_forces_tiled_pb;
  kp.gridDim = forces_wave_grid(d);
  kp.blockDim = dim3(FT_X, FT_Y);
  kp.sharedMemBytes = (unsigned)FORCES_TILED_SMEM;
  kp.kernelParams = args;
  return cudaGraphExecKernelNodeSetParams(exec, node, &kp);
}
void launch_forces_recompute(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st) {
  launch_pdl(k_forces<true>, grid_for(d), block_shape(), 0, st, P, f, noise, curl, d);
}
cudaError_t step_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_forces_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FORCES_TILED_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_forces_tiled_pb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FORCES_TILED_SMEM);
  int dev = 0, sms = 0, per_sm = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_forces_tiled, FT_X * FT_Y, FORCES_TILED_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxDevices) g_forces_wave[dev] = (per_sm > 0 ? per_sm : 1) * sms;
  for (int v = 0; v < FORCES_TILES && e == cudaSuccess; ++v)
    with_forces_depth(v, [&](auto z) {
      e = cudaFuncSetAttribute(k_forces_b<decltype(z)::value>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FORCES_TILED_SMEM);
    });
  return e;
}
// Block grids of the batched stages for a simulation of dims d with tile candidate `tile`.
dim3 step_grid(Dims d, int tile) {
  dim3 g;
  with_cell_tile(tile, [&](auto t) {
    using T = decltype(t);
    g = dim3((d.nx + T::X - 1) / T::X, (d.ny + T::Y - 1) / T::Y, (d.nz + T::Z - 1) / T::Z);
  });
  return g;
}
dim3 forces_grid(Dims d, int tile) {
  const int zd = kForcesDepth[tile >= 0 && tile < FORCES_TILES ? tile : 0];
  return dim3((d.nx + FT_X - 1) / FT_X, (d.ny + FT_Y - 1) / FT_Y, (d.nz + zd - 1) / zd);
}
void launch_adv1_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st) {
  with_cell_tile(tile, [&](auto t) {
    using T = decltype(t);
    launch_pdl(k_adv1_b<T>, dim3(m.prefix[m.n]), dim3(T::X, T::Y, T::Z), 0, st, m, I);
  });
}
void launch_adv2_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st) {
  with_cell_tile(tile, [&](auto t) {
    using T = decltype(t);
    launch_pdl(k_adv2_b<T>, dim3(m.prefix[m.n]), dim3(T::X, T::Y, T::Z), 0, st, m, I);
  });
}
void launch_forces_batch(const BatchMap& m, const StepBatch& I, const uint2* noise, const uint2* curl, int tile, cudaStream_t st) {
  with_forces_depth(tile, [&](auto z) {
    launch_pdl(k_forces_b<decltype(z)::value>, dim3(m.prefix[m.n]), dim3(FT_X, FT_Y), FORCES_TILED_SMEM, st, m, I, noise, curl);
  });
}
void launch_div_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st) {
  with_cell_tile(tile, [&](auto t) {
    using T = decltype(t);
    launch_pdl(k_div_b<T>, dim3(m.prefix[m.n]), dim3(T::X, T::Y, T::Z), 0, st, m, I);
  });
}
void launch_project_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st) {
  with_cell_tile(tile, [&](auto t) {
    using T = decltype(t);
    launch_pdl(k_project_b<T>, dim3(m.prefix[m.n]), dim3(T::X, T::Y, T::Z), 0, st, m, I);
  });
}
void launch_forces_unfused(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st) {
  launch_pdl(k_forces<false>, grid_for(d), block_shape(), 0, st, P, f, noise, curl, d);
}
void launch_div(const float* P, Fields f, float* b0, Dims d, cudaStream_t st, int* mg_counter) {
  launch_pdl(k_div, grid_for(d), block_shape(), 0, st, P, (const float4*)f.velX, b0, d, mg_counter);
}
void launch_project(const float* P, Fields f, const float* p0, Dims d, cudaStream_t st) {
  launch_pdl(k_project, grid_for(d), block_shape(), 0, st, P, (const float4*)f.velX, p0, (const unsigned char*)f.solid, f.vel, d);
}

}  // namespace fire

namespace fire {
// Verifies that this library carries a kernel image for the current device.
cudaError_t kernels_probe() {
  cudaFuncAttributes a;
  return cudaFuncGetAttributes(&a, k_div);
}
}  // namespace fire
