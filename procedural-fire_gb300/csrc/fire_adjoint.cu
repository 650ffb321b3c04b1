// Discrete adjoint of the fire step (src/sim.js:627-648) and the checkpointed reverse sweep over a rollout.
//
// The forward step is   adv1 -> adv2 -> curl+forces -> div -> pressure solve -> project.   Each stage has a
// hand-written reverse kernel here that takes the cotangents of the stage's outputs and accumulates the
// cotangents of its inputs, linearised at the forward values the stage saw:
//
//   k_proj_adj1 / k_proj_adj2   project (src/sim.js:526-550): the masks (solid, floor, |v| <= 20) of the
//                               branch taken; the pressure-gradient transpose as a gather.
//   pressure solve              p = A^-1 b with A the symmetric 7-point operator of the multigrid (open
//                               faces and the floor fold into its diagonal), so the cotangent of b is
//                               A^-1 applied to the cotangent of p: the same V-cycles run on it.
//   k_div_adj                   div (src/sim.js:399-413): transpose of the central difference, as a gather.
//   k_forces_adj1 / 2           forces (src/sim.js:214-396) with the fused curl (src/sim.js:200-211): the
//                               reverse of every source term, each min/max/clamp taking the branch the
//                               forward took; then the vorticity cotangents scattered onto velY.
//   k_adv2_adj                  MacCormack correction (src/sim.js:159-197): the limiter passes the
//                               cotangent to the branch it took (the corrected value, the own hat, or the
//                               extreme texel of the 8-texel stencil), the forward-traced sample is
//                               differentiated in its values and its position.
//   k_adv1_adj                  RK2 semi-Lagrangian advection (src/sim.js:142-157): trilinear weights
//                               scattered to the sampled texels, and the sample-position derivative carried
//                               back through both trace points into the velocity.
//
// Scatters use float4 atomics (sm_90+), so sums of cotangents are not bitwise reproducible run to run;
// every gather-shaped transpose (div, pressure gradient) is a plain per-cell gather.
//
// FireAdjoint runs a rollout of n steps through per-slot CUDA graphs that write every stage's output to a
// tape of k steps (k = checkpoint interval), keeps the state at every k-th step, and in the reverse sweep
// recomputes one segment at a time from its checkpoint (bitwise the same steps: same kernels, same blocks,
// same warm start) and runs the reverse-step graphs over it.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include "fire_device.cuh"
#include "fire_launch.cuh"
#include "fire_simobj.h"
#include "fire_nvtx.h"

namespace fire {

// Cotangent buffers.  vel/S/S2 hold the cotangent of the step's output state on entry to a reverse step and
// of its input state on exit.
struct AdjFields {
  float4 *vel, *S, *S2;        // state
  float4 *velX, *SX, *S2X;     // advection hats
  float4 *velY, *SY, *S2Y;     // advected fields (forces inputs)
  float4 *F;                   // forces output: velocity (xyz) and expansion target phi (w)
  float4 *W;                   // vorticity (xyz) and its magnitude (w)
  float4 *G;                   // masked velocity cotangent of the projection (scratch)
  float *Pp;                   // pressure p
  float *B;                    // divergence right-hand side b (also the warm start of the next solve)
  double *flux;                // spot fluxes (MAX_SPOTS), g/s
  double *loss;                // [0] loss of fire_adjoint_loss
};
// Forward values one reverse step is linearised at: the step's Fields (state, hats, advected fields,
// geometry) plus the forces output velocity and the solved pressure.
struct TapeStep {
  Fields f;
  float4* Fv;
  float* p;
};

constexpr int ABX = 32, ABY = 4, ABZ = 2;
static dim3 agrid(Dims d) { return dim3((d.nx + ABX - 1) / ABX, (d.ny + ABY - 1) / ABY, (d.nz + ABZ - 1) / ABZ); }
static dim3 ablock() { return dim3(ABX, ABY, ABZ); }

struct ACell { int i, j, k; bool ok; };
__device__ __forceinline__ ACell acell(Dims d) {
  pdl_wait();
  pdl_trigger();
  ACell c;
  c.i = blockIdx.x * ABX + threadIdx.x;
  c.j = blockIdx.y * ABY + threadIdx.y;
  c.k = blockIdx.z * ABZ + threadIdx.z;
  c.ok = c.i < d.nx && c.j < d.ny && c.k < d.nz;
  return c;
}

// ---- derivative helpers ----
__device__ __forceinline__ float dsstep(float e0, float e1, float x) {   // d/dx of sstep (same t as sstep)
  const float inv = 1.0f / (e1 - e0);
  const float t = clampf((x - e0) * inv, 0.0f, 1.0f);
  return 6.0f * t * (1.0f - t) * inv;
}
__device__ __forceinline__ bool in01(float x) { return x > 0.0f && x < 1.0f; }   // clamp(x, 0, 1) passes x
__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ bool nz4(float4 a) { return a.x != 0.0f || a.y != 0.0f || a.z != 0.0f || a.w != 0.0f; }
__device__ __forceinline__ void atomic_add4(float4* p, float4 v) { if (nz4(v)) atomicAdd(p, v); }

// Gradient of outside_fade with respect to the position (zero where the clamp saturates).
__device__ __forceinline__ f3 outside_fade_grad(f3 c, Dims d) {
  const float lo = fminf(c.x, c.z);
  const float hx = c.x - (float)d.nx, hy = c.y - (float)d.ny, hz = c.z - (float)d.nz;
  const float hi = fmaxf(hx, fmaxf(hy, hz));
  const float m = fmaxf(-lo, hi);
  const float fv = 1.0f - m;
  if (!(fv > 0.0f && fv < 1.0f)) return mk3(0.0f, 0.0f, 0.0f);
  if (-lo >= hi) return c.x <= c.z ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 0.0f, 1.0f);   // fade = 1 + min(x, z)
  if (hx >= hy && hx >= hz) return mk3(-1.0f, 0.0f, 0.0f);
  return hy >= hz ? mk3(0.0f, -1.0f, 0.0f) : mk3(0.0f, 0.0f, -1.0f);
}

// A trilinear sample with its derivatives along the three position axes (cell units).  Where the
// clamp-to-edge saturates, both taps of an axis are the same texel and the derivative vanishes by itself.
struct SampleD { float4 v, dx, dy, dz; };
__device__ __forceinline__ SampleD sample_d(const float4* __restrict__ f, const Tap& t, Dims d) {
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const size_t r00 = (size_t)t.y0 * sy + (size_t)t.z0 * sz, r10 = (size_t)t.y1 * sy + (size_t)t.z0 * sz;
  const size_t r01 = (size_t)t.y0 * sy + (size_t)t.z1 * sz, r11 = (size_t)t.y1 * sy + (size_t)t.z1 * sz;
  const float4 a00 = __ldg(f + r00 + t.x0), b00 = __ldg(f + r00 + t.x1);
  const float4 a10 = __ldg(f + r10 + t.x0), b10 = __ldg(f + r10 + t.x1);
  const float4 a01 = __ldg(f + r01 + t.x0), b01 = __ldg(f + r01 + t.x1);
  const float4 a11 = __ldg(f + r11 + t.x0), b11 = __ldg(f + r11 + t.x1);
  const float4 c00 = lerp4(a00, b00, t.fx), c10 = lerp4(a10, b10, t.fx);
  const float4 c01 = lerp4(a01, b01, t.fx), c11 = lerp4(a11, b11, t.fx);
  SampleD s;
  const float4 e0 = lerp4(c00, c10, t.fy), e1 = lerp4(c01, c11, t.fy);
  s.v = lerp4(e0, e1, t.fz);
  s.dx = lerp4(lerp4(sub4(b00, a00), sub4(b10, a10), t.fy), lerp4(sub4(b01, a01), sub4(b11, a11), t.fy), t.fz);
  s.dy = lerp4(sub4(c10, c00), sub4(c11, c01), t.fz);
  s.dz = sub4(e1, e0);
  return s;
}
// Position cotangent of a sample: lambda . d(sample)/d(position).
__device__ __forceinline__ f3 pos_cot(const SampleD& s, float4 lam) { return mk3(dot4(lam, s.dx), dot4(lam, s.dy), dot4(lam, s.dz)); }
__device__ __forceinline__ f3 pos_cot3(const SampleD& s, f3 lam) {
  return mk3(dot3(lam, xyz(s.dx)), dot3(lam, xyz(s.dy)), dot3(lam, xyz(s.dz)));
}
// Transpose of a trilinear sample: lam * weight added to each of the 8 taps.
__device__ __forceinline__ void scatter_tap(float4* __restrict__ g, const Tap& t, Dims d, float4 lam) {
  if (!nz4(lam)) return;
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const float wx[2] = {1.0f - t.fx, t.fx}, wy[2] = {1.0f - t.fy, t.fy}, wz[2] = {1.0f - t.fz, t.fz};
  const int xs[2] = {t.x0, t.x1}, ys[2] = {t.y0, t.y1}, zs[2] = {t.z0, t.z1};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int a = q & 1, b = (q >> 1) & 1, c = (q >> 2) & 1;
    const float w = wx[a] * wy[b] * wz[c];
    if (w != 0.0f) atomicAdd(g + (size_t)xs[a] + (size_t)ys[b] * sy + (size_t)zs[c] * sz, mul4(lam, w));
  }
}

// =====================================================================================================
// adv1 (src/sim.js:142-157): velX = mix(wind, vel(bt), fade), SX = S(bt) fade, S2X = S2(bt) fade with
// bt = c - vel(mid) dt/dx, mid = c - vel(c) dt/(2 dx).
__global__ void __launch_bounds__(256) k_adv1_adj(const float* __restrict__ P, TapeStep T, AdjFields a, Dims d) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
  const float4 lvX = a.velX[ci], lSX = a.SX[ci], lS2X = a.S2X[ci];
  if (!nz4(lvX) && !nz4(lSX) && !nz4(lS2X)) return;
  const float dt = __ldg(P + P_dt), dx = __ldg(P + P_dx);
  const Fields& f = T.f;
  const f3 c = mk3((float)id.i + 0.5f, (float)id.j + 0.5f, (float)id.k + 0.5f);
  const f3 v0 = xyz(__ldg(f.vel + ci));
  const f3 mid = c - v0 * (0.5f * dt) / dx;
  const Tap tm = make_tap(mid, d);
  const SampleD sm = sample_d(f.vel, tm, d);
  const f3 bt = c - xyz(sm.v) * dt / dx;
  const Tap tb = make_tap(bt, d);
  const float fade = outside_fade(bt, d);
  const float ws = sstep(0.03f, 0.4f, bt.y * dx);
  const float windX = __ldg(P + P_windX), windZ = __ldg(P + P_windZ);
  const f3 wind = mk3(windX * ws, 0.0f * ws, windZ * ws);
  const SampleD sv = sample_d(f.vel, tb, d);
  const SampleD sS = sample_d(f.S, tb, d);
  const SampleD sS2 = sample_d(f.S2, tb, d);
  // velX = wind (1 - fade) + sv fade;  SX = sS fade;  S2X = sS2 fade
  const f3 lv = xyz(lvX);
  const f3 lsv = lv * fade;
  const float4 lsS = mul4(lSX, fade), lsS2 = mul4(lS2X, fade);
  const float lfade = dot3(lv, xyz(sv.v) - wind) + dot4(lSX, sS.v) + dot4(lS2X, sS2.v);
  const float lws = (lv.x * windX + lv.z * windZ) * (1.0f - fade);
  scatter_tap(a.vel, tb, d, f4(lsv, 0.0f));
  scatter_tap(a.S, tb, d, lsS);
  scatter_tap(a.S2, tb, d, lsS2);
  f3 lbt = outside_fade_grad(bt, d) * lfade + pos_cot3(sv, lsv) + pos_cot(sS, lsS) + pos_cot(sS2, lsS2);
  lbt.y += lws * dsstep(0.03f, 0.4f, bt.y * dx) * dx;
  const f3 lv1 = lbt * (-dt / dx);
  scatter_tap(a.vel, tm, d, f4(lv1, 0.0f));
  const f3 lmid = pos_cot3(sm, lv1);
  atomic_add4(a.vel + ci, f4(lmid * (-0.5f * dt / dx), 0.0f));
}

// =====================================================================================================
// adv2 (src/sim.js:159-197).  For one channel: x = H + (own - hat(fw)) / 2 (or H if the back-trace left
// the domain), r = clamp(x, min(mn, H), max(mx, H)), out = r (velocity) or max(r, 0) (scalars).
struct LimCh {
  float lH, lown, lsamp;   // cotangents of the own hat, the own input value, the forward-traced hat sample
};
// Routes the cotangent `lr` of r through the limiter; a texel branch adds straight into the input field.
__device__ __forceinline__ LimCh limiter_adj(float lr, float x, float H, float mn, float mx, bool revert, float4* __restrict__ gin,
                                             int ch, const float4* __restrict__ fin, int b0x, int b0y, int b0z, Dims d) {
  LimCh o{0.0f, 0.0f, 0.0f};
  if (lr == 0.0f) return o;
  const float lo = fminf(mn, H), hi = fmaxf(mx, H);
  int texelMode = 0;   // 1: argmin texel, 2: argmax texel
  if (fmaxf(x, lo) > hi) {
    if (mx > H) texelMode = 2; else o.lH = lr;
  } else if (x < lo) {
    if (mn < H) texelMode = 1; else o.lH = lr;
  } else {
    o.lH = lr;
    if (!revert) { o.lown = 0.5f * lr; o.lsamp = -0.5f * lr; }
  }
  if (texelMode) {
    const float target = texelMode == 1 ? mn : mx;
    for (int q = 0; q < 8; ++q) {
      const int qx = min(max(b0x + (q & 1), 0), d.nx - 1);
      const int qy = min(max(b0y + ((q >> 1) & 1), 0), d.ny - 1);
      const int qz = min(max(b0z + ((q >> 2) & 1), 0), d.nz - 1);
      const size_t t = cell(qx, qy, qz, d.nx, d.ny);
      const float4 v = __ldg(fin + t);
      const float val = ch == 0 ? v.x : ch == 1 ? v.y : ch == 2 ? v.z : v.w;
      if (val == target) { atomicAdd(reinterpret_cast<float*>(gin + t) + ch, lr); break; }
    }
  }
  return o;
}
__device__ __forceinline__ float ch4(float4 v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }
__device__ __forceinline__ void set4(float4& v, int c, float s) { if (c == 0) v.x = s; else if (c == 1) v.y = s; else if (c == 2) v.z = s; else v.w = s; }

__global__ void __launch_bounds__(256) k_adv2_adj(const float* __restrict__ P, TapeStep T, AdjFields a, Dims d) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
  const float4 lY = a.velY[ci], lSY = a.SY[ci], lS2Y = a.S2Y[ci];
  if (!nz4(lY) && !nz4(lSY) && !nz4(lS2Y)) return;
  const float dt = __ldg(P + P_dt), dx = __ldg(P + P_dx);
  const Fields& f = T.f;
  const f3 c = mk3((float)id.i + 0.5f, (float)id.j + 0.5f, (float)id.k + 0.5f);
  const f3 v = xyz(__ldg(f.vel + ci));
  const f3 fw = c + v * dt / dx;
  const Tap tf = make_tap(fw, d);
  const float4 vH = __ldg(f.velX + ci), sH = __ldg(f.SX + ci), s2H = __ldg(f.S2X + ci);
  const SampleD hv = sample_d(f.velX, tf, d), hs = sample_d(f.SX, tf, d), hs2 = sample_d(f.S2X, tf, d);
  const float4 sOwn = __ldg(f.S + ci), s2Own = __ldg(f.S2 + ci);
  const f3 vN3 = xyz(vH) + (v - xyz(hv.v)) * 0.5f;
  const float4 sN = add4(sH, mul4(sub4(sOwn, hs.v), 0.5f));
  const float4 s2N = add4(s2H, mul4(sub4(s2Own, hs2.v), 0.5f));
  const f3 bt = backtrace(f.vel, c, v, dt, dx, d);
  const f3 b = mk3(bt.x - 0.5f, bt.y - 0.5f, bt.z - 0.5f);
  const int b0x = (int)floorf(clampf(b.x, -2.0f, (float)(d.nx + 1)));
  const int b0y = (int)floorf(clampf(b.y, -2.0f, (float)(d.ny + 1)));
  const int b0z = (int)floorf(clampf(b.z, -2.0f, (float)(d.nz + 1)));
  float4 vmn = make_float4(1e9f, 1e9f, 1e9f, 1e9f), vmx = make_float4(-1e9f, -1e9f, -1e9f, -1e9f);
  float4 smn = vmn, smx = vmx, tmn = vmn, tmx = vmx;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int qx = b0x + (q & 1), qy = b0y + ((q >> 1) & 1), qz = b0z + ((q >> 2) & 1);
    const float4 vv = ldc(f.vel, qx, qy, qz, d), ss = ldc(f.S, qx, qy, qz, d), tt = ldc(f.S2, qx, qy, qz, d);
    vmn = fmin4(vmn, vv); vmx = fmax4(vmx, vv);
    smn = fmin4(smn, ss); smx = fmax4(smx, ss);
    tmn = fmin4(tmn, tt); tmx = fmax4(tmx, tt);
  }
  const bool revert = outside_fade(mk3(b.x + 0.5f, b.y + 0.5f, b.z + 0.5f), d) < 1.0f;
  float4 lHv = make_float4(0, 0, 0, 0), lHs = lHv, lHs2 = lHv, lOv = lHv, lOs = lHv, lOs2 = lHv, lSv = lHv, lSs = lHv, lSs2 = lHv;
  const float4 vN = f4(vN3, 0.0f);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float H = ch4(vH, ch), x = revert ? H : ch4(vN, ch);
    const LimCh o = limiter_adj(ch4(lY, ch), x, H, ch4(vmn, ch), ch4(vmx, ch), revert, a.vel, ch, f.vel, b0x, b0y, b0z, d);
    set4(lHv, ch, o.lH); set4(lOv, ch, o.lown); set4(lSv, ch, o.lsamp);
  }
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    {
      const float H = ch4(sH, ch), x = revert ? H : ch4(sN, ch);
      const float r = fminf(fmaxf(x, fminf(ch4(smn, ch), H)), fmaxf(ch4(smx, ch), H));
      const float lr = r > 0.0f ? ch4(lSY, ch) : 0.0f;
      const LimCh o = limiter_adj(lr, x, H, ch4(smn, ch), ch4(smx, ch), revert, a.S, ch, f.S, b0x, b0y, b0z, d);
      set4(lHs, ch, o.lH); set4(lOs, ch, o.lown); set4(lSs, ch, o.lsamp);
    }
    {
      const float H = ch4(s2H, ch), x = revert ? H : ch4(s2N, ch);
      const float r = fminf(fmaxf(x, fminf(ch4(tmn, ch), H)), fmaxf(ch4(tmx, ch), H));
      const float lr = r > 0.0f ? ch4(lS2Y, ch) : 0.0f;
      const LimCh o = limiter_adj(lr, x, H, ch4(tmn, ch), ch4(tmx, ch), revert, a.S2, ch, f.S2, b0x, b0y, b0z, d);
      set4(lHs2, ch, o.lH); set4(lOs2, ch, o.lown); set4(lSs2, ch, o.lsamp);
    }
  }
  // forward-traced hat samples: values and position fw = c + v dt/dx
  scatter_tap(a.velX, tf, d, lSv);
  scatter_tap(a.SX, tf, d, lSs);
  scatter_tap(a.S2X, tf, d, lSs2);
  const f3 lfw = pos_cot3(hv, xyz(lSv)) + pos_cot(hs, lSs) + pos_cot(hs2, lSs2);
  atomic_add4(a.velX + ci, lHv);
  atomic_add4(a.SX + ci, lHs);
  atomic_add4(a.S2X + ci, lHs2);
  atomic_add4(a.vel + ci, f4(xyz(lOv) + lfw * (dt / dx), 0.0f));
  atomic_add4(a.S + ci, lOs);
  atomic_add4(a.S2 + ci, lOs2);
}

// =====================================================================================================
// forces (src/sim.js:214-396): the forward of fire_step.cu's forces_cell is recomputed with every
// intermediate kept, then reversed statement by statement.  Returns the cotangent of the spot sum `acc`
// (zero when the spot branch was not the one taken).
__device__ __forceinline__ float forces_adj_cell(const float* __restrict__ P, const TapeStep& Tp, const AdjFields& a,
                                                 const uint2* __restrict__ noiseT, const uint2* __restrict__ curlT, Dims d,
                                                 int i, int j, int k, f3& pos) {
  const Fields& f = Tp.f;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float dt = __ldg(P + P_dt), dx = __ldg(P + P_dx), I = __ldg(P + P_intensity);
  const float seed = __ldg(P + P_seed), time = __ldg(P + P_time);
  const float* E = P + P_STRIDE;
  const f3 p = mk3(__ldg(P + P_ox), __ldg(P + P_oy), __ldg(P + P_oz)) + mk3((float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f) * dx;
  pos = p;
  const float4 v4 = __ldg(f.velY + ci), sIn = __ldg(f.SY + ci), s2In = __ldg(f.S2Y + ci), geo = __ldg(f.geo + ci);
  const float4 lF = a.F[ci], lSo = a.S[ci], lS2o = a.S2[ci];

  // ------------------------------------------------ forward recompute
  float src = 0.0f, anchor = 0.0f;
  if (geo.x > 0.001f) {
    f3 qa = p * __ldg(P + P_anchorFreq) + mk3(seed * 0.37f, 0.0f, 0.11f);
    anchor = sstep(-0.05f, 0.25f, noise4(noiseT, qa).z);
    f3 qn = p * (__ldg(P + P_srcFreq) * 0.06f) + mk3(seed * 0.131f, 0.0f, time * __ldg(P + P_srcSpeed));
    const float th = __ldg(P + P_srcThresh);
    float pulse = sstep(th - 0.25f, th + 0.25f, noise4(noiseT, qn).x);
    src = clampf(geo.x * __ldg(P + P_logSrc) * (__ldg(P + P_srcFloor) + __ldg(P + P_anchorGain) * anchor) * mixf(0.55f, 1.0f, pulse) * 1.2f,
                 0.0f, 1.0f) * I;
    src *= 1.0f - geo.z;
  }
  const int nSpots = (int)__ldg(E + E_nSpots);
  float acc = 0.0f;
  bool spotOn = false;
  if (nSpots > 0 && p.y < __ldg(E + E_spotTop)) {
    const float spotRef = __ldg(E + E_spotRef);
    for (int q = 0; q < nSpots; ++q) {
      const float* sp = E + E_SPOTS + SPOT_STRIDE * q;
      f3 dd = p - mk3(__ldg(sp + 0), __ldg(sp + 1), __ldg(sp + 2));
      float sg = __ldg(sp + 3);
      float d2 = dot3(dd, dd);
      if (d2 < 16.0f * sg * sg) acc += (__ldg(sp + 4) / spotRef) * expf(-d2 / (2.0f * sg * sg));
    }
    const float sv = clampf(acc, 0.0f, 1.0f) * I;
    spotOn = sv > src;
    src = fmaxf(src, sv);
  }
  const float srcW = fminf(src, 1.0f);
  const float bedHot = geo.y;
  float bed = geo.y * clampf(I * 1.4f, 0.3f, 1.0f);
  if (bed > 0.001f) {
    f3 qb = p * 2.4f + mk3(0.17f, -time * 0.12f, time * 0.05f);
    bed *= sstep(0.0f, 0.3f, noise4(noiseT, qb).y);
  }
  const float fuelSrc = __ldg(P + P_fuelSrc), srcTemp = __ldg(P + P_srcTemp);
  const float cFuel = src * fuelSrc, cBedF = bed * __ldg(P + P_bedFuel);
  const float cTemp = src * srcTemp, cBedT = bedHot * __ldg(P + P_bedTemp);
  const float sy0 = sIn.y, sx0 = sIn.x;
  const float sy1 = fmaxf(sy0, cFuel), sy2 = fmaxf(sy1, cBedF);
  const float sx1 = fmaxf(sx0, cTemp), sx2 = fmaxf(sx1, cBedT);
  const float srcAll = fmaxf(srcW, bed);
  const float t1 = bed * (1.0f - srcW);
  const float w0 = s2In.w, w1 = mixf(w0, 1.0f, t1), w2 = mixf(w1, 0.0f, srcW);
  const float y0 = s2In.y, y1 = y0 * (1.0f - srcAll);
  const float x0 = s2In.x;
  const float r1 = (1.0f - sy2) * srcW, x1 = fmaxf(x0, r1);
  const float r2 = (1.0f - sy2) * bed * 0.6f, x2 = fmaxf(x1, r2);
  const float wsaRaw = srcW + bed * 0.4f, wsa = clampf(wsaRaw, 0.0f, 1.0f);
  const float pw = dt * 90.0f;
  const float wsrc = wsa > 0.0f ? 1.0f - powf(1.0f - wsa * 0.5f, pw) : 0.0f;
  const float vy0 = v4.y, srcVel = __ldg(P + P_srcVel);
  const float mv = fmaxf(vy0, srcVel);
  const float vy1 = mixf(vy0, mv, wsrc);
  const float z1 = s2In.z + geo.x * (1.0f - anchor) * __ldg(P + P_smolder) * dt * I;
  const float burstAmt = __ldg(P + P_burstAmt);
  float bw = 0.0f, sy3 = sy2, sx3 = sx2, x3 = x2, w3 = w2, y2 = y1, bsum = 0.0f, brhs = 0.0f;
  if (burstAmt > 0.0f) {
    float bd = len3(p - mk3(__ldg(P + P_burstX), __ldg(P + P_burstY), __ldg(P + P_burstZ)));
    bw = clampf(expf(-bd * bd / 0.006f) * burstAmt, 0.0f, 1.0f);
    sy3 = fmaxf(sy2, 0.17f * bw);
    sx3 = fmaxf(sx2, 0.9f * bw);
    x3 = x2 * (1.0f - bw);
    w3 = w2 * (1.0f - bw);
    bsum = sy3 + x3;
    brhs = 0.05f * bw * clampf(bsum, 0.0f, 1.0f);
    y2 = fmaxf(y1, brhs);
  }
  const float ageDen = fmaxf(sy3 + x3, 1e-4f);
  const float ageF = y2 / ageDen;
  const float T0 = 293.0f + 1000.0f * sx3;
  const float oRaw = 1.0f - sy3 - x3, o = clampf(oRaw, 0.0f, 1.0f);
  const float ignT = __ldg(P + P_ignT), rs = __ldg(P + P_rs), kMix = __ldg(P + P_kMix);
  const float ign = sstep(ignT - 50.0f, ignT + 50.0f, T0);
  const float ex = expf(-kMix * ign * dt), Ek = 1.0f - ex;
  const float orat = o / rs, bm = fminf(sy3, orat), bb = bm * Ek;
  const float x4raw = x3 + (1.0f + rs) * bb, x4 = fminf(x4raw, 1.0f);
  const float heatOut = __ldg(P + P_heatOut);
  const float limRaw = 2100.0f - T0, lim = fmaxf(limRaw, 0.0f);
  const float hb = heatOut * bb, dT = fminf(hb, lim);
  const float T1 = T0 + dT;
  const float q = dT / dt;
  const float expn = __ldg(P + P_expansion);
  const bool solid = geo.z > 0.5f;
  const float phiRaw = expn * q / T1;
  const float sootOx = __ldg(P + P_sootOx), sootForm = __ldg(P + P_sootForm);
  const float ageF2raw = ageF + dt, ageF2 = fminf(ageF2raw, 4.0f);
  const float a0 = __ldg(E + E_sootAge0), a1 = __ldg(E + E_sootAge1);
  const float gA = sstep(a0, a1, ageF2), gT = sstep(1000.0f, 1400.0f, T1);
  const float sz1 = sIn.z + sootForm * bb * gA * gT * (1.0f - w3);
  const float sk = sstep(1100.0f, 1400.0f, T1);
  const float k1 = expf(-sootOx * (0.25f + o) * sk * dt);
  const float sz2 = sz1 * k1;
  const float h1 = sstep(850.0f, 1100.0f, T1), h2 = sstep(1100.0f, 1300.0f, T1);
  const float k2 = expf(-sootOx * 0.5f * o * h1 * (1.0f - h2) * dt);
  const float sz3 = sz2 * k2;
  const float dSoot = __ldg(E + E_decaySoot);
  const float sz4 = sz3 * dSoot;
  const float th = T1 * 0.001f, radCool = __ldg(P + P_radCool);
  const float radRaw = radCool * 970.0f * sz4 * th * th * (th * th * th * th - 0.00737f);
  const float rad = fminf(radRaw, 6000.0f);
  const float T2 = T1 - rad * dt;
  const float coolRate = __ldg(P + P_coolRate);
  const float nbq = 1.0f - sstep(500.0f, 5000.0f, q);
  const float ec = expf(-coolRate * nbq * dt);
  const float T2m = T2 - 293.0f;
  const float T3 = 293.0f + fmaxf(T2m, 0.0f) * ec;
  const float sx5 = (T3 - 293.0f) * 0.001f, sw = q * 1e-4f;
  const float dFuel = __ldg(E + E_decayFuel), dVit = __ldg(E + E_decayVit), dSmoke = __ldg(E + E_decaySmoke);
  const float sy4 = sy3 - bb;
  const float sy5 = sy4 * dFuel, x5 = x4 * dVit, z2 = z1 * dSmoke;
  const float clS = sy5 + x5, cl = clampf(clS, 0.0f, 1.0f);
  const float y3 = ageF2 * cl;
  const float buoy = __ldg(P + P_buoyancy);
  f3 v = mk3(v4.x, vy1 + buoy * sx5 * dt, v4.z);
  const float visc = __ldg(P + P_visc);
  f3 lapV = mk3(0.0f, 0.0f, 0.0f);
  float nu = 0.0f, kvRaw = 0.0f, kv = 0.0f;
  if (visc > 0.0f) {
    f3 l = xyz(ldc(f.velY, i + 1, j, k, d)) + xyz(ldc(f.velY, i - 1, j, k, d));
    l = l + xyz(ldc(f.velY, i, j + 1, k, d));
    l = l + xyz(ldc(f.velY, i, j - 1, k, d));
    l = l + xyz(ldc(f.velY, i, j, k + 1, d));
    l = l + xyz(ldc(f.velY, i, j, k - 1, d));
    lapV = l - xyz(v4) * 6.0f;
    nu = visc * 1.5e-5f * powf(fmaxf(T3, 293.0f) / 293.0f, 1.7f);
    kvRaw = nu * dt / (dx * dx);
    kv = fminf(kvRaw, 0.15f);
    v = v + lapV * kv;
  }
  const float lamAge = __ldg(P + P_lamAge);
  const float lamE1 = fmaxf(lamAge, 1e-3f);
  const float lam = lamAge > 0.0f ? sstep(0.5f * lamAge, lamE1, ageF2) : 1.0f;
  const float4 wc4 = curl_at(f.velY, i, j, k, d);
  const f3 wc = xyz(wc4);
  const f3 g = mk3(curl_at(f.velY, min(i + 1, d.nx - 1), j, k, d).w - curl_at(f.velY, max(i - 1, 0), j, k, d).w,
                   curl_at(f.velY, i, min(j + 1, d.ny - 1), k, d).w - curl_at(f.velY, i, max(j - 1, 0), k, d).w,
                   curl_at(f.velY, i, j, min(k + 1, d.nz - 1), d).w - curl_at(f.velY, i, j, max(k - 1, 0), d).w);
  const float gl = len3(g);
  const float vortEps = __ldg(P + P_vortEps);
  const float sG = sstep(450.0f, 900.0f, T3), sYp = sstep(0.02f, 0.08f, p.y);
  f3 nrm = mk3(0.0f, 0.0f, 0.0f), cr = nrm;
  float gate = 0.0f;
  if (gl > 1e-6f) {
    gate = sG * (1.0f - srcAll) * sYp * lam;
    nrm = g / gl;
    cr = cross3(nrm, wc);
    v = v + cr * (vortEps * gate) * dt;
  }
  const float turbAmp = __ldg(P + P_turbAmp);
  f3 tq = (p - mk3(0.0f, time * __ldg(P + P_turbRise), 0.0f)) * __ldg(P + P_turbFreq) + mk3(0.0f, 0.0f, time * __ldg(P + P_turbEvolve));
  const f3 cn = xyz(sample_table(curlT, tq));
  const float sA = sstep(500.0f, 1100.0f, T3), sB = sstep(0.0f, 3.0f, sw);
  const float tg1 = fmaxf(sA, sB);
  const float mixc = mixf(0.6f, 1.8f, sstep(0.2f, 0.75f, p.y));
  const float tgate = tg1 * (1.0f - srcAll) * mixc * lam;
  v = v + cn * (turbAmp / 12.0f) * tgate * dt * 10.0f;
  const float windX = __ldg(P + P_windX), windZ = __ldg(P + P_windZ);
  const float windK = sstep(0.05f, 0.5f, p.y) * (1.0f + __ldg(P + P_gust));
  v.x += (windX * windK - v.x) * dt * 0.35f * windK;
  v.z += (windZ * windK - v.z) * dt * 0.35f * windK;
  const float dVel = __ldg(E + E_decayVel);
  v = v * dVel;
  if (solid) v = mk3(0.0f, 0.0f, 0.0f);
  const f3 fp = mk3((float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f);
  const float side = fminf(fminf(fp.x, (float)d.nx - fp.x), fminf(fp.z, (float)d.nz - fp.z));
  const float spc = clampf((1.0f - sstep(0.0f, 5.0f, side)) * __ldg(P + P_sponge), 0.0f, 1.0f);
  const float ks = spc > 0.0f ? 1.0f - powf(1.0f - 0.15f * spc, dt * 90.0f) : 0.0f;
  const float wsy = sstep(0.03f, 0.4f, p.y);
  v.x = mixf(v.x, windX * wsy, ks);
  v.z = mixf(v.z, windZ * wsy, ks);
  const float top = sstep((float)d.ny - 10.0f, (float)d.ny, fp.y);
  const float kt = top > 0.0f ? powf(1.0f - 0.1f * top, dt * 90.0f) : 1.0f;
  const f3 vPre = v;
  const float vl = len3(v);
  const float sz5 = sz4 * kt, z3 = z2 * kt;
  bool bad = isnan(sx5) || isnan(solid ? 0.0f : sy5) || isnan(sz5) || isnan(sw) || isnan(x5) || isnan(solid ? 0.0f : y3) ||
             isnan(z3) || isnan(w3) || isnan(vPre.x) || isnan(vPre.y) || isnan(vPre.z);
  if (bad) {   // the forward wrote zeros: no dependence on any input
    a.SY[ci] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    a.S2Y[ci] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return 0.0f;
  }

  // ------------------------------------------------ reverse
  f3 lv = xyz(lF);
  const float lphi = lF.w;
  float lsx5 = lSo.x, lsy5 = lSo.y, lsz5 = lSo.z, lsw = lSo.w;
  float lx5 = lS2o.x, ly3 = lS2o.y, lz3 = lS2o.z, lw3 = lS2o.w;
  if (vl > 15.0f) {
    const f3 u = vPre / vl;
    lv = (lv - u * dot3(u, lv)) * (15.0f / vl);
  }
  const float lsz4a = lsz5 * kt;
  const float lz2 = lz3 * kt;
  lv.x *= 1.0f - ks;
  lv.z *= 1.0f - ks;
  if (solid) { lv = mk3(0.0f, 0.0f, 0.0f); lsy5 = 0.0f; ly3 = 0.0f; }
  lv = lv * dVel;
  lv.x *= 1.0f - dt * 0.35f * windK;
  lv.z *= 1.0f - dt * 0.35f * windK;
  // turbulence
  const float ltgate = dot3(lv, cn) * (turbAmp / 12.0f) * dt * 10.0f;
  float lsrcAll = -ltgate * tg1 * mixc * lam;
  float llam = ltgate * tg1 * (1.0f - srcAll) * mixc;
  const float ltg1 = ltgate * (1.0f - srcAll) * mixc * lam;
  float lT3 = 0.0f;
  if (sA >= sB) lT3 += ltg1 * dsstep(500.0f, 1100.0f, T3); else lsw += ltg1 * dsstep(0.0f, 3.0f, sw);
  // vorticity confinement
  f3 lwc = mk3(0.0f, 0.0f, 0.0f), lg = lwc;
  if (gl > 1e-6f) {
    const f3 lcr = lv * (vortEps * gate * dt);
    const float lgate = dot3(lv, cr) * vortEps * dt;
    const f3 ln = cross3(wc, lcr);
    lwc = cross3(lcr, nrm);
    lg = (ln - nrm * dot3(nrm, ln)) / gl;
    lT3 += lgate * dsstep(450.0f, 900.0f, T3) * (1.0f - srcAll) * sYp * lam;
    lsrcAll -= lgate * sG * sYp * lam;
    llam += lgate * sG * (1.0f - srcAll) * sYp;
  }
  float lageF2 = lamAge > 0.0f ? llam * dsstep(0.5f * lamAge, lamE1, ageF2) : 0.0f;
  // viscosity
  f3 llap = mk3(0.0f, 0.0f, 0.0f);
  if (visc > 0.0f) {
    llap = lv * kv;
    if (kvRaw < 0.15f && T3 > 293.0f) lT3 += dot3(lv, lapV) * (dt / (dx * dx)) * nu * 1.7f / T3;
  }
  // buoyancy
  lsx5 += lv.y * buoy * dt;
  const float lvy1 = lv.y;
  // scalar outputs
  lageF2 += ly3 * cl;
  const float lcl = ly3 * ageF2;
  if (in01(clS)) { lsy5 += lcl; lx5 += lcl; }
  const float lz1 = lz2 * dSmoke;
  const float lx4 = lx5 * dVit;
  const float lsy4 = lsy5 * dFuel;
  float lq = lsw * 1e-4f;
  lT3 += lsx5 * 0.001f;
  // cooling
  float lT2 = 0.0f, lec = 0.0f;
  if (T2m > 0.0f) { lT2 = lT3 * ec; lec = lT3 * T2m; }
  const float lnb = lec * ec * (-coolRate * dt);
  lq -= lnb * dsstep(500.0f, 5000.0f, q);
  float lT1 = lT2;
  const float lrad = -lT2 * dt;
  float lsz4 = lsz4a;
  if (radRaw < 6000.0f) {
    const float c = radCool * 970.0f;
    const float th4 = th * th * th * th;
    lsz4 += lrad * c * th * th * (th4 - 0.00737f);
    lT1 += lrad * c * sz4 * (6.0f * th4 * th - 2.0f * 0.00737f * th) * 0.001f;
  }
  // soot
  const float lsz3 = lsz4 * dSoot;
  const float lsz2 = lsz3 * k2;
  const float larg2 = lsz3 * sz2 * k2;
  float lo = larg2 * (-sootOx * 0.5f * h1 * (1.0f - h2) * dt);
  lT1 += larg2 * (-sootOx * 0.5f * o * (1.0f - h2) * dt) * dsstep(850.0f, 1100.0f, T1);
  lT1 += larg2 * (sootOx * 0.5f * o * h1 * dt) * dsstep(1100.0f, 1300.0f, T1);
  const float lsz1 = lsz2 * k1;
  const float larg1 = lsz2 * sz1 * k1;
  lo += larg1 * (-sootOx * sk * dt);
  lT1 += larg1 * (-sootOx * (0.25f + o) * dt) * dsstep(1100.0f, 1400.0f, T1);
  const float lsz0 = lsz1;
  float lbb = lsz1 * sootForm * gA * gT * (1.0f - w3);
  lageF2 += lsz1 * sootForm * bb * gT * (1.0f - w3) * dsstep(a0, a1, ageF2);
  lT1 += lsz1 * sootForm * bb * gA * (1.0f - w3) * dsstep(1000.0f, 1400.0f, T1);
  lw3 -= lsz1 * sootForm * bb * gA * gT;
  const float lageF = ageF2raw < 4.0f ? lageF2 : 0.0f;
  // expansion target
  if (!solid && phiRaw < 60.0f) { lq += lphi * expn / T1; lT1 -= lphi * phiRaw / T1; }
  // combustion
  const float ldT = lT1 + lq / dt;
  float lT0 = lT1;
  if (hb <= lim) lbb += ldT * heatOut; else if (limRaw > 0.0f) lT0 -= ldT;
  float lx3 = 0.0f;
  if (x4raw < 1.0f) { lx3 += lx4; lbb += lx4 * (1.0f + rs); }
  float lsy3 = lsy4;
  lbb -= lsy4;
  const float lbm = lbb * Ek;
  const float lEk = lbb * bm;
  lT0 += lEk * ex * kMix * dt * dsstep(ignT - 50.0f, ignT + 50.0f, T0);
  if (sy3 <= orat) lsy3 += lbm; else lo += lbm / rs;
  if (in01(oRaw)) { lsy3 -= lo; lx3 -= lo; }
  const float lsx3 = 1000.0f * lT0;
  const float ly2 = lageF / ageDen;
  if (sy3 + x3 > 1e-4f) { const float lden = -lageF * ageF / ageDen; lsy3 += lden; lx3 += lden; }
  // burst
  float lsy2, lsx2, lx2, lw2, ly1;
  if (burstAmt > 0.0f) {
    if (y1 >= brhs) ly1 = ly2;
    else {
      ly1 = 0.0f;
      const float lc = ly2 * 0.05f * bw;
      if (in01(bsum)) { lsy3 += lc; lx3 += lc; }
    }
    lw2 = lw3 * (1.0f - bw);
    lx2 = lx3 * (1.0f - bw);
    lsx2 = sx2 >= 0.9f * bw ? lsx3 : 0.0f;
    lsy2 = sy2 >= 0.17f * bw ? lsy3 : 0.0f;
  } else {
    ly1 = ly2; lw2 = lw3; lx2 = lx3; lsx2 = lsx3; lsy2 = lsy3;
  }
  // sources
  const float lvy0 = lvy1 * (1.0f - wsrc) + (vy0 >= srcVel ? lvy1 * wsrc : 0.0f);
  const float lwsrc = lvy1 * (mv - vy0);
  float lsrcW = 0.0f;
  if (wsa > 0.0f && wsaRaw < 1.0f) lsrcW += lwsrc * pw * powf(1.0f - wsa * 0.5f, pw - 1.0f) * 0.5f;
  float lx1 = 0.0f;
  if (x1 >= r2) lx1 = lx2; else lsy2 -= lx2 * bed * 0.6f;
  float lx0 = 0.0f;
  if (x0 >= r1) lx0 = lx1; else { lsy2 -= lx1 * srcW; lsrcW += lx1 * (1.0f - sy2); }
  const float ly0 = ly1 * (1.0f - srcAll);
  lsrcAll -= ly1 * y0;
  const float lw1 = lw2 * (1.0f - srcW);
  lsrcW -= lw2 * w1;
  const float lw0 = lw1 * (1.0f - t1);
  lsrcW -= lw1 * (1.0f - w0) * bed;
  if (srcW >= bed) lsrcW += lsrcAll;
  float lsrc = 0.0f;
  const float lsx1 = sx1 >= cBedT ? lsx2 : 0.0f;
  float lsx0 = 0.0f;
  if (sx0 >= cTemp) lsx0 = lsx1; else lsrc += lsx1 * srcTemp;
  const float lsy1 = sy1 >= cBedF ? lsy2 : 0.0f;
  float lsy0 = 0.0f;
  if (sy0 >= cFuel) lsy0 = lsy1; else lsrc += lsy1 * fuelSrc;
  if (src < 1.0f) lsrc += lsrcW;
  const float lacc = (spotOn && in01(acc)) ? lsrc * I : 0.0f;

  // ------------------------------------------------ input cotangents
  a.SY[ci] = make_float4(lsx0, lsy0, lsz0, 0.0f);
  a.S2Y[ci] = make_float4(lx0, ly0, lz1, lw0);
  float4 lc = make_float4(lv.x, lvy0, lv.z, 0.0f);
  if (visc > 0.0f) {
    lc = sub4(lc, f4(llap * 6.0f, 0.0f));
    const float4 l4 = f4(llap, 0.0f);
    atomic_add4(a.velY + cell(min(i + 1, d.nx - 1), j, k, d.nx, d.ny), l4);
    atomic_add4(a.velY + cell(max(i - 1, 0), j, k, d.nx, d.ny), l4);
    atomic_add4(a.velY + cell(i, min(j + 1, d.ny - 1), k, d.nx, d.ny), l4);
    atomic_add4(a.velY + cell(i, max(j - 1, 0), k, d.nx, d.ny), l4);
    atomic_add4(a.velY + cell(i, j, min(k + 1, d.nz - 1), d.nx, d.ny), l4);
    atomic_add4(a.velY + cell(i, j, max(k - 1, 0), d.nx, d.ny), l4);
  }
  atomic_add4(a.velY + ci, lc);
  atomic_add4(a.W + ci, f4(lwc, 0.0f));
  if (lg.x != 0.0f) {
    atomicAdd(&a.W[cell(min(i + 1, d.nx - 1), j, k, d.nx, d.ny)].w, lg.x);
    atomicAdd(&a.W[cell(max(i - 1, 0), j, k, d.nx, d.ny)].w, -lg.x);
  }
  if (lg.y != 0.0f) {
    atomicAdd(&a.W[cell(i, min(j + 1, d.ny - 1), k, d.nx, d.ny)].w, lg.y);
    atomicAdd(&a.W[cell(i, max(j - 1, 0), k, d.nx, d.ny)].w, -lg.y);
  }
  if (lg.z != 0.0f) {
    atomicAdd(&a.W[cell(i, j, min(k + 1, d.nz - 1), d.nx, d.ny)].w, lg.z);
    atomicAdd(&a.W[cell(i, j, max(k - 1, 0), d.nx, d.ny)].w, -lg.z);
  }
  return lacc;
}

// Pass 1 of the forces adjoint: per-cell reverse, then the spot-flux cotangents reduced per warp.  Consumes
// the output cotangents (S, S2 are zeroed for the advection adjoints that accumulate into them next) and
// clears the hat cotangents the advection adjoints accumulate into.
__global__ void __launch_bounds__(256) k_forces_adj1(const float* __restrict__ P, TapeStep T, AdjFields a, const uint2* __restrict__ noiseT,
                                                     const uint2* __restrict__ curlT, Dims d, int consume) {
  const ACell id = acell(d);
  float lacc = 0.0f;
  f3 p = mk3(0.0f, 0.0f, 0.0f);
  if (id.ok) {
    lacc = forces_adj_cell(P, T, a, noiseT, curlT, d, id.i, id.j, id.k, p);
    if (consume) {
      const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
      const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      a.S[ci] = z; a.S2[ci] = z; a.velX[ci] = z; a.SX[ci] = z; a.S2X[ci] = z;
    }
  }
  // d acc / d flux_q = G_q / spotRef  (G_q the Gaussian of spot q at this cell, 0 beyond 4 sigma)
  if (!__any_sync(0xffffffffu, lacc != 0.0f)) return;
  const float* E = P + P_STRIDE;
  const int nSpots = (int)__ldg(E + E_nSpots);
  const float spotRef = __ldg(E + E_spotRef);
  for (int q = 0; q < nSpots; ++q) {
    float c = 0.0f;
    if (lacc != 0.0f) {
      const float* sp = E + E_SPOTS + SPOT_STRIDE * q;
      f3 dd = p - mk3(__ldg(sp + 0), __ldg(sp + 1), __ldg(sp + 2));
      float sg = __ldg(sp + 3);
      float d2 = dot3(dd, dd);
      if (d2 < 16.0f * sg * sg) c = lacc * expf(-d2 / (2.0f * sg * sg)) / spotRef;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c != 0.0f) atomicAdd(a.flux + q, (double)c);
  }
}
// Pass 2: vorticity cotangents (vector + magnitude) onto the 6 clamped velY neighbours of the curl stencil.
__global__ void __launch_bounds__(256) k_forces_adj2(TapeStep T, AdjFields a, Dims d) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float4 lW = a.W[ci];
  if (!nz4(lW)) return;
  f3 lw = xyz(lW);
  if (lW.w != 0.0f) {
    const float4 w = curl_at(T.f.velY, i, j, k, d);
    if (w.w > 0.0f) lw = lw + xyz(w) * (lW.w / w.w);
  }
  const f3 h = lw * 0.5f;
  atomic_add4(a.velY + cell(min(i + 1, d.nx - 1), j, k, d.nx, d.ny), make_float4(0.0f, h.z, -h.y, 0.0f));   // R
  atomic_add4(a.velY + cell(max(i - 1, 0), j, k, d.nx, d.ny), make_float4(0.0f, -h.z, h.y, 0.0f));          // L
  atomic_add4(a.velY + cell(i, min(j + 1, d.ny - 1), k, d.nx, d.ny), make_float4(-h.z, 0.0f, h.x, 0.0f));   // T
  atomic_add4(a.velY + cell(i, max(j - 1, 0), k, d.nx, d.ny), make_float4(h.z, 0.0f, -h.x, 0.0f));          // B
  atomic_add4(a.velY + cell(i, j, min(k + 1, d.nz - 1), d.nx, d.ny), make_float4(h.y, -h.x, 0.0f, 0.0f));   // F
  atomic_add4(a.velY + cell(i, j, max(k - 1, 0), d.nx, d.ny), make_float4(-h.y, h.x, 0.0f, 0.0f));          // K
}

// =====================================================================================================
// div (src/sim.js:399-413): b = ((R - L) + (T - B) + (F - K)) / (2 dx) - phi with clamped neighbours and
// B = -v.y on the floor row.  Its transpose gathers each cell's share of the neighbours' cotangents.
__global__ void __launch_bounds__(256) k_div_adj(const float* __restrict__ P, AdjFields a, Dims d) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float c = 1.0f / (2.0f * __ldg(P + P_dx));
  const float* lb = a.B;
  const float me = lb[ci];
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
  if (i > 0) gx += lb[ci - 1];                 // this cell is R of i-1
  if (i == d.nx - 1) gx += me;                 // R of itself (clamped)
  if (i < d.nx - 1) gx -= lb[ci + 1];          // L of i+1
  if (i == 0) gx -= me;                        // L of itself (clamped)
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  if (j > 0) gy += lb[ci - sy];                // T of j-1
  if (j == d.ny - 1) gy += me;                 // T of itself (clamped)
  if (j < d.ny - 1) gy -= lb[ci + sy];         // B of j+1
  if (j == 0) gy += me;                        // floor: B = -v.y of itself
  if (k > 0) gz += lb[ci - sz];
  if (k == d.nz - 1) gz += me;
  if (k < d.nz - 1) gz -= lb[ci + sz];
  if (k == 0) gz -= me;
  float4 F = a.F[ci];
  F.x += gx * c; F.y += gy * c; F.z += gz * c; F.w -= me;
  a.F[ci] = F;
}

// =====================================================================================================
// project (src/sim.js:526-550), pass 1: per-cell masks.  Writes the forces-output velocity cotangent (w = 0)
// and the masked cotangent G; consumes the state cotangent and clears the forces-adjoint accumulators.
__global__ void __launch_bounds__(256) k_proj_adj1(const float* __restrict__ P, TapeStep T, AdjFields a, Dims d, int consume) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const float4 lu4 = a.vel[ci];
  const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (consume) { a.vel[ci] = z; a.velY[ci] = z; a.W[ci] = z; }
  f3 lv = mk3(0.0f, 0.0f, 0.0f);
  if (!__ldg(T.f.solid + ci) && nz4(lu4)) {
    const float dx = __ldg(P + P_dx);
    const float* p0 = T.p;
    const float me = __ldg(p0 + ci);
    auto pr = [&](int x, int y, int zz) -> float {
      if (x < 0 || zz < 0 || x >= d.nx || zz >= d.nz || y >= d.ny) return -me;
      if (y < 0) return me;
      return __ldg(p0 + cell(x, y, zz, d.nx, d.ny));
    };
    const f3 g = mk3(pr(i + 1, j, k) - pr(i - 1, j, k), pr(i, j + 1, k) - pr(i, j - 1, k), pr(i, j, k + 1) - pr(i, j, k - 1)) / (2.0f * dx);
    const f3 v = xyz(__ldg(T.Fv + ci)) - g;
    f3 vf = v;
    if (j == 0) vf.y = fmaxf(v.y, 0.0f);
    const float vl = len3(vf);
    f3 lu = xyz(lu4);
    if (isnan(vl)) lu = mk3(0.0f, 0.0f, 0.0f);
    else if (vl > 20.0f) { const f3 u = vf / vl; lu = (lu - u * dot3(u, lu)) * (20.0f / vl); }
    if (j == 0 && !(v.y >= 0.0f)) lu.y = 0.0f;
    lv = lu;
  }
  a.F[ci] = f4(lv, 0.0f);
  a.G[ci] = f4(lv, 0.0f);
}
// Pass 2: pressure cotangent, the transpose of g = (pr(+) - pr(-)) / (2 dx) with the open-face (-p) and
// floor (+p) ghosts, applied to -G.
__global__ void __launch_bounds__(256) k_proj_adj2(const float* __restrict__ P, AdjFields a, Dims d) {
  const ACell id = acell(d);
  if (!id.ok) return;
  const int i = id.i, j = id.j, k = id.k;
  const size_t ci = cell(i, j, k, d.nx, d.ny);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const float c = 1.0f / (2.0f * __ldg(P + P_dx));
  const float4 me = a.G[ci];
  float s = 0.0f;
  if (i > 0) s -= a.G[ci - 1].x;
  if (i < d.nx - 1) s += a.G[ci + 1].x;
  if (i + 1 >= d.nx) s += me.x;
  if (i - 1 < 0) s -= me.x;
  if (j > 0) s -= a.G[ci - sy].y;
  if (j < d.ny - 1) s += a.G[ci + sy].y;
  if (j + 1 >= d.ny) s += me.y;
  if (j - 1 < 0) s += me.y;
  if (k > 0) s -= a.G[ci - sz].z;
  if (k < d.nz - 1) s += a.G[ci + sz].z;
  if (k + 1 >= d.nz) s += me.z;
  if (k - 1 < 0) s -= me.z;
  a.Pp[ci] = s * c;
}

// =====================================================================================================
// Loss of the inverse source fit: L = sum (1000 (S.x - S*.x))^2 + (S.z - S*.z)^2 (temperature in kelvin,
// soot as stored), its cotangent written into the state cotangents (vel and S2 zero).
__global__ void __launch_bounds__(256) k_loss(const float4* __restrict__ S, const float4* __restrict__ target, AdjFields a, Dims d) {
  const ACell id = acell(d);
  double l = 0.0;
  if (id.ok) {
    const size_t ci = cell(id.i, id.j, id.k, d.nx, d.ny);
    const float4 s = __ldg(S + ci), t = __ldg(target + ci);
    const float dT = 1000.0f * (s.x - t.x), dz = s.z - t.z;
    l = (double)dT * dT + (double)dz * dz;
    a.S[ci] = make_float4(2000.0f * dT, 0.0f, 2.0f * dz, 0.0f);
    a.S2[ci] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    a.vel[ci] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(a.loss, l);
}

// ---- launchers ----
void launch_adjoint_project(const float* P, const TapeStep& T, const AdjFields& a, Dims d, bool consume, cudaStream_t st) {
  launch_pdl(k_proj_adj1, agrid(d), ablock(), 0, st, P, T, a, d, (int)consume);
  launch_pdl(k_proj_adj2, agrid(d), ablock(), 0, st, P, a, d);
}
void launch_adjoint_div(const float* P, const AdjFields& a, Dims d, cudaStream_t st) {
  launch_pdl(k_div_adj, agrid(d), ablock(), 0, st, P, a, d);
}
void launch_adjoint_forces(const float* P, const TapeStep& T, const AdjFields& a, const uint2* noise, const uint2* curl, Dims d, bool consume,
                           cudaStream_t st) {
  launch_pdl(k_forces_adj1, agrid(d), ablock(), 0, st, P, T, a, noise, curl, d, (int)consume);
  launch_pdl(k_forces_adj2, agrid(d), ablock(), 0, st, T, a, d);
}
void launch_adjoint_adv2(const float* P, const TapeStep& T, const AdjFields& a, Dims d, cudaStream_t st) {
  launch_pdl(k_adv2_adj, agrid(d), ablock(), 0, st, P, T, a, d);
}
void launch_adjoint_adv1(const float* P, const TapeStep& T, const AdjFields& a, Dims d, cudaStream_t st) {
  launch_pdl(k_adv1_adj, agrid(d), ablock(), 0, st, P, T, a, d);
}
void launch_adjoint_loss(const float4* S, const float4* target, const AdjFields& a, Dims d, cudaStream_t st) {
  launch_pdl(k_loss, agrid(d), ablock(), 0, st, S, target, a, d);
}

}  // namespace fire

// =====================================================================================================
// Host driver behind the C ABI.
using namespace fire;
using namespace fire::rt;

struct FireAdjoint {
  FireSim* sim = nullptr;
  int nSteps = 0, K = 0, nSeg = 0;
  size_t cells = 0;
  std::vector<void*> allocs;
  float4* stateBuf = nullptr;   // (K + 1) x {vel, S, S2}: slot k is the input state of the segment's k-th step
  float4* tapeBuf = nullptr;    // K x {velX, SX, S2X, velY, SY, S2Y, forces velocity}
  float* tapeP = nullptr;       // K x pressure
  float4* ckBuf = nullptr;      // nSeg x {vel, S, S2}
  float* ckP = nullptr;         // nSeg x pressure (the warm start the segment began with)
  int* ckCounter = nullptr;     // nSeg x the solve's cycle prediction (counter slot 3)
  float* finalP = nullptr;      // pressure after the rollout, restored after the backward
  int* finalCounter = nullptr;
  float* dBlocks = nullptr;     // nSteps x BLOCK_FLOATS
  float4* target = nullptr;
  AdjFields a{};
  std::vector<cudaGraphExec_t> fwd, rev;
  std::vector<float> hBlocks;
  bool forwardDone = false;
  int tapeSeg = -1;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float fwdMs = 0, bwdMs = 0;
};

namespace {
#define ACK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return set_err(A->sim, FIRE_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

float4* state_f(FireAdjoint* A, int k, int c) { return A->stateBuf + ((size_t)k * 3 + c) * A->cells; }
float4* tape_f(FireAdjoint* A, int k, int c) { return A->tapeBuf + ((size_t)k * 7 + c) * A->cells; }
float* tape_p(FireAdjoint* A, int k) { return A->tapeP + (size_t)k * A->cells; }
int seg_len(FireAdjoint* A, int s) { return std::min(A->K, A->nSteps - s * A->K); }

// Forward Fields of tape slot k: state k in, hats and advected fields into the tape.
Fields fields_adv(FireAdjoint* A, int k) {
  Fields f = A->sim->f;
  f.vel = state_f(A, k, 0); f.S = state_f(A, k, 1); f.S2 = state_f(A, k, 2);
  f.velX = tape_f(A, k, 0); f.SX = tape_f(A, k, 1); f.S2X = tape_f(A, k, 2);
  f.velY = tape_f(A, k, 3); f.SY = tape_f(A, k, 4); f.S2Y = tape_f(A, k, 5);
  return f;
}
// Forces writes its velocity into the tape and S, S2 straight into state k+1; div/project read that
// velocity and project writes state k+1's velocity.
Fields fields_out(FireAdjoint* A, int k) {
  Fields f = fields_adv(A, k);
  f.velX = tape_f(A, k, 6);
  f.vel = state_f(A, k + 1, 0); f.S = state_f(A, k + 1, 1); f.S2 = state_f(A, k + 1, 2);
  return f;
}
TapeStep tape_step(FireAdjoint* A, int k) { return TapeStep{fields_adv(A, k), tape_f(A, k, 6), tape_p(A, k)}; }

int capture(FireAdjoint* A, bool forward, int k, cudaGraphExec_t* out) {
  FireSim* sim = A->sim;
  cudaStream_t st;
  ACK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return set_err(sim, FIRE_ERR_CUDA, "begin capture: %s", cudaGetErrorString(e)); }
  const float* P = sim->dBlock;
  const Dims d = sim->d;
  const MGLevel& L0 = sim->levels[0];
  const size_t pb = A->cells * sizeof(float);
  int rc = 0;
  if (forward) {   // record_step with the tape's buffers (src/sim.js:633-644)
    const Fields f1 = fields_adv(A, k), f2 = fields_out(A, k);
    launch_adv1(P, f1, d, st);
    launch_adv2(P, f1, d, st);
    launch_forces(P, f2, sim->noise, sim->curl, d, st);
    launch_div(P, f2, L0.b, d, st);
    rc = record_mg(sim, st);
    launch_project(P, f2, L0.p, d, st);
    cudaMemcpyAsync(tape_p(A, k), L0.p, pb, cudaMemcpyDeviceToDevice, st);
  } else {         // the reverse step
    const TapeStep T = tape_step(A, k);
    launch_adjoint_project(P, T, A->a, d, true, st);
    cudaMemcpyAsync(L0.b, A->a.Pp, pb, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(L0.p, A->a.B, pb, cudaMemcpyDeviceToDevice, st);
    rc = record_mg(sim, st);
    cudaMemcpyAsync(A->a.B, L0.p, pb, cudaMemcpyDeviceToDevice, st);
    launch_adjoint_div(P, A->a, d, st);
    launch_adjoint_forces(P, T, A->a, sim->noise, sim->curl, d, true, st);
    launch_adjoint_adv2(P, T, A->a, d, st);
    launch_adjoint_adv1(P, T, A->a, d, st);
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  cudaStreamDestroy(st);
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return set_err(sim, FIRE_ERR_CUDA, "end capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(sim, FIRE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return FIRE_OK;
}

int ensure_graphs(FireAdjoint* A) {
  if (!A->fwd.empty()) return FIRE_OK;
  A->fwd.assign(A->K, nullptr);
  A->rev.assign(A->K, nullptr);
  for (int k = 0; k < A->K; ++k) {
    int rc = capture(A, true, k, &A->fwd[k]);
    if (!rc) rc = capture(A, false, k, &A->rev[k]);
    if (rc) return rc;
  }
  return FIRE_OK;
}

int copy_state(FireAdjoint* A, float4* const dst[3], float4* const src[3], cudaStream_t st) {
  for (int c = 0; c < 3; ++c) ACK(cudaMemcpyAsync(dst[c], src[c], A->cells * sizeof(float4), cudaMemcpyDeviceToDevice, st));
  return FIRE_OK;
}
int run_step_graph(FireAdjoint* A, cudaGraphExec_t g, int n, cudaStream_t st) {
  ACK(cudaMemcpyAsync(A->sim->dBlock, A->dBlocks + (size_t)n * BLOCK_FLOATS, sizeof(float) * BLOCK_FLOATS, cudaMemcpyDeviceToDevice, st));
  ACK(cudaGraphLaunch(g, st));
  return FIRE_OK;
}
// Recomputes segment s into the tape from its checkpoint (same blocks, warm start and cycle prediction).
int recompute_segment(FireAdjoint* A, int s, cudaStream_t st) {
  float4* dst[3] = {state_f(A, 0, 0), state_f(A, 0, 1), state_f(A, 0, 2)};
  float4* src[3] = {A->ckBuf + (size_t)(s * 3 + 0) * A->cells, A->ckBuf + (size_t)(s * 3 + 1) * A->cells, A->ckBuf + (size_t)(s * 3 + 2) * A->cells};
  int rc = copy_state(A, dst, src, st);
  if (rc) return rc;
  ACK(cudaMemcpyAsync(A->sim->levels[0].p, A->ckP + (size_t)s * A->cells, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
  ACK(cudaMemcpyAsync(A->sim->dCounter + 3, A->ckCounter + s, sizeof(int), cudaMemcpyDeviceToDevice, st));
  for (int k = 0; k < seg_len(A, s); ++k)
    if ((rc = run_step_graph(A, A->fwd[k], s * A->K + k, st))) return rc;
  A->tapeSeg = s;
  return FIRE_OK;
}
float4* adj_buf4(FireAdjoint* A, int which) {
  float4* const b[12] = {A->a.vel, A->a.S, A->a.S2, A->a.velX, A->a.SX, A->a.S2X, A->a.velY, A->a.SY, A->a.S2Y, A->a.F, A->a.W, A->a.G};
  return which >= 0 && which < 12 ? b[which] : nullptr;
}
}  // namespace

extern "C" {

int fire_adjoint_create(FireSim* sim, int n_steps, int checkpoint_every, FireAdjoint** out) {
  FIRE_RANGE("fire_adjoint_create");
  if (!sim || !out || n_steps < 1 || checkpoint_every < 1 || checkpoint_every > 512) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  if (cudaSetDevice(sim->device) != cudaSuccess) return FIRE_ERR_CUDA;
  FireAdjoint* A = new FireAdjoint();
  A->sim = sim;
  A->nSteps = n_steps;
  A->K = std::min(checkpoint_every, n_steps);
  A->nSeg = (n_steps + A->K - 1) / A->K;
  A->cells = (size_t)sim->d.nx * sim->d.ny * sim->d.nz;
  const size_t c4 = A->cells * sizeof(float4), c1 = A->cells * sizeof(float);
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    A->allocs.push_back(p);
    return p;
  };
  bool ok = true;
  auto take4 = [&](size_t n) { float4* p = (float4*)alloc(n * c4); ok = ok && p; return p; };
  auto take1 = [&](size_t n) { float* p = (float*)alloc(n * c1); ok = ok && p; return p; };
  A->stateBuf = take4((size_t)(A->K + 1) * 3);
  A->tapeBuf = take4((size_t)A->K * 7);
  A->tapeP = take1(A->K);
  A->ckBuf = take4((size_t)A->nSeg * 3);
  A->ckP = take1(A->nSeg);
  A->finalP = take1(1);
  A->target = take4(1);
  float4* adj = take4(12);
  float* adj1 = take1(2);
  A->ckCounter = (int*)alloc(sizeof(int) * (A->nSeg + 1));
  A->finalCounter = A->ckCounter ? A->ckCounter + A->nSeg : nullptr;
  A->dBlocks = (float*)alloc(sizeof(float) * BLOCK_FLOATS * n_steps);
  double* dd = (double*)alloc(sizeof(double) * (MAX_SPOTS + 1));
  ok = ok && A->ckCounter && A->dBlocks && dd;
  if (!ok) { fire_adjoint_destroy(A); return FIRE_ERR_OOM; }
  float4* const bufs[12] = {adj, adj + A->cells, adj + 2 * A->cells, adj + 3 * A->cells, adj + 4 * A->cells, adj + 5 * A->cells,
                            adj + 6 * A->cells, adj + 7 * A->cells, adj + 8 * A->cells, adj + 9 * A->cells, adj + 10 * A->cells,
                            adj + 11 * A->cells};
  A->a = AdjFields{bufs[0], bufs[1], bufs[2], bufs[3], bufs[4], bufs[5], bufs[6], bufs[7], bufs[8], bufs[9], bufs[10], bufs[11],
                   adj1, adj1 + A->cells, dd, dd + MAX_SPOTS};
  for (int i = 0; i < 4; ++i)
    if (cudaEventCreate(&A->ev[i]) != cudaSuccess) { fire_adjoint_destroy(A); return FIRE_ERR_CUDA; }
  if (cudaMemset(adj, 0, 12 * c4) != cudaSuccess || cudaMemset(adj1, 0, 2 * c1) != cudaSuccess ||
      cudaMemset(dd, 0, sizeof(double) * (MAX_SPOTS + 1)) != cudaSuccess) {
    fire_adjoint_destroy(A);
    return FIRE_ERR_CUDA;
  }
  A->hBlocks.assign((size_t)BLOCK_FLOATS * n_steps, 0.0f);
  *out = A;
  return FIRE_OK;
}

int fire_adjoint_destroy(FireAdjoint* A) {
  if (!A) return FIRE_ERR_BAD_ARG;
  cudaSetDevice(A->sim->device);
  cudaDeviceSynchronize();
  for (auto g : A->fwd) if (g) cudaGraphExecDestroy(g);
  for (auto g : A->rev) if (g) cudaGraphExecDestroy(g);
  for (auto e : A->ev) if (e) cudaEventDestroy(e);
  for (void* p : A->allocs) cudaFree(p);
  delete A;
  return FIRE_OK;
}

int fire_adjoint_forward(FireAdjoint* A, float dt, void* stream) {
  FIRE_RANGE("fire_adjoint_forward");
  if (!A || !(dt > 0.0f)) return FIRE_ERR_BAD_ARG;
  FireSim* sim = A->sim;
  sim->stepStatsValid = false;   // the tape writes the simulation's fields
  ACK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  int rc;
  if (!sim->geoReady || sim->logsDirty) {
    if ((rc = upload_block(sim, dt, st, true))) return rc;
    if ((rc = ensure_geo(sim, st))) return rc;
  }
  if ((rc = ensure_graphs(A))) return rc;
  // the blocks fire_sim_step would upload, with the event envelopes advanced per step
  for (int n = 0; n < A->nSteps; ++n) {
    advance_events(sim, dt);
    fill_block(sim, dt, A->hBlocks.data() + (size_t)n * BLOCK_FLOATS);
    sim->time += dt;
    sim->frame += 1;
    sim->stepsRun += 1;
  }
  ACK(cudaMemcpyAsync(A->dBlocks, A->hBlocks.data(), sizeof(float) * A->hBlocks.size(), cudaMemcpyHostToDevice, st));
  ACK(cudaEventRecord(A->ev[0], st));
  float4* simState[3] = {sim->f.vel, sim->f.S, sim->f.S2};
  float4* slot0[3] = {state_f(A, 0, 0), state_f(A, 0, 1), state_f(A, 0, 2)};
  if ((rc = copy_state(A, slot0, simState, st))) return rc;
  for (int s = 0; s < A->nSeg; ++s) {
    if (s > 0) {
      const int kp = seg_len(A, s - 1);
      float4* last[3] = {state_f(A, kp, 0), state_f(A, kp, 1), state_f(A, kp, 2)};
      if ((rc = copy_state(A, slot0, last, st))) return rc;
    }
    float4* ck[3] = {A->ckBuf + (size_t)(s * 3 + 0) * A->cells, A->ckBuf + (size_t)(s * 3 + 1) * A->cells, A->ckBuf + (size_t)(s * 3 + 2) * A->cells};
    if ((rc = copy_state(A, ck, slot0, st))) return rc;
    ACK(cudaMemcpyAsync(A->ckP + (size_t)s * A->cells, sim->levels[0].p, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(A->ckCounter + s, sim->dCounter + 3, sizeof(int), cudaMemcpyDeviceToDevice, st));
    for (int k = 0; k < seg_len(A, s); ++k)
      if ((rc = run_step_graph(A, A->fwd[k], s * A->K + k, st))) return rc;
  }
  const int kl = seg_len(A, A->nSeg - 1);
  float4* last[3] = {state_f(A, kl, 0), state_f(A, kl, 1), state_f(A, kl, 2)};
  if ((rc = copy_state(A, simState, last, st))) return rc;
  ACK(cudaMemcpyAsync(A->finalP, sim->levels[0].p, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
  ACK(cudaMemcpyAsync(A->finalCounter, sim->dCounter + 3, sizeof(int), cudaMemcpyDeviceToDevice, st));
  ACK(cudaEventRecord(A->ev[1], st));
  A->tapeSeg = A->nSeg - 1;
  A->forwardDone = true;
  A->fwdMs = -1.0f;
  return FIRE_OK;
}

int fire_adjoint_loss(FireAdjoint* A, const float* target_S, double* loss) {
  if (!A || !target_S || !loss) return FIRE_ERR_BAD_ARG;
  FireSim* sim = A->sim;
  ACK(cudaSetDevice(sim->device));
  ACK(cudaDeviceSynchronize());
  ACK(cudaMemcpy(A->target, target_S, A->cells * sizeof(float4), cudaMemcpyHostToDevice));
  ACK(cudaMemset(A->a.loss, 0, sizeof(double)));
  launch_adjoint_loss(sim->f.S, A->target, A->a, sim->d, 0);
  ACK(cudaGetLastError());
  ACK(cudaMemcpy(loss, A->a.loss, sizeof(double), cudaMemcpyDeviceToHost));
  return FIRE_OK;
}

int fire_adjoint_seed(FireAdjoint* A, const float* d_vel, const float* d_S, const float* d_S2) {
  if (!A) return FIRE_ERR_BAD_ARG;
  ACK(cudaSetDevice(A->sim->device));
  ACK(cudaDeviceSynchronize());
  const float* src[3] = {d_vel, d_S, d_S2};
  float4* dst[3] = {A->a.vel, A->a.S, A->a.S2};
  for (int c = 0; c < 3; ++c) {
    if (src[c]) ACK(cudaMemcpy(dst[c], src[c], A->cells * sizeof(float4), cudaMemcpyHostToDevice));
    else ACK(cudaMemset(dst[c], 0, A->cells * sizeof(float4)));
  }
  return FIRE_OK;
}

int fire_adjoint_backward(FireAdjoint* A, void* stream) {
  FIRE_RANGE("fire_adjoint_backward");
  if (!A) return FIRE_ERR_BAD_ARG;
  FireSim* sim = A->sim;
  sim->stepStatsValid = false;   // the tape writes the simulation's fields
  if (!A->forwardDone) return set_err(sim, FIRE_ERR_STATE, "fire_adjoint_backward before fire_adjoint_forward");
  ACK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  int rc;
  const size_t c4 = A->cells * sizeof(float4);
  ACK(cudaEventRecord(A->ev[2], st));
  for (float4* b : {A->a.velX, A->a.SX, A->a.S2X, A->a.velY, A->a.W}) ACK(cudaMemsetAsync(b, 0, c4, st));
  ACK(cudaMemsetAsync(A->a.B, 0, A->cells * sizeof(float), st));
  ACK(cudaMemsetAsync(A->a.flux, 0, sizeof(double) * MAX_SPOTS, st));
  for (int s = A->nSeg - 1; s >= 0; --s) {
    if (A->tapeSeg != s && (rc = recompute_segment(A, s, st))) return rc;
    for (int k = seg_len(A, s) - 1; k >= 0; --k)
      if ((rc = run_step_graph(A, A->rev[k], s * A->K + k, st))) return rc;
  }
  // the simulation keeps the rollout's final pressure (its warm start) and cycle prediction
  ACK(cudaMemcpyAsync(sim->levels[0].p, A->finalP, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
  ACK(cudaMemcpyAsync(sim->dCounter + 3, A->finalCounter, sizeof(int), cudaMemcpyDeviceToDevice, st));
  ACK(cudaEventRecord(A->ev[3], st));
  A->bwdMs = -1.0f;
  return FIRE_OK;
}

int fire_adjoint_grad_spots(FireAdjoint* A, double* out, int n) {
  if (!A || !out || n < 0 || n > MAX_SPOTS) return FIRE_ERR_BAD_ARG;
  ACK(cudaSetDevice(A->sim->device));
  ACK(cudaDeviceSynchronize());
  if (n) ACK(cudaMemcpy(out, A->a.flux, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return FIRE_OK;
}

int fire_adjoint_io(FireAdjoint* A, int which, void* host, size_t bytes, int dir) {
  if (!A || !host || which < 0 || which >= FIRE_ADJ_COUNT || (dir != 0 && dir != 1)) return FIRE_ERR_BAD_ARG;
  void* dev = which < 12 ? (void*)adj_buf4(A, which) : which == FIRE_ADJ_P ? (void*)A->a.Pp : (void*)A->a.B;
  const size_t need = A->cells * (which < 12 ? sizeof(float4) : sizeof(float));
  if (bytes != need) return set_err(A->sim, FIRE_ERR_BAD_ARG, "adjoint buffer %d holds %zu bytes", which, need);
  ACK(cudaSetDevice(A->sim->device));
  ACK(cudaDeviceSynchronize());
  if (dir == 0) ACK(cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost));
  else ACK(cudaMemcpy(dev, host, bytes, cudaMemcpyHostToDevice));
  return FIRE_OK;
}

int fire_adjoint_clear(FireAdjoint* A) {
  if (!A) return FIRE_ERR_BAD_ARG;
  ACK(cudaSetDevice(A->sim->device));
  ACK(cudaDeviceSynchronize());
  ACK(cudaMemset(A->a.vel, 0, 12 * A->cells * sizeof(float4)));
  ACK(cudaMemset(A->a.Pp, 0, 2 * A->cells * sizeof(float)));
  ACK(cudaMemset(A->a.flux, 0, sizeof(double) * (MAX_SPOTS + 1)));
  return FIRE_OK;
}

int fire_adjoint_stage(FireAdjoint* A, int stage, float dt, int arg, void* stream) {
  FIRE_RANGE("fire_adjoint_stage");
  if (!A || !(dt > 0.0f)) return FIRE_ERR_BAD_ARG;
  FireSim* sim = A->sim;
  sim->stepStatsValid = false;   // stage runs may write the simulation's fields
  ACK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  int rc = upload_block(sim, dt, st, false);
  if (rc) return rc;
  const float* P = sim->dBlock;
  const TapeStep T{sim->f, sim->f.velX, sim->levels[0].p};
  const MGLevel& L0 = sim->levels[0];
  switch (stage) {
    case FIRE_STAGE_ADV1: launch_adjoint_adv1(P, T, A->a, sim->d, st); break;
    case FIRE_STAGE_ADV2: launch_adjoint_adv2(P, T, A->a, sim->d, st); break;
    case FIRE_STAGE_CURL:
    case FIRE_STAGE_FORCES: launch_adjoint_forces(P, T, A->a, sim->noise, sim->curl, sim->d, false, st); break;
    case FIRE_STAGE_DIV: launch_adjoint_div(P, A->a, sim->d, st); break;
    case FIRE_STAGE_PROJECT: launch_adjoint_project(P, T, A->a, sim->d, false, st); break;
    case FIRE_STAGE_VCYCLE:
      if (arg < 1) return FIRE_ERR_BAD_ARG;
      ACK(cudaMemcpyAsync(L0.b, A->a.Pp, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
      ACK(cudaMemcpyAsync(L0.p, A->a.B, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
      for (int c = 0; c < arg; ++c) record_vcycle(sim, st);
      ACK(cudaMemcpyAsync(A->a.B, L0.p, A->cells * sizeof(float), cudaMemcpyDeviceToDevice, st));
      break;
    default: return FIRE_ERR_BAD_ARG;
  }
  ACK(cudaGetLastError());
  return FIRE_OK;
}

int fire_adjoint_timing(FireAdjoint* A, float* forward_ms, float* backward_ms) {
  if (!A) return FIRE_ERR_BAD_ARG;
  ACK(cudaSetDevice(A->sim->device));
  if (A->fwdMs < 0.0f) { ACK(cudaEventSynchronize(A->ev[1])); ACK(cudaEventElapsedTime(&A->fwdMs, A->ev[0], A->ev[1])); }
  if (A->bwdMs < 0.0f) { ACK(cudaEventSynchronize(A->ev[3])); ACK(cudaEventElapsedTime(&A->bwdMs, A->ev[2], A->ev[3])); }
  if (forward_ms) *forward_ms = A->fwdMs;
  if (backward_ms) *backward_ms = A->bwdMs;
  return FIRE_OK;
}

}  // extern "C"
