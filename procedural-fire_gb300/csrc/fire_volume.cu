// Volume rendering of the simulation (the renderer's fire light extraction, flame prefilter and
// emission-absorption ray march: src/renderer.js:104-165, 173-192, 194-326) as CUDA kernels writing a
// headless image buffer instead of a WebGPU texture.
//
//   k_lights   one CTA per height band (8): the emission-weighted centroid, spread and radiant intensity
//              of the band, temporally filtered, as 8 point lights (pLights)
//   k_sharpen  s + k (s - mean of the 6 neighbours), clamped to the local range (pSharpen; flameSharp > 0)
//   k_volume   one thread per volume pixel: camera ray, box clip, jittered march with the curl-noise detail
//              warp, soot emission from the blackbody LUT, blue chemiluminescence, single scattering of the
//              8 lights off soot and smoke, Beer-Lambert absorption (pVolume)
//
// There is no surface pass (logs, stones, ground are rasterised geometry of the page): the depth the march
// stops at is a caller-supplied buffer, or unbounded.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fire_sim.h"
#include "fire_device.cuh"
#include "fire_launch.cuh"
#include "fire_nvtx.h"

namespace fire {
namespace {

constexpr int NLIGHTS = 8;                 // src/renderer.js:30
constexpr float kPIf = 3.14159265f;

// Renderer uniforms the volume passes read (RP_FIELDS subset, src/renderer.js:8-16), all f32.
struct VolU {
  float width, height, vw, vh, time, frame;
  float camX, camY, camZ, tanFov, fwdX, fwdY, fwdZ, aspect, rgtX, rgtY, rgtZ, jitX, upX, upY, upZ, jitY;
  float ox, oy, oz, dx, sx, sy, sz, tempScale, nx, ny, nz, nLights;
  float stepMul, sootAbs, sootEmit, emitK, blueK, smokeScat, smokeG, detailAmt, detailFreq, detailSpeed, lightK;
  float bbTmin, bbTmax, bbN, emitTempLo, sootScat, sootEdge, cubic, flameSharp, lightDt, flickerK, lensX, lensY, focus;
  float depthW, depthH;   // caller depth buffer size (0: none)
};
constexpr int VOLU_FLOATS = sizeof(VolU) / sizeof(float);

__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ f3 vmul(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }

// bbRow (src/renderer.js:74-80): linear interpolation in the 2-row LUT; row 0 blackbody, row 1 soot.
__device__ __forceinline__ f3 bb_row(const VolU& R, const float4* __restrict__ lut, float T, int row) {
  const float x = clampf((T - R.bbTmin) / (R.bbTmax - R.bbTmin), 0.0f, 1.0f) * (R.bbN - 1.0f);
  const unsigned i = (unsigned)floorf(x);
  const float f = x - floorf(x);
  const unsigned n = (unsigned)R.bbN;
  const float4 a = __ldg(lut + row * n + i), b = __ldg(lut + row * n + min(i + 1u, n - 1u));
  return mk3(mixf(a.x, b.x, f), mixf(a.y, b.y, f), mixf(a.z, b.z, f));
}
__device__ __forceinline__ float lum(f3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

__global__ void __launch_bounds__(256) k_lights(VolU R, const float4* __restrict__ S, const float4* __restrict__ lut,
                                                float4* __restrict__ lights, float4* __restrict__ lstate) {
  __shared__ float4 accP[256], accC[256];
  const unsigned li = threadIdx.x, wg = blockIdx.x;
  const unsigned nx = (unsigned)R.nx, ny = (unsigned)R.ny, nz = (unsigned)R.nz;
  const unsigned bandH = ny / NLIGHTS, y0 = wg * bandH;
  float4 P = make_float4(0.f, 0.f, 0.f, 0.f), C = P;
  const unsigned hx = nx / 2u, hb = bandH / 2u, total = hx * hb * (nz / 2u);
  for (unsigned i = li; i < total; i += 256u) {
    const unsigned ix = (i % hx) * 2u, iy = ((i / hx) % hb) * 2u + y0, iz = (i / (hx * hb)) * 2u;
    const float4 s = __ldg(S + ix + nx * (iy + ny * iz));
    const float T = 293.0f + s.x * R.tempScale;
    if (T < 700.0f) continue;
    const f3 e = bb_row(R, lut, T, 1) * (s.z * R.sootEmit) * R.emitK;
    const float w = lum(e);
    const f3 pos = mk3(R.ox, R.oy, R.oz) + (mk3((float)ix, (float)iy, (float)iz) + mk3(1.0f, 1.0f, 1.0f)) * R.dx;
    P = make_float4(P.x + pos.x * w, P.y + pos.y * w, P.z + pos.z * w, P.w + w);
    C = make_float4(C.x + e.x, C.y + e.y, C.z + e.z, C.w + dot3(pos, pos) * w);
  }
  accP[li] = P;
  accC[li] = C;
  __syncthreads();
  for (unsigned s = 128u; s > 0u; s >>= 1u) {
    if (li < s) {
      const float4 a = accP[li + s], c = accC[li + s];
      accP[li] = make_float4(accP[li].x + a.x, accP[li].y + a.y, accP[li].z + a.z, accP[li].w + a.w);
      accC[li] = make_float4(accC[li].x + c.x, accC[li].y + c.y, accC[li].z + c.z, accC[li].w + c.w);
    }
    __syncthreads();
  }
  if (li != 0u) return;
  const float w = accP[0].w;
  const f3 cen = w > 1e-6f ? mk3(accP[0].x, accP[0].y, accP[0].z) / w : mk3(0.0f, ((float)y0 + (float)bandH * 0.5f) * R.dx, 0.0f);
  const float spread = w > 1e-6f ? fmaxf(accC[0].w / w - dot3(cen, cen), 0.0f) : 0.04f;
  const f3 J = mk3(accC[0].x, accC[0].y, accC[0].z) * ((float)(nx * bandH * nz) / (float)total) * R.dx * R.dx * R.dx;
  float4 sp = lstate[wg], sc = lstate[NLIGHTS + wg], sm = lstate[2 * NLIGHTS + wg];
  if (R.lightDt < 0.0f || sm.w <= 0.0f) {
    sp = make_float4(cen.x, cen.y, cen.z, spread);
    sc = make_float4(J.x, J.y, J.z, 0.0f);
    sm = make_float4(J.x, J.y, J.z, 1.0f);
  } else {
    const float a = 1.0f - expf(-R.lightDt / 0.08f), ap = 1.0f - expf(-R.lightDt / 0.15f), am = 1.0f - expf(-R.lightDt / 1.5f);
    sp = make_float4(mixf(sp.x, cen.x, ap), mixf(sp.y, cen.y, ap), mixf(sp.z, cen.z, ap), mixf(sp.w, spread, ap));
    sc = make_float4(mixf(sc.x, J.x, a), mixf(sc.y, J.y, a), mixf(sc.z, J.z, a), 0.0f);
    sm = make_float4(mixf(sm.x, J.x, am), mixf(sm.y, J.y, am), mixf(sm.z, J.z, am), 1.0f);
  }
  lstate[wg] = sp;
  lstate[NLIGHTS + wg] = sc;
  lstate[2 * NLIGHTS + wg] = sm;
  const float ratio = lum(mk3(sc.x, sc.y, sc.z)) / fmaxf(lum(mk3(sm.x, sm.y, sm.z)), 1e-9f);
  const f3 Jc = mk3(sc.x, sc.y, sc.z) * powf(fmaxf(ratio, 1e-4f), R.flickerK - 1.0f);
  const float wl = lum(Jc);
  const bool on = wl > 1e-3f * lum(mk3(sm.x, sm.y, sm.z)) && wl > 0.0f;
  lights[2 * wg] = make_float4(sp.x, sp.y, sp.z, on ? wl : 0.0f);
  lights[2 * wg + 1] = make_float4(on ? Jc.x : 0.0f, on ? Jc.y : 0.0f, on ? Jc.z : 0.0f, sp.w);
}

__global__ void __launch_bounds__(256) k_sharpen(float k, const float4* __restrict__ in, float4* __restrict__ out, Dims d) {
  const int x = blockIdx.x * 8 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z * 4 + threadIdx.z;
  if (x >= d.nx || y >= d.ny || z >= d.nz) return;
  const float4 s = __ldg(in + cell(x, y, z, d.nx, d.ny));
  float4 n = make_float4(0.f, 0.f, 0.f, 0.f), lo = s, up = s;
#pragma unroll
  for (int q = 0; q < 6; ++q) {   // -x, +x, -y, +y, -z, +z as the reference's loop
    const int sgn = (q & 1) == 0 ? -1 : 1, ax = q / 2;
    const float4 v = ldc(in, x + (ax == 0 ? sgn : 0), y + (ax == 1 ? sgn : 0), z + (ax == 2 ? sgn : 0), d);
    n = add4(n, v);
    lo = fmin4(lo, v);
    up = fmax4(up, v);
  }
  const float4 t = add4(s, mul4(sub4(s, mul4(n, 1.0f / 6.0f)), k));
  out[cell(x, y, z, d.nx, d.ny)] = fmin4(fmax4(t, lo), up);
}

// Cubic B-spline reconstruction from 8 trilinear fetches (src/renderer.js:213-232); g in cell units.
__device__ __forceinline__ float4 sample_cubic(const float4* __restrict__ f, f3 g, Dims d) {
  const f3 dims = mk3((float)d.nx, (float)d.ny, (float)d.nz);
  const f3 c = g - mk3(0.5f, 0.5f, 0.5f);
  const f3 i = mk3(floorf(c.x), floorf(c.y), floorf(c.z));
  const f3 fr = c - i;
  const f3 f2 = vmul(fr, fr), f3v = vmul(f2, fr);
  auto W = [&](float a, float b, float cc, float dd) {
    return mk3((a + b * fr.x + cc * f2.x + dd * f3v.x) / 6.0f, (a + b * fr.y + cc * f2.y + dd * f3v.y) / 6.0f,
               (a + b * fr.z + cc * f2.z + dd * f3v.z) / 6.0f);
  };
  const f3 w0 = W(1.0f, -3.0f, 3.0f, -1.0f), w1 = W(4.0f, 0.0f, -6.0f, 3.0f), w2 = W(1.0f, 3.0f, 3.0f, -3.0f);
  const f3 w3 = mk3(f3v.x / 6.0f, f3v.y / 6.0f, f3v.z / 6.0f);
  const f3 g0 = w0 + w1, g1 = w2 + w3;
  const f3 h0 = mk3((i.x - 0.5f + w1.x / g0.x) / dims.x, (i.y - 0.5f + w1.y / g0.y) / dims.y, (i.z - 0.5f + w1.z / g0.z) / dims.z);
  const f3 h1 = mk3((i.x + 1.5f + w3.x / g1.x) / dims.x, (i.y + 1.5f + w3.y / g1.y) / dims.y, (i.z + 1.5f + w3.z / g1.z) / dims.z);
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const bool ox = k & 1, oy = k & 2, oz = k & 4;
    const f3 p = mk3(ox ? h1.x : h0.x, oy ? h1.y : h0.y, oz ? h1.z : h0.z);
    const float wv = (ox ? g1.x : g0.x) * (oy ? g1.y : g0.y) * (oz ? g1.z : g0.z);
    acc = add4(acc, mul4(sample(f, make_tap(vmul(p, dims), d), d), wv));
  }
  return acc;
}
__device__ __forceinline__ float hg(float c, float g) {
  const float g2 = g * g;
  return (1.0f - g2) / (4.0f * kPIf * powf(1.0f + g2 - 2.0f * g * c, 1.5f));
}

__global__ void __launch_bounds__(64) k_volume(VolU R, const float4* __restrict__ S, const float4* __restrict__ S2, Dims d,
                                               const uint2* __restrict__ curlT, const float4* __restrict__ lut,
                                               const float4* __restrict__ lights, const float* __restrict__ depth,
                                               float4* __restrict__ vol, float2* __restrict__ aux) {
  const unsigned ix = blockIdx.x * 8 + threadIdx.x, iy = blockIdx.y * 8 + threadIdx.y;
  if ((float)ix >= R.vw || (float)iy >= R.vh) return;
  const float pxx = (float)ix + 0.5f + R.jitX * (R.vw / R.width), pxy = (float)iy + 0.5f + R.jitY * (R.vw / R.width);
  // camRay (src/renderer.js:207-211) and the thin lens (lensRay, src/renderer.js:87-95)
  const float ndx = pxx / R.vw * 2.0f - 1.0f, ndy = 1.0f - pxy / R.vh * 2.0f;
  const f3 fwd = mk3(R.fwdX, R.fwdY, R.fwdZ), rgt = mk3(R.rgtX, R.rgtY, R.rgtZ), upv = mk3(R.upX, R.upY, R.upZ);
  f3 dPin = fwd + rgt * ndx * R.tanFov * R.aspect + upv * ndy * R.tanFov;
  dPin = dPin / sqrtf(dot3(dPin, dPin));
  f3 ro = mk3(R.camX, R.camY, R.camZ), rd = dPin;
  if (R.focus > 0.0f) {
    const f3 o = ro + rgt * R.lensX + upv * R.lensY;
    const f3 q = ro + dPin * (R.focus / dot3(dPin, fwd));
    const f3 dq = q - o;
    ro = o;
    rd = dq / sqrtf(dot3(dq, dq));
  }
  float sd = 1e9f;
  if (depth && R.depthW > 0.0f) {
    const int dw = (int)R.depthW, dh = (int)R.depthH;
    const int fx = min(max((int)(pxx / R.vw * R.depthW), 0), dw - 1), fy = min(max((int)(pxy / R.vh * R.depthH), 0), dh - 1);
    sd = __ldg(depth + fx + dw * fy);
  }
  const f3 bmin = mk3(R.ox, R.oy, R.oz), bmax = bmin + mk3(R.sx, R.sy, R.sz);
  const f3 inv = mk3(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
  const f3 t0 = vmul(bmin - ro, inv), t1 = vmul(bmax - ro, inv);
  const float tn = fmaxf(fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z)), 0.0f);
  const float tf = fminf(fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z)), sd);
  f3 L = mk3(0.f, 0.f, 0.f);
  float Tr = 1.0f, haze = 0.0f;
  if (tf > tn) {
    const float ds = R.dx * R.stepMul;
    // interleaved gradient noise (src/shaders/lib.js IGN)
    const float ipx = (float)ix + 5.588238f * fmodf(R.frame, 64.0f), ipy = (float)iy + 5.588238f * fmodf(R.frame, 64.0f);
    const float jit = fractf(52.9829189f * fractf(ipx * 0.06711056f + ipy * 0.00583715f));
    float t = tn + ds * jit;
    const f3 dims = mk3(R.nx, R.ny, R.nz);
    const int nlit = (int)R.nLights;
    for (int it = 0; it < 1200; ++it) {
      if (t > tf || Tr < 0.003f) break;
      const f3 p = ro + rd * t;
      f3 g = (p - bmin) / R.dx;
      float mottle = 0.0f;
      if (R.detailAmt > 0.0f) {   // divergence-free detail warp, two cross-faded phases
        const float rise = R.detailSpeed * (0.5f + 1.5f * sstep(0.0f, 1.0f, p.y));
        const float ph = R.time / 0.7f;
        const float f0 = fractf(ph), f1 = fractf(ph + 0.5f);
        const float w0 = 1.0f - fabsf(2.0f * f0 - 1.0f);
        const f3 o0 = mk3(0.37f, 0.0f, 0.61f) * floorf(ph), o1 = mk3(0.71f, 0.0f, 0.29f) * floorf(ph + 0.5f);
        const f3 q0 = (p - mk3(0.0f, rise * f0 * 0.7f, 0.0f)) * R.detailFreq * 0.25f + o0;
        const f3 q1 = (p - mk3(0.0f, rise * f1 * 0.7f, 0.0f)) * R.detailFreq * 0.25f + o1;
        const float4 c0 = sample_table(curlT, q0), c1 = sample_table(curlT, q1);
        const float4 cw = add4(mul4(c0, w0), mul4(c1, 1.0f - w0));
        g = g + vmul(xyz(cw) * (R.detailAmt * 0.12f), mk3(1.0f, 0.6f, 1.0f));
        mottle = cw.w * 0.08f - 0.6f;
      }
      float4 s = R.cubic > 0.5f ? sample_cubic(S, g, d) : sample(S, make_tap(g, d), d);
      const float edge = fminf(fminf(g.x, dims.x - g.x), fminf(g.z, dims.z - g.z));
      const float fade = sstep(0.02f, 0.15f, edge * R.dx) * sstep(0.0f, 0.4f, (dims.y - g.y) * R.dx);
      s = mul4(s, fade);
      const float T = 293.0f + s.x * R.tempScale + mottle * 60.0f * R.detailAmt * (s.x >= 0.3f ? 1.0f : 0.0f);
      float soot = s.z;
      if (R.sootEdge > 0.0f) soot *= sstep(0.6f * R.sootEdge, 1.4f * R.sootEdge, soot);
      float smoke = 0.0f;
      if (R.smokeScat > 0.0f) smoke = sample(S2, make_tap(g, d), d).z * fade;
      if (soot > 1e-4f || s.w > 1e-3f || smoke > 1e-4f) {
        const float sigSoot = soot * R.sootAbs;
        const float sigS = sigSoot * R.sootScat + smoke * R.smokeScat;
        const float sigT = sigSoot + smoke * R.smokeScat * 1.1f + 1e-6f;
        f3 e = mk3(0.f, 0.f, 0.f);
        if (T > R.emitTempLo) e = bb_row(R, lut, T, 1) * (soot * R.sootEmit) * R.emitK;
        e = e + mk3(0.15f, 0.3f, 1.0f) * powf(s.w, 1.6f) * (R.blueK / 3.0f) * expf(-soot * 2.0f);
        f3 ins = mk3(0.f, 0.f, 0.f);
        if (sigS * Tr > 1e-6f) {
          for (int k = 0; k < nlit; ++k) {
            const float4 lp = __ldg(lights + 2 * k), lc = __ldg(lights + 2 * k + 1);
            const f3 toL = xyz(lp) - p;
            const float r2 = dot3(toL, toL) + lc.w * 0.6f + 0.004f;
            ins = ins + xyz(lc) * hg(dot3(rd, toL * rsqrtf(r2)), R.smokeG) / r2;
          }
          ins = ins * (sigS * R.lightK);
        }
        const float a = expf(-sigT * ds);
        const float w = sigT * ds < 1e-4f ? ds : (1.0f - a) / sigT;
        L = L + (e + ins) * Tr * w;
        Tr *= a;
      }
      haze += fmaxf(s.x - 0.05f, 0.0f) * ds;
      t += ds;
    }
  }
  vol[ix + (unsigned)R.vw * iy] = make_float4(L.x, L.y, L.z, Tr);
  aux[ix + (unsigned)R.vw * iy] = make_float2(haze, sd);
}

}  // namespace
}  // namespace fire

using namespace fire;

// Renderer parameter names this module reads and their defaults (RP_DEFAULTS, src/renderer.js:18-25).
namespace {
struct NamedParam { const char* name; int offset; float def; };
#define VP(n, d) {#n, (int)(offsetof(VolU, n) / sizeof(float)), d}
const NamedParam kVolParams[] = {
  VP(stepMul, 0.7f), VP(sootAbs, 4.0f), VP(sootEmit, 10.0f), VP(emitK, 4.0f), VP(blueK, 0.05f), VP(smokeScat, 0.02f),
  VP(smokeG, 0.5f), VP(detailAmt, 0.6f), VP(detailFreq, 2.2f), VP(detailSpeed, 0.9f), VP(lightK, 1.0f), VP(tempScale, 1000.0f),
  VP(emitTempLo, 900.0f), VP(sootScat, 0.015f), VP(sootEdge, 0.0f), VP(cubic, 0.0f), VP(flameSharp, 0.0f), VP(flickerK, 0.35f),
  VP(lensX, 0.0f), VP(lensY, 0.0f), VP(focus, 0.0f),
};
#undef VP
}  // namespace

struct FireVolume {
  FireSim* sim = nullptr;
  int device = 0;
  int w = 0, h = 0, vw = 0, vh = 0;
  VolU U{};
  float4* dLut = nullptr;        // 2 x n blackbody rows
  int lutN = 1024;
  float4* dLights = nullptr;     // NLIGHTS x (pos+w, colour+spread)
  float4* dLstate = nullptr;     // 3 NLIGHTS temporal filter states
  float4* dVol = nullptr;        // vw x vh: radiance rgb, transmittance
  float2* dAux = nullptr;        // vw x vh: haze, depth
  float4* dSharp = nullptr;      // prefiltered S (flameSharp > 0 with cubic)
  const float* depth = nullptr;  // caller depth buffer (optional)
  double lastLightTime = -1e300;
  bool haveLight = false;
};

extern "C" {

int fire_volume_create(FireSim* sim, int width, int height, float vol_scale, float white_balance_k, FireVolume** out) {
  FIRE_RANGE("fire_volume_create");
  if (!sim || !out || width < 1 || height < 1 || !(vol_scale > 0.0f)) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  FireInfo info;
  if (fire_sim_info(sim, &info) != FIRE_OK) return FIRE_ERR_BAD_ARG;
  FireVolume* v = new FireVolume();
  v->sim = sim;
  cudaGetDevice(&v->device);
  v->w = width; v->h = height;
  v->vw = std::max(8, (int)std::lround(width * (double)vol_scale));   // src/renderer.js:580
  v->vh = std::max(8, (int)std::lround(height * (double)vol_scale));
  for (const NamedParam& p : kVolParams) reinterpret_cast<float*>(&v->U)[p.offset] = p.def;
  std::vector<float> lut((size_t)v->lutN * 2 * 4);
  fire_blackbody_lut(v->lutN, 400.0f, 3000.0f, white_balance_k, lut.data());
  v->U.bbTmin = 400.0f; v->U.bbTmax = 3000.0f; v->U.bbN = (float)v->lutN;
  const size_t px = (size_t)v->vw * v->vh;
  if (cudaMalloc((void**)&v->dLut, lut.size() * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void**)&v->dLights, sizeof(float4) * 2 * NLIGHTS) != cudaSuccess ||
      cudaMalloc((void**)&v->dLstate, sizeof(float4) * 3 * NLIGHTS) != cudaSuccess ||
      cudaMalloc((void**)&v->dVol, sizeof(float4) * px) != cudaSuccess || cudaMalloc((void**)&v->dAux, sizeof(float2) * px) != cudaSuccess ||
      cudaMemcpy(v->dLut, lut.data(), lut.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(v->dLstate, 0, sizeof(float4) * 3 * NLIGHTS) != cudaSuccess) {
    fire_volume_destroy(v);
    return FIRE_ERR_OOM;
  }
  *out = v;
  return FIRE_OK;
}

int fire_volume_destroy(FireVolume* v) {
  if (!v) return FIRE_ERR_BAD_ARG;
  cudaDeviceSynchronize();
  cudaFree(v->dLut); cudaFree(v->dLights); cudaFree(v->dLstate); cudaFree(v->dVol); cudaFree(v->dAux);
  if (v->dSharp) cudaFree(v->dSharp);
  delete v;
  return FIRE_OK;
}

int fire_volume_size(FireVolume* v, int* vw, int* vh) {
  if (!v || !vw || !vh) return FIRE_ERR_BAD_ARG;
  *vw = v->vw; *vh = v->vh;
  return FIRE_OK;
}

int fire_volume_set_params(FireVolume* v, const char* const* names, const float* values, int n) {
  if (!v || n < 0 || (n > 0 && (!names || !values))) return FIRE_ERR_BAD_ARG;
  for (int i = 0; i < n; ++i) {
    bool found = false;
    for (const NamedParam& p : kVolParams)
      if (names[i] && std::strcmp(names[i], p.name) == 0) { reinterpret_cast<float*>(&v->U)[p.offset] = values[i]; found = true; }
    if (!found) return FIRE_ERR_BAD_PARAM;
  }
  return FIRE_OK;
}

// lookAt (src/camera.js:6-17): forward, right = forward x (0, 1, 0), up = right x forward; fov in degrees.
int fire_volume_set_camera(FireVolume* v, const double pos[3], const double target[3], double fov_deg, float jit_x, float jit_y) {
  if (!v || !pos || !target) return FIRE_ERR_BAD_ARG;
  auto norm = [](double* a) {
    double l = std::hypot(std::hypot(a[0], a[1]), a[2]);
    if (l == 0.0) l = 1.0;
    a[0] /= l; a[1] /= l; a[2] /= l;
  };
  double f[3] = {target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]};
  norm(f);
  double r[3] = {f[1] * 0.0 - f[2] * 1.0, f[2] * 0.0 - f[0] * 0.0, f[0] * 1.0 - f[1] * 0.0};
  norm(r);
  const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
  VolU& U = v->U;
  U.camX = (float)pos[0]; U.camY = (float)pos[1]; U.camZ = (float)pos[2];
  U.fwdX = (float)f[0]; U.fwdY = (float)f[1]; U.fwdZ = (float)f[2];
  U.rgtX = (float)r[0]; U.rgtY = (float)r[1]; U.rgtZ = (float)r[2];
  U.upX = (float)u[0]; U.upY = (float)u[1]; U.upZ = (float)u[2];
  U.tanFov = (float)std::tan(fov_deg * 3.141592653589793 / 180.0 / 2.0);
  U.aspect = (float)((double)v->w / (double)v->h);
  U.jitX = jit_x; U.jitY = jit_y;
  return FIRE_OK;
}

int fire_volume_set_depth(FireVolume* v, const float* depth_dev, int width, int height) {
  if (!v || (depth_dev && (width < 1 || height < 1))) return FIRE_ERR_BAD_ARG;
  v->depth = depth_dev;
  v->U.depthW = depth_dev ? (float)width : 0.0f;
  v->U.depthH = depth_dev ? (float)height : 0.0f;
  return FIRE_OK;
}

// The uniforms of the next render (renderer.uploadParams, src/renderer.js:634-650); 64 floats.
int fire_volume_uniforms(FireVolume* v, double time, int frame, float* out, int n) {
  if (!v || !out || n < VOLU_FLOATS) return FIRE_ERR_BAD_ARG;
  FireInfo info;
  if (fire_sim_info(v->sim, &info) != FIRE_OK) return FIRE_ERR_STATE;
  VolU U = v->U;
  U.width = (float)v->w; U.height = (float)v->h; U.vw = (float)v->vw; U.vh = (float)v->vh;
  U.time = (float)time; U.frame = (float)frame;
  U.ox = info.origin[0]; U.oy = info.origin[1]; U.oz = info.origin[2]; U.dx = info.dx;
  U.sx = info.size[0]; U.sy = info.size[1]; U.sz = info.size[2];
  U.nx = (float)info.res[0]; U.ny = (float)info.res[1]; U.nz = (float)info.res[2];
  U.nLights = (float)NLIGHTS;
  // light smoothing step: time since the last render, -1 resets the filter (src/renderer.js:636)
  const bool reset = !v->haveLight || time < v->lastLightTime || time - v->lastLightTime > 0.5;
  U.lightDt = reset ? -1.0f : (float)(time - v->lastLightTime);
  std::memcpy(out, &U, sizeof U);
  return VOLU_FLOATS;
}

// One render: lights, the optional prefilter, the march (renderHDR's fire passes, src/renderer.js:666-690).
int fire_volume_render(FireVolume* v, double time, int frame, void* stream) {
  FIRE_RANGE("fire_volume_render");
  if (!v) return FIRE_ERR_BAD_ARG;
  float raw[VOLU_FLOATS];
  if (fire_volume_uniforms(v, time, frame, raw, VOLU_FLOATS) < 0) return FIRE_ERR_STATE;
  VolU U;
  std::memcpy(&U, raw, sizeof U);
  v->lastLightTime = time;
  v->haveLight = true;
  FireFieldDesc fs, fs2, fc;
  if (fire_sim_field(v->sim, FIRE_FIELD_S, &fs) || fire_sim_field(v->sim, FIRE_FIELD_S2, &fs2) || fire_sim_field(v->sim, FIRE_FIELD_CURL, &fc))
    return FIRE_ERR_STATE;
  const Dims d{fs.dims[0], fs.dims[1], fs.dims[2]};
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const float4* S = (const float4*)fs.data;
  k_lights<<<NLIGHTS, 256, 0, st>>>(U, S, v->dLut, v->dLights, v->dLstate);
  const float4* Svol = S;
  if (U.flameSharp > 0.0f && U.cubic > 0.5f) {
    if (!v->dSharp && cudaMalloc((void**)&v->dSharp, sizeof(float4) * (size_t)d.nx * d.ny * d.nz) != cudaSuccess) return FIRE_ERR_OOM;
    k_sharpen<<<dim3((d.nx + 7) / 8, (d.ny + 7) / 8, (d.nz + 3) / 4), dim3(8, 8, 4), 0, st>>>(U.flameSharp, S, v->dSharp, d);
    Svol = v->dSharp;
  }
  k_volume<<<dim3((v->vw + 7) / 8, (v->vh + 7) / 8), dim3(8, 8), 0, st>>>(U, Svol, (const float4*)fs2.data, d, (const uint2*)fc.data,
                                                                        v->dLut, v->dLights, v->depth, v->dVol, v->dAux);
  return cudaGetLastError() == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

// which: 0 volume image (vw x vh x 4: radiance, transmittance), 1 aux (vw x vh x 2: haze, depth),
// 2 lights (8 x 8), 3 blackbody LUT (2 x n x 4).  Synchronous.
int fire_volume_download(FireVolume* v, int which, float* host, size_t bytes) {
  if (!v || !host) return FIRE_ERR_BAD_ARG;
  const size_t px = (size_t)v->vw * v->vh;
  const void* src = nullptr;
  size_t need = 0;
  switch (which) {
    case 0: src = v->dVol; need = px * sizeof(float4); break;
    case 1: src = v->dAux; need = px * sizeof(float2); break;
    case 2: src = v->dLights; need = sizeof(float4) * 2 * NLIGHTS; break;
    case 3: src = v->dLut; need = sizeof(float4) * 2 * (size_t)v->lutN; break;
    default: return FIRE_ERR_BAD_ARG;
  }
  if (bytes != need) return FIRE_ERR_BAD_ARG;
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(host, src, need, cudaMemcpyDeviceToHost) != cudaSuccess) return FIRE_ERR_CUDA;
  return FIRE_OK;
}

}  // extern "C"
