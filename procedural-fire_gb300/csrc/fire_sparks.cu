// Burning sparks carried by the simulation's velocity field: the particle update of src/sparks.js:55-142
// (sparkUpdate) as two kernels per step.
//
// A spark is 4 float4 (64 B, the reference's storage layout): p = (position, age), v = (velocity, burn time
// left), q = (previous position, temperature K), m = (diameter mm, seed, alive, flicker Hz).
//
// Spawning: the reference hands spawn slots 0, 1, ... to dead particles with an atomic counter, so which
// particle gets which slot depends on execution order, while the slot alone drives the spawned spark's
// randomness.  Here the k-th dead particle in index order takes slot k (a block count pass and a per-block
// prefix), which is one of the orders the reference can produce and is deterministic.
#include "fire_device.cuh"
#include "fire_launch.cuh"

namespace fire {
namespace {

constexpr int SPT = 256;   // threads per CTA
constexpr float kTwoPi = 6.2831853f;

__device__ __forceinline__ uint32_t pcg1(uint32_t n) {   // src/shaders/lib.js:11-15
  const uint32_t s = n * 747796405u + 2891336453u;
  const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
__device__ __forceinline__ float rand2(uint32_t n, uint32_t m) { return __uint2float_rn(pcg1(n ^ pcg1(m))) * kInvU32; }   // lib.js:18

struct SparkRng {
  uint32_t seed, frame;
  __device__ float r(uint32_t slot, uint32_t k) const { return rand2(slot * 7919u + k * 104729u + seed, frame); }
  __device__ float gauss(uint32_t slot, uint32_t k) const {
    const float u1 = fmaxf(r(slot, k), 1e-6f), u2 = r(slot, k + 1u);
    return sqrtf(-2.0f * logf(u1)) * cosf(kTwoPi * u2);
  }
};

__device__ __forceinline__ f3 normalize3(f3 v) { return v / sqrtf(dot3(v, v)); }

// Fluid velocity at world position p (src/sparks.js:70-78): the velocity field sampled linearly with
// clamp-to-edge inside the box; above the box near the axis a slowing column; zero elsewhere.
__device__ __forceinline__ f3 fluid_vel(const SparkU& S, const float4* __restrict__ vel, Dims d, f3 p) {
  const f3 g = mk3((p.x - S.ox) / S.sx, (p.y - S.oy) / S.sy, (p.z - S.oz) / S.sz);
  if (g.x < 0.0f || g.y < 0.0f || g.z < 0.0f || g.x > 1.0f || g.y > 1.0f || g.z > 1.0f) {
    if (g.y > 1.0f && sqrtf(p.x * p.x + p.z * p.z) < 0.5f) return mk3(0.0f, 1.6f / (1.0f + (g.y - 1.0f) * 1.5f), 0.0f);
    return mk3(0.0f, 0.0f, 0.0f);
  }
  const f3 c = mk3(g.x * (float)d.nx, g.y * (float)d.ny, g.z * (float)d.nz);   // texel i centred at i + 0.5
  return xyz(sample(vel, make_tap(c, d), d));
}

// Dead particles per CTA.
__global__ void __launch_bounds__(SPT) k_spark_count(const float4* __restrict__ sp, int count, int* __restrict__ dead) {
  pdl_wait();
  pdl_trigger();
  const int i = blockIdx.x * SPT + threadIdx.x;
  const bool d = i < count && __ldg(sp + 4 * i + 3).z < 0.5f;
  const int n = __syncthreads_count(d);
  if (threadIdx.x == 0) dead[blockIdx.x] = n;
}

__global__ void __launch_bounds__(SPT) k_spark_update(float4* __restrict__ sp, SparkU S, const int* __restrict__ dead,
                                                      const float4* __restrict__ vel, Dims d, const uint2* __restrict__ curlT) {
  __shared__ int swarp[SPT / 32];
  __shared__ int sbase;
  pdl_wait();
  pdl_trigger();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int i = blockIdx.x * SPT + tid;
  const int count = (int)S.count;
  float4 P = make_float4(0.f, 0.f, 0.f, 0.f), V = P, Q = P, M = P;
  if (i < count) { P = sp[4 * i]; V = sp[4 * i + 1]; Q = sp[4 * i + 2]; M = sp[4 * i + 3]; }
  const bool isDead = i < count && M.z < 0.5f;
  // slot of a dead particle = number of dead particles before it
  {
    int acc = 0;
    for (int b = tid; b < (int)blockIdx.x; b += SPT) acc += __ldg(dead + b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) swarp[wid] = acc;
    __syncthreads();
    if (tid == 0) {
      int s = 0;
      for (int w = 0; w < SPT / 32; ++w) s += swarp[w];
      sbase = s;
    }
    __syncthreads();
  }
  const unsigned ball = __ballot_sync(0xffffffffu, isDead);
  if (lane == 0) swarp[wid] = __popc(ball);
  __syncthreads();
  int before = sbase;
  for (int w = 0; w < wid; ++w) before += swarp[w];
  before += __popc(ball & ((1u << lane) - 1u));
  if (i >= count) return;

  const float dt = S.dt;
  const SparkRng R{(uint32_t)S.seed, (uint32_t)S.frame};
  if (isDead) {   // src/sparks.js:82-111
    const uint32_t want = (uint32_t)(S.nBase + S.nBurst);
    if (want == 0u) return;
    const uint32_t slot = (uint32_t)before;
    if (slot >= want) return;
    const bool burst = slot >= (uint32_t)S.nBase;
    f3 p, v;
    if (burst) {
      p = mk3(S.burstX, S.burstY, S.burstZ) +
          (mk3(R.r(slot, 7u), R.r(slot, 8u), R.r(slot, 9u)) - mk3(0.5f, 0.5f, 0.5f)) * S.burstRadius * 2.0f;
      f3 radial = mk3(p.x, 0.0f, p.z);
      radial = len3(radial) > 1e-3f ? normalize3(radial) : mk3(0.0f, 0.0f, 0.0f);
      const f3 aim = mk3(S.aimX, 0.0f, S.aimZ);
      const f3 dir = normalize3(mk3(R.gauss(slot, 1u), fabsf(R.gauss(slot, 3u)) * 1.2f + 0.7f, R.gauss(slot, 5u)) + (radial + aim) * S.burstFan);
      v = dir * S.burstSpeed * (0.5f + 0.8f * R.r(slot, 10u));
    } else {
      const float a = R.r(slot, 1u) * kTwoPi, rr = sqrtf(R.r(slot, 2u)) * S.bedRadius;
      p = mk3(cosf(a) * rr, 0.05f + R.r(slot, 3u) * 0.12f, sinf(a) * rr);
      v = mk3(R.gauss(slot, 4u) * 0.4f, 0.6f + R.r(slot, 6u) * 1.8f, R.gauss(slot, 11u) * 0.4f);
    }
    const float dmm = clampf(0.5f * expf(0.55f * R.gauss(slot, 13u)) * S.sizeK * (burst ? S.burstSize : 1.0f), 0.15f, 2.5f);
    const float tb = (0.25f + 2.0f * dmm * dmm) * (0.6f + 0.8f * R.r(slot, 15u)) * S.lifeK;
    const float T0 = 1230.0f + 70.0f * R.gauss(slot, 16u) + (burst ? 80.0f : 0.0f);
    const float fl = R.r(slot, 20u) < 0.45f ? 5.0f + 15.0f * R.r(slot, 18u) : 0.0f;
    sp[4 * i] = make_float4(p.x, p.y, p.z, 0.0f);
    sp[4 * i + 1] = make_float4(v.x, v.y, v.z, tb);
    sp[4 * i + 2] = make_float4(p.x, p.y, p.z, T0);
    sp[4 * i + 3] = make_float4(dmm, R.r(slot, 19u), 1.0f, fl);
    return;
  }
  // alive: integrate (src/sparks.js:113-141)
  const float dmm = M.x;
  f3 p = xyz(P), v = xyz(V);
  const float tau = fmaxf(0.4f * dmm * dmm, 0.01f);
  f3 u = fluid_vel(S, vel, d, p) * S.upK;
  const f3 tq = p * 0.9f + mk3(0.0f, -S.time * 0.5f, S.time * 0.13f + M.y * 3.0f);
  const float turbAmp = S.turb * (0.3f + 3.0f * sstep(0.4f, 1.2f, p.y)) / 12.0f;
  u = u + xyz(sample_table(curlT, tq)) * turbAmp;
  const float k = 1.0f - expf(-dt / tau);
  v = mk3(mixf(v.x, u.x, k), mixf(v.y, u.y, k), mixf(v.z, u.z, k));
  v.y -= 9.81f * (1.0f - 0.004f) * dt * (dmm < 0.3f ? 0.2f : 1.0f);
  const float4 qn = make_float4(p.x, p.y, p.z, Q.w);
  p = p + v * dt;
  float T = Q.w;
  const float tb = V.w - dt;
  if (tb > 0.0f) {
    const float rel = len3(u - v);
    T = mixf(T, 1180.0f + 60.0f * fminf(rel, 3.0f) + 60.0f * (M.y - 0.5f), 1.0f - expf(-dt / 0.3f));
  } else {
    T = 293.0f + (T - 293.0f) * expf(-dt / (0.06f + 0.08f * dmm));
  }
  const float age = P.w + dt;
  const float alive = (T < 760.0f || p.y < 0.0f || p.y > 4.5f || sqrtf(p.x * p.x + p.z * p.z) > 3.0f || age > 12.0f) ? 0.0f : 1.0f;
  sp[4 * i] = make_float4(p.x, p.y, p.z, age);
  sp[4 * i + 1] = make_float4(v.x, v.y, v.z, tb);
  sp[4 * i + 2] = make_float4(qn.x, qn.y, qn.z, T);
  sp[4 * i + 3] = make_float4(M.x, M.y, alive, M.w);
}

}  // namespace

int spark_blocks(int count) { return (count + SPT - 1) / SPT; }
void launch_sparks(float4* sp, const SparkU& S, int* dead, const float4* vel, Dims d, const uint2* curl, cudaStream_t st) {
  const int count = (int)S.count;
  if (count <= 0) return;
  const dim3 g(spark_blocks(count));
  launch_pdl(k_spark_count, g, dim3(SPT), 0, st, (const float4*)sp, count, dead);
  launch_pdl(k_spark_update, g, dim3(SPT), 0, st, sp, S, (const int*)dead, vel, d, curl);
}

}  // namespace fire
