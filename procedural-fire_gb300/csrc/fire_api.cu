// Host runtime behind the C ABI (include/fire_sim.h): the GB300 counterpart of FireSim (src/sim.js:48-649)
// and of the page-level event and diagnostics API (src/main.js).
//
// Design:
//   * All fields and multigrid levels live in one device arena (dense float4 / float arrays).
//   * The per-step parameter block (SIM_FIELDS + extension, 800 bytes) is staged in a pinned ring and
//     copied to the device ahead of each step on the caller's stream, replacing queue.writeBuffer of the
//     uniform buffer (src/gpu.js:70).  The step body reads it through a fixed device pointer, so the
//     whole step is captured once as a CUDA graph and replayed every step.
//   * The emitter geometry runs outside the graph, only when stale (src/sim.js:632).
//   * The residual-driven multigrid mode loops V-cycles inside the graph with a conditional WHILE node;
//     the loop condition is set on the device from the FP64 residual norm, so no host round trip.
#include <cmath>
#include <cstdio>
#include <cstdarg>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cuda_runtime.h>
#include "../../include/fire_sim.h"
#include "fire_internal.h"

namespace fire {

const char* const kParamNames[P_COUNT] = {
  "nx", "ny", "nz", "dx", "dt", "time", "frame", "seed",
  "ox", "oy", "oz", "nLogs",
  "fuelSrc", "bedFuel", "srcTemp", "bedTemp", "srcVel", "srcFreq", "srcSpeed", "srcThresh",
  "ignT", "kMix", "rs", "heatOut", "expansion", "sootForm", "sootOx", "radCool",
  "coolRate", "sootDissip", "smokeDissip", "vitDecay", "fuelDissip", "buoyancy", "vortEps", "turbAmp",
  "turbFreq", "turbRise", "turbEvolve", "windX", "windZ", "gust", "intensity", "velDissip",
  "bedRadius", "logSrc", "burstX", "burstY", "burstZ", "burstAmt", "smolder", "sponge", "hotR0", "hotR1", "hotY1",
  "visc", "lamAge", "anchorFreq", "srcFloor", "anchorGain",
};

// SIM_DEFAULTS (src/sim.js:25-44) in SIM_FIELDS order; simulation-owned entries are 0 (seed: `?? 0`).
const float kParamDefaults[P_STRIDE] = {
  0, 0, 0, 0, 0, 0, 0, 0,                       // nx ny nz dx dt time frame seed
  0, 0, 0, 0,                                   // ox oy oz nLogs
  0.13f, 0.16f, 0.75f, 0.82f, 0.25f, 35.0f, 0.06f, 0.0f,       // fuelSrc bedFuel srcTemp bedTemp srcVel srcFreq srcSpeed srcThresh
  550.0f, 30.0f, 4.7f, 7700.0f, 0.7f, 25.0f, 30.0f, 0.25f,     // ignT kMix rs heatOut expansion sootForm sootOx radCool
  3.0f, 0.4f, 0.3f, 1.5f, 0.3f, 26.8f, 8.0f, 0.8f,             // coolRate sootDissip smokeDissip vitDecay fuelDissip buoyancy vortEps turbAmp
  1.5f, 1.5f, 0.6f, 0.0f, 0.0f, 0.0f, 1.0f, 0.05f,             // turbFreq turbRise turbEvolve windX windZ gust intensity velDissip
  0.22f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.02f, 1.0f, 0.12f, 0.45f, 0.5f,   // bedRadius logSrc burstX..burstAmt smolder sponge hotR0 hotR1 hotY1
  0.0f, 0.0f, 1.6f, 0.25f, 0.95f,                              // visc lamAge anchorFreq srcFloor anchorGain
  0, 0, 0, 0,                                                   // padding to 64
};

// ---- kernels defined in other translation units that the runtime launches directly ----
cudaError_t kernels_probe();
void launch_mg_counter_reset(int* counter, cudaStream_t st);
void launch_residual_decide(const MGLevel& L, double* partials, double* sums2, double tol, int max_cycles, int* counter,
                            double* rel_out, cudaGraphConditionalHandle h, cudaStream_t st);

}  // namespace fire

using namespace fire;

namespace {
constexpr size_t ALIGN = 256;
size_t align_up(size_t v) { return (v + ALIGN - 1) / ALIGN * ALIGN; }
}  // namespace

#include "fire_simobj.h"
#include "fire_nvtx.h"

namespace fire {
namespace rt {

int set_err(FireSim* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return code;
}
#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return set_err(sim, FIRE_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

float* field_ptr4(FireSim* s, int which) {
  switch (which) {
    case FIRE_FIELD_VEL: return (float*)s->f.vel;
    case FIRE_FIELD_VELX: return (float*)s->f.velX;
    case FIRE_FIELD_VELY: return (float*)s->f.velY;
    case FIRE_FIELD_S: return (float*)s->f.S;
    case FIRE_FIELD_SX: return (float*)s->f.SX;
    case FIRE_FIELD_SY: return (float*)s->f.SY;
    case FIRE_FIELD_S2: return (float*)s->f.S2;
    case FIRE_FIELD_S2X: return (float*)s->f.S2X;
    case FIRE_FIELD_S2Y: return (float*)s->f.S2Y;
    case FIRE_FIELD_VORT: return (float*)s->f.vort;
    case FIRE_FIELD_GEO: return (float*)s->f.geo;
    default: return nullptr;
  }
}

// Fill the simulation-owned entries of the block, as uploadUniforms does (src/sim.js:620-624), and apply
// the event envelopes for this step.
void fill_block(FireSim* s, float dt, float* out) {
  float* P = out;
  std::memcpy(P, s->params, sizeof(float) * P_STRIDE);
  P[P_nx] = (float)s->res[0]; P[P_ny] = (float)s->res[1]; P[P_nz] = (float)s->res[2];
  P[P_dx] = (float)s->dx; P[P_dt] = dt; P[P_time] = (float)s->time; P[P_frame] = (float)s->frame;
  P[P_ox] = s->origin[0]; P[P_oy] = s->origin[1]; P[P_oz] = s->origin[2];
  P[P_nLogs] = (float)s->nLogs;
  std::memcpy(P + P_STRIDE, s->ext, sizeof(float) * E_COUNT);
  // per-step constants shared by every cell, evaluated once here in FP32 as the per-cell code would
  float* E = P + P_STRIDE;
  E[E_decaySoot] = std::exp(-P[P_sootDissip] * dt);
  E[E_decayFuel] = std::exp(-P[P_fuelDissip] * dt);
  E[E_decayVit] = std::exp(-P[P_vitDecay] * dt);
  E[E_decaySmoke] = std::exp(-P[P_smokeDissip] * dt);
  E[E_decayVel] = std::exp(-P[P_velDissip] * dt);
  E[E_turbK] = P[P_turbAmp] / 12.0f;                                        // src/sim.js:368
  {
    const float ign0 = P[P_ignT] - 50.0f, ign1 = P[P_ignT] + 50.0f;         // src/sim.js:302
    const float th0 = P[P_srcThresh] - 0.25f, th1 = P[P_srcThresh] + 0.25f;   // src/sim.js:252
    E[E_invIgn] = 1.0f / (ign1 - ign0);
    E[E_invPulse] = 1.0f / (th1 - th0);
    E[E_invSootAge] = 1.0f / (E[E_sootAge1] - E[E_sootAge0]);
  }
  float top = -1e30f;
  for (int i = 0; i < (int)E[E_nSpots]; ++i) {
    const float* sp = E + E_SPOTS + SPOT_STRIDE * i;
    top = std::max(top, sp[1] + 4.0f * sp[3]);
  }
  E[E_spotTop] = top;
}

void advance_events(FireSim* s, float dt) {
  // burst: burstAmt held while the simulated time is before burstUntil (src/main.js:404, 461)
  if (s->burstActive) {
    if (s->time < s->burstUntil) s->params[P_burstAmt] = s->burstAmt;
    else { s->params[P_burstAmt] = 0.0f; s->burstActive = false; }
  }
  // gust: windT counts down before the envelope is evaluated (src/main.js:459-461)
  if (s->gustActive) {
    s->gustLeft = std::max(0.0, s->gustLeft - (double)dt);
    double gw = s->gustLeft > 0 ? std::sin(3.141592653589793 * (1.0 - s->gustLeft / s->gustDur)) : 0.0;
    s->params[P_windX] = (float)(s->windBase[0] + -1.4 * gw * s->gustStrength);
    s->params[P_windZ] = (float)(s->windBase[1] + 0.5 * gw * s->gustStrength);
    if (s->gustLeft <= 0) {
      s->gustActive = false;
      s->params[P_windX] = s->windBase[0];
      s->params[P_windZ] = s->windBase[1];
    }
  }
}

// Stage a slot of the pinned ring (waiting if its previous copy has not run yet).
int ring_slot(FireSim* sim, float** slot, cudaEvent_t* ev) {
  int k = sim->ringPos;
  sim->ringPos = (k + 1) % RING_SLOTS;
  if (sim->ringUsed[k]) CK(cudaEventSynchronize(sim->ringEv[k]));
  sim->ringUsed[k] = true;
  *slot = sim->hRing + (size_t)k * SLOT_FLOATS;
  *ev = sim->ringEv[k];
  return FIRE_OK;
}

int upload_block(FireSim* sim, float dt, cudaStream_t st, bool with_logs, const float** staged) {
  float* slot;
  cudaEvent_t ev;
  int rc = ring_slot(sim, &slot, &ev);
  if (rc) return rc;
  fill_block(sim, dt, slot);
  if (staged) *staged = slot;
  CK(cudaMemcpyAsync(sim->dBlock, slot, sizeof(float) * BLOCK_FLOATS, cudaMemcpyHostToDevice, st));
  if (with_logs) {
    std::memcpy(slot + BLOCK_FLOATS, sim->logs, sizeof(float) * MAX_LOGS * 8);
    CK(cudaMemcpyAsync(sim->dLogs, slot + BLOCK_FLOATS, sizeof(float) * MAX_LOGS * 8, cudaMemcpyHostToDevice, st));
  }
  CK(cudaEventRecord(ev, st));
  return FIRE_OK;
}

// `iters` red-black sweeps of level l (src/sim.js:576-586): colour 0 then colour 1, one launch each; with
// first_done the first colour-0 sweep has already been applied (by the fused restriction).
void record_smooth(FireSim* s, int l, int iters, cudaStream_t st, bool first_done = false) {
  for (int k = 0; k < iters; ++k) {
    if (k > 0 || !first_done) launch_smooth(s->levels[l], 0, st);
    launch_smooth(s->levels[l], 1, st);
  }
}
// One V(2,2) cycle (src/sim.js:588-599).  Levels [tailFirst, n) run inside one tail kernel.  A restriction
// onto a level that is smoothed by launches also applies that level's first colour-0 sweep.
void record_vcycle(FireSim* s, cudaStream_t st) {
  const int n = (int)s->levels.size();
  const int T = s->tailFirst;
  const int top = std::min(T, n - 1);
  for (int i = 0; i < top; ++i) {
    record_smooth(s, i, 2, st, i > 0);
    if (i + 1 < top) launch_restrict_smooth(s->levels[i], s->levels[i + 1], st);
    else launch_restrict(s->levels[i], s->levels[i + 1], st);
  }
  if (T < n) launch_tail(s->levels.data(), T, n, 2, 2, s->coarseIters, s->dCounter + 2, st, false, nullptr, s->tailWaitPolls);
  else record_smooth(s, n - 1, s->coarseIters, st);
  for (int i = top - 1; i >= 0; --i) { launch_prolong(s->levels[i], s->levels[i + 1], st); record_smooth(s, i, 2, st); }
}

int record_ev(FireSim* sim, int idx, cudaStream_t st, bool prof) {
  if (prof) CK(cudaEventRecordWithFlags(sim->stageEv[idx], st, cudaEventRecordExternal));
  return FIRE_OK;
}

// Records the multigrid solve: a fixed number of cycles, or (residual-driven mode) a conditional
// WHILE loop whose body is one cycle plus the FP64 residual norm and the device-side decision.  The loop
// counts its cycles from zero: counter_cleared says a divergence kernel recorded just before has cleared the
// count (launch_div with the counter), else a clearing kernel is recorded here.
int record_mg(FireSim* sim, cudaStream_t st, bool counter_cleared) {
  if (sim->mg_max_cycles <= 0) {
    for (int c = 0; c < sim->vcycles; ++c) record_vcycle(sim, st);
    return FIRE_OK;
  }
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps;
  size_t ndeps;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  if (cs != cudaStreamCaptureStatusActive) return set_err(sim, FIRE_ERR_STATE, "residual-driven solve needs graph capture");
  if (!counter_cleared) launch_mg_counter_reset(sim->dCounter, st);
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  // capture the loop body on the side stream into the body graph
  cudaStream_t bs = sim->capStream;
  CK(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  record_vcycle(sim, bs);
  launch_residual_decide(sim->levels[0], sim->dPartials, sim->dSmall, sim->mg_tol, sim->mg_max_cycles, sim->dCounter,
                         sim->dSmall + 19, h, bs);
  cudaGraph_t outg;
  CK(cudaStreamEndCapture(bs, &outg));
  return FIRE_OK;
}

// Records one step body (src/sim.js:633-644) on `st`: the parameter block must already be on the device.
int record_step(FireSim* sim, cudaStream_t st, bool prof) {
  int rc;
  const Dims d = sim->d;
  const float* P = sim->dBlock;
  if ((rc = record_ev(sim, 0, st, prof))) return rc;
  launch_adv1(P, sim->f, d, st);
  if ((rc = record_ev(sim, 1, st, prof))) return rc;
  launch_adv2(P, sim->f, d, st);
  if ((rc = record_ev(sim, 2, st, prof))) return rc;
  if ((rc = record_ev(sim, 3, st, prof))) return rc;    // curl is fused into forces
  {
    // the block is a kernel parameter here; fire_sim_step sets each step's on the instantiated graph
    ParamBlock pb;
    std::memset(&pb, 0, sizeof pb);
    launch_forces_pb(pb, sim->f, sim->noise, sim->curl, d, st);
    CK(cudaGetLastError());
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &ndeps));
    if (cs != cudaStreamCaptureStatusActive || ndeps != 1) return set_err(sim, FIRE_ERR_STATE, "forces node not captured");
    sim->forcesNode = deps[0];
  }
  if ((rc = record_ev(sim, 4, st, prof))) return rc;
  if (sim->stepStats) {
    // S is final after the forces stage (projection only changes vel): its diagnostics run on a branch that
    // overlaps the divergence, the pressure solve and the projection, and joins at the end of the step
    CK(cudaEventRecord(sim->forkEv, st));
    CK(cudaStreamWaitEvent(sim->sideStream, sim->forkEv, 0));
    launch_diag(sim->f.S, d, (float)sim->dx, sim->dDiagPartials, sim->dSmall + 24, sim->sideStream);
    CK(cudaGetLastError());
    CK(cudaEventRecord(sim->joinEv, sim->sideStream));
  }
  launch_div(P, sim->f, sim->levels[0].b, d, st, sim->mg_max_cycles > 0 ? sim->dCounter : nullptr);
  if ((rc = record_ev(sim, 5, st, prof))) return rc;
  if ((rc = record_mg(sim, st, sim->mg_max_cycles > 0))) return rc;
  if ((rc = record_ev(sim, 6, st, prof))) return rc;
  launch_project(P, sim->f, sim->levels[0].p, d, st);
  if ((rc = record_ev(sim, 7, st, prof))) return rc;
  if (sim->stepStats) CK(cudaStreamWaitEvent(st, sim->joinEv, 0));
  CK(cudaGetLastError());
  return FIRE_OK;
}

void drop_graph(FireSim* s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->exec = nullptr;
  s->graph = nullptr;
  s->forcesNode = nullptr;
}

int build_graph(FireSim* sim) {
  drop_graph(sim);
  // the main capture runs on a private stream; the residual loop body is captured on capStream
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return set_err(sim, FIRE_ERR_CUDA, "begin capture: %s", cudaGetErrorString(e)); }
  int rc = record_step(sim, st, sim->profiling);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  cudaStreamDestroy(st);
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return set_err(sim, FIRE_ERR_CUDA, "end capture: %s", cudaGetErrorString(e));
  sim->graph = g;
  e = cudaGraphInstantiate(&sim->exec, g, 0);
  if (e != cudaSuccess) { drop_graph(sim); return set_err(sim, FIRE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  sim->graphProfiled = sim->profiling;
  return FIRE_OK;
}

int ensure_geo(FireSim* sim, cudaStream_t st) {
  if (sim->geoReady && !sim->logsDirty) return FIRE_OK;
  // geometry uses the current block (dx, origin, hot radii, nLogs) and the log buffer
  launch_geo(sim->dBlock, sim->dLogs, sim->f.geo, sim->f.solid, sim->d, st);
  CK(cudaGetLastError());
  sim->geoReady = true;
  sim->logsDirty = false;
  return FIRE_OK;
}

}  // namespace rt
}  // namespace fire
using namespace fire::rt;

// =====================================================================================================
extern "C" {

const char* fire_version(void) { return "procedural-fire-gb300 0.1 (sm_103a)"; }

int fire_param_index(const char* name) {
  if (!name) return -1;
  for (int i = 0; i < P_COUNT; ++i)
    if (std::strcmp(name, kParamNames[i]) == 0) return i;
  return -1;
}
const char* fire_param_name(int index) { return (index >= 0 && index < P_COUNT) ? kParamNames[index] : nullptr; }
int fire_param_defaults(float* block64) {
  if (!block64) return FIRE_ERR_BAD_ARG;
  std::memcpy(block64, kParamDefaults, sizeof(float) * P_STRIDE);
  return FIRE_OK;
}

int fire_device_ok(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return 0;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return 0;
  if (p.major != 10 || p.minor != 3) return 0;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  cudaError_t e = kernels_probe();
  cudaSetDevice(prev);
  return e == cudaSuccess ? 1 : 0;
}

int fire_sim_create(const FireConfig* cfg, const float* logs, int n_logs, FireSim** out) {
  FIRE_RANGE("fire_sim_create");
  FireSim* sim = nullptr;
  if (!cfg || !out) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  for (int i = 0; i < 3; ++i)
    if (cfg->res[i] < 2 || cfg->size[i] <= 0.0f) return FIRE_ERR_BAD_ARG;
  // the stencil kernels address cells with 32-bit offsets
  if ((long long)cfg->res[0] * cfg->res[1] * cfg->res[2] > 0x7fffffffLL) return FIRE_ERR_BAD_ARG;
  if (n_logs < 0 || n_logs > MAX_LOGS || (n_logs > 0 && !logs)) return FIRE_ERR_BAD_ARG;
  if (cfg->vcycles < 0 || cfg->mg_max_cycles < 0) return FIRE_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FIRE_ERR_NO_DEVICE;
  if (cfg->device < 0 || cfg->device >= ndev) return FIRE_ERR_BAD_ARG;
  if (!fire_device_ok(cfg->device)) return FIRE_ERR_NO_DEVICE;

  sim = new FireSim();
  sim->device = cfg->device;
  if (cudaSetDevice(sim->device) != cudaSuccess) { delete sim; return FIRE_ERR_NO_DEVICE; }
  for (int i = 0; i < 3; ++i) { sim->res[i] = cfg->res[i]; sim->size[i] = cfg->size[i]; }
  sim->dx = (double)cfg->size[0] / (double)cfg->res[0];                        // src/sim.js:53
  sim->origin[0] = -cfg->size[0] / 2; sim->origin[1] = 0; sim->origin[2] = -cfg->size[2] / 2;   // src/sim.js:54
  sim->vcycles = cfg->vcycles;
  sim->mg_max_cycles = cfg->mg_max_cycles;
  sim->mg_tol = cfg->mg_tol;
  std::memcpy(sim->params, kParamDefaults, sizeof sim->params);
  std::memset(sim->ext, 0, sizeof sim->ext);
  sim->ext[E_sootAge0] = 0.015f;
  sim->ext[E_sootAge1] = 0.05f;
  sim->ext[E_bedGain] = 1.0f;
  sim->ext[E_spotRef] = 4.0f;
  std::memset(sim->logs, 0, sizeof sim->logs);
  if (n_logs > 0) std::memcpy(sim->logs, logs, sizeof(float) * 8 * n_logs);
  sim->nLogs = n_logs;
  sim->d = Dims{cfg->res[0], cfg->res[1], cfg->res[2]};

  // multigrid hierarchy (src/sim.js:79-87): halve while every dim is even and the smallest > 6
  {
    int x = cfg->res[0], y = cfg->res[1], z = cfg->res[2];
    double h = sim->dx;
    while (true) {
      MGLevel L{x, y, z, (float)h, nullptr, nullptr};
      sim->levels.push_back(L);
      if (x % 2 || y % 2 || z % 2 || std::min(x, std::min(y, z)) <= 6) break;
      x /= 2; y /= 2; z /= 2; h *= 2;
    }
    const MGLevel& C = sim->levels.back();
    const double PI = 3.14159265358979323846;
    double mu = (std::cos(PI / C.nx) + std::cos(PI / (2.0 * C.ny)) + std::cos(PI / C.nz)) / 3.0;   // src/sim.js:91-92
    sim->coarseIters = (int)std::max(8.0, std::min(64.0, std::ceil(std::log(0.05) / std::log(mu * mu))));
    const int n = (int)sim->levels.size();
    sim->tailFirst = tail_first(sim->levels.data(), n);
  }

  // device arena
  const size_t cells = (size_t)cfg->res[0] * cfg->res[1] * cfg->res[2];
  size_t off = 0;
  std::vector<size_t> fieldOff(11);
  for (int i = 0; i < 11; ++i) { fieldOff[i] = off; off = align_up(off + cells * sizeof(float4)); }
  std::vector<size_t> pOff(sim->levels.size()), bOff(sim->levels.size());
  for (size_t l = 0; l < sim->levels.size(); ++l) {
    size_t c = (size_t)sim->levels[l].nx * sim->levels[l].ny * sim->levels[l].nz;
    pOff[l] = off; off = align_up(off + c * sizeof(float));
    bOff[l] = off; off = align_up(off + c * sizeof(float));
  }
  const size_t tabBytes = (size_t)TABLE_N * TABLE_N * TABLE_N * sizeof(uint2);
  size_t solidOff = off; off = align_up(off + cells);
  size_t noiseOff = off; off = align_up(off + tabBytes);
  size_t curlOff = off; off = align_up(off + tabBytes);
  size_t blockOff = off; off = align_up(off + sizeof(float) * BLOCK_FLOATS);
  size_t logsOff = off; off = align_up(off + sizeof(float) * MAX_LOGS * 8);
  sim->partialsCount = std::max(stats_partials_count(sim->d), residual_partials_count(sim->levels[0]));
  size_t partOff = off; off = align_up(off + sizeof(double) * 16 * (size_t)sim->partialsCount);
  size_t diagPartOff = off; off = align_up(off + sizeof(double) * 16 * (size_t)stats_partials_count(sim->d));
  size_t smallOff = off; off = align_up(off + sizeof(double) * 48);
  size_t cntOff = off; off = align_up(off + sizeof(int) * 4);
  sim->arenaBytes = off;
  cudaError_t e = cudaMalloc(&sim->arena, off);
  if (e != cudaSuccess) { delete sim; return FIRE_ERR_OOM; }
  char* A = (char*)sim->arena;
  float4** fp[11] = {&sim->f.vel, &sim->f.velX, &sim->f.velY, &sim->f.S, &sim->f.SX, &sim->f.SY,
                     &sim->f.S2, &sim->f.S2X, &sim->f.S2Y, &sim->f.vort, &sim->f.geo};
  for (int i = 0; i < 11; ++i) *fp[i] = (float4*)(A + fieldOff[i]);
  for (size_t l = 0; l < sim->levels.size(); ++l) {
    sim->levels[l].p = (float*)(A + pOff[l]);
    sim->levels[l].b = (float*)(A + bOff[l]);
  }
  sim->noise = (uint2*)(A + noiseOff);
  sim->curl = (uint2*)(A + curlOff);
  sim->f.solid = (unsigned char*)(A + solidOff);
  sim->dBlock = (float*)(A + blockOff);
  sim->dLogs = (float*)(A + logsOff);
  sim->dPartials = (double*)(A + partOff);
  sim->dSmall = (double*)(A + smallOff);
  sim->dDiagPartials = (double*)(A + diagPartOff);
  sim->dCounter = (int*)(A + cntOff);

  auto fail = [&](int code) { fire_sim_destroy(sim); return code; };
  if (cudaHostAlloc((void**)&sim->hRing, sizeof(float) * SLOT_FLOATS * RING_SLOTS, cudaHostAllocDefault) != cudaSuccess) return fail(FIRE_ERR_OOM);
  if (cudaHostAlloc((void**)&sim->hSmall, sizeof(double) * 32, cudaHostAllocDefault) != cudaSuccess) return fail(FIRE_ERR_OOM);
  if (cudaHostAlloc((void**)&sim->hCounter, sizeof(int) * 4, cudaHostAllocDefault) != cudaSuccess) return fail(FIRE_ERR_OOM);
  for (int k = 0; k < RING_SLOTS; ++k) {
    sim->ringUsed[k] = false;
    if (cudaEventCreateWithFlags(&sim->ringEv[k], cudaEventDisableTiming) != cudaSuccess) return fail(FIRE_ERR_CUDA);
  }
  for (int k = 0; k <= FIRE_STAGE_COUNT; ++k)
    if (cudaEventCreate(&sim->stageEv[k]) != cudaSuccess) return fail(FIRE_ERR_CUDA);
  if (cudaEventCreateWithFlags(&sim->doneEv, cudaEventDisableTiming) != cudaSuccess) return fail(FIRE_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&sim->capStream, cudaStreamNonBlocking) != cudaSuccess) return fail(FIRE_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&sim->sideStream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&sim->forkEv, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&sim->joinEv, cudaEventDisableTiming) != cudaSuccess)
    return fail(FIRE_ERR_CUDA);
  if (mg_configure(TAIL_SMEM_BUDGET) != cudaSuccess) return fail(set_err(sim, FIRE_ERR_CUDA, "tail kernel smem opt-in failed"));
  if (step_configure() != cudaSuccess) return fail(set_err(sim, FIRE_ERR_CUDA, "forces kernel smem opt-in failed"));

  // zero state (reset semantics), bake the tables (src/noise.js), upload logs
  cudaStream_t st = sim->capStream;
  if (cudaMemsetAsync(sim->arena, 0, sim->arenaBytes, st) != cudaSuccess) return fail(FIRE_ERR_CUDA);
  launch_noise_table(sim->noise, TABLE_N, cfg->noise_seed, st);
  launch_curl_table(sim->noise, sim->curl, TABLE_N, st);
  if (cudaGetLastError() != cudaSuccess) return fail(FIRE_ERR_CUDA);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(set_err(sim, FIRE_ERR_CUDA, "table bake failed"));
  sim->geoReady = false;
  sim->logsDirty = true;
  *out = sim;
  return FIRE_OK;
}

int fire_sim_destroy(FireSim* sim) {
  if (!sim) return FIRE_ERR_BAD_ARG;
  cudaSetDevice(sim->device);
  cudaDeviceSynchronize();
  drop_graph(sim);
  for (int k = 0; k < RING_SLOTS; ++k) if (sim->ringEv[k]) cudaEventDestroy(sim->ringEv[k]);
  for (int k = 0; k <= FIRE_STAGE_COUNT; ++k) if (sim->stageEv[k]) cudaEventDestroy(sim->stageEv[k]);
  if (sim->doneEv) cudaEventDestroy(sim->doneEv);
  if (sim->capStream) cudaStreamDestroy(sim->capStream);
  if (sim->sideStream) cudaStreamDestroy(sim->sideStream);
  if (sim->forkEv) cudaEventDestroy(sim->forkEv);
  if (sim->joinEv) cudaEventDestroy(sim->joinEv);
  if (sim->hRing) cudaFreeHost(sim->hRing);
  if (sim->hSmall) cudaFreeHost(sim->hSmall);
  if (sim->hCounter) cudaFreeHost(sim->hCounter);
  if (sim->arena) cudaFree(sim->arena);
  delete sim;
  return FIRE_OK;
}

int fire_sim_step(FireSim* sim, float dt, int n_steps, void* stream) {
  FIRE_RANGE("fire_sim_step");
  if (!sim || n_steps < 0 || !(dt > 0.0f)) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  if (!sim->exec || sim->graphProfiled != sim->profiling) {
    int rc = build_graph(sim);
    if (rc) return rc;
  }
  for (int s = 0; s < n_steps; ++s) {
    advance_events(sim, dt);
    const bool geo = !sim->geoReady || sim->logsDirty;
    const float* staged = nullptr;
    int rc = upload_block(sim, dt, st, geo, &staged);
    if (rc) return rc;
    if (geo && (rc = ensure_geo(sim, st))) return rc;
    ParamBlock pb;
    std::memcpy(pb.v, staged, sizeof pb.v);
    CK(forces_pb_set(sim->exec, sim->forcesNode, pb, sim->f, sim->noise, sim->curl, sim->d));
    CK(cudaGraphLaunch(sim->exec, st));
    sim->stepStatsValid = sim->stepStats;
    sim->time += dt;                                                          // src/sim.js:646-647
    sim->frame += 1;
    sim->stepsRun += 1;
  }
  if (sim->profiling) { CK(cudaEventRecord(sim->doneEv, st)); sim->profiledStepPending = n_steps > 0; }
  return FIRE_OK;
}

int fire_sim_sync(FireSim* sim) {
  if (!sim) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  // device-side bounded waits report through counter slot 2 instead of hanging
  int err = 0;
  CK(cudaMemcpy(&err, sim->dCounter + 2, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    CK(cudaMemset(sim->dCounter + 2, 0, sizeof(int)));
    return set_err(sim, FIRE_ERR_CUDA, "a device-side wait timed out (multigrid tail bulk copy)");
  }
  return FIRE_OK;
}

int fire_sim_set_params(FireSim* sim, const char* const* names, const float* values, int n) {
  if (!sim || n < 0 || (n > 0 && (!names || !values))) return FIRE_ERR_BAD_ARG;
  int idx[P_COUNT * 4];
  if (n > (int)(sizeof idx / sizeof idx[0])) return set_err(sim, FIRE_ERR_BAD_ARG, "too many parameters");
  for (int i = 0; i < n; ++i) {
    idx[i] = fire_param_index(names[i]);
    if (idx[i] < 0) return set_err(sim, FIRE_ERR_BAD_PARAM, "unknown uniform SimParams.%s", names[i] ? names[i] : "(null)");
  }
  for (int i = 0; i < n; ++i) {
    const int k = idx[i];
    if (k == P_hotR0 || k == P_hotR1 || k == P_hotY1 || k == P_bedRadius) sim->geoReady = false;   // src/sim.js:602
    sim->params[k] = values[i];
    if (k == P_windX && !sim->gustActive) sim->windBase[0] = values[i];
    if (k == P_windZ && !sim->gustActive) sim->windBase[1] = values[i];
    if (k == P_burstAmt) sim->burstActive = false;   // an explicit burstAmt overrides a pending inject
  }
  return FIRE_OK;
}
int fire_sim_get_param(FireSim* sim, const char* name, float* value) {
  if (!sim || !value) return FIRE_ERR_BAD_ARG;
  int k = fire_param_index(name);
  if (k < 0) return set_err(sim, FIRE_ERR_BAD_PARAM, "unknown uniform SimParams.%s", name ? name : "(null)");
  *value = sim->params[k];
  return FIRE_OK;
}
int fire_sim_set_param_block(FireSim* sim, const float* block64) {
  if (!sim || !block64) return FIRE_ERR_BAD_ARG;
  const char* names[P_COUNT];
  float vals[P_COUNT];
  int n = 0;
  for (int k = P_seed; k < P_COUNT; ++k) {
    if (k >= P_ox && k <= P_nLogs) continue;
    names[n] = kParamNames[k];
    vals[n++] = block64[k];
  }
  // only mark the geometry stale when a geometry parameter actually changes
  bool geoChange = block64[P_hotR0] != sim->params[P_hotR0] || block64[P_hotR1] != sim->params[P_hotR1] ||
                   block64[P_hotY1] != sim->params[P_hotY1] || block64[P_bedRadius] != sim->params[P_bedRadius];
  bool was = sim->geoReady;
  int rc = fire_sim_set_params(sim, names, vals, n);
  if (rc == FIRE_OK && !geoChange) sim->geoReady = was;
  return rc;
}
int fire_sim_get_param_block(FireSim* sim, float* block64) {
  if (!sim || !block64) return FIRE_ERR_BAD_ARG;
  std::memcpy(block64, sim->params, sizeof(float) * P_STRIDE);
  return FIRE_OK;
}
int fire_sim_peek_block(FireSim* sim, float dt, float* out) {
  if (!sim || !out) return FIRE_ERR_BAD_ARG;
  static_assert(BLOCK_FLOATS == FIRE_BLOCK_FLOATS, "block size mismatch");
  fill_block(sim, dt, out);
  return FIRE_OK;
}
int fire_sim_set_soot_age(FireSim* sim, float age0, float age1) {
  if (!sim || !(age1 > age0)) return FIRE_ERR_BAD_ARG;
  sim->ext[E_sootAge0] = age0;
  sim->ext[E_sootAge1] = age1;
  return FIRE_OK;
}
int fire_sim_set_bed_gain(FireSim* sim, float gain) {
  if (!sim || gain < 0.0f) return FIRE_ERR_BAD_ARG;
  sim->ext[E_bedGain] = gain;
  sim->geoReady = false;
  return FIRE_OK;
}
int fire_sim_set_mg_omega(FireSim* sim, float omega) {
  if (!sim || !(omega > 0.0f && omega < 2.0f)) return FIRE_ERR_BAD_ARG;
  for (MGLevel& L : sim->levels) L.omega = omega;
  drop_graph(sim);   // the smoother launches carry omega as an argument
  return FIRE_OK;
}

int fire_sim_set_tail_wait_limit(FireSim* sim, int polls) {
  if (!sim || polls < 0) return FIRE_ERR_BAD_ARG;
  sim->tailWaitPolls = polls;
  drop_graph(sim);   // the tail launch carries the limit in its descriptor
  return FIRE_OK;
}

int fire_sim_set_spots(FireSim* sim, const float* spots, int n) {
  if (!sim || n < 0 || n > MAX_SPOTS || (n > 0 && !spots)) return FIRE_ERR_BAD_ARG;
  for (int i = 0; i < n; ++i)
    if (!(spots[5 * i + 3] > 0.0f) || spots[5 * i + 4] < 0.0f) return set_err(sim, FIRE_ERR_BAD_ARG, "spot %d: sigma must be > 0 and flux >= 0", i);
  std::memset(sim->ext + E_SPOTS, 0, sizeof(float) * MAX_SPOTS * SPOT_STRIDE);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 5; ++c) sim->ext[E_SPOTS + SPOT_STRIDE * i + c] = spots[5 * i + c];
  sim->ext[E_nSpots] = (float)n;
  return FIRE_OK;
}

int fire_sim_inject(FireSim* sim, float x, float y, float z, float amount, float duration) {
  if (!sim || amount < 0.0f || duration < 0.0f) return FIRE_ERR_BAD_ARG;
  sim->params[P_burstX] = x; sim->params[P_burstY] = y; sim->params[P_burstZ] = z;
  sim->burstAmt = amount;
  sim->burstUntil = sim->time + duration;
  sim->burstActive = true;
  return FIRE_OK;
}
int fire_sim_stoke(FireSim* sim, int log_index, float s) {
  if (!sim || log_index < 0 || log_index >= sim->nLogs || s < 0.0f || s > 1.0f) return FIRE_ERR_BAD_ARG;
  // applyLogs (src/main.js:135-150) with logOffsetsAt's offsets (src/timeline.js:126-133)
  const float footOut = 0.02f, topDrop = 0.04f, topOut = 0.012f;
  float* a = sim->logs + 8 * log_index;
  float ox = a[0], oz = a[2];
  float l = std::hypot(ox, oz);
  if (l == 0.0f) l = 1.0f;
  float dxn = ox / l, dzn = oz / l;
  a[0] += dxn * footOut * s; a[2] += dzn * footOut * s; a[1] -= 0.004f * s;
  a[4] += dxn * topOut * s; a[6] += dzn * topOut * s; a[5] -= topDrop * s;
  sim->logsDirty = true;
  return fire_sim_inject(sim, a[0], 0.08f, a[2], 1.0f, 0.25f);   // the log-shift burst (src/main.js:404)
}
int fire_sim_gust(FireSim* sim, float strength, float duration) {
  if (!sim || !(duration > 0.0f)) return FIRE_ERR_BAD_ARG;
  if (!sim->gustActive) { sim->windBase[0] = sim->params[P_windX]; sim->windBase[1] = sim->params[P_windZ]; }
  sim->gustActive = true;
  sim->gustLeft = duration;
  sim->gustDur = duration;
  sim->gustStrength = strength;
  return FIRE_OK;
}

int fire_sim_reset(FireSim* sim) {
  if (!sim) return FIRE_ERR_BAD_ARG;
  sim->stepStatsValid = false;
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  const size_t cells = (size_t)sim->res[0] * sim->res[1] * sim->res[2];
  for (int w = FIRE_FIELD_VEL; w <= FIRE_FIELD_VORT; ++w) CK(cudaMemset(field_ptr4(sim, w), 0, cells * sizeof(float4)));
  for (auto& L : sim->levels) CK(cudaMemset(L.p, 0, sizeof(float) * (size_t)L.nx * L.ny * L.nz));
  sim->time = 0;
  sim->frame = 0;
  return FIRE_OK;
}

// ---- checkpoint / resume ----
namespace {
// Header of a saved state; the payload follows: vel, S, S2 (float4 per cell each) and level-0 p (float).
struct SaveHeader {
  char magic[8];
  uint32_t version, header_bytes;
  int32_t res[3];
  float size[3];
  double time;
  int64_t frame, stepsRun;
  float params[P_STRIDE];
  float ext[E_COUNT];
  float logs[MAX_LOGS * 8];
  int32_t nLogs;
  double burstUntil;
  float burstAmt;
  int32_t burstActive;
  double gustLeft, gustDur;
  float gustStrength;
  int32_t gustActive;
  float windBase[2];
  int32_t counters[4];   // the residual loop's counters (cumulative cycles, first cycle the next step tests)
  int32_t lastCycles;
  double lastRel;
};
const char kSaveMagic[8] = {'F', 'I', 'R', 'E', 'S', 'I', 'M', '1'};
size_t save_bytes(const FireSim* s) {
  const size_t cells = (size_t)s->res[0] * s->res[1] * s->res[2];
  return sizeof(SaveHeader) + cells * (3 * sizeof(float4) + sizeof(float));
}
}  // namespace

int fire_sim_save(FireSim* sim, void* buf, size_t capacity, size_t* bytes_out) {
  FIRE_RANGE("fire_sim_save");
  if (!sim || !bytes_out) return FIRE_ERR_BAD_ARG;
  const size_t need = save_bytes(sim);
  *bytes_out = need;
  if (!buf) return FIRE_OK;
  if (capacity < need) return set_err(sim, FIRE_ERR_BAD_ARG, "save: need %zu bytes, got %zu", need, capacity);
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  SaveHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kSaveMagic, sizeof h.magic);
  h.version = 1;
  h.header_bytes = (uint32_t)sizeof h;
  for (int i = 0; i < 3; ++i) { h.res[i] = sim->res[i]; h.size[i] = sim->size[i]; }
  h.time = sim->time;
  h.frame = sim->frame;
  h.stepsRun = sim->stepsRun;
  std::memcpy(h.params, sim->params, sizeof h.params);
  std::memcpy(h.ext, sim->ext, sizeof h.ext);
  std::memcpy(h.logs, sim->logs, sizeof h.logs);
  h.nLogs = sim->nLogs;
  h.burstUntil = sim->burstUntil; h.burstAmt = sim->burstAmt; h.burstActive = sim->burstActive;
  h.gustLeft = sim->gustLeft; h.gustDur = sim->gustDur; h.gustStrength = sim->gustStrength; h.gustActive = sim->gustActive;
  h.windBase[0] = sim->windBase[0]; h.windBase[1] = sim->windBase[1];
  CK(cudaMemcpy(h.counters, sim->dCounter, sizeof h.counters, cudaMemcpyDeviceToHost));
  h.counters[0] = 0;
  h.counters[2] = 0;   // per-step cycle count and wait-timeout flag are not state
  h.lastCycles = sim->lastCycles;
  h.lastRel = sim->lastRel;
  char* o = static_cast<char*>(buf);
  std::memcpy(o, &h, sizeof h);
  o += sizeof h;
  const size_t cells = (size_t)sim->res[0] * sim->res[1] * sim->res[2];
  for (const float4* f : {sim->f.vel, sim->f.S, sim->f.S2}) {
    CK(cudaMemcpy(o, f, cells * sizeof(float4), cudaMemcpyDeviceToHost));
    o += cells * sizeof(float4);
  }
  CK(cudaMemcpy(o, sim->levels[0].p, cells * sizeof(float), cudaMemcpyDeviceToHost));
  return FIRE_OK;
}

int fire_sim_load(FireSim* sim, const void* buf, size_t bytes) {
  FIRE_RANGE("fire_sim_load");
  if (!sim || !buf) return FIRE_ERR_BAD_ARG;
  if (bytes != save_bytes(sim)) return set_err(sim, FIRE_ERR_BAD_ARG, "load: %zu bytes, this simulation's state is %zu", bytes, save_bytes(sim));
  SaveHeader h;
  std::memcpy(&h, buf, sizeof h);
  sim->stepStatsValid = false;
  if (std::memcmp(h.magic, kSaveMagic, sizeof h.magic) != 0 || h.version != 1 || h.header_bytes != sizeof h)
    return set_err(sim, FIRE_ERR_BAD_ARG, "load: not a saved simulation state of this version");
  for (int i = 0; i < 3; ++i)
    if (h.res[i] != sim->res[i] || h.size[i] != sim->size[i]) return set_err(sim, FIRE_ERR_BAD_ARG, "load: saved for another grid");
  if (h.nLogs < 0 || h.nLogs > MAX_LOGS) return set_err(sim, FIRE_ERR_BAD_ARG, "load: bad log count");
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  const char* in = static_cast<const char*>(buf) + sizeof h;
  const size_t cells = (size_t)sim->res[0] * sim->res[1] * sim->res[2];
  for (float4* f : {sim->f.vel, sim->f.S, sim->f.S2}) {
    CK(cudaMemcpy(f, in, cells * sizeof(float4), cudaMemcpyHostToDevice));
    in += cells * sizeof(float4);
  }
  CK(cudaMemcpy(sim->levels[0].p, in, cells * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(sim->dCounter, h.counters, sizeof h.counters, cudaMemcpyHostToDevice));
  sim->time = h.time;
  sim->frame = h.frame;
  sim->stepsRun = h.stepsRun;
  std::memcpy(sim->params, h.params, sizeof h.params);
  std::memcpy(sim->ext, h.ext, sizeof h.ext);
  std::memcpy(sim->logs, h.logs, sizeof h.logs);
  sim->nLogs = h.nLogs;
  sim->burstUntil = h.burstUntil; sim->burstAmt = h.burstAmt; sim->burstActive = h.burstActive != 0;
  sim->gustLeft = h.gustLeft; sim->gustDur = h.gustDur; sim->gustStrength = h.gustStrength; sim->gustActive = h.gustActive != 0;
  sim->windBase[0] = h.windBase[0]; sim->windBase[1] = h.windBase[1];
  sim->lastCycles = h.lastCycles;
  sim->lastRel = h.lastRel;
  sim->geoReady = false;    // the emitter geometry is rebuilt from the restored logs at the next step
  sim->logsDirty = true;
  return FIRE_OK;
}

int fire_sim_upload_logs(FireSim* sim, const float* logs, int n_logs) {
  if (!sim || n_logs < 0 || n_logs > MAX_LOGS || (n_logs > 0 && !logs)) return FIRE_ERR_BAD_ARG;
  std::memset(sim->logs, 0, sizeof sim->logs);
  if (n_logs > 0) std::memcpy(sim->logs, logs, sizeof(float) * 8 * n_logs);
  sim->nLogs = n_logs;
  sim->logsDirty = true;
  return FIRE_OK;
}

int fire_sim_field(FireSim* sim, int which, FireFieldDesc* out) {
  if (!sim || !out) return FIRE_ERR_BAD_ARG;
  std::memset(out, 0, sizeof *out);
  if (which >= FIRE_FIELD_VEL && which <= FIRE_FIELD_GEO) {
    out->data = field_ptr4(sim, which);
    for (int i = 0; i < 3; ++i) out->dims[i] = sim->res[i];
    out->channels = 4; out->elem_bytes = 4;
  } else if (which == FIRE_FIELD_P || which == FIRE_FIELD_B) {
    out->data = which == FIRE_FIELD_P ? sim->levels[0].p : sim->levels[0].b;
    for (int i = 0; i < 3; ++i) out->dims[i] = sim->res[i];
    out->channels = 1; out->elem_bytes = 4;
  } else if (which == FIRE_FIELD_NOISE || which == FIRE_FIELD_CURL) {
    out->data = which == FIRE_FIELD_NOISE ? (void*)sim->noise : (void*)sim->curl;
    for (int i = 0; i < 3; ++i) out->dims[i] = TABLE_N;
    out->channels = 4; out->elem_bytes = 2;
  } else {
    return set_err(sim, FIRE_ERR_BAD_ARG, "unknown field %d", which);
  }
  out->strides[0] = (size_t)out->channels * out->elem_bytes;
  out->strides[1] = out->strides[0] * out->dims[0];
  out->strides[2] = out->strides[1] * out->dims[1];
  out->bytes = out->strides[2] * out->dims[2];
  return FIRE_OK;
}

int fire_sim_download(FireSim* sim, int which, void* host, size_t bytes) {
  FireFieldDesc d;
  int rc = fire_sim_field(sim, which, &d);
  if (rc) return rc;
  if (!host || bytes != d.bytes) return set_err(sim, FIRE_ERR_BAD_ARG, "download: need %zu bytes, got %zu", d.bytes, bytes);
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(host, d.data, bytes, cudaMemcpyDeviceToHost));
  return FIRE_OK;
}
int fire_sim_upload(FireSim* sim, int which, const void* host, size_t bytes) {
  FireFieldDesc d;
  int rc = fire_sim_field(sim, which, &d);
  if (rc) return rc;
  if (!host || bytes != d.bytes) return set_err(sim, FIRE_ERR_BAD_ARG, "upload: need %zu bytes, got %zu", d.bytes, bytes);
  sim->stepStatsValid = false;
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(d.data, host, bytes, cudaMemcpyHostToDevice));
  if (which == FIRE_FIELD_GEO) {   // caller-provided geometry: derive the solid mask, skip the rebuild
    launch_solid_mask(sim->f.geo, sim->f.solid, sim->d, nullptr);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    sim->geoReady = true;
    sim->logsDirty = false;
  }
  return FIRE_OK;
}

int fire_sim_info(FireSim* sim, FireInfo* out) {
  if (!sim || !out) return FIRE_ERR_BAD_ARG;
  std::memset(out, 0, sizeof *out);
  for (int i = 0; i < 3; ++i) { out->res[i] = sim->res[i]; out->size[i] = sim->size[i]; out->origin[i] = sim->origin[i]; }
  out->dx = (float)sim->dx;
  out->time = sim->time;
  out->frame = sim->frame;
  out->n_levels = (int)sim->levels.size();
  out->coarse_iters = sim->coarseIters;
  out->vcycles = sim->vcycles;
  if (sim->mg_max_cycles > 0) {
    cudaSetDevice(sim->device);
    cudaDeviceSynchronize();
    int cnt[2] = {0, 0};
    double rel = -1;
    cudaMemcpy(cnt, sim->dCounter, 2 * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(&rel, sim->dSmall + 19, sizeof(double), cudaMemcpyDeviceToHost);
    sim->lastCycles = cnt[0];
    sim->lastRel = rel;
    out->total_cycles = cnt[1];
  } else {
    sim->lastCycles = sim->vcycles;
    out->total_cycles = (long long)sim->stepsRun * sim->vcycles;
  }
  out->last_cycles = sim->lastCycles;
  out->last_rel_residual = sim->lastRel;
  return FIRE_OK;
}

const char* fire_sim_last_error(FireSim* sim) { return sim ? sim->err.c_str() : "null handle"; }

int fire_sim_run_stage(FireSim* sim, int stage, float dt, void* stream) {
  FIRE_RANGE("fire_sim_run_stage");
  if (!sim || stage < 0 || stage >= FIRE_STAGE_COUNT) return FIRE_ERR_BAD_ARG;
  sim->stepStatsValid = false;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  int rc = upload_block(sim, dt, st, stage == FIRE_STAGE_GEO);
  if (rc) return rc;
  const float* P = sim->dBlock;
  static const char* const kStageRange[FIRE_STAGE_COUNT] = {"stage:geo", "stage:adv1", "stage:adv2", "stage:curl",
                                                            "stage:forces", "stage:div", "stage:vcycle", "stage:project"};
  FIRE_RANGE(kStageRange[stage]);
  switch (stage) {
    case FIRE_STAGE_GEO: sim->geoReady = false; rc = ensure_geo(sim, st); if (rc) return rc; break;
    case FIRE_STAGE_ADV1: launch_adv1(P, sim->f, sim->d, st); break;
    case FIRE_STAGE_ADV2: launch_adv2(P, sim->f, sim->d, st); break;
    case FIRE_STAGE_CURL: launch_curl(sim->f, sim->d, st); break;
    case FIRE_STAGE_FORCES: launch_forces(P, sim->f, sim->noise, sim->curl, sim->d, st); break;
    case FIRE_STAGE_DIV: launch_div(P, sim->f, sim->levels[0].b, sim->d, st); break;
    case FIRE_STAGE_VCYCLE: record_vcycle(sim, st); break;
    case FIRE_STAGE_PROJECT: launch_project(P, sim->f, sim->levels[0].p, sim->d, st); break;
  }
  CK(cudaGetLastError());
  return FIRE_OK;
}

int fire_sim_run_mg(FireSim* sim, int op, int level, int arg, void* stream) {
  FIRE_RANGE("fire_sim_run_mg");
  if (!sim || level < 0 || level >= (int)sim->levels.size()) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  const int n = (int)sim->levels.size();
  switch (op) {
    case 1: if (arg != 0 && arg != 1) return FIRE_ERR_BAD_ARG; launch_smooth(sim->levels[level], arg, st); break;
    case 2: if (level >= n - 1) return FIRE_ERR_BAD_ARG; launch_restrict(sim->levels[level], sim->levels[level + 1], st); break;
    case 3: if (level >= n - 1) return FIRE_ERR_BAD_ARG; launch_prolong(sim->levels[level], sim->levels[level + 1], st); break;
    case 6:   // level-0 residual norms into the device scratch, asynchronously (timing aid)
      launch_residual(sim->levels[0], sim->dPartials, sim->dSmall, st);
      break;
    case 5:   // `arg` red-black sweeps (each = colour 0 then colour 1), as the V-cycle runs them
      if (arg < 1) return FIRE_ERR_BAD_ARG;
      record_smooth(sim, level, arg, st);
      break;
    case 4:   // the shared-memory V-cycle from `level` down, if it fits
      if (!tail_fits(sim->levels.data(), level, n)) return FIRE_ERR_BAD_ARG;
      launch_tail(sim->levels.data(), level, n, 2, 2, sim->coarseIters, sim->dCounter + 2, st, false, nullptr, sim->tailWaitPolls);
      break;
    default: return FIRE_ERR_BAD_ARG;
  }
  CK(cudaGetLastError());
  return FIRE_OK;
}

int fire_sim_level_dims(FireSim* sim, int level, int dims3[3], float* h) {
  if (!sim || !dims3 || level < 0 || level >= (int)sim->levels.size()) return FIRE_ERR_BAD_ARG;
  dims3[0] = sim->levels[level].nx; dims3[1] = sim->levels[level].ny; dims3[2] = sim->levels[level].nz;
  if (h) *h = sim->levels[level].h;
  return FIRE_OK;
}

int fire_sim_level_io(FireSim* sim, int level, int which, void* host, size_t bytes, int to_device) {
  if (!sim || !host || level < 0 || level >= (int)sim->levels.size() || (which != 0 && which != 1)) return FIRE_ERR_BAD_ARG;
  const MGLevel& L = sim->levels[level];
  size_t need = sizeof(float) * (size_t)L.nx * L.ny * L.nz;
  if (bytes != need) return set_err(sim, FIRE_ERR_BAD_ARG, "level io: need %zu bytes", need);
  CK(cudaSetDevice(sim->device));
  CK(cudaDeviceSynchronize());
  float* dptr = which ? L.b : L.p;
  if (to_device) CK(cudaMemcpy(dptr, host, bytes, cudaMemcpyHostToDevice));
  else CK(cudaMemcpy(host, dptr, bytes, cudaMemcpyDeviceToHost));
  return FIRE_OK;
}

int fire_sim_profile(FireSim* sim, int enable) {
  if (!sim) return FIRE_ERR_BAD_ARG;
  sim->profiling = enable != 0;
  return FIRE_OK;
}
int fire_sim_stage_times(FireSim* sim, float* ms, int n) {
  if (!sim || !ms || n < FIRE_STAGE_COUNT) return FIRE_ERR_BAD_ARG;
  if (!sim->graphProfiled || !sim->profiledStepPending) return set_err(sim, FIRE_ERR_STATE, "no profiled step has run");
  CK(cudaSetDevice(sim->device));
  CK(cudaEventSynchronize(sim->doneEv));
  // event k marks the start of stage slot k: 0 adv1, 1 adv2, 2 (curl, fused), 3 forces, 4 div, 5 mg, 6 project, 7 end
  float t[FIRE_STAGE_COUNT];
  for (int k = 0; k < 7; ++k) CK(cudaEventElapsedTime(&t[k], sim->stageEv[k], sim->stageEv[k + 1]));
  ms[FIRE_STAGE_GEO] = 0.0f;
  ms[FIRE_STAGE_ADV1] = t[0];
  ms[FIRE_STAGE_ADV2] = t[1];
  ms[FIRE_STAGE_CURL] = t[2];
  ms[FIRE_STAGE_FORCES] = t[3];
  ms[FIRE_STAGE_DIV] = t[4];
  ms[FIRE_STAGE_VCYCLE] = t[5];
  ms[FIRE_STAGE_PROJECT] = t[6];
  for (int k = FIRE_STAGE_COUNT; k < n; ++k) ms[k] = 0.0f;
  return FIRE_OK;
}

int fire_sim_residual(FireSim* sim, double* rel, void* stream) {
  FIRE_RANGE("fire_sim_residual");
  if (!sim || !rel) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  launch_residual(sim->levels[0], sim->dPartials, sim->dSmall, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(sim->hSmall, sim->dSmall, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *rel = sim->hSmall[1] > 0 ? std::sqrt(sim->hSmall[0] / sim->hSmall[1]) : 0.0;
  return FIRE_OK;
}

int fire_sim_stats(FireSim* sim, int which, double* out16, void* stream) {
  FIRE_RANGE("fire_sim_stats");
  if (!sim || !out16) return FIRE_ERR_BAD_ARG;
  float* f = field_ptr4(sim, which);
  if (!f) return set_err(sim, FIRE_ERR_BAD_ARG, "stats: field %d is not a 4-channel grid field", which);
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  launch_stats((const float4*)f, sim->d, sim->dPartials, sim->dSmall + 2, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(sim->hSmall + 2, sim->dSmall + 2, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::memcpy(out16, sim->hSmall + 2, 16 * sizeof(double));
  return FIRE_OK;
}
int fire_sim_hrr(FireSim* sim, double* q_kw, void* stream) {
  FIRE_RANGE("fire_sim_hrr");
  if (!sim || !q_kw) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  launch_hrr(sim->f.S, sim->d, (float)sim->dx, sim->dPartials, sim->dSmall + 18, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(sim->hSmall + 18, sim->dSmall + 18, sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *q_kw = sim->hSmall[18];
  return FIRE_OK;
}
int fire_sim_height_profile(FireSim* sim, double* rows6, int max_rows, int* n_rows, void* stream) {
  FIRE_RANGE("fire_sim_height_profile");
  if (!sim || !rows6 || !n_rows) return FIRE_ERR_BAD_ARG;
  const int n = height_profile_rows(sim->d);
  *n_rows = n;
  if (max_rows < n) return set_err(sim, FIRE_ERR_BAD_ARG, "height profile needs %d rows", n);
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  double* d = nullptr;
  CK(cudaMallocAsync(&d, sizeof(double) * 6 * (size_t)n, st));
  launch_height_profile(sim->f.S, sim->d, sim->dx, d, st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(rows6, d, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_err(sim, FIRE_ERR_CUDA, "height profile: %s", cudaGetErrorString(e));
  return FIRE_OK;
}
int fire_sim_stats_async(FireSim* sim, double* pinned_out17, void* stream) {
  FIRE_RANGE("fire_sim_stats_async");
  if (!sim || !pinned_out17) return FIRE_ERR_BAD_ARG;
  CK(cudaSetDevice(sim->device));
  cudaStream_t st = as_stream(stream);
  if (sim->stepStats && sim->stepStatsValid) {   // the last step's graph formed them (same kernels)
    CK(cudaMemcpyAsync(pinned_out17, sim->dSmall + 24, 17 * sizeof(double), cudaMemcpyDeviceToHost, st));
    return FIRE_OK;
  }
  launch_diag(sim->f.S, sim->d, (float)sim->dx, sim->dPartials, sim->dSmall + 2, st);   // dSmall[2..18]
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(pinned_out17, sim->dSmall + 2, 17 * sizeof(double), cudaMemcpyDeviceToHost, st));
  return FIRE_OK;
}

int fire_sim_set_step_stats(FireSim* sim, int enable) {
  if (!sim || (enable != 0 && enable != 1)) return FIRE_ERR_BAD_ARG;
  if (sim->stepStats != (enable == 1)) {
    CK(cudaSetDevice(sim->device));
    CK(cudaDeviceSynchronize());   // no replay of the current graph is in flight when it is replaced
    drop_graph(sim);
  }
  sim->stepStats = enable == 1;
  sim->stepStatsValid = false;
  return FIRE_OK;
}

}  // extern "C"

// ==================================================================================================
// Ensemble: many independent simulations of uneven sizes advanced together.  Every stage of a step is
// one launch over all members (a BatchMap concatenates their block grids), the multigrid levels outside
// each member's shared-memory tail are batched level by level, and the tails of all members run in one
// launch per tail form; the whole step is one CUDA graph.  Members are ordinary FireSim handles (created
// and owned by the ensemble) so their parameters, spots, events, fields and diagnostics use the FireSim
// API; their parameter blocks are staged into one contiguous device array and copied with one copy.
constexpr int ENS_STAGES = 5;   // adv1, adv2, forces, div, project
struct FireEnsemble {
  int device = 0;
  std::vector<FireSim*> sims;
  float* dBlocks = nullptr;                 // n x BLOCK_FLOATS on the device
  float* hRing = nullptr;                   // ENS_RING slots of n x BLOCK_FLOATS, pinned
  cudaEvent_t ringEv[4] = {};
  bool ringUsed[4] = {};
  int ringPos = 0;
  void* dTail[2] = {nullptr, nullptr};      // tail descriptors by form (single CTA, cluster)
  int tailCount[2] = {0, 0};
  size_t tailSmem[2] = {0, 0};
  int* dErr = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long steps = 0;
  // tile candidate per batched stage (adv1, adv2, forces, div, project), chosen by timing every candidate
  // on the first step (autotune) or set by the caller
  int tiles[ENS_STAGES] = {0, 0, 0, 0, 0};
  float tileMs[ENS_STAGES][CELL_TILES] = {};
  int tuneAt = 8;        // the step index that runs the tuning (-1: never)
  bool tuned = false;
  std::string err;
};

namespace {
constexpr int ENS_RING = 4;

// Appends simulation `inst` with a gx x gy x gz block grid to a map.
void map_add(BatchMap& m, int inst, dim3 g) {
  const int k = m.n++;
  m.inst[k] = inst;
  m.gx[k] = (int)g.x;
  m.gy[k] = (int)g.y;
  m.prefix[k + 1] = m.prefix[k] + (int)(g.x * g.y * g.z);
}
BatchMap map_empty() {
  BatchMap m;
  std::memset(&m, 0, sizeof m);
  return m;
}

int ens_err(FireEnsemble* e, int code, const char* msg) {
  if (e) e->err = msg;
  return code;
}

// Records one ensemble step (src/sim.js:633-644 for every member): adv1, adv2, curl + forces, div,
// `vcycles` V(2,2) cycles, project.
// Launch descriptions of one ensemble step: the members' stage pointers, one BatchMap per tile candidate,
// and the multigrid's per-level maps and level tables.
struct EnsCtx {
  StepBatch SB;
  BatchMap cell[CELL_TILES], forces[FORCES_TILES];
  int depth = 0;
  std::vector<BatchMap> smoothMap, coarseMap;
  std::vector<LevelBatch> LB;
};
void ens_context(FireEnsemble* e, EnsCtx& c) {
  const int n = (int)e->sims.size();
  std::memset(&c.SB, 0, sizeof c.SB);
  for (auto& m : c.cell) m = map_empty();
  for (auto& m : c.forces) m = map_empty();
  c.depth = 0;
  for (int i = 0; i < n; ++i) {
    FireSim* s = e->sims[i];
    c.SB.s[i] = StepInst{e->dBlocks + (size_t)i * BLOCK_FLOATS, s->f, s->d, s->levels[0].b, s->levels[0].p};
    for (int v = 0; v < CELL_TILES; ++v) map_add(c.cell[v], i, step_grid(s->d, v));
    for (int v = 0; v < FORCES_TILES; ++v) map_add(c.forces[v], i, forces_grid(s->d, v));
    c.depth = std::max(c.depth, std::min(s->tailFirst, (int)s->levels.size() - 1));
  }
  // per level: the members that have it outside their tail, and every member's level l and l + 1
  c.smoothMap.assign(c.depth, map_empty());
  c.coarseMap.assign(c.depth, map_empty());
  c.LB.assign(c.depth + 1, LevelBatch{});
  for (int l = 0; l <= c.depth; ++l) std::memset(&c.LB[l], 0, sizeof(LevelBatch));
  for (int i = 0; i < n; ++i) {
    FireSim* s = e->sims[i];
    const int top = std::min(s->tailFirst, (int)s->levels.size() - 1);
    for (int l = 0; l <= c.depth && l < (int)s->levels.size(); ++l) c.LB[l].l[i] = s->levels[l];
    for (int l = 0; l < top; ++l) {
      map_add(c.smoothMap[l], i, smooth_grid(s->levels[l]));
      map_add(c.coarseMap[l], i, coarse_grid(s->levels[l + 1]));
    }
  }
}
void ens_stage(FireEnsemble* e, const EnsCtx& c, int stage, int tile, cudaStream_t st) {
  switch (stage) {
    case 0: launch_adv1_batch(c.cell[tile], c.SB, tile, st); break;
    case 1: launch_adv2_batch(c.cell[tile], c.SB, tile, st); break;
    case 2: launch_forces_batch(c.forces[tile], c.SB, e->sims[0]->noise, e->sims[0]->curl, tile, st); break;
    case 3: launch_div_batch(c.cell[tile], c.SB, tile, st); break;
    default: launch_project_batch(c.cell[tile], c.SB, tile, st); break;
  }
}
void ens_mg(FireEnsemble* e, const EnsCtx& c, cudaStream_t st) {
  const int V = e->sims[0]->vcycles;
  for (int cy = 0; cy < V; ++cy) {
    for (int l = 0; l < c.depth; ++l) {
      for (int k = 0; k < 2; ++k) { launch_smooth_batch(c.smoothMap[l], c.LB[l], 0, st); launch_smooth_batch(c.smoothMap[l], c.LB[l], 1, st); }
      launch_restrict_batch(c.coarseMap[l], c.LB[l], c.LB[l + 1], st);
    }
    for (int kind = 0; kind < 2; ++kind)
      launch_tail_batch(kind, e->dTail[kind], e->tailCount[kind], e->tailSmem[kind], 2, 2, e->dErr, st);
    for (int l = c.depth - 1; l >= 0; --l) {
      launch_prolong_batch(c.coarseMap[l], c.LB[l], c.LB[l + 1], st);
      for (int k = 0; k < 2; ++k) { launch_smooth_batch(c.smoothMap[l], c.LB[l], 0, st); launch_smooth_batch(c.smoothMap[l], c.LB[l], 1, st); }
    }
  }
}

int record_ensemble_step(FireEnsemble* e, cudaStream_t st) {
  EnsCtx c;
  ens_context(e, c);
  for (int s = 0; s < 4; ++s) ens_stage(e, c, s, e->tiles[s], st);
  ens_mg(e, c, st);
  ens_stage(e, c, 4, e->tiles[4], st);
  return cudaGetLastError() == cudaSuccess ? FIRE_OK : ens_err(e, FIRE_ERR_CUDA, "ensemble step launch failed");
}

// The autotuner: runs one step eagerly, timing every tile candidate of every batched stage (3 launches each,
// CUDA events, the mean) and keeping the fastest.  Each stage reads only what the previous stages wrote and
// every candidate computes the same per-cell arithmetic, so running all candidates of a stage back to back
// leaves exactly the state one step leaves.
int tune_ensemble(FireEnsemble* e, cudaStream_t st) {
  EnsCtx c;
  ens_context(e, c);
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return ens_err(e, FIRE_ERR_CUDA, "autotune: event create failed");
  }
  constexpr int R = 3;
  int rc = FIRE_OK;
  for (int s = 0; s < ENS_STAGES && !rc; ++s) {
    if (s == 4) ens_mg(e, c, st);
    const int count = s == 2 ? FORCES_TILES : CELL_TILES;
    int best = 0;
    float bestMs = 1e30f;
    for (int v = 0; v < count; ++v) {
      float ms = 0.0f;
      if (cudaEventRecord(a, st) != cudaSuccess) { rc = FIRE_ERR_CUDA; break; }
      for (int r = 0; r < R; ++r) ens_stage(e, c, s, v, st);
      if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
          cudaEventElapsedTime(&ms, a, b) != cudaSuccess) { rc = FIRE_ERR_CUDA; break; }
      e->tileMs[s][v] = ms / R;
      if (ms < bestMs) { bestMs = ms; best = v; }
    }
    e->tiles[s] = best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!rc && cudaGetLastError() != cudaSuccess) rc = FIRE_ERR_CUDA;
  e->tuned = true;
  return rc ? ens_err(e, rc, "autotune step failed") : FIRE_OK;
}

int build_ensemble_graph(FireEnsemble* e) {
  if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
  if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return FIRE_ERR_CUDA;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaStreamDestroy(st); return FIRE_ERR_CUDA; }
  const int rc = record_ensemble_step(e, st);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  cudaStreamDestroy(st);
  if (rc || ce != cudaSuccess) { if (g) cudaGraphDestroy(g); return rc ? rc : ens_err(e, FIRE_ERR_CUDA, "ensemble capture failed"); }
  e->graph = g;
  if (cudaGraphInstantiate(&e->exec, g, 0) != cudaSuccess) return ens_err(e, FIRE_ERR_CUDA, "ensemble graph instantiate failed");
  return FIRE_OK;
}
}  // namespace

extern "C" {

int fire_ensemble_destroy(FireEnsemble* e) {
  if (!e) return FIRE_ERR_BAD_ARG;
  cudaSetDevice(e->device);
  cudaDeviceSynchronize();
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  for (int k = 0; k < ENS_RING; ++k) if (e->ringEv[k]) cudaEventDestroy(e->ringEv[k]);
  if (e->hRing) cudaFreeHost(e->hRing);
  if (e->dBlocks) cudaFree(e->dBlocks);
  for (int k = 0; k < 2; ++k) if (e->dTail[k]) cudaFree(e->dTail[k]);
  if (e->dErr) cudaFree(e->dErr);
  for (FireSim* s : e->sims) fire_sim_destroy(s);
  delete e;
  return FIRE_OK;
}

int fire_ensemble_create(const FireConfig* cfgs, int n, FireEnsemble** out) {
  FIRE_RANGE("fire_ensemble_create");
  if (!cfgs || !out || n < 1 || n > BATCH_MAX) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    // fixed cycle counts only (the residual-driven loop is per simulation), one device and table seed
    if (cfgs[i].mg_max_cycles != 0 || cfgs[i].vcycles != cfgs[0].vcycles || cfgs[i].device != cfgs[0].device ||
        cfgs[i].noise_seed != cfgs[0].noise_seed)
      return FIRE_ERR_BAD_ARG;
  }
  FireEnsemble* e = new FireEnsemble();
  e->device = cfgs[0].device;
  for (int i = 0; i < n; ++i) {
    FireSim* s = nullptr;
    const int rc = fire_sim_create(&cfgs[i], nullptr, 0, &s);
    if (rc) { fire_ensemble_destroy(e); return rc; }
    e->sims.push_back(s);
    // members' tails run side by side in one launch: let each start at the finest level that fits
    s->tailFirst = tail_first(s->levels.data(), (int)s->levels.size(), false, 1L << 40);
    if (s->tailFirst >= (int)s->levels.size()) { fire_ensemble_destroy(e); return FIRE_ERR_BAD_ARG; }   // needs a tail
  }
  cudaSetDevice(e->device);
  const size_t blkBytes = sizeof(float) * BLOCK_FLOATS * (size_t)n;
  if (cudaMalloc((void**)&e->dBlocks, blkBytes) != cudaSuccess || cudaMalloc((void**)&e->dErr, sizeof(int)) != cudaSuccess ||
      cudaMemset(e->dErr, 0, sizeof(int)) != cudaSuccess ||
      cudaHostAlloc((void**)&e->hRing, blkBytes * ENS_RING, cudaHostAllocDefault) != cudaSuccess) {
    fire_ensemble_destroy(e);
    return FIRE_ERR_OOM;
  }
  for (int k = 0; k < ENS_RING; ++k)
    if (cudaEventCreateWithFlags(&e->ringEv[k], cudaEventDisableTiming) != cudaSuccess) { fire_ensemble_destroy(e); return FIRE_ERR_CUDA; }
  // tail descriptors, grouped by form
  std::vector<unsigned char> desc[2];
  for (int i = 0; i < n; ++i) {
    FireSim* s = e->sims[i];
    const int L = (int)s->levels.size();
    const int kind = tail_kind(s->levels.data(), s->tailFirst, L);
    const size_t sz = tail_desc_size(kind);
    desc[kind].resize(desc[kind].size() + sz);
    tail_desc_fill(s->levels.data(), s->tailFirst, L, s->coarseIters, desc[kind].data() + desc[kind].size() - sz);
    e->tailCount[kind] += 1;
    e->tailSmem[kind] = std::max(e->tailSmem[kind], tail_smem_bytes(s->levels.data(), s->tailFirst, L));
  }
  for (int k = 0; k < 2; ++k) {
    if (!e->tailCount[k]) continue;
    if (cudaMalloc(&e->dTail[k], desc[k].size()) != cudaSuccess ||
        cudaMemcpy(e->dTail[k], desc[k].data(), desc[k].size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      fire_ensemble_destroy(e);
      return FIRE_ERR_CUDA;
    }
  }
  *out = e;
  return FIRE_OK;
}

int fire_ensemble_size(FireEnsemble* e) { return e ? (int)e->sims.size() : FIRE_ERR_BAD_ARG; }

int fire_ensemble_sim(FireEnsemble* e, int i, FireSim** out) {
  if (!e || !out || i < 0 || i >= (int)e->sims.size()) return FIRE_ERR_BAD_ARG;
  *out = e->sims[i];
  return FIRE_OK;
}

int fire_ensemble_step(FireEnsemble* e, float dt, int n_steps, void* stream) {
  FIRE_RANGE("fire_ensemble_step");
  if (!e || n_steps < 0 || !(dt > 0.0f)) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return FIRE_ERR_CUDA;
  cudaStream_t st = as_stream(stream);
  const int n = (int)e->sims.size();
  for (FireSim* s : e->sims) s->stepStatsValid = false;   // members are stepped by the ensemble's graph
  for (int step = 0; step < n_steps; ++step) {
    const int k = e->ringPos;
    e->ringPos = (k + 1) % ENS_RING;
    if (e->ringUsed[k] && cudaEventSynchronize(e->ringEv[k]) != cudaSuccess) return FIRE_ERR_CUDA;
    e->ringUsed[k] = true;
    float* slot = e->hRing + (size_t)k * BLOCK_FLOATS * n;
    for (int i = 0; i < n; ++i) {
      FireSim* s = e->sims[i];
      advance_events(s, dt);
      fill_block(s, dt, slot + (size_t)i * BLOCK_FLOATS);
      if (!s->geoReady || s->logsDirty) {   // emitter geometry from this member's own block and logs
        int rc = upload_block(s, dt, st, true);
        if (rc) return rc;
        if ((rc = ensure_geo(s, st))) return rc;
      }
    }
    if (cudaMemcpyAsync(e->dBlocks, slot, sizeof(float) * BLOCK_FLOATS * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaEventRecord(e->ringEv[k], st) != cudaSuccess)
      return FIRE_ERR_CUDA;
    if (e->tuneAt >= 0 && !e->tuned && e->steps >= e->tuneAt) {   // eager step that picks the graph's tiles
      if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
      const int rc = tune_ensemble(e, st);
      if (rc) return rc;
    } else {
      if (!e->exec) {
        const int rc = build_ensemble_graph(e);
        if (rc) return rc;
      }
      if (cudaGraphLaunch(e->exec, st) != cudaSuccess) return FIRE_ERR_CUDA;
    }
    for (FireSim* s : e->sims) {                                               // src/sim.js:646-647
      s->time += dt;
      s->frame += 1;
      s->stepsRun += 1;
    }
    e->steps += 1;
  }
  return FIRE_OK;
}

int fire_ensemble_set_autotune(FireEnsemble* e, int at_step) {
  if (!e || at_step < -1) return FIRE_ERR_BAD_ARG;
  e->tuneAt = at_step;
  e->tuned = false;
  return FIRE_OK;
}
int fire_ensemble_set_tiles(FireEnsemble* e, const int* tiles) {
  if (!e || !tiles) return FIRE_ERR_BAD_ARG;
  for (int s = 0; s < ENS_STAGES; ++s)
    if (tiles[s] < 0 || tiles[s] >= (s == 2 ? FORCES_TILES : CELL_TILES)) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FIRE_ERR_CUDA;
  std::memcpy(e->tiles, tiles, sizeof e->tiles);
  e->tuned = true;
  if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
  if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
  return FIRE_OK;
}
int fire_ensemble_tiles(FireEnsemble* e, int* tiles, float* ms) {
  if (!e || !tiles) return FIRE_ERR_BAD_ARG;
  std::memcpy(tiles, e->tiles, sizeof e->tiles);
  if (ms) std::memcpy(ms, e->tileMs, sizeof e->tileMs);
  return e->tuned ? FIRE_OK : FIRE_ERR_STATE;
}

int fire_ensemble_sync(FireEnsemble* e) {
  if (!e) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FIRE_ERR_CUDA;
  int err = 0;
  if (cudaMemcpy(&err, e->dErr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return FIRE_ERR_CUDA;
  if (err) {
    cudaMemset(e->dErr, 0, sizeof(int));
    return ens_err(e, FIRE_ERR_CUDA, "a device-side wait timed out (multigrid tail bulk copy)");
  }
  return FIRE_OK;
}

const char* fire_ensemble_last_error(FireEnsemble* e) { return e ? e->err.c_str() : "null ensemble"; }

}  // extern "C"

// ==================================================================================================
// Sparks (src/sparks.js): particles carried by a simulation's velocity field.  The host keeps the spawn
// bookkeeping of Sparks.step (src/sparks.js:250-274) in doubles as the page does; the device runs the
// particle update (fire_sparks.cu).
struct SparkBurstRec {
  double t0;
  int n, emitted;
  float pos[3], speed, radius, dur, fan, size, aim[3];
  bool hasAim;
};
struct FireSparks {
  FireSim* sim = nullptr;
  int count = 0;
  float4* dSp = nullptr;
  int* dDead = nullptr;
  double rate = 3.0, carry = 0.0, time = 0.0;   // src/sparks.js:24-28
  long long frame = 0;
  float turb = 1.0f, lifeK = 1.0f, sizeK = 1.0f, upK = 1.0f;
  std::vector<SparkBurstRec> bursts;
};

namespace {
// The uniforms of the next step (src/sparks.js:250-270); with commit, the bookkeeping advances too.
SparkU spark_uniforms(FireSparks* s, float dt, bool commit) {
  double carry = s->carry + s->rate * (double)dt;
  const double nBase = std::floor(carry);
  carry -= nBase;
  std::vector<SparkBurstRec> bursts = s->bursts;
  int nBurst = 0;
  const SparkBurstRec* B = nullptr;
  for (SparkBurstRec& b : bursts) {
    const double frac = std::min((s->time + (double)dt - b.t0) / (double)b.dur, 1.0);
    const int due = std::min(b.n, (int)std::floor((double)b.n * frac + 0.5));   // Math.round
    const int k = due - b.emitted;
    if (k > 0 && !B) { B = &b; nBurst = k; b.emitted += k; }
  }
  SparkU U;
  U.dt = dt; U.time = (float)s->time; U.frame = (float)s->frame; U.count = (float)s->count;
  U.nBase = (float)nBase; U.nBurst = (float)nBurst;
  U.burstX = B ? B->pos[0] : 0.0f; U.burstY = B ? B->pos[1] : 0.0f; U.burstZ = B ? B->pos[2] : 0.0f;
  U.burstSpeed = B ? B->speed : 0.0f; U.burstRadius = B ? B->radius : 0.0f;
  U.ox = s->sim->origin[0]; U.oy = s->sim->origin[1]; U.oz = s->sim->origin[2];
  U.sx = s->sim->size[0]; U.sy = s->sim->size[1]; U.sz = s->sim->size[2];
  U.turb = s->turb; U.lifeK = s->lifeK; U.bedRadius = 0.2f; U.seed = 1234.0f; U.sizeK = s->sizeK; U.upK = s->upK;
  U.burstFan = B ? B->fan : 0.0f; U.burstSize = B ? B->size : 1.0f;
  U.aimX = (B && B->hasAim) ? B->aim[0] : 0.0f; U.aimZ = (B && B->hasAim) ? B->aim[2] : 0.0f;
  if (commit) {
    s->carry = carry;
    bursts.erase(std::remove_if(bursts.begin(), bursts.end(), [](const SparkBurstRec& b) { return b.emitted >= b.n; }), bursts.end());
    s->bursts = bursts;
  }
  return U;
}
}  // namespace

extern "C" {

int fire_sparks_create(FireSim* sim, int count, FireSparks** out) {
  FIRE_RANGE("fire_sparks_create");
  if (!sim || !out || count < 1 || count > (1 << 24)) return FIRE_ERR_BAD_ARG;
  *out = nullptr;
  CK(cudaSetDevice(sim->device));
  FireSparks* s = new FireSparks();
  s->sim = sim;
  s->count = count;
  if (cudaMalloc((void**)&s->dSp, sizeof(float4) * 4 * (size_t)count) != cudaSuccess ||
      cudaMalloc((void**)&s->dDead, sizeof(int) * (size_t)spark_blocks(count)) != cudaSuccess ||
      cudaMemset(s->dSp, 0, sizeof(float4) * 4 * (size_t)count) != cudaSuccess) {
    if (s->dSp) cudaFree(s->dSp);
    if (s->dDead) cudaFree(s->dDead);
    delete s;
    return FIRE_ERR_OOM;
  }
  *out = s;
  return FIRE_OK;
}

int fire_sparks_destroy(FireSparks* s) {
  if (!s) return FIRE_ERR_BAD_ARG;
  cudaSetDevice(s->sim->device);
  cudaDeviceSynchronize();
  cudaFree(s->dSp);
  cudaFree(s->dDead);
  delete s;
  return FIRE_OK;
}

int fire_sparks_reset(FireSparks* s) {   // src/sparks.js:38-41
  if (!s) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(s->sim->device) != cudaSuccess || cudaMemset(s->dSp, 0, sizeof(float4) * 4 * (size_t)s->count) != cudaSuccess)
    return FIRE_ERR_CUDA;
  s->carry = 0.0;
  s->bursts.clear();
  s->time = 0.0;
  s->frame = 0;
  return FIRE_OK;
}

int fire_sparks_burst(FireSparks* s, int n, const float pos[3], float speed, float radius, float dur, float fan, float size,
                      const float* aim3) {   // src/sparks.js:44-46
  if (!s || !pos || n < 0 || !(dur > 0.0f)) return FIRE_ERR_BAD_ARG;
  SparkBurstRec b;
  b.t0 = s->time;
  b.n = n;
  b.emitted = 0;
  for (int i = 0; i < 3; ++i) { b.pos[i] = pos[i]; b.aim[i] = aim3 ? aim3[i] : 0.0f; }
  b.speed = speed; b.radius = radius; b.dur = dur; b.fan = fan; b.size = size;
  b.hasAim = aim3 != nullptr;
  s->bursts.push_back(b);
  return FIRE_OK;
}

int fire_sparks_set(FireSparks* s, float rate, float turb, float lifeK, float sizeK, float upK) {
  if (!s || !(rate >= 0.0f)) return FIRE_ERR_BAD_ARG;
  s->rate = rate; s->turb = turb; s->lifeK = lifeK; s->sizeK = sizeK; s->upK = upK;
  return FIRE_OK;
}

int fire_sparks_set_rate(FireSparks* s, float rate) {   // simStep: sparks.rate = 1.0 * intensity
  if (!s || !(rate >= 0.0f)) return FIRE_ERR_BAD_ARG;
  s->rate = rate;
  return FIRE_OK;
}

int fire_sparks_peek(FireSparks* s, float dt, float* out27) {
  if (!s || !out27) return FIRE_ERR_BAD_ARG;
  const SparkU U = spark_uniforms(s, dt, false);
  std::memcpy(out27, &U, sizeof U);
  return FIRE_OK;
}

// One spark step after the simulation's step on the same stream (it reads the simulation's velocity).
int fire_sparks_step(FireSparks* s, float dt, void* stream) {
  FIRE_RANGE("fire_sparks_step");
  if (!s || !(dt > 0.0f)) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(s->sim->device) != cudaSuccess) return FIRE_ERR_CUDA;
  const SparkU U = spark_uniforms(s, dt, true);
  launch_sparks(s->dSp, U, s->dDead, s->sim->f.vel, s->sim->d, s->sim->curl, as_stream(stream));
  s->time += dt;
  s->frame += 1;
  return cudaGetLastError() == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

int fire_sparks_buffer(FireSparks* s, void** dev_ptr, int* count) {
  if (!s || !dev_ptr || !count) return FIRE_ERR_BAD_ARG;
  *dev_ptr = s->dSp;
  *count = s->count;
  return FIRE_OK;
}

int fire_sparks_io(FireSparks* s, float* host, size_t bytes, int to_device) {
  if (!s || !host || bytes != sizeof(float4) * 4 * (size_t)s->count) return FIRE_ERR_BAD_ARG;
  if (cudaSetDevice(s->sim->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FIRE_ERR_CUDA;
  const cudaError_t e = to_device ? cudaMemcpy(s->dSp, host, bytes, cudaMemcpyHostToDevice) : cudaMemcpy(host, s->dSp, bytes, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

}  // extern "C"
