// The simulation object behind the C ABI (include/fire_sim.h) and the host helpers that the runtime's
// translation units share (fire_api.cu defines them; the adjoint driver in fire_adjoint.cu uses them).
#pragma once
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/fire_sim.h"
#include "fire_internal.h"

namespace fire {
constexpr int RING_SLOTS = 256;
constexpr int SLOT_FLOATS = BLOCK_FLOATS + MAX_LOGS * 8;   // param block + log buffer (1312 bytes)
}  // namespace fire

struct FireSim {
  // (the fields of FireSim (src/sim.js:48-101) plus the runtime's device arena, graph and staging state)
  int device = 0;
  int res[3] = {0, 0, 0};
  float size[3] = {0, 0, 0};
  double dx = 0;
  float origin[3] = {0, 0, 0};
  int vcycles = 2;
  int mg_max_cycles = 0;
  double mg_tol = 0;
  double time = 0;
  long long frame = 0;
  float params[fire::P_STRIDE];
  float ext[fire::E_COUNT];
  float logs[fire::MAX_LOGS * 8];
  int nLogs = 0;
  bool geoReady = false;
  bool logsDirty = true;

  // device
  void* arena = nullptr;
  size_t arenaBytes = 0;
  fire::Fields f{};
  fire::Dims d{};
  std::vector<fire::MGLevel> levels;
  int coarseIters = 8;
  int tailFirst = 0;
  int tailWaitPolls = fire::TAIL_WAIT_POLLS;   // bound of the tail's first bulk-copy wait (fire_sim_set_tail_wait_limit)
  uint2* noise = nullptr;
  uint2* curl = nullptr;
  float* dBlock = nullptr;
  float* dLogs = nullptr;
  double* dPartials = nullptr;
  int partialsCount = 0;
  double* dSmall = nullptr;     // [0..1] residual sums, [2..17] stats, [18] hrr, [19] rel residual,
                                // [24..40] the step graph's diagnostics (per-step diagnostics mode)
  double* dDiagPartials = nullptr;   // scratch of the step graph's diagnostics branch (it runs beside the solve)
  int* dCounter = nullptr;      // [0] V-cycles of this step's residual-driven loop, [1] cycles since creation,
                                // [2] device wait timeout flag, [3] first cycle the next step tests

  // host staging
  float* hRing = nullptr;
  cudaEvent_t ringEv[fire::RING_SLOTS];
  bool ringUsed[fire::RING_SLOTS];
  int ringPos = 0;
  double* hSmall = nullptr;     // pinned mirror of dSmall
  int* hCounter = nullptr;

  cudaStream_t capStream = nullptr;
  // per-step diagnostics: the step graph forms fire_sim_stats_async's values on a branch beside the solve
  bool stepStats = false;
  bool stepStatsValid = false;   // dSmall[24..40] hold the diagnostics of the current S
  cudaStream_t sideStream = nullptr;
  cudaEvent_t forkEv = nullptr, joinEv = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t forcesNode = nullptr;   // the step graph's forces launch, which takes the block by value
  bool graphProfiled = false;
  bool profiling = false;
  cudaEvent_t stageEv[FIRE_STAGE_COUNT + 1];
  cudaEvent_t doneEv = nullptr;
  bool profiledStepPending = false;

  // events (src/main.js:401-407, 456-461)
  double burstUntil = -1;
  float burstAmt = 0;
  bool burstActive = false;
  double gustLeft = 0, gustDur = 2.4;
  float gustStrength = 1;
  bool gustActive = false;
  float windBase[2] = {0, 0};

  int lastCycles = 0;
  double lastRel = -1;
  long long stepsRun = 0;
  std::string err;
};

namespace fire {
namespace rt {
// Records the error message on the handle and returns `code`.
int set_err(FireSim* s, int code, const char* fmt, ...);
// Fills the 208-float block of the next step (uniforms + extension) for time step dt.
void fill_block(FireSim* s, float dt, float* out);
// Advances the burst and gust envelopes by one step (src/main.js:401-407, 456-461).
void advance_events(FireSim* s, float dt);
// Records the pressure solve of one step on `st` (fixed V-cycles, or the residual-driven loop, which needs
// stream capture).
int record_mg(FireSim* sim, cudaStream_t st, bool counter_cleared = false);
// Rebuilds the emitter geometry when stale (src/sim.js:632).
int ensure_geo(FireSim* sim, cudaStream_t st);
// Stages the block for dt (and the log buffer) in the pinned ring and copies it to the device on `st`;
// `staged` (optional) receives the host copy of the block.
int upload_block(FireSim* sim, float dt, cudaStream_t st, bool with_logs, const float** staged = nullptr);
// One V(2,2) cycle of the pressure solve (src/sim.js:588-599) on `st`.
void record_vcycle(FireSim* s, cudaStream_t st);
cudaStream_t as_stream(void* s);
}  // namespace rt
}  // namespace fire
