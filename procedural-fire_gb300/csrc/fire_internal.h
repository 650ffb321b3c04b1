// Internal declarations shared by the host runtime and the CUDA kernels of the fire simulation step.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace fire {

// SIM_FIELDS order (src/sim.js:14-23): the index of every scalar in the 64-float parameter block.
enum ParamIndex {
  P_nx, P_ny, P_nz, P_dx, P_dt, P_time, P_frame, P_seed, P_ox, P_oy, P_oz, P_nLogs,
  P_fuelSrc, P_bedFuel, P_srcTemp, P_bedTemp, P_srcVel, P_srcFreq, P_srcSpeed, P_srcThresh,
  P_ignT, P_kMix, P_rs, P_heatOut, P_expansion, P_sootForm, P_sootOx, P_radCool,
  P_coolRate, P_sootDissip, P_smokeDissip, P_vitDecay, P_fuelDissip, P_buoyancy, P_vortEps, P_turbAmp,
  P_turbFreq, P_turbRise, P_turbEvolve, P_windX, P_windZ, P_gust, P_intensity, P_velDissip,
  P_bedRadius, P_logSrc, P_burstX, P_burstY, P_burstZ, P_burstAmt, P_smolder, P_sponge, P_hotR0, P_hotR1, P_hotY1,
  P_visc, P_lamAge, P_anchorFreq, P_srcFloor, P_anchorGain, P_COUNT
};
static_assert(P_COUNT == 60, "SIM_FIELDS has 60 entries");
constexpr int P_STRIDE = 64;

// Extension block appended after the 64-float parameter block (no counterpart in the reference): the soot
// age gate, coal-bed gain and spots, plus per-step constants the host derives from the uniforms: the five
// decay factors exp(-k dt) that are the same for every cell (src/sim.js:318, 327-329, 375; computed with the
// same expf the oracle uses), the height above which no spot contributes (max spot y + 4 sigma), and the
// uniform divisions of the forces physics (turbAmp / 12 and the reciprocals 1 / (e1 - e0) of the smoothsteps
// whose edges are parameters: ignition, source pulse, soot age), in the FP32 operations the kernel would use.
enum ExtIndex {
  E_sootAge0 = 0, E_sootAge1, E_bedGain, E_nSpots, E_spotRef, E_spotTop,
  E_decaySoot, E_decayFuel, E_decayVit, E_decaySmoke, E_decayVel,
  E_turbK, E_invIgn, E_invPulse, E_invSootAge,
  E_SPOTS = 16
};
static_assert(E_invSootAge < E_SPOTS, "per-step constants fit before the spot table");
constexpr int MAX_SPOTS = 16;
constexpr int SPOT_STRIDE = 8;
constexpr int E_COUNT = E_SPOTS + MAX_SPOTS * SPOT_STRIDE;   // 144
constexpr int BLOCK_FLOATS = P_STRIDE + E_COUNT;            // 208 floats uploaded per step

constexpr int TABLE_N = 128;          // noise / curl tables: 128^3 (src/main.js:36-37)
constexpr int MAX_LOGS = 16;          // packLogs max (src/scene.js:92)

extern const char* const kParamNames[P_COUNT];
extern const float kParamDefaults[P_STRIDE];

// Device view of the simulation buffers.  All rgba fields are float4, x fastest.
struct Fields {
  float4* vel; float4* velX; float4* velY;
  float4* S; float4* SX; float4* SY;
  float4* S2; float4* S2X; float4* S2Y;
  float4* vort; float4* geo;
  unsigned char* solid;   // geo.b > 0.5 as one byte per cell (what projection reads)
};
struct Dims { int nx, ny, nz; };

struct MGLevel {
  int nx, ny, nz;
  float h;
  float* p;
  float* b;
  float omega = 1.0f;   // over-relaxation of the launch-per-sweep smoother (1: Gauss-Seidel, the reference's)
  // 0: the simulation's multigrid (mgSmooth / mgProlong, src/sim.js:417-437, 468-495).  1: the variant of the
  // reference's convergence studies (research/webgpu-bench/poisson.mjs:28-65, wgsl/mg.wgsl smoothRB /
  // prolongAdd): ghost values from the cell's old value, p <- mix(p, (sum_nb - h^2 b) / 6, omega), and
  // clamp-to-edge trilinear prolongation without sign flips.  Only the standalone solver's FP32 form sets it.
  int study = 0;
};

// ---- batched launches over many independent simulations ----
// A batched launch is one 1D grid whose flat blocks are the concatenated block grids of n simulations:
// simulation inst[k] owns flat blocks [prefix[k], prefix[k+1]) laid out as its own gx x gy x gz grid.
constexpr int BATCH_MAX = 64;
struct BatchMap {
  int n;
  int prefix[BATCH_MAX + 1];
  int gx[BATCH_MAX], gy[BATCH_MAX];
  int inst[BATCH_MAX];
};
// What the step stages of one simulation need (device-resident array, one entry per simulation).
struct StepInst {
  const float* P;     // parameter block
  Fields f;
  Dims d;
  float* b0;          // level-0 right-hand side (written by div)
  const float* p0;    // level-0 pressure (read by project)
};
// Passed by value as a kernel parameter (it lives in the constant bank, so a CTA's simulation pointers
// cost no registers to hold).
struct StepBatch { StepInst s[BATCH_MAX]; };
// One multigrid level of each simulation of a batch, by simulation index (kernel parameter).
struct LevelBatch { MGLevel l[BATCH_MAX]; };

// Uniforms of one spark update (SPARK_FIELDS order, src/sparks.js:9-13), all f32 as the reference uploads them.
struct SparkU {
  float dt, time, frame, count, nBase, nBurst, burstX, burstY, burstZ, burstSpeed, burstRadius;
  float ox, oy, oz, sx, sy, sz, turb, lifeK, bedRadius, seed, sizeK, upK, burstFan, burstSize, aimX, aimZ;
};
static_assert(sizeof(SparkU) == 27 * sizeof(float), "27 spark uniforms");
// ---- kernel launchers (fire_sparks.cu) ----
int spark_blocks(int count);
// One spark step (dead-count pass + update); `dead` holds spark_blocks(count) ints.
void launch_sparks(float4* sp, const SparkU& S, int* dead, const float4* vel, Dims d, const uint2* curl, cudaStream_t st);

// ---- kernel launchers (fire_tables.cu) ----
void launch_noise_table(uint2* noise, int N, int seed, cudaStream_t st);
void launch_curl_table(const uint2* noise, uint2* curl, int N, cudaStream_t st);
void launch_geo(const float* P, const float* logs, float4* geo, unsigned char* solid, Dims d, cudaStream_t st);
// Rebuilds the solid mask from a caller-provided geometry field.
void launch_solid_mask(const float4* geo, unsigned char* solid, Dims d, cudaStream_t st);

// ---- kernel launchers (fire_step.cu) ----
void launch_adv1(const float* P, Fields f, Dims d, cudaStream_t st);
void launch_adv2(const float* P, Fields f, Dims d, cudaStream_t st);
void launch_curl(Fields f, Dims d, cudaStream_t st);
void launch_forces(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st);
// The parameter block as a kernel parameter (BLOCK_FLOATS floats, 832 bytes): the step graph's forces launch
// takes it by value, and the host sets it on the instantiated graph before each step (forces_pb_set; `node`
// is the kernel node that launch_forces_pb captured).
struct ParamBlock { float v[BLOCK_FLOATS]; };
void launch_forces_pb(const ParamBlock& pb, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st);
cudaError_t forces_pb_set(cudaGraphExec_t exec, cudaGraphNode_t node, const ParamBlock& pb, Fields f, const uint2* noise,
                          const uint2* curl, Dims d);
void launch_forces_unfused(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st);
void launch_forces_recompute(const float* P, Fields f, const uint2* noise, const uint2* curl, Dims d, cudaStream_t st);
// Opts the shared-memory kernels of fire_step.cu into their dynamic shared memory on the current device.
cudaError_t step_configure();
void launch_div(const float* P, Fields f, float* b0, Dims d, cudaStream_t st, int* mg_counter = nullptr);
void launch_project(const float* P, Fields f, const float* p0, Dims d, cudaStream_t st);
// Tile candidates of the batched stages: CELL_TILES cell tiles for adv1, adv2, div and project (0 is the
// per-simulation kernels' 32x4x2; then 32x8x1, 32x2x4, 64x4x1) and FORCES_TILES z-march depths of the forces
// tile (16, 8, 32).  Every candidate computes the same per-cell arithmetic.
constexpr int CELL_TILES = 4, FORCES_TILES = 3;
// Block grids of the per-cell stages (adv1, adv2, div, project) and of the tiled forces stage, per candidate.
dim3 step_grid(Dims d, int tile = 0);
dim3 forces_grid(Dims d, int tile = 0);
void launch_adv1_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st);
void launch_adv2_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st);
void launch_forces_batch(const BatchMap& m, const StepBatch& I, const uint2* noise, const uint2* curl, int tile, cudaStream_t st);
void launch_div_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st);
void launch_project_batch(const BatchMap& m, const StepBatch& I, int tile, cudaStream_t st);

// ---- kernel launchers (fire_mg.cu) ----
cudaError_t launch_smooth(const MGLevel& L, int color, cudaStream_t st);
cudaError_t launch_restrict(const MGLevel& F, const MGLevel& C, cudaStream_t st);
// Restriction fused with the coarse level's first colour-0 sweep (bit-identical to launch_restrict followed
// by launch_smooth(C, 0)); not for study levels.
cudaError_t launch_restrict_smooth(const MGLevel& F, const MGLevel& C, cudaStream_t st);
cudaError_t launch_prolong(const MGLevel& F, const MGLevel& C, cudaStream_t st);
// One launch runs the V-cycle over levels [first, n) out of shared memory: a single CTA when every level
// fits in its shared memory, or a thread-block cluster whose CTAs each hold a z-slab of the finer tail
// levels (distributed shared memory for the slab edges) with the coarsest levels gathered on CTA 0.
// tail_fits: whether [first, n) can run as one tail launch; tail_first: the finest `first` that fits and has
// at most max_cells cells (n if none) — for one simulation, larger levels are cheaper as their own launches.
// coarse64: the coarsest level is solved in FP64: exactly with `cinv` (its dense inverse, transposed, in
// global memory) when given, else by `coarse` FP64 sweeps on a double copy in shared memory.
bool tail_fits(const MGLevel* levels, int first, int n, bool coarse64 = false);
constexpr long TAIL_FIRST_CELLS = 8192;
int tail_first(const MGLevel* levels, int n, bool coarse64 = false, long max_cells = TAIL_FIRST_CELLS);
// Shared memory per CTA of the tail launch for [first, n).
size_t tail_smem_bytes(const MGLevel* levels, int first, int n, bool coarse64 = false);
// `err` receives 1 if the single-CTA kernel's bounded wait for its bulk copies ran out (the kernel then
// waits, at the full bound, for the copies in flight and returns without running the cycle).  wait_polls
// bounds the first wait (TAIL_WAIT_POLLS; a fault-injection test lowers it).
constexpr int TAIL_WAIT_POLLS = 1 << 22;
cudaError_t launch_tail(const MGLevel* levels, int first, int n, int pre, int post, int coarse, int* err, cudaStream_t st,
                        bool coarse64 = false, const double* cinv = nullptr, int wait_polls = TAIL_WAIT_POLLS);
// Opts the tail kernels into `max_tail_smem` bytes of dynamic shared memory on the current device.
cudaError_t mg_configure(size_t max_tail_smem);
// Batched forms: one launch per level operation over the simulations of a BatchMap.
dim3 smooth_grid(const MGLevel& L);
dim3 coarse_grid(const MGLevel& C);   // restriction into / prolongation from level C
void launch_smooth_batch(const BatchMap& m, const LevelBatch& L, int color, cudaStream_t st);
void launch_restrict_batch(const BatchMap& m, const LevelBatch& F, const LevelBatch& C, cudaStream_t st);
void launch_prolong_batch(const BatchMap& m, const LevelBatch& F, const LevelBatch& C, cudaStream_t st);
// Tails of many simulations in one launch: kind 0 = single-CTA form, 1 = cluster form.  The host fills
// tail_desc_size(kind) bytes per simulation with tail_desc_fill (with that simulation's coarsest sweeps),
// copies them to the device, and launches `count` of them with the largest tail_smem_bytes among them.
int tail_kind(const MGLevel* levels, int first, int n);
size_t tail_desc_size(int kind);
void tail_desc_fill(const MGLevel* levels, int first, int n, int coarse, void* out);
void launch_tail_batch(int kind, const void* dev_descs, int count, size_t smem, int pre, int post, int* err, cudaStream_t st);
constexpr size_t TAIL_SMEM_BUDGET = 200 * 1024;
// Residual / RHS sums of squares on a level: partial sums per CTA then a fixed-order final sum.
int residual_partials_count(const MGLevel& L);
void launch_residual(const MGLevel& L, double* partials, double* out2, cudaStream_t st);

// ---- diagnostics (fire_stats.cu) ----
int stats_partials_count(Dims d);
void launch_stats(const float4* f, Dims d, double* partials, double* out16, cudaStream_t st);
void launch_hrr(const float4* S, Dims d, float dx, double* partials, double* out1, cudaStream_t st);
// FIRE.profile's height profile rows (6 doubles each, height_profile_rows of them) into device memory.
int height_profile_rows(Dims d);
void launch_height_profile(const float4* S, Dims d, double dx, double* rows6, cudaStream_t st);
// launch_stats of S and launch_hrr in one pass over S (same results); out17 = the 16 stats, then the heat release.
void launch_diag(const float4* S, Dims d, float dx, double* partials, double* out17, cudaStream_t st);

}  // namespace fire
