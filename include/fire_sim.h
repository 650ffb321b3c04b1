/*
 * fire_sim.h - C ABI of the GB300-native procedural-fire simulation step.
 *
 * This is the drop-in boundary for the reference's `FireSim` class (src/sim.js) and the parts of the
 * deterministic page API that drive it (src/main.js `window.FIRE`).  Every entry point uses plain C types:
 * pointers, sizes and status codes; CUDA streams are passed as `void*` (a cudaStream_t, or NULL for the
 * legacy default stream).  Each declaration names the reference interface it replaces (file:line,
 * relative to the reference project).
 *
 * Threading: a FireSim handle is not thread-safe; drive each handle from one host thread.  Several
 * handles may run concurrently on different streams.
 *
 * Errors: every function returns FIRE_OK (0) or a FIRE_ERR_* code; fire_sim_last_error() gives a
 * message for the most recent failure on a handle (the reference only logs WebGPU validation errors,
 * src/gpu.js:25-26, 102-104).
 */
#ifndef FIRE_SIM_H
#define FIRE_SIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------------- */
#define FIRE_OK 0
#define FIRE_ERR_BAD_ARG 1     /* null pointer, bad dims, wrong buffer size, unknown field id       */
#define FIRE_ERR_BAD_PARAM 2   /* unknown parameter name (src/gpu.js:65 throws `unknown uniform`)    */
#define FIRE_ERR_CUDA 3        /* a CUDA runtime call failed (message in fire_sim_last_error)        */
#define FIRE_ERR_NO_DEVICE 4   /* no CUDA device, or the device is not an sm_103 part               */
#define FIRE_ERR_OOM 5         /* device or pinned-host allocation failed                            */
#define FIRE_ERR_STATE 6       /* call not valid in the current state (e.g. stage before geometry)  */

/* ---- parameter block ---------------------------------------------------------------------------
 * The 60 scalar parameters in SIM_FIELDS order (src/sim.js:14-23), padded to 64 floats exactly like
 * the reference's uniform buffer (UniformStruct, src/gpu.js:48-61).  Defaults: SIM_DEFAULTS
 * (src/sim.js:25-44).  The first 12 entries (nx..nLogs) are owned by the simulation and rewritten
 * every step, as uploadUniforms does (src/sim.js:620-624).                                         */
#define FIRE_PARAM_COUNT 60
#define FIRE_PARAM_STRIDE 64

/* Build-defined extension block: the soot age gate, a coal-bed gain and Gaussian pyrolysis spots.
 * These have no counterpart in the reference uniform; with their defaults (0.015, 0.05, 1, no spots)
 * the step is the reference step.                                                                   */
#define FIRE_MAX_SPOTS 16
#define FIRE_MAX_LOGS 16

/* ---- fields --------------------------------------------------------------------------------------
 * The reference's 3D textures (src/sim.js:71-76) and multigrid level 0 (src/sim.js:79-87).  Layout in
 * device memory: dense, x fastest, then y, then z; 4 channels per cell for the rgba fields (float32
 * each), 1 channel for P/B; noise/curl tables are 128^3 texels of 4 IEEE halves (rgba16float).       */
enum FireField {
  FIRE_FIELD_VEL = 0,   /* xyz velocity (m/s), w = 0 after projection          sim.vel  */
  FIRE_FIELD_VELX = 1,  /* forward-advected hats, then pre-projection velocity sim.velX */
  FIRE_FIELD_VELY = 2,  /* MacCormack-corrected velocity                       sim.velY */
  FIRE_FIELD_S = 3,     /* theta, fuel, soot, heat release                     sim.S    */
  FIRE_FIELD_SX = 4,
  FIRE_FIELD_SY = 5,
  FIRE_FIELD_S2 = 6,    /* products, gas age, smoke, CO fraction               sim.S2   */
  FIRE_FIELD_S2X = 7,
  FIRE_FIELD_S2Y = 8,
  FIRE_FIELD_VORT = 9,  /* curl of velY; written only by the stand-alone curl stage (the step fuses it) */
  FIRE_FIELD_GEO = 10,  /* band, bed, solid, sdf                               sim.geo  */
  FIRE_FIELD_P = 11,    /* pressure, multigrid level 0                         levels[0].p */
  FIRE_FIELD_B = 12,    /* divergence right-hand side, level 0                 levels[0].b */
  FIRE_FIELD_NOISE = 13,/* 128^3 rgba16f noise table (src/noise.js:6-64)                  */
  FIRE_FIELD_CURL = 14, /* 128^3 rgba16f curl table  (src/noise.js:67-90)                 */
  FIRE_FIELD_COUNT = 15
};

/* Pipeline stages (the dispatches of FireSim.step, src/sim.js:632-644), for stage-level runs and
 * per-stage timing.  FIRE_STAGE_FORCES is the fused curl + forces kernel.                            */
enum FireStage {
  FIRE_STAGE_GEO = 0, FIRE_STAGE_ADV1 = 1, FIRE_STAGE_ADV2 = 2, FIRE_STAGE_CURL = 3,
  FIRE_STAGE_FORCES = 4, FIRE_STAGE_DIV = 5, FIRE_STAGE_VCYCLE = 6, FIRE_STAGE_PROJECT = 7,
  FIRE_STAGE_COUNT = 8
};

typedef struct FireSim FireSim;

/* Construction options: the FireSim constructor's {res, size, vcycles} (src/sim.js:49) plus the noise
 * table seed the page passes to makeNoiseTexture (src/main.js:36).                                  */
typedef struct FireConfig {
  int res[3];          /* cells in x, y, z                                                        */
  float size[3];       /* domain size in metres; dx = size[0] / res[0] (src/sim.js:53)            */
  int vcycles;         /* multigrid V(2,2) cycles per step (src/sim.js:55, 642)                    */
  int device;          /* CUDA device ordinal                                                     */
  int noise_seed;      /* seed of the baked noise table (reference page: 1)                        */
  int mg_max_cycles;   /* > 0: residual-driven solve, at most this many cycles (0 = fixed vcycles) */
  double mg_tol;       /* relative residual ||b - A p|| / ||b|| target of the residual-driven mode   */
} FireConfig;
/* The residual-driven solve runs inside the step graph (a conditional loop decided on the device) and stops
 * only on a tested residual <= mg_tol or after mg_max_cycles.  The test is skipped on cycles the previous
 * steps predict are still needed, with periodic probes one cycle earlier; a step whose need fell since the
 * last probe runs one cycle more than it needs.                                                      */

typedef struct FireFieldDesc {
  void* data;          /* device pointer, owned by the simulation, valid until destroy              */
  int dims[3];         /* texels in x, y, z                                                        */
  int channels;        /* 4 (rgba) or 1                                                            */
  int elem_bytes;      /* bytes per channel: 4 (float32) or 2 (float16)                             */
  size_t strides[3];   /* byte strides of x, y, z                                                  */
  size_t bytes;        /* total size                                                                */
} FireFieldDesc;

typedef struct FireInfo {
  int res[3];
  float size[3];
  float dx;
  float origin[3];     /* (-sx/2, 0, -sz/2) (src/sim.js:54)                                        */
  double time;         /* sim.time (src/sim.js:57, 646)                                            */
  long long frame;     /* sim.frame                                                                 */
  int n_levels;        /* multigrid levels (src/sim.js:79-87)                                       */
  int coarse_iters;    /* red-black sweeps on the coarsest level (src/sim.js:88-92)                 */
  int vcycles;
  int last_cycles;     /* V-cycles run by the most recent step (residual-driven mode)               */
  double last_rel_residual; /* relative residual after the most recent step (if measured)          */
  long long total_cycles;   /* V-cycles run since creation (residual-driven mode; else steps x vcycles) */
} FireInfo;

/* ---- lifetime ------------------------------------------------------------------------------------ */
/* new FireSim(device, {res, size, logs, vcycles, noiseTex, curlTex}) (src/sim.js:49-101).  Bakes the noise
 * and curl tables on the device (makeNoiseTexture/makeCurlTexture, src/noise.js:6-90).  `logs` holds
 * n_logs capsules of 8 floats (a.xyz, r, b.xyz, burn) as packLogs writes them (src/scene.js:92-98);
 * the reference passes all 16 packed slots, so n_logs = 16 with zero padding reproduces it.
 * FIRE_ERR_BAD_ARG for a resolution below 2 on any axis or of more than 2^31 - 1 cells.           */
int fire_sim_create(const FireConfig* cfg, const float* logs, int n_logs, FireSim** out);
int fire_sim_destroy(FireSim* sim);

/* FireSim.step(enc, dt) x n_steps (src/sim.js:627-648): each step uploads the parameter block, rebuilds
 * the emitter geometry if it is stale (src/sim.js:632), then runs advection, forces, divergence, the
 * multigrid solve and projection as one CUDA graph on `stream`.  Asynchronous.                      */
int fire_sim_step(FireSim* sim, float dt, int n_steps, void* stream);
/* Waits for all work the handle queued (FIRE.step's onSubmittedWorkDone, src/main.js:244).         */
int fire_sim_sync(FireSim* sim);

/* ---- parameters (FireSim.setParams, src/sim.js:601-604) ----------------------------------------- */
/* Merges name/value pairs.  An unknown name fails with FIRE_ERR_BAD_PARAM and changes nothing.
 * Setting hotR0, hotR1, hotY1 or bedRadius marks the geometry stale, as the reference does.         */
int fire_sim_set_params(FireSim* sim, const char* const* names, const float* values, int n);
int fire_sim_get_param(FireSim* sim, const char* name, float* value);
/* Whole block in SIM_FIELDS order (64 floats); entries 0..11 are ignored on set.                   */
int fire_sim_set_param_block(FireSim* sim, const float* block64);
int fire_sim_get_param_block(FireSim* sim, float* block64);
/* The block the next step would upload for time step dt (uniforms + extension, FIRE_BLOCK_FLOATS
 * floats): what uploadUniforms writes (src/sim.js:620-624), before this step's event envelopes.     */
#define FIRE_BLOCK_FLOATS 208
int fire_sim_peek_block(FireSim* sim, float dt, float* out);
/* SIM_FIELDS index of a name, or -1; and the name of an index (src/sim.js:14-23).                   */
int fire_param_index(const char* name);
const char* fire_param_name(int index);
/* SIM_DEFAULTS in SIM_FIELDS order (src/sim.js:25-44); simulation-owned entries are 0.              */
int fire_param_defaults(float* block64);

/* Extensions with no counterpart in the reference (defaults reproduce the reference step):
 * soot formation age gate smoothstep(age0, age1, age) (reference constants 0.015, 0.05 at
 * src/sim.js:314) and a gain on the coal bed of the emitter geometry (1 = reference, 0 = no bed).   */
int fire_sim_set_soot_age(FireSim* sim, float age0, float age1);
int fire_sim_set_bed_gain(FireSim* sim, float gain);
/* Gaussian pyrolysis spots: n records of (x, y, z, sigma_m, flux_g_per_s).  A spot adds a pyrolysis
 * source of peak weight flux / ref_flux (ref_flux = 4 g/s) with a Gaussian profile of width sigma;
 * it feeds the same source path as the log pyrolysis band (src/sim.js:246-284).                    */
int fire_sim_set_spots(FireSim* sim, const float* spots, int n);
/* Over-relaxation factor of every red-black sweep of the step's V-cycle (pre/post smoothing and the
 * coarsest-level sweeps): p += omega (p_GS - p), 0 < omega < 2.  1 (default) is the reference's
 * Gauss-Seidel (src/sim.js:417-437) bit for bit; a larger value can cut the cycles a residual-driven solve
 * needs (no counterpart in the reference).                                                            */
int fire_sim_set_mg_omega(FireSim* sim, float omega);
/* Fault-injection hook for the device-side bounded wait (no counterpart in the reference, which logs
 * WebGPU device loss, src/gpu.js:25-26): the multigrid's single-CTA tail waits for the TMA bulk copies that
 * stage its first level into shared memory for at most `polls` polls (default 4194304, and about a second)
 * before it records a timeout, waits again at the full bound for the copies in flight and returns without
 * running the cycle; fire_sim_sync then reports FIRE_ERR_CUDA ("a device-side wait timed out") and clears
 * the flag.  0 makes the first wait give up at once, so a test can exercise that path on a healthy GPU.   */
int fire_sim_set_tail_wait_limit(FireSim* sim, int polls);

/* ---- events (src/main.js:401-407, 456-461; src/timeline.js:126-157) ---------------------------- */
/* inject: a burst puff (burstX/Y/Z, burstAmt; forces at src/sim.js:288-296) of `amount` lasting
 * `duration` seconds of simulated time (the page holds burstAmt = 1 for 250 ms, src/main.js:404, 461). */
int fire_sim_inject(FireSim* sim, float x, float y, float z, float amount, float duration);
/* stoke: moves log `log_index` as applyLogs does (src/main.js:135-150) with the timeline's offsets
 * scaled by s in [0, 1] (src/timeline.js:126-133: foot 2 cm out, top 1.2 cm out and 4 cm down), marks
 * the geometry stale, and injects a 0.25 s burst at the log's foot.                                   */
int fire_sim_stoke(FireSim* sim, int log_index, float s);
/* gust: the page's wind envelope windX = -1.4 g, windZ = 0.5 g with g = sin(pi (1 - t_left / dur))
 * (src/main.js:405, 459-461), advanced per step in simulated time and scaled by `strength`.          */
int fire_sim_gust(FireSim* sim, float strength, float duration);

/* ---- state ------------------------------------------------------------------------------------- */
/* FireSim.reset (src/sim.js:606-618): zero every velocity/scalar/vorticity field and every pressure
 * level; time = frame = 0.                                                                         */
int fire_sim_reset(FireSim* sim);
/* Rewrite the log buffer and mark the geometry stale (src/main.js:147-149).                          */
int fire_sim_upload_logs(FireSim* sim, const float* logs, int n_logs);

/* Zero-copy view of a field's device buffer (the reference binds sim.vel/S/S2 into the renderer and
 * sparks, src/renderer.js:603-610, src/sparks.js:245).                                               */
int fire_sim_field(FireSim* sim, int which, FireFieldDesc* out);
/* Synchronous copies between a field and host memory (`bytes` must equal FireFieldDesc.bytes).
 * Readback as FIRE.stats does it (src/main.js:268-294); upload sets state for tests and restarts.  */
int fire_sim_download(FireSim* sim, int which, void* host, size_t bytes);
/* Checkpoint and resume (no counterpart in the reference, which resumes a capture by re-simulating from
 * the start, tools/render_video.mjs:79-82).  fire_sim_save writes the state a later step depends on into a
 * host buffer: time and frame, the parameter block and its extension, the logs, the event envelopes, the
 * residual-driven loop's cycle prediction, vel, S, S2 and the level-0 pressure (the warm start).  With
 * buf = NULL it only reports the size in *bytes.  fire_sim_load restores it into a simulation created with
 * the same grid and size (other configuration, e.g. the solver settings, is the caller's); the emitter
 * geometry is rebuilt from the restored logs at the next step.  Steps after a load give the same bits as the
 * saved simulation's steps would have.  Both synchronise the device.                                   */
int fire_sim_save(FireSim* sim, void* buf, size_t capacity, size_t* bytes);
int fire_sim_load(FireSim* sim, const void* buf, size_t bytes);
int fire_sim_upload(FireSim* sim, int which, const void* host, size_t bytes);
int fire_sim_info(FireSim* sim, FireInfo* out);
const char* fire_sim_last_error(FireSim* sim);

/* ---- stage-level access and profiling (src/sim.js:629-644 profileStages; src/gpu.js:128-171) -- */
/* Runs one stage with the current parameter block and dt (no time advance).  FIRE_STAGE_VCYCLE runs
 * one V(2,2) cycle.  Synchronous with respect to `stream`'s previous work only.                     */
int fire_sim_run_stage(FireSim* sim, int stage, float dt, void* stream);
/* Multigrid pieces on level `level` (1 = smooth colour `arg`, 2 = restrict level -> level+1,
 * 3 = prolong level+1 -> level, 4 = shared-memory V-cycle from `level` to the coarsest level,
 * 5 = `arg` red-black sweeps, 6 = level-0 residual norms into device scratch without waiting), for
 * kernel-level parity tests and timing (mgSmooth/mgRestrict/mgProlong, src/sim.js:417-495).        */
int fire_sim_run_mg(FireSim* sim, int op, int level, int arg, void* stream);
/* Level arrays (which: 0 = p, 1 = b) of any multigrid level, as float32 host arrays.               */
int fire_sim_level_io(FireSim* sim, int level, int which, void* host, size_t bytes, int to_device);
int fire_sim_level_dims(FireSim* sim, int level, int dims3[3], float* h);
/* Per-stage GPU milliseconds of the most recent profiled step: enable, then read FIRE_STAGE_COUNT
 * floats (waits for that step).  Stage 3 (curl) is fused into stage 4 and reads 0.                 */
int fire_sim_profile(FireSim* sim, int enable);
int fire_sim_stage_times(FireSim* sim, float* ms, int n);
/* Relative residual ||b - A p||_2 / ||b||_2 of multigrid level 0 (FP64 sums, fixed order).        */
int fire_sim_residual(FireSim* sim, double* rel, void* stream);

/* ---- diagnostics (FIRE.stats / FIRE.profile, src/main.js:268-355) ------------------------------ */
/* Per-channel min, max, mean and non-finite count of a 4-channel field: out[16] = 4 x (min, max,
 * mean, bad).  Deterministic device reduction; synchronous.                                        */
int fire_sim_stats(FireSim* sim, int which, double* out16, void* stream);
/* Heat release rate in kW: sum of 354800 q / T dV over cells with q > 0 (src/main.js:347-352).     */
int fire_sim_hrr(FireSim* sim, double* q_kw, void* stream);
/* Queue the stats of S and the heat release into a pinned host buffer without waiting:
 * out[0..15] = S stats as in fire_sim_stats, out[16] = heat release (kW).  The values are valid once
 * `stream` has reached this point (fire_sim_sync or a stream/event wait).                          */
int fire_sim_stats_async(FireSim* sim, double* pinned_out17, void* stream);
/* Per-step diagnostics (enable = 1): every fire_sim_step forms the values of fire_sim_stats_async (same
 * kernels, same bits) on a graph branch that runs beside the divergence, pressure solve and projection,
 * and fire_sim_stats_async after a step only queues their copy to the host.  A call that changes S
 * through the API (upload, load, reset, stage runs, the adjoint, an ensemble step) makes the next
 * fire_sim_stats_async compute them again; writes through fire_sim_field's pointer are not seen, so call
 * this with 0 before writing S that way.  The change takes effect at the next step (the step graph is
 * rebuilt; this call synchronises the device).  Off by default.                                        */
int fire_sim_set_step_stats(FireSim* sim, int enable);
/* FIRE.profile's height profile (src/main.js:322-340): for rows j = 0, 4, 8, ... of y, over the x-z plane
 * of S, with T = 293 + 1000 S.x: h = (j + 0.5) dx, the mean T of the centreline cells (|i - nx/2| < 3 and
 * |k - nz/2| < 3), the maximum T (from 0), the maximum soot S.z and fuel S.y (from 0) and the count of
 * cells above 1000 K.  rows6 receives n = ceil(ny / 4) rows of 6 doubles (h, Tc, Tmax, soot, fuel, hot);
 * FIRE_ERR_BAD_ARG if max_rows < n.  T, Tc and the comparisons are FP64 like the reference's JS; the
 * reference rounds the values for display (Tc, Tmax to integers, h, soot, fuel to 0.01), this does not.
 * Synchronous.                                                                                      */
int fire_sim_height_profile(FireSim* sim, double* rows6, int max_rows, int* n_rows, void* stream);

/* ---- scene helpers (src/scene.js) ------------------------------------------------------------- */
/* buildCampfire(seed) + packLogs (src/scene.js:13-42, 92-98): writes max_logs*8 floats (8 real logs,
 * zero-padded); returns the number of real logs.                                                    */
int fire_build_campfire(uint32_t seed, float* out, int max_logs);
/* Seeded floor spots for the spot emitter: n records (x, 0, z, sigma, flux) with positions uniform
 * on a disc of `radius` around the origin and flux uniform in [flux_lo, flux_hi] g/s.  Uses the
 * reference's pcg hash (src/shaders/lib.js:11-18).                                                 */
int fire_make_spots(uint32_t seed, int n, float flux_lo, float flux_hi, float sigma, float radius, float* out);

/* ---- pressure solve without device allocation --------------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate device memory when they
 * need a pressure solve - hosts whose device memory belongs to another allocator (a caching or pooled
 * allocator that must not be bypassed), frame loops that fixed their memory budget up front, or code
 * recording into a CUDA graph, where cudaMalloc is not allowed.
 *
 * Runs `cycles` V(2,2) cycles of the step's multigrid on caller-owned level-0 device arrays: `p` (pressure,
 * updated in place) and `b` (right-hand side, read only), both nx*ny*nz floats, x fastest; `h` is the cell
 * size in metres.  The level rules, coarse sweep count and kernels are those of fire_sim_step; the sweeps
 * are the reference's plain Gauss-Seidel (omega 1, fire_sim_step's default; fire_sim_set_mg_omega does not
 * apply here).  Every coarser level lives in one file-scope device array of FIRE_NOALLOC_SCRATCH_BYTES that
 * the library holds on every GPU that loads it until the process exits; nothing is allocated or freed.
 *   - The first call on a device (the one current when it is called) sets that device up: it resolves the
 *     array's device address and opts the coarse-level kernel into its shared memory.  Make that first call
 *     before any stream capture.
 *   - Grids whose coarse levels do not fit the array (level-0 grids beyond roughly 7 million cells) are
 *     rejected with FIRE_ERR_BAD_ARG before any work is queued.
 *   - All calls share the array and it keeps the last call's contents; each cycle rewrites the coarse
 *     levels before reading them, so nothing needs clearing between calls.  Calls whose work overlaps on the
 *     GPU (concurrent streams, or several host threads) race on the array: serialise them.
 * Asynchronous on `stream` (a cudaStream_t, or NULL).
 * Returns FIRE_ERR_CUDA if a launch failed (an error left by the caller's earlier work is not blamed on it).
 * If the coarse-level kernel's bounded wait for its staging copies ever runs out, that cycle skips its coarse
 * correction and the kernel records it in a flag at the end of the array: fire_poisson_noalloc_status reports
 * it (FIRE_ERR_CUDA) after waiting for `stream`, and clears it.                                            */
#define FIRE_NOALLOC_SCRATCH_BYTES (8u * 1024u * 1024u)
int fire_poisson_vcycles_noalloc(float* p, const float* b, int nx, int ny, int nz, float h, int cycles, void* stream);
/* Waits for `stream` and reports (FIRE_ERR_CUDA) and clears a bulk-copy wait timeout recorded by the calls
 * above on the current device; FIRE_OK if none.  Allocates nothing; synchronous.                         */
int fire_poisson_noalloc_status(void* stream);

/* ---- ensembles of independent simulations ------------------------------------------------------
 * n (<= 64) simulations of possibly different grids advanced together: each stage of a step is one
 * kernel launch over all members, the multigrid levels are batched level by level and the members'
 * shared-memory tails run in one launch per tail form, all captured in one CUDA graph per step.  The
 * members are FireSim handles owned by the ensemble: configure them (params, spots, soot age, events) and
 * read them (fields, stats) with the fire_sim_* functions, but step them only through the ensemble and do
 * not destroy them.  Every member must use fixed V-cycles (mg_max_cycles = 0) with the same count, the
 * same device and the same noise_seed (the noise/curl tables are shared).  The batched kernels run the
 * per-simulation kernels' bodies, so a member's fields are those fire_sim_step gives it alone up to FP32
 * rounding (FMA contraction may differ between the two compiled forms).  No counterpart in the reference
 * (one FireSim per page).                                                                               */
typedef struct FireEnsemble FireEnsemble;
int fire_ensemble_create(const FireConfig* cfgs, int n, FireEnsemble** out);
int fire_ensemble_destroy(FireEnsemble* e);
int fire_ensemble_size(FireEnsemble* e);
int fire_ensemble_sim(FireEnsemble* e, int index, FireSim** out);
/* n_steps steps of dt seconds for every member, asynchronous on `stream`.  Step number `at_step` of
 * fire_ensemble_set_autotune (default 8, once the fires have developed) is the tuning step: it runs
 * eagerly, times every tile candidate of every batched stage on the members' current state and keeps the
 * fastest (the call waits for those timings); the step's results are those of any other step.  Steps
 * before it use tile 0 everywhere.                                                                      */
int fire_ensemble_step(FireEnsemble* e, float dt, int n_steps, void* stream);
int fire_ensemble_sync(FireEnsemble* e);
const char* fire_ensemble_last_error(FireEnsemble* e);
/* Tile candidates of the batched stages (adv1, adv2, forces, div, project): cell tiles 0-3 (32x4x2, 32x8x1,
 * 32x2x4, 64x4x1 threads) for the per-cell stages, z-march depths 0-2 (16, 8, 32 planes) for forces.
 * fire_ensemble_tiles reports the chosen ones (FIRE_ERR_STATE before the tuning step) and, if ms is not
 * NULL, the measured mean launch time of each candidate (5 x 4 floats, ms; unused entries 0).          */
#define FIRE_ENSEMBLE_STAGES 5
int fire_ensemble_set_autotune(FireEnsemble* e, int at_step);   /* -1: no tuning; re-arms a new tuning */
int fire_ensemble_set_tiles(FireEnsemble* e, const int* tiles);
int fire_ensemble_tiles(FireEnsemble* e, int* tiles, float* ms);

/* ---- sparks (src/sparks.js) ---------------------------------------------------------------------
 * Burning sparks carried by a simulation's velocity field: the particle update of Sparks.step
 * (src/sparks.js:55-142, 250-274).  A spark is 16 floats: position+age, velocity+burn time left,
 * previous position+temperature (K), diameter (mm)+seed+alive+flicker (Hz).  fire_sparks_step reads the
 * simulation's velocity: queue it after fire_sim_step on the same stream.  The drawing of the streaks
 * (src/sparks.js:146-221) is a rasterisation pass and is not part of this library.                   */
typedef struct FireSparks FireSparks;
int fire_sparks_create(FireSim* sim, int count, FireSparks** out);        /* Sparks constructor (count)  */
int fire_sparks_destroy(FireSparks* s);
int fire_sparks_reset(FireSparks* s);                                      /* src/sparks.js:38-41       */
/* burst({n, pos, speed, radius, dur, fan, size, aim}) (src/sparks.js:44-46); aim3 may be NULL.      */
int fire_sparks_burst(FireSparks* s, int n, const float pos[3], float speed, float radius, float dur, float fan, float size,
                      const float* aim3);
/* rate (sparks/s, the page sets 1 x intensity) and params.turb / lifeK / sizeK / upK.               */
int fire_sparks_set(FireSparks* s, float rate, float turb, float lifeK, float sizeK, float upK);
int fire_sparks_step(FireSparks* s, float dt, void* stream);               /* src/sparks.js:250-274     */
/* The 27 uniforms (SPARK_FIELDS order) the next step would use, without advancing anything.         */
int fire_sparks_peek(FireSparks* s, float dt, float* out27);
int fire_sparks_buffer(FireSparks* s, void** dev_ptr, int* count);          /* zero-copy device view     */
int fire_sparks_io(FireSparks* s, float* host, size_t bytes, int to_device);   /* count * 16 floats, sync */
int fire_sparks_set_rate(FireSparks* s, float rate);                        /* sparks.rate alone         */

/* ---- volume rendering of the fire (src/renderer.js pLights, pSharpen, pVolume) -------------------
 * The renderer's fire light extraction (8 temporally filtered point lights, one per height band), the
 * optional flame prefilter and the emission-absorption ray march of S (soot, temperature, heat release)
 * and S2 (smoke) with single scattering of the lights, into a headless image of vw x vh pixels
 * (vw = max(8, round(width * vol_scale))): per pixel radiance rgb and transmittance, plus haze and depth.
 * The page's surfaces (logs, stones, ground), composite, bloom and tone map are rasterisation and display
 * and are not part of this library; a caller may give the depth the march stops at.                    */
typedef struct FireVolume FireVolume;
/* white_balance_k: the camera white balance (the renderer uses 5000 K; 0 = none).                       */
int fire_volume_create(FireSim* sim, int width, int height, float vol_scale, float white_balance_k, FireVolume** out);
int fire_volume_destroy(FireVolume* v);
int fire_volume_size(FireVolume* v, int* vw, int* vh);
/* Renderer parameters (RP_FIELDS names): stepMul sootAbs sootEmit emitK blueK smokeScat smokeG detailAmt
 * detailFreq detailSpeed lightK tempScale emitTempLo sootScat sootEdge cubic flameSharp flickerK lensX
 * lensY focus.  Unknown names: FIRE_ERR_BAD_PARAM.                                                       */
int fire_volume_set_params(FireVolume* v, const char* const* names, const float* values, int n);
/* lookAt (src/camera.js:6-17); jitter in full-resolution pixels.                                        */
int fire_volume_set_camera(FireVolume* v, const double pos[3], const double target[3], double fov_deg, float jit_x, float jit_y);
int fire_volume_set_depth(FireVolume* v, const float* depth_dev, int width, int height);   /* NULL: none */
/* The f32 uniforms the next render would use (returns their count, at most 64).                         */
int fire_volume_uniforms(FireVolume* v, double time, int frame, float* out, int n);
int fire_volume_render(FireVolume* v, double time, int frame, void* stream);
/* which: 0 image (vw*vh*4 floats), 1 aux (vw*vh*2: haze, depth), 2 lights (8 * 8: pos+power,
 * colour+spread), 3 blackbody LUT (2 * 1024 * 4).  Synchronous.                                          */
int fire_volume_download(FireVolume* v, int which, float* host, size_t bytes);
/* blackbodyLUT (src/blackbody.js:78-93): 2 rows (blackbody, soot) x n x (r, g, b, Y) over [tmin, tmax].   */
int fire_blackbody_lut(int n, float tmin, float tmax, float white_balance_k, float* out);

/* ---- the cinematic's timeline (src/timeline.js) and its capture-mode driver (src/main.js:128-160) ----
 * Host-only and deterministic.  Events: the scripted cue sheet plus the seeded background pops, sorted by
 * time.  fire_timeline_step(j) is capStep(j): the simulation's parameters (simAt) and log offsets
 * (logOffsetsAt, applied to the base logs and re-uploaded when they change) at t = j / (30 n), the spark
 * bursts of the events in [t, t + 1/(30 n)), then one fire_sim_step and one fire_sparks_step (sparks may
 * be NULL) of 1 / (30 n) seconds.  No GPU work of its own.                                              */
enum { FIRE_EVENT_POP = 0, FIRE_EVENT_CRACKLE_BURST = 1, FIRE_EVENT_LOG_SHIFT = 2, FIRE_EVENT_GUST = 3, FIRE_EVENT_IGNITE = 4 };
typedef struct {
  double t;                 /* seconds                                                                */
  int type;                 /* FIRE_EVENT_*                                                           */
  double strength;
  double pos[3];
  int has_aim;
  double aim[3];
  int log;                  /* log-shift: the log that moves                                          */
  double dur;               /* gust: duration (s)                                                     */
} FireTimelineEvent;
int fire_timeline_event_count(void);
int fire_timeline_events(FireTimelineEvent* out, int max);                 /* returns the number written */
double fire_timeline_intensity_at(double t);                               /* src/timeline.js:118-129   */
/* simAt (src/timeline.js:147-170): intensity, burstAmt, burstX, burstY, burstZ, windX, windZ.          */
int fire_timeline_sim_at(double t, double* out7);
/* logOffsetsAt (src/timeline.js:136-144): returns 1 and the offsets after the log shift, else 0.       */
int fire_timeline_log_offsets_at(double t, int* index, double* s, double* foot_out, double* top_drop, double* top_out);
int fire_timeline_camera_at(double t, double* pos3, double* target3, double* fov_deg);   /* cameraAt    */
int fire_timeline_lens_at(double t, double* focus, double* aperture, double* fmm, double* fnum);   /* lensAt */
double fire_timeline_exposure_at(double t);                                /* exposureAt                */
double fire_timeline_preroll(void);                                        /* PREROLL (s)               */
typedef struct FireTimeline FireTimeline;
/* base_logs: the campfire's packed logs (8 floats each); steps_per_frame: n (dt = 1 / (30 n)).          */
int fire_timeline_create(const float* base_logs, int n_logs, int steps_per_frame, FireTimeline** out);
int fire_timeline_destroy(FireTimeline* tl);
double fire_timeline_step_dt(FireTimeline* tl);
double fire_timeline_step_time(FireTimeline* tl, long long j);
int fire_timeline_step(FireTimeline* tl, FireSim* sim, FireSparks* sparks, long long j, void* stream);

/* ---- standalone pressure Poisson solver --------------------------------------------------------
 * The step's pressure equation (src/sim.js:415-495, 576-599: cell-centred 7-point Laplacian, p = 0 on the
 * side and top faces, zero gradient at the floor, levels halved while every dimension is even and the
 * smallest exceeds 6) solved on its own to a relative residual ||b - A x||_2 / ||b||_2 <= tol.
 *   FIRE_POISSON_FP32  the step's V(2,2) cycle (the reference's multigrid, coarseIters coarsest sweeps) on x
 *                      and b directly, repeated until the tolerance is met (research/webgpu-bench/poisson.mjs
 *                      iterates the same cycle).  An FP32 x cannot represent the solution to much better
 *                      than ~1e-5 relative residual on large grids (its rounding alone leaves that much), so
 *                      this form stalls there.
 *   FIRE_POISSON_FP16 / FIRE_POISSON_BF16 / FIRE_POISSON_IR32  iterative refinement: the solution is an FP32
 *                      pair (x, x_lo) updated with error-free additions and the residual is formed from
 *                      neighbour differences, all in FP32 arithmetic; each correction A e = r is one V(2,2)
 *                      cycle whose level arrays are stored in IEEE half / bfloat16 / FP32 (arithmetic in FP32
 *                      registers), with r scaled by the previous residual's RMS so it stays inside half's
 *                      range, and the coarsest level solved exactly in FP64 (dense inverse; FP64 sweeps when
 *                      it has more than 512 cells).  These reach 1e-6 and below.
 * Residual norms and the RHS mean are double-float (FP32 pair) reductions in a fixed order: deterministic,
 * ~44 significant bits.  The solve loop runs on the device (a CUDA graph with a conditional WHILE node):
 * fire_poisson_solve queues it on `stream` and returns; fire_poisson_result waits and reports.
 * No counterpart in the reference as an entry point: it exists there only inside FireSim.step and the
 * research multigrid benchmarks.                                                                        */
enum { FIRE_POISSON_FP32 = 0, FIRE_POISSON_FP16 = 1, FIRE_POISSON_BF16 = 2, FIRE_POISSON_IR32 = 3 };
typedef struct FirePoisson FirePoisson;
typedef struct {
  int iterations;              /* V-cycles (FP32) or refinement steps (FP16/BF16) of the last solve     */
  double rel_residual;         /* ||b - A x|| / ||b|| after the last solve                             */
  double rel_residual_initial; /* before it                                                             */
  double b_norm;               /* ||b||_2                                                               */
} FirePoissonResult;
/* res: grid (x fastest, then y, then z); h: cell size in metres; device: CUDA ordinal.                  */
int fire_poisson_create(const int res[3], float h, int precision, int device, FirePoisson** out);
int fire_poisson_destroy(FirePoisson* ps);
/* x (in: initial guess, out: solution) and b are device arrays of res[0]*res[1]*res[2] floats, x 16-byte
 * aligned.  x_lo (refinement forms; may be NULL): the low half of the solution pair, in/out like x; with
 * NULL the pair starts at (x, 0) and only its rounded sum x is returned.  inner_cycles: V-cycles per
 * refinement step (1..16; ignored by FIRE_POISSON_FP32, as is x_lo).                                      */
int fire_poisson_solve(FirePoisson* ps, const float* b, float* x, float* x_lo, double tol, int max_iters, int inner_cycles,
                       void* stream);
int fire_poisson_result(FirePoisson* ps, FirePoissonResult* out);
/* Relative residual of (b, x + x_lo) (x_lo may be NULL), double-float norms; synchronous.                  */
int fire_poisson_residual(FirePoisson* ps, const float* b, const float* x, const float* x_lo, double* rel);
/* Seeded zero-mean right-hand side on the device: n_sources Gaussian sources (centres uniform over the
 * grid, sigma uniform in [1, 4] cells, amplitude standard normal) plus `noise` times per-cell standard
 * normal noise, then the mean removed.  Asynchronous on `stream`.                                       */
int fire_poisson_make_rhs(FirePoisson* ps, float* b, unsigned seed, int n_sources, float noise, void* stream);
/* The sources of fire_poisson_make_rhs as 5 floats each (centre x, y, z in cells, sigma in cells,
 * amplitude); host only.                                                                                */
int fire_poisson_sources(unsigned seed, int n_sources, const int res[3], float* out);
/* FIRE_POISSON_FP32 form only: runs the V-cycle variant of the reference's multigrid convergence studies
 * instead of the simulation's (research/webgpu-bench/poisson.mjs:28-75 rbgs / prolongAdd / vcycle and
 * research/webgpu-bench/wgsl/mg.wgsl:20-35 smoothRB, 97-105 prolongAdd): the red-black update takes ghost
 * values from the cell's old value, p <- mix(p, (sum_nb - h^2 b) / 6, omega), prolongation is clamp-to-edge
 * trilinear without sign flips, and the coarsest level gets `coarse_sweeps` sweeps (poisson.mjs: 30,
 * bench.js benchMG: 16).  Restriction and the level hierarchy are unchanged.  With h = 1 the levels have
 * h^2 = 4^l as in the studies.  Lets the GPU reproduce the studies' recorded residual histories.           */
int fire_poisson_set_study(FirePoisson* ps, int coarse_sweeps);

/* ---- discrete adjoint of the step and checkpointed rollouts -----------------------------------------
 * Reverse-mode derivatives of FireSim.step (src/sim.js:627-648) over a rollout of n steps: the adjoint of
 * each stage (advect, sources, projection) linearised at the branch the forward took (every min / max /
 * clamp, the MacCormack limiter, the speed clamps), the pressure solve treated as p = A^-1 b with A the
 * multigrid's symmetric operator (so its adjoint is the same solve).  The rollout keeps the state every
 * `checkpoint_every` steps; the backward recomputes one segment at a time into a tape and runs the
 * adjoint steps over it.  No counterpart in the reference (it has no derivatives).
 *
 *   fire_adjoint_forward   n steps of dt from the simulation's current state (per-step parameter blocks
 *                          and event envelopes as fire_sim_step), leaving the simulation in the final state.
 *   fire_adjoint_loss      L = sum over cells (1000 (S.x - T.x))^2 + (S.z - T.z)^2 (temperature in kelvin,
 *                          soot) against a target S field; seeds the final-state cotangents with dL.
 *   fire_adjoint_seed      or seeds arbitrary final-state cotangents (vel, S, S2; NULL = zero).
 *   fire_adjoint_backward  the reverse sweep: afterwards FIRE_ADJ_VEL / S / S2 hold the cotangents of the
 *                          rollout's initial state and fire_adjoint_grad_spots the spot-flux gradients.
 * Cotangent buffers (float4 per cell unless noted), read and written with fire_adjoint_io:                */
enum {
  FIRE_ADJ_VEL = 0, FIRE_ADJ_S = 1, FIRE_ADJ_S2 = 2,            /* state                                  */
  FIRE_ADJ_VELX = 3, FIRE_ADJ_SX = 4, FIRE_ADJ_S2X = 5,         /* advection hats                          */
  FIRE_ADJ_VELY = 6, FIRE_ADJ_SY = 7, FIRE_ADJ_S2Y = 8,         /* advected fields                         */
  FIRE_ADJ_F = 9,                                               /* forces output velocity (xyz), phi (w)   */
  FIRE_ADJ_W = 10,                                              /* vorticity (xyz) and its magnitude (w)   */
  FIRE_ADJ_G = 11,                                              /* projection scratch                      */
  FIRE_ADJ_P = 12, FIRE_ADJ_B = 13,                             /* pressure p, divergence b (1 float)      */
  FIRE_ADJ_COUNT = 14
};
typedef struct FireAdjoint FireAdjoint;
/* n_steps >= 1, 1 <= checkpoint_every <= 512 (k >= n_steps keeps the whole rollout on the tape: no
 * recomputation, 2 CUDA graphs per step captured once).  Device memory: (k + 1) * 3 + k * 7 + 12 float4 fields plus
 * (n_steps / k + 1) * 3 checkpoint fields.  The solve mode (fixed V-cycles or residual-driven) is the
 * simulation's at creation.                                                                             */
int fire_adjoint_create(FireSim* sim, int n_steps, int checkpoint_every, FireAdjoint** out);
int fire_adjoint_destroy(FireAdjoint* adj);
int fire_adjoint_forward(FireAdjoint* adj, float dt, void* stream);
/* target_S: host float4 field (x fastest); loss: out, synchronous.                                       */
int fire_adjoint_loss(FireAdjoint* adj, const float* target_S, double* loss);
int fire_adjoint_seed(FireAdjoint* adj, const float* d_vel, const float* d_S, const float* d_S2);
int fire_adjoint_backward(FireAdjoint* adj, void* stream);
/* dL/d(flux) of each spot in g/s (n <= the simulation's spot count), synchronous.                         */
int fire_adjoint_grad_spots(FireAdjoint* adj, double* out, int n);
/* dir 0: device -> host, 1: host -> device; bytes must be the buffer's size.                              */
int fire_adjoint_io(FireAdjoint* adj, int which, void* host, size_t bytes, int dir);
/* Zeroes every cotangent buffer and the spot gradients.                                                   */
int fire_adjoint_clear(FireAdjoint* adj);
/* One stage's adjoint at the simulation's own current fields (the stage-level counterpart of
 * fire_sim_run_stage), with parameter block for dt: FIRE_STAGE_ADV1 / ADV2 / FORCES (with the curl) / DIV /
 * PROJECT, or FIRE_STAGE_VCYCLE: `arg` V-cycles of the pressure solve on FIRE_ADJ_P into FIRE_ADJ_B.
 * Each reads the cotangents of the stage's outputs and adds into those of its inputs: ADV1 velX,SX,S2X ->
 * vel,S,S2; ADV2 velY,SY,S2Y -> vel,S,S2 and the hats; FORCES F,S,S2 -> velY (added), SY,S2Y (written),
 * spot gradients; DIV B -> F (added); PROJECT vel -> F (written), P.                                         */
int fire_adjoint_stage(FireAdjoint* adj, int stage, float dt, int arg, void* stream);
/* Timing of the last forward / backward (GPU milliseconds, CUDA events on the call's stream).              */
int fire_adjoint_timing(FireAdjoint* adj, float* forward_ms, float* backward_ms);

/* ---- library ----------------------------------------------------------------------------------- */
/* 1 if the library's kernels were built for the current device's architecture, else 0.             */
int fire_device_ok(int device);
const char* fire_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FIRE_SIM_H */
