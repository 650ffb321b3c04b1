// The 20 s cinematic's cue sheet and the capture-mode driver of the simulation (src/timeline.js, and
// capStep / applyLogs / fireEvent / simStep of src/main.js:70-90, 128-158): deterministic host code that
// sets the simulation's parameters, moves the logs, throws spark bursts and steps the simulation and the
// sparks, so the cinematic's simulation runs end to end through the C ABI.
//
// The tables (shots, intensity keys, scripted events) are the reference's cue sheet restated as data; the
// background pops come from the same seeded generator with JavaScript number semantics (unsigned 32-bit
// LCG, doubles, toFixed rounding).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fire_sim.h"
#include "fire_nvtx.h"

namespace {

constexpr double kPI = 3.141592653589793;
constexpr int kFPS = 30;             // src/timeline.js:6-8
constexpr double kDuration = 20.0;
constexpr double kPreroll = 5.0;

struct Cam { double pos[3], target[3], fov; };
struct Shot { double t0, t1; Cam a, b; double N, ev; };
const Shot kShots[] = {   // src/timeline.js:11-25
  {0.0, 2.4, {{0.62, 0.30, 1.05}, {0, 0.40, 0}, 42}, {{0.55, 0.28, 0.93}, {0, 0.38, 0}, 42}, 8.0, -0.3},
  {2.4, 5.6, {{0.45, 0.25, 0.95}, {0, 0.30, 0}, 38}, {{0.40, 1.00, 0.95}, {0, 1.05, 0}, 38}, 7.0, 0.0},
  {5.6, 8.4, {{-0.56, 0.16, -0.05}, {0, 0.12, 0}, 50}, {{-0.48, 0.15, -0.04}, {0, 0.11, 0}, 50}, 8.0, -0.9},
  {8.4, 13.4, {{-0.94, 0.60, 1.29}, {0, 0.40, 0}, 46}, {{-0.835, 0.55, 1.149}, {0, 0.40, 0}, 46}, 11.0, 0.0},
  {13.4, 16.6, {{0.75, 0.10, 0.95}, {0, 0.68, 0}, 50}, {{0.80, 0.12, 0.88}, {0, 0.72, 0}, 50}, 8.0, -0.2},
  {16.6, 20.0, {{0.90, 0.38, 1.55}, {0, 0.45, 0}, 42}, {{0.62, 0.30, 1.05}, {0, 0.40, 0}, 42}, 8.0, -0.3},
};
constexpr int kNShots = sizeof(kShots) / sizeof(kShots[0]);

const double kIntensity[][2] = {   // src/timeline.js:28-31
  {-kPreroll, 1.0}, {0.0, 1.0}, {1.0, 1.0}, {2.0, 1.12}, {6.0, 1.12}, {8.6, 1.0}, {9.0, 1.2}, {9.6, 1.05},
  {11.0, 1.08}, {12.6, 1.08}, {14.0, 1.05}, {18.3, 1.05}, {18.5, 1.15}, {19.2, 1.0}, {20.0, 1.0},
};
constexpr int kNIntensity = sizeof(kIntensity) / sizeof(kIntensity[0]);

struct Event {
  double t;
  int type;                 // FIRE_EVENT_*
  double strength;
  double pos[3];
  bool hasAim;
  double aim[3];
  int log;                  // log-shift: the log index
  double dur;               // gust: duration
};
Event ev(double t, int type, double s, double x, double y, double z) {
  Event e{};
  e.t = t; e.type = type; e.strength = s; e.pos[0] = x; e.pos[1] = y; e.pos[2] = z; e.log = 3; e.dur = 1.6;
  return e;
}
std::vector<Event> scripted() {   // src/timeline.js:34-47
  std::vector<Event> v;
  Event e = ev(0.30, FIRE_EVENT_POP, 1.0, 0.06, 0.14, 0.12);
  e.hasAim = true; e.aim[0] = 0.5; e.aim[2] = 0.86;
  v.push_back(e);
  v.push_back(ev(2.433, FIRE_EVENT_POP, 0.5, -0.08, 0.12, 0.10));
  v.push_back(ev(4.6, FIRE_EVENT_POP, 0.6, 0.10, 0.16, 0.02));
  v.push_back(ev(5.633, FIRE_EVENT_POP, 0.45, -0.05, 0.10, 0.12));
  v.push_back(ev(7.2, FIRE_EVENT_CRACKLE_BURST, 0.5, -0.10, 0.08, 0.06));
  v.push_back(ev(8.433, FIRE_EVENT_POP, 0.5, 0.06, 0.12, 0.10));
  v.push_back(ev(9.0, FIRE_EVENT_LOG_SHIFT, 1.0, 0.05, 0.12, 0.0));
  v.push_back(ev(11.0, FIRE_EVENT_GUST, 1.0, 0, 0.3, 0));
  v.push_back(ev(13.433, FIRE_EVENT_POP, 0.5, 0.08, 0.13, -0.05));
  v.push_back(ev(15.2, FIRE_EVENT_POP, 0.85, -0.06, 0.15, 0.08));
  v.push_back(ev(16.633, FIRE_EVENT_POP, 0.5, 0.02, 0.12, 0.12));
  e = ev(18.5, FIRE_EVENT_POP, 1.0, 0.06, 0.14, 0.12);
  e.hasAim = true; e.aim[0] = 0.5; e.aim[2] = 0.86;
  v.push_back(e);
  return v;
}
// Number.prototype.toFixed then unary plus: the double nearest the decimal rounded to `digits` places.
double to_fixed(double x, int digits) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*f", digits, x);
  return std::strtod(buf, nullptr);
}
// Clustered Poisson background pops (src/timeline.js:51-71), JavaScript number semantics.
std::vector<Event> random_pops(const std::vector<Event>& S, uint32_t seed = 20261025u) {
  uint32_t st = seed;
  auto rnd = [&]() { st = st * 1664525u + 1013904223u; return (double)st / 4294967296.0; };
  std::vector<Event> out;
  double t = 0.6;
  while (t < kDuration - 0.3) {
    t += -std::log(1.0 - rnd()) / 0.8;
    if (t >= kDuration - 0.3) break;
    const double strength = std::min(0.6, 0.12 + 0.45 * std::pow(rnd(), 2.2));
    const double a = rnd() * kPI * 2, r = std::sqrt(rnd()) * 0.2;
    const double px = std::cos(a) * r, py = 0.07 + rnd() * 0.15, pz = std::sin(a) * r;
    out.push_back(ev(to_fixed(t, 3), FIRE_EVENT_POP, to_fixed(strength, 2), px, py, pz));
    if (rnd() < 0.25) {   // aftershock
      const double t2 = t + 0.05 + rnd() * 0.25;
      out.push_back(ev(to_fixed(t2, 3), FIRE_EVENT_POP, to_fixed(strength * 0.5, 2), std::cos(a) * r, 0.1, std::sin(a) * r));
    }
  }
  std::vector<Event> kept;   // clear of the hero events
  for (const Event& e : out) {
    bool near = false;
    for (const Event& s : S) near = near || std::fabs(s.t - e.t) < 0.35;
    if (!near) kept.push_back(e);
  }
  return kept;
}
const std::vector<Event>& events() {   // src/timeline.js:72, sorted stably by time
  static const std::vector<Event> E = [] {
    std::vector<Event> s = scripted();
    std::vector<Event> all = s;
    const std::vector<Event> r = random_pops(s);
    all.insert(all.end(), r.begin(), r.end());
    std::stable_sort(all.begin(), all.end(), [](const Event& a, const Event& b) { return a.t < b.t; });
    return all;
  }();
  return E;
}
const Event* find_type(int type) {
  for (const Event& e : events()) if (e.type == type) return &e;
  return nullptr;
}

const Shot& shot_at(double t) {   // src/timeline.js:75-78
  for (const Shot& s : kShots) if (t < s.t1) return s;
  return kShots[kNShots - 1];
}
double lerp(double a, double b, double u) { return a + (b - a) * u; }

double intensity_at(double t) {   // src/timeline.js:118-129
  if (t <= kIntensity[0][0]) return kIntensity[0][1];
  for (int i = 0; i < kNIntensity - 1; ++i) {
    if (t <= kIntensity[i + 1][0]) {
      const double u = (t - kIntensity[i][0]) / (kIntensity[i + 1][0] - kIntensity[i][0]);
      const double s = u * u * (3 - 2 * u);
      return kIntensity[i][1] + (kIntensity[i + 1][1] - kIntensity[i][1]) * s;
    }
  }
  return kIntensity[kNIntensity - 1][1];
}

}  // namespace

struct FireTimeline {
  std::vector<float> baseLogs;
  int nLogs = 0;
  int n = 8;                 // simulation steps per frame
  std::string logKey;        // the log offsets last applied (applyLogs skips unchanged ones)
};

extern "C" {

int fire_timeline_event_count(void) { return (int)events().size(); }

int fire_timeline_events(FireTimelineEvent* out, int max) {
  if (!out || max < 0) return FIRE_ERR_BAD_ARG;
  const std::vector<Event>& E = events();
  const int n = std::min(max, (int)E.size());
  for (int i = 0; i < n; ++i) {
    const Event& e = E[i];
    FireTimelineEvent& o = out[i];
    o.t = e.t; o.type = e.type; o.strength = e.strength;
    for (int k = 0; k < 3; ++k) { o.pos[k] = e.pos[k]; o.aim[k] = e.aim[k]; }
    o.has_aim = e.hasAim ? 1 : 0;
    o.log = e.log;
    o.dur = e.dur;
  }
  return n;
}

double fire_timeline_intensity_at(double t) { return intensity_at(t); }

// simAt (src/timeline.js:147-170): intensity, burstAmt, burstX, burstY, burstZ, windX, windZ.
int fire_timeline_sim_at(double t, double* out7) {
  if (!out7) return FIRE_ERR_BAD_ARG;
  double p[7] = {intensity_at(t), 0, 0, 0, 0, 0, 0};
  for (const Event& e : events()) {
    const double dt = t - e.t;
    if (dt < 0 || dt > 0.4) continue;
    if (e.type == FIRE_EVENT_LOG_SHIFT || e.type == FIRE_EVENT_POP || e.type == FIRE_EVENT_CRACKLE_BURST) {
      const bool ls = e.type == FIRE_EVENT_LOG_SHIFT;
      const double w = (ls ? 1.0 : 0.6) * e.strength * std::exp(-dt / (ls ? 0.12 : 0.04));
      if (w > p[1]) { p[1] = w; p[2] = e.pos[0]; p[3] = e.pos[1]; p[4] = e.pos[2]; }
    }
  }
  p[5] = 0.28 * std::sin(t * 0.23 + 1.0) + 0.14 * std::sin(t * 0.61 + 0.4);   // slow wandering draft
  p[6] = 0.18 * std::sin(t * 0.17 + 2.3);
  if (const Event* g = find_type(FIRE_EVENT_GUST)) {
    const double dt = t - g->t, dur = g->dur;
    const double w = (dt > 0 && dt < dur + 1.2) ? std::pow(std::sin(kPI * std::min(dt / (dur + 0.6), 1.0)), 1.5) * g->strength : 0.0;
    p[5] += 2.8 * w;
  }
  std::memcpy(out7, p, sizeof p);
  return FIRE_OK;
}

// logOffsetsAt (src/timeline.js:136-144): 1 and (index, s, footOut, topDrop, topOut) after the log shift,
// else 0.
int fire_timeline_log_offsets_at(double t, int* index, double* s, double* foot_out, double* top_drop, double* top_out) {
  const Event* e = find_type(FIRE_EVENT_LOG_SHIFT);
  if (!e || t < e->t) return 0;
  const double u = std::min((t - e->t) / 0.12, 1.0);
  if (index) *index = e->log;
  if (s) *s = u * u * (3 - 2 * u);
  if (foot_out) *foot_out = 0.02;
  if (top_drop) *top_drop = 0.04;
  if (top_out) *top_out = 0.012;
  return 1;
}

// cameraAt (src/timeline.js:80-101): position, target, vertical field of view (degrees).
int fire_timeline_camera_at(double t, double* pos3, double* target3, double* fov) {
  const Shot& s = shot_at(t);
  double u = std::min(std::max((t - s.t0) / (s.t1 - s.t0), 0.0), 1.0);
  u = u + (u * u * (3 - 2 * u) - u) * 0.3;
  double pos[3], tgt[3];
  for (int i = 0; i < 3; ++i) { pos[i] = lerp(s.a.pos[i], s.b.pos[i], u); tgt[i] = lerp(s.a.target[i], s.b.target[i], u); }
  const double f = lerp(s.a.fov, s.b.fov, u);
  auto n = [t](double fr, double ph) {
    return std::sin(t * fr + ph) * 0.5 + std::sin(t * fr * 2.13 + ph * 1.7) * 0.3 + std::sin(t * fr * 4.7 + ph * 0.3) * 0.2;
  };
  const double d = std::hypot(std::hypot(pos[0] - tgt[0], pos[1] - tgt[1]), pos[2] - tgt[2]);
  const double jit[3] = {n(1.1, 0.3) * 0.0022, n(0.9, 2.1) * 0.0022, n(1.3, 4.2) * 0.0022};
  const double aim[3] = {n(0.7, 1.7) * 0.0028 * d, n(0.8, 3.3) * 0.0028 * d, n(0.6, 5.1) * 0.0028 * d};
  const Event* lb = find_type(FIRE_EVENT_LOG_SHIFT);
  const double bump = (lb && t >= lb->t && t < lb->t + 0.2) ? 0.003 * std::exp(-(t - lb->t) / 0.05) : 0.0;
  for (int i = 0; i < 3; ++i) {
    if (pos3) pos3[i] = pos[i] + jit[i] + (i == 1 ? -bump : 0.0);
    if (target3) target3[i] = tgt[i] + aim[i] + (i == 1 ? -bump * 0.5 : 0.0);
  }
  if (fov) *fov = f;
  return FIRE_OK;
}

// lensAt (src/timeline.js:104-110) and exposureAt (src/timeline.js:132-134).
int fire_timeline_lens_at(double t, double* focus, double* aperture, double* fmm, double* fnum) {
  double pos[3], tgt[3], fov;
  fire_timeline_camera_at(t, pos, tgt, &fov);
  const double N = shot_at(t).N;
  const double f = 18.0 / std::tan((fov * kPI / 180.0) / 2.0);
  if (focus) *focus = std::hypot(std::hypot(tgt[0] - pos[0], tgt[1] - pos[1]), tgt[2] - pos[2]);
  if (aperture) *aperture = f / (2.0 * N) / 1000.0;
  if (fmm) *fmm = f;
  if (fnum) *fnum = N;
  return FIRE_OK;
}
double fire_timeline_exposure_at(double t) { return std::pow(2.0, shot_at(t).ev); }

int fire_timeline_create(const float* base_logs, int n_logs, int steps_per_frame, FireTimeline** out) {
  if (!out || n_logs < 0 || n_logs > 16 || (n_logs > 0 && !base_logs) || steps_per_frame < 1) return FIRE_ERR_BAD_ARG;
  FireTimeline* tl = new FireTimeline();
  tl->baseLogs.assign(base_logs ? base_logs : nullptr, base_logs ? base_logs + 8 * n_logs : nullptr);
  tl->nLogs = n_logs;
  tl->n = steps_per_frame;
  *out = tl;
  return FIRE_OK;
}
int fire_timeline_destroy(FireTimeline* tl) {
  if (!tl) return FIRE_ERR_BAD_ARG;
  delete tl;
  return FIRE_OK;
}
double fire_timeline_step_dt(FireTimeline* tl) { return tl ? 1.0 / (kFPS * tl->n) : 0.0; }
double fire_timeline_step_time(FireTimeline* tl, long long j) { return tl ? (double)j / (kFPS * tl->n) : 0.0; }
double fire_timeline_preroll(void) { return kPreroll; }

// applyLogs (src/main.js:131-150): the log-shift offsets applied to the base logs, uploaded when changed.
static int apply_logs(FireTimeline* tl, FireSim* sim, double t) {
  int idx = 0;
  double s = 0, footOut = 0, topDrop = 0, topOut = 0;
  const bool on = fire_timeline_log_offsets_at(t, &idx, &s, &footOut, &topDrop, &topOut) != 0;
  char key[64] = "";
  if (on) std::snprintf(key, sizeof key, "%d:%.3f", idx, s);
  if (tl->logKey == key) return FIRE_OK;
  tl->logKey = key;
  std::vector<float> arr = tl->baseLogs;
  if (on && idx < tl->nLogs) {
    const int i = idx * 8;
    const double ox = arr[i], oz = arr[i + 2];
    double l = std::hypot(ox, oz);
    if (l == 0.0) l = 1.0;
    const double dx = ox / l, dz = oz / l;
    arr[i] = (float)(arr[i] + dx * footOut * s);
    arr[i + 2] = (float)(arr[i + 2] + dz * footOut * s);
    arr[i + 1] = (float)(arr[i + 1] - 0.004 * s);
    arr[i + 4] = (float)(arr[i + 4] + dx * topOut * s);
    arr[i + 6] = (float)(arr[i + 6] + dz * topOut * s);
    arr[i + 5] = (float)(arr[i + 5] - topDrop * s);
  }
  return fire_sim_upload_logs(sim, arr.empty() ? nullptr : arr.data(), tl->nLogs);
}

// fireEvent (src/main.js:80-87): spark bursts for an event.
static int fire_event(FireSparks* sp, const FireTimelineEvent& e) {
  if (!sp) return FIRE_OK;
  const double s = e.strength;
  const float pos[3] = {(float)e.pos[0], (float)e.pos[1], (float)e.pos[2]};
  const float aim[3] = {(float)e.aim[0], (float)e.aim[1], (float)e.aim[2]};
  auto rnd = [](double x) { return (int)std::floor(x + 0.5); };   // Math.round
  switch (e.type) {
    case FIRE_EVENT_IGNITE: return fire_sparks_burst(sp, 140, pos, 3.2f, 0.12f, 0.5f, 0.6f, 1.3f, nullptr);
    case FIRE_EVENT_POP:
      if (s >= 0.8)
        return fire_sparks_burst(sp, rnd(110 * s), pos, (float)(3.5 + 2.5 * s), 0.03f, 0.05f, 0.9f, 1.4f, e.has_aim ? aim : nullptr);
      return fire_sparks_burst(sp, rnd(3 + 12 * s), pos, (float)(3 + 3 * s), 0.02f, 0.04f, 0.8f, 1.4f, nullptr);
    case FIRE_EVENT_LOG_SHIFT: return fire_sparks_burst(sp, rnd(190 * s), pos, 4.5f, 0.12f, 0.15f, 0.7f, 1.5f, nullptr);
    case FIRE_EVENT_CRACKLE_BURST: return fire_sparks_burst(sp, rnd(12 * s), pos, 3.0f, 0.08f, 0.3f, 0.6f, 1.3f, nullptr);
    default: return FIRE_OK;
  }
}

// capStep(j) (src/main.js:153-160): parameters and log offsets at t = j / (FPS n), the events in
// [t, t_next), then one simulation step and one spark step (simStep, src/main.js:70-76) of 1 / (FPS n).
int fire_timeline_step(FireTimeline* tl, FireSim* sim, FireSparks* sparks, long long j, void* stream) {
  FIRE_RANGE("fire_timeline_step");
  if (!tl || !sim) return FIRE_ERR_BAD_ARG;
  const double t = fire_timeline_step_time(tl, j), tNext = fire_timeline_step_time(tl, j + 1);
  double p[7];
  fire_timeline_sim_at(t, p);
  static const char* const names[7] = {"intensity", "burstAmt", "burstX", "burstY", "burstZ", "windX", "windZ"};
  float vals[7];
  for (int i = 0; i < 7; ++i) vals[i] = (float)p[i];
  int rc = fire_sim_set_params(sim, names, vals, 7);
  if (rc) return rc;
  if ((rc = apply_logs(tl, sim, t))) return rc;
  const std::vector<Event>& E = events();
  for (size_t i = 0; i < E.size(); ++i) {
    if (E[i].t >= t && E[i].t < tNext) {
      FireTimelineEvent e = {};
      e.t = E[i].t; e.type = E[i].type; e.strength = E[i].strength;
      for (int k = 0; k < 3; ++k) { e.pos[k] = E[i].pos[k]; e.aim[k] = E[i].aim[k]; }
      e.has_aim = E[i].hasAim ? 1 : 0;
      e.log = E[i].log;
      e.dur = E[i].dur;
      if ((rc = fire_event(sparks, e))) return rc;
    }
  }
  const float dt = (float)fire_timeline_step_dt(tl);
  if ((rc = fire_sim_step(sim, dt, 1, stream))) return rc;
  if (sparks) {
    float intensity = 1.0f;
    fire_sim_get_param(sim, "intensity", &intensity);
    // sparks.rate = 1.0 * intensity; the other spark parameters keep their values
    if ((rc = fire_sparks_set_rate(sparks, intensity))) return rc;
    if ((rc = fire_sparks_step(sparks, dt, stream))) return rc;
  }
  return FIRE_OK;
}

}  // extern "C"
