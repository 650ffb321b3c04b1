// Pressure V-cycles on caller-owned arrays with no device allocation.
//
// Some callers cannot call cudaMalloc when they need a pressure solve: a host whose device memory is owned
// by another allocator (a caching or pooled allocator that must not be bypassed), a frame loop that has
// fixed its memory budget up front, or code that is recording work into a CUDA graph, where allocation is
// not permitted.  fire_poisson_vcycles_noalloc serves them: the caller passes the level-0 pressure and
// right-hand side; every coarser multigrid level lives in one file-scope device array of fixed size that
// the library holds on every GPU that loads it, until the process exits.
//
// The V-cycle is the step's own (same kernels, same level rules, same coarse sweep count) with the
// reference's Gauss-Seidel sweeps (omega 1), so the result equals the V-cycle fire_sim_step runs on the same
// arrays with its default smoother, bit for bit.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>
#include <algorithm>
#include "../../include/fire_sim.h"
#include "fire_internal.h"
#include "fire_nvtx.h"

namespace fire {

// 8 MiB of scratch: the coarse levels (p and b) of a level-0 grid of up to ~7 million cells.
constexpr size_t NOALLOC_BYTES = (size_t)FIRE_NOALLOC_SCRATCH_BYTES;
constexpr size_t NOALLOC_FLAG_BYTES = 256;   // the tail kernel's wait-timeout flag lives at the end
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {
struct DeviceSetup {
  bool ready = false;
  unsigned char* base = nullptr;   // device address of g_noalloc_scratch on that device
};
std::mutex g_setup_mutex;
DeviceSetup g_setup[64];

// Once per device, with that device current: resolve the array's device address (in host code the
// symbol name is only a host-side stand-in) and opt the tail kernel into its shared memory.  No stream work
// is issued: a file-scope device array starts zeroed when the module loads, so the timeout flag starts clear.
int setup_device(int dev, unsigned char** base) {
  if (dev < 0 || dev >= 64) return FIRE_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || ptr == nullptr) return FIRE_ERR_CUDA;
    if (mg_configure(TAIL_SMEM_BUDGET) != cudaSuccess) return FIRE_ERR_CUDA;
    s.base = static_cast<unsigned char*>(ptr);
    s.ready = true;
  }
  *base = s.base;
  return FIRE_OK;
}
bool device_ready(int dev) {
  if (dev < 0 || dev >= 64) return false;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  return g_setup[dev].ready;
}
size_t align256(size_t v) { return (v + 255) / 256 * 256; }
}  // namespace
}  // namespace fire

using namespace fire;

extern "C" int fire_poisson_vcycles_noalloc(float* p, const float* b, int nx, int ny, int nz, float h, int cycles, void* stream) {
  FIRE_RANGE("fire_poisson_vcycles_noalloc");
  if (!p || !b || nx < 2 || ny < 2 || nz < 2 || !(h > 0.0f) || cycles < 0) return FIRE_ERR_BAD_ARG;
  // level hierarchy and coarse sweep count as the simulation builds them (src/sim.js:79-92)
  std::vector<MGLevel> levels;
  {
    int x = nx, y = ny, z = nz;
    double hh = h;
    while (true) {
      levels.push_back(MGLevel{x, y, z, (float)hh, nullptr, nullptr});
      if (x % 2 || y % 2 || z % 2 || std::min(x, std::min(y, z)) <= 6) break;
      x /= 2; y /= 2; z /= 2; hh *= 2;
    }
  }
  const int n = (int)levels.size();
  size_t need = 0;
  for (int l = 1; l < n; ++l) need += 2 * align256(sizeof(float) * (size_t)levels[l].nx * levels[l].ny * levels[l].nz);
  if (need > NOALLOC_BYTES - NOALLOC_FLAG_BYTES) return FIRE_ERR_BAD_ARG;   // beyond the fixed scratch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FIRE_ERR_CUDA;
  unsigned char* base = nullptr;
  int rc = setup_device(dev, &base);
  if (rc) return rc;

  levels[0].p = p;
  levels[0].b = const_cast<float*>(b);   // read only: smoothing and restriction read b, nothing writes it
  size_t off = 0;
  for (int l = 1; l < n; ++l) {
    const size_t bytes = align256(sizeof(float) * (size_t)levels[l].nx * levels[l].ny * levels[l].nz);
    levels[l].p = reinterpret_cast<float*>(base + off); off += bytes;
    levels[l].b = reinterpret_cast<float*>(base + off); off += bytes;
  }
  int* err = reinterpret_cast<int*>(base + NOALLOC_BYTES - NOALLOC_FLAG_BYTES);
  const MGLevel& C = levels.back();
  const double PI = 3.14159265358979323846;
  const double mu = (std::cos(PI / C.nx) + std::cos(PI / (2.0 * C.ny)) + std::cos(PI / C.nz)) / 3.0;
  const int coarse = (int)std::max(8.0, std::min(64.0, std::ceil(std::log(0.05) / std::log(mu * mu))));
  const int T = tail_first(levels.data(), n);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int top = std::min(T, n - 1);
  // every launch's own status is checked, so an error left by the caller's earlier work is neither blamed on
  // this call nor cleared by it
  bool ok = true;
  auto sweeps = [&](const MGLevel& L, int iters) {
    for (int k = 0; k < iters && ok; ++k) ok = launch_smooth(L, 0, st) == cudaSuccess && launch_smooth(L, 1, st) == cudaSuccess;
  };
  for (int c = 0; c < cycles && ok; ++c) {   // V(2,2) (src/sim.js:588-599), as the simulation records it
    for (int i = 0; i < top && ok; ++i) {
      sweeps(levels[i], 2);
      ok = ok && launch_restrict(levels[i], levels[i + 1], st) == cudaSuccess;
    }
    if (!ok) break;
    if (T < n) ok = launch_tail(levels.data(), T, n, 2, 2, coarse, err, st) == cudaSuccess;
    else sweeps(levels[n - 1], coarse);
    for (int i = top - 1; i >= 0 && ok; --i) {
      ok = launch_prolong(levels[i], levels[i + 1], st) == cudaSuccess;
      sweeps(levels[i], 2);
    }
  }
  return ok ? FIRE_OK : FIRE_ERR_CUDA;
}

// Waits for `stream`, then reports and clears the timeout flag that the coarse-level kernel of the calls
// above sets when its bounded wait for its staging copies runs out (it then skips that cycle's coarse
// correction).  Synchronous; allocates nothing.
extern "C" int fire_poisson_noalloc_status(void* stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FIRE_ERR_CUDA;
  if (!device_ready(dev)) return FIRE_OK;   // no call ran on this device
  if (cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)) != cudaSuccess) return FIRE_ERR_CUDA;
  int flag = 0;
  const size_t at = NOALLOC_BYTES - NOALLOC_FLAG_BYTES;
  if (cudaMemcpyFromSymbol(&flag, g_noalloc_scratch, sizeof flag, at) != cudaSuccess) return FIRE_ERR_CUDA;
  if (!flag) return FIRE_OK;
  const int zero = 0;
  if (cudaMemcpyToSymbol(g_noalloc_scratch, &zero, sizeof zero, at) != cudaSuccess) return FIRE_ERR_CUDA;
  return FIRE_ERR_CUDA;
}
