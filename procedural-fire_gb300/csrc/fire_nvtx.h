// NVTX ranges on the host entry points, in the "fire" domain.
//
// Each public call that queues GPU work opens a range named after itself for its whole duration, so a
// profiler's timeline shows which call launched which kernels, and `ncu --nvtx --nvtx-include
// "fire@fire_sim_run_stage/"` (for example) restricts a capture to one entry point.  Stage-level runs add
// a nested range named after the stage.  NVTX3 is header-only: without an attached tool every push and pop
// is one predictable branch on a null function pointer, so the ranges stay in the release build.
//
// The step itself is a CUDA graph, so ranges cannot name its kernels one by one; they name the
// graph launch, and the per-kernel split comes from fire_sim_profile's events.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace fire {

inline nvtxDomainHandle_t nvtx_domain() {
  static nvtxDomainHandle_t d = nvtxDomainCreateA("fire");
  return d;
}

class NvtxRange {
 public:
  explicit NvtxRange(const char* name) {
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = name;
    nvtxDomainRangePushEx(nvtx_domain(), &a);
  }
  ~NvtxRange() { nvtxDomainRangePop(nvtx_domain()); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace fire

#define FIRE_NVTX_CAT2(a, b) a##b
#define FIRE_NVTX_CAT(a, b) FIRE_NVTX_CAT2(a, b)
// Opens a range for the rest of the enclosing scope.
#define FIRE_RANGE(name) ::fire::NvtxRange FIRE_NVTX_CAT(fire_nvtx_range_, __LINE__)(name)
