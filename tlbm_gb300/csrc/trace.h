// trace.h -- NVTX ranges around the engine's host calls (create, run, step, outputs, ensemble
// steps), so a timeline profiler shows what each stretch of kernels belongs to.  NVTX v3 is
// header-only and a no-op unless a profiler is attached.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace tlbm {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace tlbm
