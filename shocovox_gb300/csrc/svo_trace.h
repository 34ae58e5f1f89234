// svo_trace.h -- NVTX ranges around the library's phases (upload, sync, cast enqueue, batched cast,
// server admission / launch / retirement), so that a profiler's timeline shows them beside the
// kernels.  NVTX v3 is header-only: without a tool attached a range costs one branch.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace svo {

// One NVTX range for the lifetime of the object.
class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace svo
