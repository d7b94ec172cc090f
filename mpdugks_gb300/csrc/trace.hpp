// NVTX ranges around the library's host-side phases: a step call, a reduction,
// a download, a checkpoint, a serving chunk, a FlowField write.  NVTX 3 is
// header-only; the calls do nothing unless a profiler (Nsight Systems) has
// injected itself into the process.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace dugks {

struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace dugks
