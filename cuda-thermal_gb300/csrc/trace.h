// trace.h - NVTX ranges around the host-side phases (solver and batch
// set-up, set_dt, solves), so a timeline tool (Nsight Systems) shows them
// beside the kernels. Header-only NVTX 3: without a tool attached each range
// costs a function call and nothing else.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace ct {

struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace ct
