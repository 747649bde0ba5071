// irr_trace.cuh -- NVTX ranges around the library's phases (set-up, steps,
// read-back, batch and MD calls), so that a profiler's timeline shows them;
// with no tool attached a range costs a null check.  The reference prints
// wall-clock phase times instead (irregular_runtime.cu:303,334-338,380).
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace irr {

class TraceRange {
public:
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace irr
