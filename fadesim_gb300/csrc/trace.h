// Host-timeline ranges (NVTX v3, header-only) around the library's entry
// points, so that a profiler's timeline or an ncu --nvtx filter can pick out
// one call.  Without an attached tool the calls return at once.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace fadesim {

struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace fadesim
