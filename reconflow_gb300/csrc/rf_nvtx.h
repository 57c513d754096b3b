// NVTX ranges (header-only NVTX3, a no-op unless a profiler is attached):
// every public entry point's host work, and per level / warp while a
// schedule is enqueued.  In graph mode (the default) the per-level ranges
// are recorded once, when the schedule is captured, and every replay shows
// under the entry point's range; RF_USE_GRAPHS=0 runs the schedule eagerly,
// so each level's and warp's kernels sit inside their own range.
#pragma once

#include <cstdarg>
#include <cstdio>

#include <nvtx3/nvToolsExt.h>

namespace rf {

class NvtxRange {
public:
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    NvtxRange(const char* fmt, int a, int b = -1) {
        char buf[64];
        if (b < 0) std::snprintf(buf, sizeof buf, fmt, a);
        else std::snprintf(buf, sizeof buf, fmt, a, b);
        nvtxRangePushA(buf);
    }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace rf
