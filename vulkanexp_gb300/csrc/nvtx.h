// nvtx.h — NVTX ranges around the public entry points, so a profiler can
// filter and label the launches of one call (ncu --nvtx --nvtx-include
// "ddgi_update/"); header-only NVTX 3, inert without a profiler attached.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace ddgi {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace ddgi
