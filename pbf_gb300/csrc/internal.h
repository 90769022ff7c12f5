// internal.h — helpers shared between the translation units of the library.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace pbf {

// Sets the message pbf_last_error(NULL) returns (thread-local).
void set_last_error(const char* msg);

// NVTX range around a host-side scope: the entry points show up by name on a
// profiler's timeline (no cost when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace pbf
