// ref_host_select.cpp — the reference's probe selection,
// IrradianceProbes::selectProbesToUpdate (src/IrradianceProbes.cpp:396-424),
// compiled from its own source text: oracle/build_ref_glsl.py copies the
// function's definition out of the reference's file into
// oracle/_ref/src/selectProbesToUpdate.inc, and it compiles here as a member
// of a stand-in class that holds exactly the members it reads (the probe-
// state readback, the offset, the per-update cap, the list upload).  Test
// infrastructure: built into oracle/_ref/libref_glsl.so.
//
// The function keeps its loop index in a function-local static, as the
// reference does, so a process's calls form one sequence starting at 0.
#include <stdint.h>
#include <string.h>

#include <vector>

namespace refhost {

struct StateReadback {  // _probeInfoMemory: map() returns the states
    const void* data = nullptr;
    void* map(size_t) { return const_cast<void*>(data); }
    void unmap() {}
};
struct ListUpload {  // _probesToUpdateMemory: fill() receives the list
    std::vector<uint32_t> values;
    void fill(const uint32_t* p, size_t n) { values.assign(p, p + n); }
};

class IrradianceProbes {
  public:
    struct ProbeInfo {
        uint32_t state;
    };
    uint32_t ProbesPerUpdate = 0;
    uint32_t probe_count = 0;
    uint32_t getProbeCount() const { return probe_count; }
    uint32_t selectProbesToUpdate();

    StateReadback _probeInfoMemory;
    ListUpload _probesToUpdateMemory;
    std::vector<ProbeInfo> _probesState;
    uint32_t _lastUpdateOffset = 0;
};

#include "selectProbesToUpdate.inc"

}  // namespace refhost

extern "C" {

// K successive selections on one object: call k reads states[k n ...] with
// the cap caps[k] (0 = no cap) and writes its list to lists[k n ...], its
// length to counts[k] and the offset it leaves to offsets[k].
void ref_select_sequence(const uint32_t* states, uint32_t n, uint32_t K, const uint32_t* caps, uint32_t* lists,
                         uint32_t* counts, uint32_t* offsets) {
    refhost::IrradianceProbes p;
    p.probe_count = n;
    for (uint32_t k = 0; k < K; ++k) {
        p._probeInfoMemory.data = states + (size_t)k * n;
        p.ProbesPerUpdate = caps[k];
        p._probesToUpdateMemory.values.clear();
        const uint32_t c = p.selectProbesToUpdate();
        counts[k] = c;
        offsets[k] = p._lastUpdateOffset;
        memset(lists + (size_t)k * n, 0xFF, n * sizeof(uint32_t));
        if (c) memcpy(lists + (size_t)k * n, p._probesToUpdateMemory.values.data(), c * sizeof(uint32_t));
    }
}

}  // extern "C"
