// trace.hh — optional host-side phase timing of the registration drivers,
// and NVTX ranges.
// Phase timing is enabled by the environment variable MGR_TRACE=1; each
// scope then waits for its stream at exit and adds its wall-clock time to a
// named phase.  trace_report() prints the phases to stderr and clears them.
// Every scope is also an NVTX range of the same name (and NvtxRange marks
// the entry points and kernel launches), which a profiler such as Nsight
// Systems shows on its timeline; without a profiler attached the NVTX calls
// do nothing.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <chrono>

namespace mgr {

bool trace_enabled();
void trace_add(const char *phase, double ms);
// a counted quantity (reported like a phase, in its own unit)
void trace_count(const char *name, double value);
void trace_report(const char *title);

struct TraceScope {
    const char *name;
    cudaStream_t st;
    bool on;
    std::chrono::steady_clock::time_point t0;
    bool ranged = true;
    TraceScope(const char *n, cudaStream_t s) : name(n), st(s), on(trace_enabled())
    {
        nvtxRangePushA(n);
        if (on) {
            cudaStreamSynchronize(st);
            t0 = std::chrono::steady_clock::now();
        }
    }
    TraceScope(const TraceScope &) = delete;
    TraceScope &operator=(const TraceScope &) = delete;
    // record the phase now (the destructor then records nothing)
    void stop()
    {
        if (on) {
            cudaStreamSynchronize(st);
            trace_add(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
            on = false;
        }
        if (ranged) {
            nvtxRangePop();
            ranged = false;
        }
    }
    ~TraceScope() { stop(); }
};

// an NVTX range over a scope (entry points, kernel launches)
struct NvtxRange {
    explicit NvtxRange(const char *n) { nvtxRangePushA(n); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
    ~NvtxRange() { nvtxRangePop(); }
};

}  // namespace mgr
