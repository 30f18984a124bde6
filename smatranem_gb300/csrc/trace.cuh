/*
 * Named ranges on the host timeline (NVTX) around the library's long-running
 * entry points: plan creation, runs, autotuning, the adjoint's forward and
 * backward passes, group runs, the port mode solver and the layer transfer.
 * NVTX3 is header-only: with no profiler attached a range costs a call into
 * an empty stub; nsys or ncu (--nvtx) show the ranges by these names.
 */
#ifndef SMATRAN_TRACE_CUH
#define SMATRAN_TRACE_CUH

#include <nvtx3/nvToolsExt.h>

namespace smat {

/* a range open for the lifetime of the object (scope) */
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

} // namespace smat

#endif
