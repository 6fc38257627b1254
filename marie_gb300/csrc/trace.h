// Host-side NVTX ranges around the phases of the J-VIE path: operator
// assembly, each solve entry point, each restart cycle of the batched GMRES
// and each refinement step of the mixed-precision solve.  The reference times
// the same phases with tic/toc (assembly_nop.m:33-142, JVIE_Solver.m:321-335);
// here a profiler that records NVTX (Nsight Systems, ncu --nvtx) shows them on
// the timeline.  Without a profiler attached a range costs a test of a
// function pointer; ranges are host calls, so they are legal inside stream
// capture and put nothing into a CUDA graph.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace marie {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace marie

#define MARIE_TRACE_CAT2(a, b) a##b
#define MARIE_TRACE_CAT(a, b) MARIE_TRACE_CAT2(a, b)
#define MARIE_TRACE(name) ::marie::TraceRange MARIE_TRACE_CAT(marie_trace_range_, __LINE__)(name)
