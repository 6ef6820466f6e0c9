// NVTX ranges of the C entry points.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace gb {

// An NVTX range around every entry point, named after it (the reference annotates
// the same hooks with NVTX.@annotate: remaining_tendency.jl:15,48,
// implicit_tendency.jl:36, jacobian.jl:74,78, constrain_state.jl:59).  Without a
// profiler attached a push or pop is one test of a function pointer.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace gb

#define GB_RANGE() ::gb::NvtxRange gb_nvtx_range_(__func__)
