// NVTX ranges over the C ABI's entry points, so a profiler's timeline shows
// which call a kernel belongs to (for example `ncu --nvtx --nvtx-include
// "gx_run/"` captures only the superstep loop's kernels).  NVTX v3 is
// header-only; with no tool attached a range costs one branch.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace gx {

struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace gx
