// NVTX ranges around the C ABI's entry points, so a profiler (ncu --nvtx,
// Nsight Systems) shows which library call enqueued which kernels.  NVTX v3
// is header-only: without an attached tool a range costs a null-pointer
// check.  Where the toolkit has no NVTX headers the ranges compile away.
#pragma once

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define PDQ_HAVE_NVTX 1
#endif
#endif

namespace pdq {

// Pushes a named range for the lifetime of the object (one per entry-point call).
struct NvtxRange {
#if defined(PDQ_HAVE_NVTX)
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
#else
  explicit NvtxRange(const char*) {}
#endif
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace pdq
