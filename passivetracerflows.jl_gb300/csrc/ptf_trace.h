// NVTX ranges around the library's entry points, so a profiler's timeline
// (ncu's --nvtx filters, nsys) shows which API call issued which kernels.
// NVTX v3 is header-only: with no tool attached each range is a call through
// a no-op function pointer.  Without the NVTX headers the ranges compile away.
#pragma once

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define PTF_HAVE_NVTX 1
#endif
#endif

namespace ptf {

struct TraceRange {
  explicit TraceRange(const char* name) {
#ifdef PTF_HAVE_NVTX
    nvtxRangePushA(name);
#else
    (void)name;
#endif
  }
  ~TraceRange() {
#ifdef PTF_HAVE_NVTX
    nvtxRangePop();
#endif
  }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace ptf
