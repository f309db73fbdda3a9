// nvtx.h -- named ranges on the host thread around the solver's dispatch
// steps (node upload, relaxation launch, result download, completion, the
// device frontier's graph replays), for timeline profilers. NVTX v3 from the
// CUDA toolkit is header-only and costs a branch per range unless a profiler
// is attached. Define GBX_NO_NVTX to compile the ranges out.
#pragma once

#if !defined(GBX_NO_NVTX) && defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define GBX_HAVE_NVTX 1
#endif
#endif

namespace gpuboscia {
namespace detail {

// One range for the lifetime of the object (push at construction, pop at
// destruction), so early returns and exceptions close it.
class NvtxRange {
public:
    explicit NvtxRange(const char* name) {
#ifdef GBX_HAVE_NVTX
        nvtxRangePushA(name);
#else
        (void)name;
#endif
    }
    ~NvtxRange() {
#ifdef GBX_HAVE_NVTX
        nvtxRangePop();
#endif
    }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace detail
}  // namespace gpuboscia
