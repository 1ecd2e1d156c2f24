// xct_check.cuh -- the bounds-checked build of the library (-DXCT_CHECKED, libxct_checked.so).
//
// Several kernels form shared-memory addresses from geometry -- a sample's floor bits, a
// window origin bounded by the tile corners -- instead of testing an index against a size,
// because the geometry proves the bound.  The checked build tests each such access against
// its buffer anyway: an access outside is skipped and the first one per translation unit is
// recorded in that unit's check word (site, index, bounds), which xct_check_report reads.
// In the standard build the checks compile to nothing.
#pragma once
#include <cuda_runtime.h>

#include "xct_internal.h"

#ifdef XCT_CHECKED
static __device__ XctCheckWord g_xct_check;

static __device__ __noinline__ void xct_check_fail(int site, long long v, long long lo, long long hi)
{
    if (atomicAdd(&g_xct_check.count, 1ull) == 0ull) {
        g_xct_check.site = site;
        g_xct_check.value = v;
        g_xct_check.lo = lo;
        g_xct_check.hi = hi;
    }
}

// true when lo <= v <= hi; otherwise records the event and yields false (skip the access)
#define XCT_IN(v, lo, hi, site)                                                                            \
    ((((long long)(v)) >= ((long long)(lo)) && ((long long)(v)) <= ((long long)(hi)))                     \
         ? true                                                                                             \
         : (xct_check_fail((site), (long long)(v), (long long)(lo), (long long)(hi)), false))

// Host reader of this translation unit's check word (one per .cu file that includes this).
#define XCT_CHECK_READER(name)                                                                             \
    int name(XctCheckWord *out, bool reset)                                                                \
    {                                                                                                      \
        if (cudaMemcpyFromSymbol(out, g_xct_check, sizeof(XctCheckWord)) != cudaSuccess) return -1;       \
        if (reset) {                                                                                       \
            const XctCheckWord z = {};                                                                     \
            if (cudaMemcpyToSymbol(g_xct_check, &z, sizeof z) != cudaSuccess) return -1;                   \
        }                                                                                                  \
        return 0;                                                                                          \
    }
#else
#define XCT_IN(v, lo, hi, site) true
#define XCT_CHECK_READER(name)
#endif
