// gx_debug.cuh -- device-side checks of the debug build.
//
// The library's kernels test every index that comes from a caller's array
// (queue orders, system ids, release offsets and counts) before they use it,
// and skip what is out of range.  Built with -DGX_DEBUG_CHECKS (the debug
// library, libgala_gb300_debug.so) each failed test is also recorded in a
// status record of its translation unit in device memory: the first failure's
// code, source line, index and bound, and the number of failures.  The
// persistent queues add every orbit they complete to a count, a sum and a sum
// of squares of (orbit id + 1) and a step total, from which the host checks
// that every orbit was integrated exactly once and took its steps.  Nothing
// traps and nothing waits; gx_debug_read returns the records summed over the
// translation units.  In the release build the checks are the plain range
// tests and no record exists.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gx {

enum DbgCode : uint32_t {
    DBG_ORDER = 1,   // an orbit id in a queue order outside [0, n) (and not the -1 padding)
    DBG_SYSTEM = 2,  // a system id outside the release grid
    DBG_OFFSET = 3,  // release offsets inconsistent with the particle array or the system size
    DBG_COUNT = 4,   // a release count that overruns the stream's particles
};

struct DbgRecord {
    unsigned long long first;  // code << 32 | source line of the first failure (0: none)
    long long index, bound;    // the first failure's index and bound
    unsigned long long fails;  // failed checks
    unsigned long long done, id_sum, id_sq, steps;  // orbits completed by the queues
};

// Host side: one reader per translation unit (registered at load time).
using DbgReader = int (*)(DbgRecord *out, bool reset);
void dbg_register(DbgReader r);

#ifdef GX_DEBUG_CHECKS

static __device__ DbgRecord g_dbg;

__device__ __forceinline__ bool dbg_check(bool ok, uint32_t code, long long index, long long bound, int line) {
    if (ok) return true;
    const unsigned long long tag = ((unsigned long long)code << 32) | (unsigned)line;
    if (atomicCAS(&g_dbg.first, 0ull, tag) == 0ull) {
        g_dbg.index = index;
        g_dbg.bound = bound;
    }
    atomicAdd(&g_dbg.fails, 1ull);
    return false;
}

__device__ __forceinline__ void dbg_done(long long id, long long steps) {
    const unsigned long long k = (unsigned long long)(id + 1);
    atomicAdd(&g_dbg.done, 1ull);
    atomicAdd(&g_dbg.id_sum, k);
    atomicAdd(&g_dbg.id_sq, k * k);
    atomicAdd(&g_dbg.steps, (unsigned long long)steps);
}

static int dbg_read_this_unit(DbgRecord *out, bool reset) {
    if (cudaMemcpyFromSymbol(out, g_dbg, sizeof(DbgRecord)) != cudaSuccess) return -1;
    if (reset) {
        const DbgRecord zero = {};
        if (cudaMemcpyToSymbol(g_dbg, &zero, sizeof(DbgRecord)) != cudaSuccess) return -1;
    }
    return 0;
}

namespace {
struct DbgRegistration {
    DbgRegistration() { dbg_register(&dbg_read_this_unit); }
};
static DbgRegistration g_dbg_registration;
}  // namespace

#define GX_DBG_CHECK(ok, code, index, bound) \
    ::gx::dbg_check((ok), (code), (long long)(index), (long long)(bound), __LINE__)
#define GX_DBG_DONE(id, steps) ::gx::dbg_done((long long)(id), (long long)(steps))

#else

#define GX_DBG_CHECK(ok, code, index, bound) (ok)
#define GX_DBG_DONE(id, steps) ((void)0)

#endif

}  // namespace gx
