// gx_queue.cuh -- the work queue of the batched integrators (gx_batch.cu,
// gx_fixed.cu).
//
// The caller's order holds chunks of orbits sorted longest first, each chunk
// `chunk` orbits of one integrator (a multiple of 32: `subs` = chunk / 32
// blocks of 32, one orbit per lane).  A persistent grid pulls work from
// counters in the caller's scratch (GX_BATCH_QUEUE_WORDS int32, zeroed by the
// launch):
//   queue[0]       claims of the main region, whole chunks [n_lead, n_chunks)
//   queue[1]       claims of the lead region, the 32-orbit blocks of chunks
//                  [0, n_lead), n_lead = min(n_chunks, 4 x multiprocessors / subs)
//   queue[2 + s]   one flag per SM sub-partition s = 4 * smid + (warp slot & 3)
// The first warp that reaches a sub-partition's flag takes a lead block (one of
// the longest, at most one per sub-partition); every other warp starts in the
// main region.  The run time of a batch of uneven orbits is that of its
// longest orbits, whose dependent chains leave most issue slots of their
// sub-partition free: two of them on one sub-partition run at about half
// speed, while a lead warp next to warps with shorter work loses little.
// Placement is a hint (the warp slot register is the scheduler's current slot);
// every block is still taken exactly once: lead blocks that no lead warp took
// are taken after the main region runs dry.  Both regions hand out their work
// in order, so what a run took is the first min(queue[1], n_lead * subs) lead
// blocks and the first min(queue[0], n_chunks - n_lead) main chunks, also
// after a cancelled launch.
#pragma once

#include <cstdint>

#include "../../include/gala_gb300.h"

namespace gx {

constexpr int QUEUE_SLOTS = GX_BATCH_QUEUE_WORDS - 2;

__device__ __forceinline__ unsigned smsp_slot() {
    unsigned sm, w;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(w));
    return sm * 4u + (w & 3u);
}

// The next work item for this warp (called by one lane): chunk c and block
// `sub` >= 0 of it (a lead block), or chunk c whole (sub = -1); c = -1 when
// nothing is left.  `phase` starts at 0 and is kept by the caller.
__device__ __forceinline__ int64_t queue_next(int32_t *queue, int64_t n_chunks, int64_t n_lead, int subs, int &phase,
                                              int &sub) {
    const int64_t n_lead_blocks = n_lead * subs;
    sub = -1;
    if (phase == 0) {
        phase = 1;
        const unsigned s = smsp_slot();
        if (s < (unsigned)QUEUE_SLOTS && atomicCAS(&queue[2 + s], 0, 1) == 0) {
            const int l = atomicAdd(&queue[1], 1);
            if (l < n_lead_blocks) {
                sub = l % subs;
                return l / subs;
            }
        }
    }
    if (phase == 1) {
        const int m = atomicAdd(&queue[0], 1);
        if (m < n_chunks - n_lead) return n_lead + m;
        phase = 2;
    }
    const int l = atomicAdd(&queue[1], 1);
    if (l < n_lead_blocks) {
        sub = l % subs;
        return l / subs;
    }
    return -1;
}

// Host: n_lead, the lead region's chunks on the current device.
int64_t queue_lead_chunks(int64_t n_chunks, int32_t chunk);

}  // namespace gx
