// grid_sync.cuh -- bounded grid barrier for the cooperative sweeps
// (k_pgs_fast, k_gs_levels, and the grid form of k_pgs_mixed).
//
// Arrivals count up monotonically in DCount::bar_count (zeroed before each
// launch); a block leaves once the count reaches its own target, so the last
// block to arrive needs no second round trip to release the others.  Every
// wait is bounded: after 2^spin_log2 polls (DCount::spin_log2, 24 when 0) the
// block records AM_E_TIMEOUT and leaves; a block still waiting sees the error
// word at its next poll and leaves too, so one expiry ends every wait at once.
// All blocks pass the same sequence of barriers (their control flow depends
// only on values read after a barrier), so the targets agree.
#pragma once
#include "am_ctx.hpp"

namespace am {

__device__ __forceinline__ bool grid_barrier_counted(DCount* dc, int nblocks, unsigned& target) {
    if (nblocks == 1) {   // one block: the block barrier orders global memory too
        __syncthreads();
        return *(volatile int*)&dc->error == 0;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        target += (unsigned)nblocks;
        unsigned* ctr = (unsigned*)&dc->bar_count;
        unsigned seen = atomicAdd(ctr, 1u) + 1u;
        const int lg = *(volatile int*)&dc->spin_log2;
        const long long limit = 1ll << (lg > 0 && lg < 40 ? lg : 24);
        long long spins = 0;
        while ((int)(seen - target) < 0) {
            if (++spins > limit) { atomicExch(&dc->error, AM_E_TIMEOUT); break; }
            if (*(volatile int*)&dc->error) break;   // another block gave up
            __nanosleep(20);
            seen = *(volatile unsigned*)ctr;
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&dc->error == 0;
}

}  // namespace am
