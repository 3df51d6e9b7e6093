// grid_sync.cuh -- bounded grid barrier for the cooperative FP64 sweeps
// (k_pgs_fast, k_gs_levels).
//
// Arrivals count up monotonically in DCount::bar_count (zeroed before each
// launch); a block leaves once the count reaches its own target, so the last
// block to arrive needs no second round trip to release the others.  Every
// wait is bounded: on expiry the block records AM_E_TIMEOUT and every block
// leaves at its next barrier check.  All blocks pass the same sequence of
// barriers (their control flow depends only on values read after a barrier),
// so the targets agree.
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
        long long spins = 0;
        while ((int)(seen - target) < 0) {
            if (++spins > (1ll << 24)) { atomicExch(&dc->error, AM_E_TIMEOUT); break; }
            __nanosleep(20);
            seen = *(volatile unsigned*)ctr;
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&dc->error == 0;
}

}  // namespace am
