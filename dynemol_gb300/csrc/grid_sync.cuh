// Bounded grid-wide barrier for cooperative persistent kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/elhl_prop.h"

namespace elhl {

constexpr unsigned long long kBarrierNs = 5000000000ULL;  // give up after 5 s

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Sense-reversing barrier over all CTAs of a cooperative launch.  Returns
// false (and sets *err = ELHL_ERR_TIMEOUT) if the other CTAs do not arrive
// within limit_ns (kBarrierNs unless the launch sets a shorter limit), so a
// stuck launch ends with an error instead of hanging.
__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned *gen, unsigned nblocks, int *err,
                                             unsigned long long limit_ns = kBarrierNs) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned prev = atomicAdd(count, 1u);
        if (prev == nblocks - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const unsigned long long t0 = globaltimer_ns();
            while (*vgen == g) {
                if (globaltimer_ns() - t0 > limit_ns) {
                    atomicExch(err, ELHL_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(40);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int *)err == 0;
}

}  // namespace elhl
