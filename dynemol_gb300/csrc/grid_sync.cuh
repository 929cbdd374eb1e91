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

// Barrier over all CTAs of a cooperative launch on a count that only grows:
// `count` is two 32-bit words read as one 64-bit count (8-byte aligned, zero
// at the launch).  Thread 0 arrives for its CTA by a release add, which
// returns the arrivals before it: all nblocks arrivals of one barrier lie in
// [nblocks e, nblocks (e + 1)), so the CTA polls (relaxed loads, then one
// acquire fence) until the count reaches nblocks (e + 1).  The last arrival
// itself releases the others (no reset, no generation word).  Returns false
// (and sets *err = ELHL_ERR_TIMEOUT) if the other CTAs do not arrive within limit_ns
// (kBarrierNs unless the launch sets a shorter limit), so a stuck launch ends
// with an error instead of hanging.
__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned nblocks, int *err,
                                             unsigned long long limit_ns = kBarrierNs) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long *c = reinterpret_cast<unsigned long long *>(count);
        unsigned long long prev;
        asm volatile("atom.add.release.gpu.global.u64 %0, [%1], 1;" : "=l"(prev) : "l"(c) : "memory");
        const unsigned long long target = (prev / nblocks + 1) * nblocks;
        const unsigned long long t0 = globaltimer_ns();
        while (true) {
            unsigned long long v;
            asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(c) : "memory");
            if (v >= target) break;
            if (globaltimer_ns() - t0 > limit_ns) {
                atomicExch(err, ELHL_ERR_TIMEOUT);
                break;
            }
            __nanosleep(40);
        }
        __threadfence();  // acquire: the other CTAs' writes before their arrivals
    }
    __syncthreads();
    return *(volatile int *)err == 0;
}

}  // namespace elhl
