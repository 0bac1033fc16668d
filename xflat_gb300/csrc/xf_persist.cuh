// Grid-wide barrier with a bounded wait, and the stage-point geometry as a
// pass of a persistent kernel (xf_persist.cu, xf_batch.cu).
//
// Every wait is bounded: a block whose wait runs past the limit raises the
// timeout flag and returns false, and the blocks still waiting see the flag
// and return false too, so the launch ends and the host reports XF_ETIMEOUT
// with the context intact.  The kernels that use it are launched
// cooperatively (every block resident), so a wait ends unless a block has
// stopped.
#pragma once
#include "xf_common.cuh"

namespace xf {
namespace detail {

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed(const int* p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Barrier on an arrival counter that is zero when the launch starts: the
// gen-th barrier of the launch opens when gen * (gridDim.x + extra) blocks
// have arrived (extra > 0 only in the tests, for arrivals that never come).
// Returns false when this block's wait ran out or another block's did.
__device__ inline bool grid_barrier(unsigned int* count, int* timeout, unsigned& gen, unsigned extra,
                                    unsigned long long limit_ns)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ++gen;
        const unsigned target = gen * (gridDim.x + extra);
        __threadfence();  // this block's writes before its arrival
        atomicAdd(count, 1u);
        const unsigned long long t0 = globaltimer_ns();
        int ok = 1;
        for (unsigned polls = 1;; ++polls) {
            if (ld_acquire(count) >= target) break;
            if (ld_relaxed(timeout)) {
                ok = 0;
                break;
            }
            if ((polls & 31) == 0 && globaltimer_ns() - t0 > limit_ns) {
                atomicExch(timeout, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();  // the other blocks' writes before this block's next loads
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The geometry of the three stage points for `n` angles, 64 angles x 3 points
// per block pass; angle i is (instance, angle) = at(i).
template <typename At>
__device__ inline void geometry_pass(int n, At at)
{
    __shared__ double s_c[3 * 64];
    const int slot = threadIdx.x % 64, pt = threadIdx.x / 64;
    const int groups = (n + 63) / 64;
    for (int g = blockIdx.x; g < groups; g += gridDim.x) {
        const int i = g * 64 + slot;
        const bool live = pt < 3 && i < n;
        int ang = -1;
        const Dev* d = at(live ? i : 0, ang);
        geometry_point(*d, live ? ang : -1, pt < 3 ? pt : 0, slot, 64, s_c);
        __syncthreads();  // s_c is rewritten by the next pass
    }
}

}  // namespace detail
}  // namespace xf
