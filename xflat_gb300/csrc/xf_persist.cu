// Persistent form of the device-controlled loop (FP64 and double-float): one
// cooperative launch runs up to k stepper iterations, each the geometry of
// the three stage points, phases A, B and C (src/Nmr.cpp:153-249), the phases
// separated by grid-wide barriers instead of kernel boundaries.  Small grids
// (the config-0 shape: 1,024 beams) spend most of a three-launch iteration in
// launch gaps, prologues and reduction tails; here every block stays resident
// and goes on to the next phase as soon as the barrier opens.
//
// Every barrier wait is bounded: a block whose wait runs past the limit
// (default 2 s, set by the "barrier_timeout_ms" option) raises the control
// block's timeout flag and returns, and the blocks still waiting see the flag
// and return too, so the launch ends and the host reports XF_ETIMEOUT with
// the context intact.  A cooperative launch guarantees that every block is
// resident, so the waits end unless a block has stopped; the
// "debug_barrier_extra" option makes each barrier wait for arrivals that never
// come, which is how the tests exercise the limit.
#include <cuda_runtime.h>

#include "xf_df.cuh"
#include "xf_fp64.cuh"
#include "xf_mixed.h"

namespace xf {
namespace {

using namespace detail;

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

// Grid-wide barrier on the control block's arrival counter (reset to zero
// before each launch).  Returns false when this block's wait ran out or
// another block's did.
__device__ bool grid_barrier(Ctl* ctl, unsigned& gen, unsigned extra, unsigned long long limit_ns)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ++gen;
        const unsigned target = gen * (gridDim.x + extra);
        __threadfence();  // this block's writes before its arrival
        atomicAdd(&ctl->bar, 1u);
        const unsigned long long t0 = globaltimer_ns();
        int ok = 1;
        for (unsigned polls = 1;; ++polls) {
            if (ld_acquire(&ctl->bar) >= target) break;
            if (ld_relaxed(&ctl->bar_timeout)) {
                ok = 0;
                break;
            }
            if ((polls & 31) == 0 && globaltimer_ns() - t0 > limit_ns) {
                atomicExch(&ctl->bar_timeout, 1);
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

// The geometry of the three stage points, 64 angles x 3 points per block pass.
__device__ void geometry_all(const Dev& d)
{
    __shared__ double s_c[3 * 64];
    const int slot = threadIdx.x % 64, pt = threadIdx.x / 64;
    const int groups = (d.A + 63) / 64;
    for (int g = blockIdx.x; g < groups; g += gridDim.x) {
        const int ang = g * 64 + slot;
        geometry_point(d, (pt < 3 && ang < d.A) ? ang : -1, pt < 3 ? pt : 0, slot, 64, s_c);
        __syncthreads();  // s_c is rewritten by the next pass
    }
}

template <int PREC, int GEOM>
__global__ void __launch_bounds__(256, 2) k_persist(Dev d, int iters, unsigned extra, unsigned long long limit_ns)
{
    Ctl* ctl = d.ctl;
    unsigned gen = 0;
    const int w0 = blockIdx.x * (blockDim.x >> 5), ws = gridDim.x * (blockDim.x >> 5);
    for (int i = 0; i < iters; ++i) {
        geometry_all(d);
        if (!grid_barrier(ctl, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseA_body<GEOM>(d, w0, ws, grid_target(d, PH_A));
        else fp64::phaseA_body<GEOM>(d, w0, ws, grid_target(d, PH_A));
        if (!grid_barrier(ctl, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseB_body<GEOM>(d, w0, ws, grid_target(d, PH_B));
        else fp64::phaseB_body<GEOM>(d, w0, ws, grid_target(d, PH_B));
        if (!grid_barrier(ctl, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseC_body<GEOM>(d, w0, ws, grid_target(d, PH_C));
        else fp64::phaseC_body<GEOM>(d, w0, ws, grid_target(d, PH_C));
        if (!grid_barrier(ctl, gen, extra, limit_ns)) return;
        if (ld_relaxed(&ctl->done)) return;
    }
}

template <int PREC, int GEOM>
void* persist_fn()
{
    return reinterpret_cast<void*>(k_persist<PREC, GEOM>);
}

void* kernel_of(const Dev& d)
{
    if (d.df) return d.geom == 0 ? persist_fn<XF_PREC_DF, 0>() : persist_fn<XF_PREC_DF, 1>();
    return d.geom == 0 ? persist_fn<XF_PREC_FP64, 0>() : persist_fn<XF_PREC_FP64, 1>();
}

}  // namespace

// Blocks of the persistent kernel: every block resident (2 of 256 threads per
// SM at most), no more than the beams fill (one warp per beam).
int persist_blocks(const Dev& d)
{
    int dev = 0, sms = 152, occ = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_of(d), 256, 0) != cudaSuccess || occ < 1) return 0;
    const int need = (d.nbeams + 7) / 8;
    return std::max(1, std::min(need, occ * sms));
}

cudaError_t launch_persist(const Dev& d, int blocks, int iters, unsigned extra, unsigned long long limit_ns,
                           cudaStream_t st)
{
    Dev dd = d;
    void* args[] = {&dd, &iters, &extra, &limit_ns};
    return cudaLaunchCooperativeKernel(kernel_of(d), dim3(blocks), dim3(256), args, 0, st);
}

}  // namespace xf
