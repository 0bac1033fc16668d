// Persistent form of the device-controlled loop (FP64 and double-float): one
// cooperative launch runs up to k stepper iterations, each the geometry of
// the three stage points, phases A, B and C (src/Nmr.cpp:153-249), the phases
// separated by grid-wide barriers instead of kernel boundaries.  Small grids
// (the config-0 shape: 1,024 beams) spend most of a three-launch iteration in
// launch gaps, prologues and reduction tails; here every block stays resident
// and goes on to the next phase as soon as the barrier opens.
//
// Every barrier wait is bounded (grid_barrier, xf_persist.cuh): the limit is
// 2 s by default, set by the "barrier_timeout_ms" option; the flag and the
// arrival counter live in the control block.  The "debug_barrier_extra"
// option makes each barrier wait for arrivals that never come, which is how
// the tests exercise the limit.
#include <cuda_runtime.h>

#include "xf_df.cuh"
#include "xf_fp64.cuh"
#include "xf_mixed.h"
#include "xf_persist.cuh"

namespace xf {
namespace {

using namespace detail;

template <int PREC, int GEOM>
__global__ void __launch_bounds__(256, 2) k_persist(Dev d, int iters, unsigned extra, unsigned long long limit_ns)
{
    Ctl* ctl = d.ctl;
    unsigned gen = 0;
    const int w0 = blockIdx.x * (blockDim.x >> 5), ws = gridDim.x * (blockDim.x >> 5);
    const auto at = [&](int i, int& ang) {
        ang = i;
        return &d;
    };
    unsigned* bar = &ctl->bar;
    int* tmo = &ctl->bar_timeout;
    for (int i = 0; i < iters; ++i) {
        geometry_pass(d.A, at);
        if (!grid_barrier(bar, tmo, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseA_body<GEOM>(d, w0, ws, grid_target(d, PH_A));
        else fp64::phaseA_body<GEOM>(d, w0, ws, grid_target(d, PH_A));
        if (!grid_barrier(bar, tmo, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseB_body<GEOM>(d, w0, ws, grid_target(d, PH_B));
        else fp64::phaseB_body<GEOM>(d, w0, ws, grid_target(d, PH_B));
        if (!grid_barrier(bar, tmo, gen, extra, limit_ns)) return;
        if (PREC == XF_PREC_DF) dfp::phaseC_body<GEOM>(d, w0, ws, grid_target(d, PH_C));
        else fp64::phaseC_body<GEOM>(d, w0, ws, grid_target(d, PH_C));
        if (!grid_barrier(bar, tmo, gen, extra, limit_ns)) return;
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
