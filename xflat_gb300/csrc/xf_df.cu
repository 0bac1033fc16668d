// Double-float path kernels (bodies in xf_df.cuh): one warp per beam, the
// grid one reduction group, launched with programmatic dependent launch.
#include "xf_df.cuh"
#include "xf_launch.cuh"
#include "xf_mixed.h"

namespace xf {
namespace {

using namespace detail;

__global__ void __launch_bounds__(256, 2) k_dfA(Dev d)
{
    pdl_enter();
    dfp::phaseA_body<0>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_A));
}

__global__ void __launch_bounds__(256, 2) k_dfB(Dev d)
{
    pdl_enter();
    dfp::phaseB_body<0>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_B));
}

__global__ void __launch_bounds__(256, 2) k_dfC(Dev d)
{
    pdl_enter();
    dfp::phaseC_body<0>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_C));
}

}  // namespace

void df_launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (phase == PH_A) launch_pdl(k_dfA, sh.blocks, sh.threads, st, d);
    else if (phase == PH_B) launch_pdl(k_dfB, sh.blocks, sh.threads, st, d);
    else launch_pdl(k_dfC, sh.blocks, sh.threads, st, d);
}

}  // namespace xf
