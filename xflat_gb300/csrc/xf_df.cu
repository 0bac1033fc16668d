// Double-float path kernels (bodies in xf_df.cuh): one warp per beam, the
// grid one reduction group, launched with programmatic dependent launch.
// The grid is one wave of resident blocks (every SM holds the same number of
// blocks for the whole kernel, the warps striding over the beams), which
// avoids the partly filled last wave of a one-block-per-8-beams grid.
#include "xf_df.cuh"
#include "xf_launch.cuh"
#include "xf_mixed.h"

namespace xf {
namespace {

using namespace detail;

// 3 resident blocks of 256 threads per SM (at most 85 registers per thread,
// no spills); phase B, which holds two propagators' constants, also in a form
// with 2 (128 registers), 7 % slower on GB300
constexpr int kDfMinBlocks = 3;

template <int GEOM>
__global__ void __launch_bounds__(256, kDfMinBlocks) k_dfA(Dev d)
{
    pdl_enter();
    dfp::phaseA_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_A));
}

template <int GEOM, int OCC>
__global__ void __launch_bounds__(256, OCC) k_dfB(Dev d)
{
    pdl_enter();
    dfp::phaseB_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_B));
}

template <int GEOM>
__global__ void __launch_bounds__(256, kDfMinBlocks) k_dfC(Dev d)
{
    pdl_enter();
    dfp::phaseC_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_C));
}

template <int GEOM>
void launch_geom(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    const int blocks = sh.phase_blocks[phase] > 0 ? sh.phase_blocks[phase] : sh.blocks;
    if (phase == PH_A) launch_pdl(k_dfA<GEOM>, blocks, sh.threads, st, d);
    else if (phase == PH_B && sh.df_b_occ == 2) launch_pdl(k_dfB<GEOM, 2>, blocks, sh.threads, st, d);
    else if (phase == PH_B) launch_pdl(k_dfB<GEOM, 3>, blocks, sh.threads, st, d);
    else launch_pdl(k_dfC<GEOM>, blocks, sh.threads, st, d);
}

template <typename K>
int resident(K kernel, int threads, int fallback)
{
    int o = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, threads, 0) == cudaSuccess && o > 0 ? o : fallback;
}

}  // namespace

void df_launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (d.geom == 0) launch_geom<0>(phase, d, sh, st);
    else launch_geom<1>(phase, d, sh, st);
}

// One wave per phase kernel: the blocks of `threads` threads that can be
// resident per SM times the SM count, capped by the blocks the beams fill
// (one warp per beam).
void df_default_shape(int nbeams, Shape& sh)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int t = sh.threads;
    const int need = std::max(1, (nbeams + t / 32 - 1) / (t / 32));
    const int occ[3] = {resident(k_dfA<0>, t, kDfMinBlocks),
                        sh.df_b_occ == 2 ? resident(k_dfB<0, 2>, t, 2) : resident(k_dfB<0, 3>, t, 3),
                        resident(k_dfC<0>, t, kDfMinBlocks)};
    // the partial-sum buffer holds rows for this many blocks (xf_handle::init)
    const int cap = std::max(max_phase_blocks(nbeams, 256), 152 * 4);
    for (int p = 0; p < 3; ++p) sh.phase_blocks[p] = std::min(std::min(need, sms * occ[p]), cap);
    sh.blocks = sh.blocks_ab = sh.phase_blocks[0];
}

}  // namespace xf
