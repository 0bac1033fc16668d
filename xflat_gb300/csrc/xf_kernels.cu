// FP64 kernels of the per-radius-step hot path (MA and MAA geometries).
//
// One stepper iteration of the reference (src/Nmr.cpp:153-206: stages S1..S11,
// five beam sweeps, four Hamiltonian reductions and an error sweep) runs as
// three phase kernels, separated by the three global reductions the data
// dependencies require:
//
//   phase A  psi1 = U(h0,dl1) psi0, psi3 = U(h0,dl0) psi0 and their angular
//            moments (S1, S2, S6 -> S3, S7)
//   phase B  psi1 <- (U(h1,dl1) psi0 + psi1)/2, psi4 = U(h3,dl1) psi0 and its
//            moments (S4/S5, S8 -> S9)
//   phase C  psi4 <- (U(h4,dl2) psi3 + psi4)/2, per-beam error against psi1,
//            max over beams, moments of the candidate (S10/S11, error sweep)
//
// Each phase assigns one warp per beam (grid-stride over beams); a lane owns
// energies lane, lane+32, ...  Per-beam energy sums are reduced with a
// warp-level reduce-scatter, weighted into the angular moments by the lanes
// that own them, combined per block in shared memory and across blocks by the
// last block to finish (fixed order, so results are bitwise reproducible).
//
// The 2x2 SU(2) propagator of src/NBeam.cpp:360-393 needs cos(x) and
// sin(x)/lambda with x = lambda*dl.  GB300 executes FP64 at about 1/58 of its
// FP32 rate, so the hot path avoids sqrt, sincos and the division: both are
// entire functions of t = x^2 and are evaluated from their Taylor series
// (coefficients 1/(2k)! and 1/(2k+1)!), truncated where the remainder is below
// half an ulp for t <= kSeriesT.  Larger t takes the direct sqrt/sincos path.
#include "xf_kernels.h"

#include "xf_common.cuh"
#include "xf_launch.cuh"
#include "xf_fp64.cuh"

#include <algorithm>

namespace xf {

namespace {

using namespace detail;
// ------------------------------------------------------------------ geometry

// phy::calcAngleBins at r, r+dr/2, r+dr and phy::calcDeltaLs for the three
// path segments (src/Nmr.cpp:153-173, src/Phy_MA.cpp:172-227,
// src/Phy_MAA.cpp:194-241).  Under device control the threads of angle 0 also
// evaluate the matter term at the three points (src/Matt.cpp:31-64).  Blocks
// of kGeoAngles angle bins x 3 stage points (geometry_point): the square roots
// and divisions of one angle run on three threads, and the launch spreads
// over A/32 SMs (one thread per angle on 128-thread blocks took 13 us per
// launch at A = 256 on GB300, FP64-pipe bound on two SMs).
constexpr int kGeoAngles = 32;

__global__ void __launch_bounds__(3 * kGeoAngles) k_geometry(Dev d)
{
    pdl_enter();
    __shared__ double s_c[3 * kGeoAngles];
    const int slot = threadIdx.x % kGeoAngles, pt = threadIdx.x / kGeoAngles;
    const int ang = blockIdx.x * kGeoAngles + slot;
    geometry_point(d, ang < d.A ? ang : -1, pt, slot, kGeoAngles, s_c);
}

// ------------------------------------------------------------------ phases

// Single-simulation phase kernels: grid-stride over beams, the grid is one
// reduction group.
template <int GEOM>
__global__ void __launch_bounds__(256) k_phaseA(Dev d)
{
    pdl_enter();
    fp64::phaseA_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_A));
}

template <int GEOM, int FUSE>
__global__ void __launch_bounds__(256) k_phaseB(Dev d)
{
    pdl_enter();
    fp64::phaseB_body<GEOM, FUSE>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5),
                                  grid_target(d, PH_B));
}

// Phase C holds fewer values across the energy loop than A and B: capped at
// 3 (MA) or 4 (MAA) resident blocks per SM it needs at most 80 registers
// with little or no spilling, and the extra warps hide FP64 latency (measured
// on GB300: 0.535 -> 0.498 ms at 4.19M MA bins, 1.094 -> 1.024 ms at 8.39M
// MAA bins; the same caps slow phases A and B).
template <int GEOM, int FUSE>
__global__ void __launch_bounds__(256, GEOM == 0 ? 3 : 4) k_phaseC(Dev d)
{
    pdl_enter();
    fp64::phaseC_body<GEOM, FUSE>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5),
                                  grid_target(d, PH_C));
}

// ------------------------------------------------------------------ helpers

// NBeam::calcESum (src/NBeam.cpp:812-840) for every beam of psi: S[b][4].
__global__ void __launch_bounds__(256) k_esum(Dev d, const double* __restrict__ psi, double* __restrict__ S)
{
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + (threadIdx.x >> 5), tw = gridDim.x * nw;
    const int epad = d.epad;
    for (int b = gw; b < d.nbeams; b += tw) {
        const double* in = psi + (size_t)b * 4 * epad;
        const double* fvp = d.fv + (b & 3) * epad;
        double v[4] = {0., 0., 0., 0.};
        for (int e = lane; e < epad; e += 32) fp64::acc_rho(fp64::load_psi(in, epad, e), fvp[e], v[1], v[2], v[3]);
        v[1] *= .5;
        warp_reduce_scatter<4>(v, lane);
        const int myv = lane >> 3;
        if ((lane & 7) == 0) S[(size_t)b * 4 + (myv == 0 ? 1 : comp_of(myv - 1))] = (myv == 0) ? 0. : v[0];
    }
}

// Angular moments from per-beam energy sums at stage point pt: the reduction of
// phy::getHvv_partial (src/Phy_MA.cpp:388-446, src/Phy_MAA.cpp:468-562).
template <int GEOM>
__global__ void __launch_bounds__(256) k_moments(Dev d, const double* __restrict__ Sarg, int pt, double* Jout,
                                                 int conditional)
{
    pdl_enter();
    moments_body<GEOM>(d, blockIdx.x * blockDim.x, gridDim.x * blockDim.x, grid_target(d, PH_MOM), Sarg, pt, Jout,
                       conditional);
}

// Accept under host control: psi0 <-> psi4, S0 <-> S4, J0 <- JC.
__global__ void k_accept(Dev d)
{
    Ctl* ctl = d.ctl;
    double* t = ctl->psi0;
    ctl->psi0 = ctl->psi4;
    ctl->psi4 = t;
    double* ts = ctl->S0;
    ctl->S0 = ctl->S4;
    ctl->S4 = ts;
    for (int i = 0; i < kNJ; ++i) ctl->J0[i] = ctl->JC[i];
}

// phy::getHvv for every (theta, phi) bin (src/Phy_MA.cpp:467-473,
// src/Phy_MAA.cpp:608-619): hvv[(ang*P+phi)*4 + z].
template <int GEOM>
__global__ void k_hvv_eval(Dev d, const double* __restrict__ J, int pt, double* __restrict__ hvv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.A * d.P) return;
    BeamIdx bi;
    bi.ang = i / d.P;
    bi.phi = i - bi.ang * d.P;
    bi.p = 0;
    double H[3];
    beam_hvv<GEOM>(d, J, pt, bi, H);
    hvv[4 * i + 0] = H[0];
    hvv[4 * i + 1] = 0.;
    hvv[4 * i + 2] = H[1];
    hvv[4 * i + 3] = H[2];
}

// Reads psi0 through the control block, so the copy follows the role swaps of
// accepted steps without a host round trip.
__global__ void k_stage_state(Dev d, int mixed, int big_endian, double* __restrict__ dst)
{
    const Ctl* ctl = d.ctl;
    const size_t n = (size_t)d.nbeams * 4 * d.epad;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const float* __restrict__ hi = ctl->m0hi;
    const float* __restrict__ lo = ctl->m0lo;
    const double* __restrict__ src = ctl->psi0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const size_t r = i / d.epad;
        const double v = mixed ? pair_at(d, hi, lo, (int)(r / 4), (int)(r % 4), (int)(i - r * d.epad)) : src[i];
        dst[i] = big_endian ? byte_reversed(v) : v;
    }
}

// One warp per beam; src/IO_f.cpp:346 weights beam i*4 + p with the spectrum
// of particle p % 2 (an operator-precedence quirk kept for file parity).
__global__ void k_survival(Dev d, int mixed, double* __restrict__ out)
{
    const Ctl* ctl = d.ctl;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int epad = d.epad;
    for (int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < d.nbeams; b += nw) {
        const double* fv = d.fv + (size_t)((b & 3) % 2) * epad;
        const size_t base = (size_t)b * 4 * epad;
        double s = 0.;
        for (int e = lane; e < epad; e += 32) {
            double ar, ai;
            if (mixed) {
                ar = pair_at(d, ctl->m0hi, ctl->m0lo, b, 0, e);
                ai = pair_at(d, ctl->m0hi, ctl->m0lo, b, 1, e);
            } else {
                ar = ctl->psi0[base + e];
                ai = ctl->psi0[base + epad + e];
            }
            s = fma(ar * ar + ai * ai, fv[e], s);
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
        if (lane == 0) out[b] = s;
    }
}

// A record decided at the last accepted step of a device-controlled run has
// no following phase A to stage it: the same staging, one warp per beam.
__global__ void k_stage_pending(Dev d, int mixed)
{
    const Ctl* ctl = d.ctl;
    const int kind = ctl->stage_kind;
    if (!kind) return;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < d.nbeams; b += nw)
        stage_beam(d, ctl, kind, b, lane, mixed ? nullptr : ctl->psi0, ctl->m0hi, ctl->m0lo);
}

}  // namespace

int max_phase_blocks(int nbeams, int threads)
{
    const int warps = threads / 32;
    const int need = (nbeams + warps - 1) / warps;
    return std::max(1, std::min(need, 152 * 16));
}

// The mixed-precision phases A and B run best as a single wave of resident
// blocks (5 per SM; measured on GB300: 0.054 / 0.037 ms at 4.19M MA bins
// with 760 blocks against 0.058 / 0.040 with one block per 8 beams, 0.130 /
// 0.093 against 0.152 / 0.099 at 8.39M MAA bins); phase C, and the FP64
// phases, limited by the FP64 pipe, with one block per 8 beams.
Shape default_shape(int nbeams, int epad, bool mixed)
{
    (void)epad;
    Shape s;
    s.threads = 256;
    s.blocks = max_phase_blocks(nbeams, s.threads);
    s.blocks_ab = mixed ? std::min(s.blocks, 152 * 5) : s.blocks;
    return s;
}

void launch_geometry(const Dev& d, cudaStream_t st)
{
    launch_pdl(k_geometry, (d.A + kGeoAngles - 1) / kGeoAngles, 3 * kGeoAngles, st, d);
}

void launch_esum(const Dev& d, const double* psi, double* S, cudaStream_t st)
{
    k_esum<<<max_phase_blocks(d.nbeams, 256), 256, 0, st>>>(d, psi, S);
}

void launch_moments(const Dev& d, const double* S, int pt, double* Jout, cudaStream_t st, int conditional)
{
    const int t = 256;
    const int blocks = std::max(1, std::min((d.nbeams + t - 1) / t, 152 * 4));
    if (d.geom == 0) launch_pdl(k_moments<0>, blocks, t, st, d, S, pt, Jout, conditional);
    else launch_pdl(k_moments<1>, blocks, t, st, d, S, pt, Jout, conditional);
}

template <int GEOM, int FUSE>
void launch_phase_t(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (phase == PH_A) launch_pdl(k_phaseA<GEOM>, sh.blocks, sh.threads, st, d);
    else if (phase == PH_B) launch_pdl(k_phaseB<GEOM, FUSE>, sh.blocks, sh.threads, st, d);
    else launch_pdl(k_phaseC<GEOM, FUSE>, sh.blocks, sh.threads, st, d);
}

void launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (d.geom == 0) {
        if (sh.fp64_fused) launch_phase_t<0, 1>(phase, d, sh, st);
        else launch_phase_t<0, 0>(phase, d, sh, st);
    } else {
        if (sh.fp64_fused) launch_phase_t<1, 1>(phase, d, sh, st);
        else launch_phase_t<1, 0>(phase, d, sh, st);
    }
}

void launch_accept(const Dev& d, cudaStream_t st) { k_accept<<<1, 1, 0, st>>>(d); }

void launch_stage_state(const Dev& d, int mixed, int big_endian, double* dst, cudaStream_t st)
{
    k_stage_state<<<152 * 4, 256, 0, st>>>(d, mixed, big_endian, dst);
}

void launch_stage_pending(const Dev& d, int mixed, cudaStream_t st)
{
    k_stage_pending<<<max_phase_blocks(d.nbeams, 256), 256, 0, st>>>(d, mixed);
}

void launch_survival(const Dev& d, int mixed, double* out, cudaStream_t st)
{
    k_survival<<<max_phase_blocks(d.nbeams, 256), 256, 0, st>>>(d, mixed, out);
}

void launch_hvv_eval(const Dev& d, const double* J, int pt, double* hvv, cudaStream_t st)
{
    const int n = d.A * d.P, t = 128;
    if (d.geom == 0) k_hvv_eval<0><<<(n + t - 1) / t, t, 0, st>>>(d, J, pt, hvv);
    else k_hvv_eval<1><<<(n + t - 1) / t, t, 0, st>>>(d, J, pt, hvv);
}

}  // namespace xf
