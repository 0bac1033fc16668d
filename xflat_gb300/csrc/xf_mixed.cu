// Mixed-precision path: FP32 SU(2) rotations and beam state (an FP32 value
// plus an FP32 compensation word per component), with FP64 where the
// stability of the method needs it: the moment reduction (Kahan-compensated
// FP32 partial sums per thread, FP64 across threads, beams and blocks), the
// step-error estimate's reduction and max, accept/reject and dr control,
// radius accumulation and the periodic unitarity renormalisation.
//
// Same stage schedule as the FP64 path (src/Nmr.cpp:153-206), written in
// increments: every propagator is U = I + K with K = (C-1) - i S sigma(h),
// evaluated from the Taylor series of C-1 and S in t = (lambda dl)^2, so that
// each increment K psi carries FP32 precision relative to its own (small)
// size.  Phases A and B only need the angular moments of psi1, psi3 and psi4
// and recompute their stage states from psi0; phase C builds the candidate
// psi0 + (d3' + d4m)/2 and the error estimate delta = psi4 - psi1.
//
// The error estimate cannot be formed as the difference of two FP32 states:
// their rounding (~6e-8) sits far above the tolerance eps0 = 1e-9 on
// sqrt(sum fv |delta|^2).  It is rebuilt exactly as a sum of operator
// differences.  With psi1 = psi0 + (K(h1,l1) + K(h0,l1)) psi0 / 2 and the
// candidate above, and using 2 K(h,l) - K(h,2l) + K(h,l)^2 = 0 (U(h,2l) =
// U(h,l)^2) to cancel the second-order terms analytically,
//   2 delta = [K(h3,l1) - K(h1,l1)] psi0 + [K(h4,l2) - K(h0,l0)] psi3
//           + [K(h0,2l0) - K(h0,l1)] psi0,                 psi3 = psi0 + d3,
// where K(h4,l2) - K(h0,l0) = [K(h4,l2) - K(h0,l2)] + [K(h0,l2) - K(h0,l0)]
// and the last bracket vanishes in MA (l1 = 2 l0).  Each bracket is
// evaluated in FP32 through divided differences of the series, with the
// Hamiltonian and path-length differences taken in FP64, so every term has
// FP32 precision relative to its own (first-order small) size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xf_common.cuh"
#include "xf_launch.cuh"
#include "xf_mixed.cuh"
#include "xf_engine.h"
#include "xf_kernels.h"
#include "xf_mixed.h"

namespace xf {

namespace {

using namespace detail;
using mixed::KSum;
// ------------------------------------------------------------------ phases

// The phase kernels are latency-bound (dependent FP32 chains and state loads,
// one warp per beam); register caps that raise the resident warps per SM beat
// the few spills they cause (measured on GB300 at 2048 x 4 x 512 bins: phase C
// 0.165 ms at 2 blocks/SM, 0.119 ms at 4).  Minimum resident blocks per SM by
// phase (A, B, C) and geometry (MA/SA, MAA).
constexpr int mix_min_blocks(int phase, int geom)
{
    return geom == 0 ? (phase == 0 ? 5 : phase == 1 ? 6 : 4) : (phase == 0 ? 5 : phase == 1 ? 6 : 4);
}

template <int GEOM>
__global__ void __launch_bounds__(256, mix_min_blocks(0, GEOM)) k_mixA(Dev d)
{
    pdl_enter();
    mixed::phaseA_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_A));
}

template <int GEOM>
__global__ void __launch_bounds__(256, mix_min_blocks(1, GEOM)) k_mixB(Dev d)
{
    pdl_enter();
    mixed::phaseB_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_B));
}

template <int GEOM>
__global__ void __launch_bounds__(256, mix_min_blocks(2, GEOM)) k_mixC(Dev d)
{
    pdl_enter();
    mixed::phaseC_body<GEOM>(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), grid_target(d, PH_C));
}

// ------------------------------------------------------------------ helpers

// Exact FP64 energy sums of psi0 from its compensated pairs (NBeam::calcESum,
// src/NBeam.cpp:812-840), optionally after the unitarity renormalisation of
// every bin (|a|^2 + |b|^2 = 1 in FP64, written back as compensated pairs).
// With `conditional` set it acts only when the step controller flagged a
// renormalisation (every renorm_every accepted steps under device control).
__global__ void __launch_bounds__(256) k_mix_esum(Dev d, int renorm, int conditional)
{
    pdl_enter();
    mixed::esum_body(d, blockIdx.x * (blockDim.x >> 5), gridDim.x * (blockDim.x >> 5), renorm, conditional);
}

// Accept under host control: swap the state, sum and moment roles.
__global__ void k_mix_accept(Dev d)
{
    Ctl* c = d.ctl;
    float* t = c->m0hi;
    c->m0hi = c->m4hi;
    c->m4hi = t;
    t = c->m0lo;
    c->m0lo = c->m4lo;
    c->m4lo = t;
    double* ts = c->S0;
    c->S0 = c->S4;
    c->S4 = ts;
    float2* tf = c->S0f;
    c->S0f = c->S4f;
    c->S4f = tf;
    for (int i = 0; i < kNJ; ++i) c->J0[i] = c->JC[i];
}

}  // namespace

// ------------------------------------------------------------------ host side

struct Mixed {
    float* hi[2] = {nullptr, nullptr};
    float* lo[2] = {nullptr, nullptr};
    float* fvf = nullptr;
    float* fvf_lo = nullptr;
    float* hvf = nullptr;
    float* hvf_lo = nullptr;
    double* S[2] = {nullptr, nullptr};
    float2* Sf[2] = {nullptr, nullptr};
};

#define XM_CUDA(h, call)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return (h)->fail(XF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

Mixed* mixed_create(xf_handle* h)
{
    Mixed* m = new Mixed();
    const size_t n = (size_t)h->nbeams * 4 * h->epad;
    const bool df = h->cfg.precision == XF_PREC_DF;
    bool ok = true;
    for (int i = 0; i < 2 && ok; ++i) {
        if (df) {
            // double-float: one buffer in the bin layout ([beam][epad][8] floats,
            // pair_at); lo points at its second half and is not read on its own
            ok = ok && cudaMalloc(&m->hi[i], 2 * n * sizeof(float)) == cudaSuccess &&
                 cudaMemset(m->hi[i], 0, 2 * n * sizeof(float)) == cudaSuccess;
            if (ok) m->lo[i] = m->hi[i] + n;
        } else {
            ok = ok && cudaMalloc(&m->hi[i], n * sizeof(float)) == cudaSuccess &&
                 cudaMemset(m->hi[i], 0, n * sizeof(float)) == cudaSuccess;
            ok = ok && cudaMalloc(&m->lo[i], n * sizeof(float)) == cudaSuccess &&
                 cudaMemset(m->lo[i], 0, n * sizeof(float)) == cudaSuccess;
        }
        ok = ok && cudaMalloc(&m->S[i], 4 * (size_t)h->nbeams * sizeof(double)) == cudaSuccess;
        ok = ok && cudaMalloc(&m->Sf[i], 4 * (size_t)h->nbeams * sizeof(float2)) == cudaSuccess &&
             cudaMemset(m->Sf[i], 0, 4 * (size_t)h->nbeams * sizeof(float2)) == cudaSuccess;
    }
    std::vector<float> fvf(4 * (size_t)h->epad, 0.f), fvf_lo(4 * (size_t)h->epad, 0.f), hvf(2 * (size_t)h->epad, 0.f),
        hvf_lo(2 * (size_t)h->epad, 0.f);
    for (int p = 0; p < 4; ++p)
        for (int e = 0; e < h->ne; ++e) {
            const double f = h->tab.fv[(size_t)p * h->ne + e];
            fvf[(size_t)p * h->epad + e] = (float)f;
            fvf_lo[(size_t)p * h->epad + e] = (float)(f - (double)(float)f);
        }
    for (int e = 0; e < h->ne; ++e)
        for (int k = 0; k < 2; ++k) {
            const double v = h->tab.hvac[2 * (size_t)e + k];
            hvf[k * h->epad + e] = (float)v;
            hvf_lo[k * h->epad + e] = (float)(v - (double)(float)v);
        }
    ok = ok && cudaMalloc(&m->fvf, fvf.size() * sizeof(float)) == cudaSuccess &&
         cudaMemcpy(m->fvf, fvf.data(), fvf.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMalloc(&m->fvf_lo, fvf_lo.size() * sizeof(float)) == cudaSuccess &&
         cudaMemcpy(m->fvf_lo, fvf_lo.data(), fvf_lo.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMalloc(&m->hvf, hvf.size() * sizeof(float)) == cudaSuccess &&
         cudaMemcpy(m->hvf, hvf.data(), hvf.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMalloc(&m->hvf_lo, hvf_lo.size() * sizeof(float)) == cudaSuccess &&
         cudaMemcpy(m->hvf_lo, hvf_lo.data(), hvf_lo.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        h->fail(XF_ENOMEM, "mixed-precision state allocation failed");
        mixed_destroy(m);
        return nullptr;
    }
    h->dev.fvf = m->fvf;
    h->dev.fvf_lo = m->fvf_lo;
    h->dev.hvf = m->hvf;
    h->dev.hvf_lo = m->hvf_lo;
    h->h_ctl->m0hi = m->hi[0];
    h->h_ctl->m0lo = m->lo[0];
    h->h_ctl->m4hi = m->hi[1];
    h->h_ctl->m4lo = m->lo[1];
    h->h_ctl->S0 = m->S[0];
    h->h_ctl->S4 = m->S[1];
    h->h_ctl->S0f = m->Sf[0];
    h->h_ctl->S4f = m->Sf[1];
    if (cudaMemcpy(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice) != cudaSuccess) {
        h->fail(XF_ECUDA, "control block upload failed");
        mixed_destroy(m);
        return nullptr;
    }
    return m;
}

void mixed_destroy(Mixed* m)
{
    if (!m) return;
    for (int i = 0; i < 2; ++i) {
        const bool shared = m->lo[i] && m->hi[i] && m->lo[i] > m->hi[i];  // double-float: lo inside hi's buffer
        if (m->hi[i]) cudaFree(m->hi[i]);
        if (m->lo[i] && !shared) cudaFree(m->lo[i]);
        if (m->S[i]) cudaFree(m->S[i]);
        if (m->Sf[i]) cudaFree(m->Sf[i]);
    }
    if (m->fvf) cudaFree(m->fvf);
    if (m->fvf_lo) cudaFree(m->fvf_lo);
    if (m->hvf) cudaFree(m->hvf);
    if (m->hvf_lo) cudaFree(m->hvf_lo);
    delete m;
}

int mixed_set_state(xf_handle* h, Mixed* m, const double* psi)
{
    (void)m;
    int rc;
    if ((rc = h->pull_ctl())) return rc;
    const size_t n = (size_t)h->nbeams * 4 * h->epad;
    if (h->dev.df) {
        // bin layout: [beam][epad][hi0..hi3, lo0..lo3]
        std::vector<float> bins(2 * n, 0.f);
        for (size_t r = 0; r < (size_t)h->nbeams * 4; ++r)
            for (int e = 0; e < h->ne; ++e) {
                const double x = psi[r * h->ne + e];
                const float xh = (float)x;
                float* p = &bins[((r / 4) * h->epad + e) * 8];
                p[r % 4] = xh;
                p[4 + r % 4] = (float)(x - (double)xh);
            }
        XM_CUDA(h, cudaMemcpy(h->h_ctl->m0hi, bins.data(), 2 * n * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> hi(n, 0.f), lo(n, 0.f);
        for (size_t r = 0; r < (size_t)h->nbeams * 4; ++r)
            for (int e = 0; e < h->ne; ++e) {
                const double x = psi[r * h->ne + e];
                const float xh = (float)x;
                hi[r * h->epad + e] = xh;
                lo[r * h->epad + e] = (float)(x - (double)xh);
            }
        XM_CUDA(h, cudaMemcpy(h->h_ctl->m0hi, hi.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        XM_CUDA(h, cudaMemcpy(h->h_ctl->m0lo, lo.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    }
    k_mix_esum<<<max_phase_blocks(h->nbeams, 256), 256, 0, h->st>>>(h->dev, 0, 0);
    XM_CUDA(h, cudaGetLastError());
    XM_CUDA(h, cudaStreamSynchronize(h->st));
    h->j0_valid = false;
    return XF_OK;
}

int mixed_get_state(xf_handle* h, Mixed* m, int which, double* psi)
{
    (void)m;
    if (which != 0 && which != 4) return h->fail(XF_EUNSUPPORTED, "the mixed path keeps only psi0 and the candidate (which = 0 or 4)");
    int rc;
    if ((rc = h->pull_ctl())) return rc;
    const size_t n = (size_t)h->nbeams * 4 * h->epad;
    if (h->dev.df) {
        std::vector<float> bins(2 * n);
        XM_CUDA(h, cudaMemcpy(bins.data(), which == 0 ? h->h_ctl->m0hi : h->h_ctl->m4hi, 2 * n * sizeof(float),
                              cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < (size_t)h->nbeams * 4; ++r)
            for (int e = 0; e < h->ne; ++e) {
                const float* p = &bins[((r / 4) * h->epad + e) * 8];
                psi[r * h->ne + e] = (double)p[r % 4] + (double)p[4 + r % 4];
            }
        return XF_OK;
    }
    std::vector<float> hi(n), lo(n);
    XM_CUDA(h, cudaMemcpy(hi.data(), which == 0 ? h->h_ctl->m0hi : h->h_ctl->m4hi, n * sizeof(float), cudaMemcpyDeviceToHost));
    XM_CUDA(h, cudaMemcpy(lo.data(), which == 0 ? h->h_ctl->m0lo : h->h_ctl->m4lo, n * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t r = 0; r < (size_t)h->nbeams * 4; ++r)
        for (int e = 0; e < h->ne; ++e) psi[r * h->ne + e] = (double)hi[r * h->epad + e] + (double)lo[r * h->epad + e];
    return XF_OK;
}

void mixed_launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (d.df) {
        df_launch_phase(phase, d, sh, st);
        return;
    }
    const int ab = sh.blocks_ab > 0 ? sh.blocks_ab : sh.blocks;
    if (d.geom == 0) {
        if (phase == PH_A) launch_pdl(k_mixA<0>, ab, sh.threads, st, d);
        else if (phase == PH_B) launch_pdl(k_mixB<0>, ab, sh.threads, st, d);
        else launch_pdl(k_mixC<0>, sh.blocks, sh.threads, st, d);
    } else {
        if (phase == PH_A) launch_pdl(k_mixA<1>, ab, sh.threads, st, d);
        else if (phase == PH_B) launch_pdl(k_mixB<1>, ab, sh.threads, st, d);
        else launch_pdl(k_mixC<1>, sh.blocks, sh.threads, st, d);
    }
}

void mixed_launch_accept(const Dev& d, cudaStream_t st) { k_mix_accept<<<1, 1, 0, st>>>(d); }

void mixed_launch_renorm(const Dev& d, int conditional, cudaStream_t st)
{
    // The conditional form runs every iteration of a device-controlled graph
    // and usually finds nothing to do: a grid of two blocks per SM keeps that
    // empty launch cheap, and covers the beams grid-stride when it does work.
    const int blocks = conditional ? std::min(max_phase_blocks(d.nbeams, 256), 2 * 152)
                                   : max_phase_blocks(d.nbeams, 256);
    launch_pdl(k_mix_esum, blocks, 256, st, d, 1, conditional);
}

}  // namespace xf
