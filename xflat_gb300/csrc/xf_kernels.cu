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

#include <algorithm>

namespace xf {

namespace {

using namespace detail;
constexpr double kSeriesT = 0.25;

// cos(sqrt(t)) and sin(sqrt(t))/sqrt(t) for 0 <= t <= kSeriesT, degree 7 in t.
// Truncation error below 7.3e-19 (cos) and 4.3e-20 (sinc) at t = 0.25.
__device__ __forceinline__ void series_cs(double t, double& c, double& s)
{
    c = -1.0 / 87178291200.0;
    c = fma(c, t, 1.0 / 479001600.0);
    c = fma(c, t, -1.0 / 3628800.0);
    c = fma(c, t, 1.0 / 40320.0);
    c = fma(c, t, -1.0 / 720.0);
    c = fma(c, t, 1.0 / 24.0);
    c = fma(c, t, -0.5);
    c = fma(c, t, 1.0);
    s = -1.0 / 1307674368000.0;
    s = fma(s, t, 1.0 / 6227020800.0);
    s = fma(s, t, -1.0 / 39916800.0);
    s = fma(s, t, 1.0 / 362880.0);
    s = fma(s, t, -1.0 / 5040.0);
    s = fma(s, t, 1.0 / 120.0);
    s = fma(s, t, -1.0 / 6.0);
    s = fma(s, t, 1.0);
}

// Coefficients (C, S) of U = C - i S H for H = [[h00, h01],[h01*, -h00]],
// h01 = h01r + i h01i, over the path length dl: C = cos(lambda dl),
// S = sin(lambda dl)/lambda, lambda = |H| (src/NBeam.cpp:366-369).
__device__ __forceinline__ void su2_coeffs(double h00, double h01r, double h01i, double dl, double& C, double& S)
{
    const double lam2 = h00 * h00 + (h01r * h01r + h01i * h01i);
    const double t = lam2 * (dl * dl);
    if (t <= kSeriesT) {
        double s;
        series_cs(t, C, s);
        S = s * dl;
    } else {
        const double lam = sqrt(lam2);
        double sn, cs;
        sincos(lam * dl, &sn, &cs);
        C = cs;
        S = sn / lam;
    }
}

// psi' = U psi with the matrix entries of src/NBeam.cpp:371-392.
struct Psi {
    double ar, ai, br, bi;
};

__device__ __forceinline__ Psi su2_apply(double C, double S, double h00, double h01r, double h01i, const Psi& x)
{
    const double m1 = -h00 * S;
    const double m2 = h01i * S;
    const double m3 = -h01r * S;
    Psi y;
    y.ar = (C * x.ar - m1 * x.ai) + (m2 * x.br - m3 * x.bi);
    y.ai = (C * x.ai + m1 * x.ar) + (m2 * x.bi + m3 * x.br);
    y.br = (-m2 * x.ar - m3 * x.ai) + (C * x.br + m1 * x.bi);
    y.bi = (-m2 * x.ai + m3 * x.ar) + (C * x.bi - m1 * x.br);
    return y;
}

// Accumulates fv * rho(psi) (first row of the density matrix, src/NBeam.cpp:314-322);
// component 0 is accumulated without the factor 1/2, applied once per beam.
__device__ __forceinline__ void acc_rho(const Psi& x, double fv, double& s0, double& s2, double& s3)
{
    const double d0 = (x.ar * x.ar + x.ai * x.ai) - (x.br * x.br + x.bi * x.bi);
    const double d2 = x.ar * x.br + x.ai * x.bi;
    const double d3 = x.ai * x.br - x.ar * x.bi;
    s0 = fma(d0, fv, s0);
    s2 = fma(d2, fv, s2);
    s3 = fma(d3, fv, s3);
}

__device__ __forceinline__ Psi load_psi(const double* __restrict__ base, int epad, int e)
{
    Psi x;
    x.ar = base[e];
    x.ai = base[epad + e];
    x.br = base[2 * epad + e];
    x.bi = base[3 * epad + e];
    return x;
}

__device__ __forceinline__ void store_psi(double* __restrict__ base, int epad, int e, const Psi& x)
{
    base[e] = x.ar;
    base[epad + e] = x.ai;
    base[2 * epad + e] = x.br;
    base[3 * epad + e] = x.bi;
}

// ------------------------------------------------------------------ geometry

// phy::calcAngleBins at r, r+dr/2, r+dr and phy::calcDeltaLs for the three
// path segments (src/Nmr.cpp:153-173, src/Phy_MA.cpp:172-227,
// src/Phy_MAA.cpp:194-241).  Under device control thread 0 also evaluates the
// matter term at the three points (src/Matt.cpp:31-64).
__global__ void k_geometry(Dev d)
{
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    const double r = ctl->r, dr = ctl->dr;
    const double dr2 = .5 * dr;
    const double rdr = r + dr;
    const double rdr2 = r + dr2;
    const double rp[3] = {r, rdr2, rdr};
    const int ang = blockIdx.x * blockDim.x + threadIdx.x;
    if (d.device_control && ang == 0) {
#pragma unroll
        for (int pt = 0; pt < 3; ++pt) {
            double hm = 0.;
            if (d.has_matter) {
                const double R = 10. / rp[pt];
                const double far = d.nbfar * (R * R * R);
                const double near = d.nb0 * exp((d.Rv - rp[pt]) / d.hNS);
                hm = d.mat_coeff * (far + near) * .5;
            }
            ctl->hm[pt] = hm;
        }
    }
    if (ang >= d.A) return;
    double c[3];
#pragma unroll
    for (int pt = 0; pt < 3; ++pt) {
        const double ra = d.Rv / rp[pt];
        const double r2 = ra * ra;
        c[pt] = sqrt(1. - r2 * (1. - d.cos2R[ang]));
        d.geo[geo_idx(0, pt, ang, d.A)] = c[pt];
        d.geo[geo_idx(1, pt, ang, d.A)] = ra * d.sinR[ang];
        d.geo[geo_idx(2, pt, ang, d.A)] = .5 * (1. / c[pt]) * r2 * d.dcos2R[ang];
    }
    if (d.geom == 0) {
        d.geo[geo_idx(3, 0, ang, d.A)] = dr2 / (c[0]);
        d.geo[geo_idx(3, 1, ang, d.A)] = dr / (c[0]);
        d.geo[geo_idx(3, 2, ang, d.A)] = dr2 / (c[1]);
    } else {
        d.geo[geo_idx(3, 0, ang, d.A)] = dr2 / ((c[0] + c[1]) * .5);
        d.geo[geo_idx(3, 1, ang, d.A)] = dr / ((c[0] + c[2]) * .5);
        d.geo[geo_idx(3, 2, ang, d.A)] = dr2 / ((c[1] + c[2]) * .5);
    }
}

// ------------------------------------------------------------------ phase A

// S1 (H of psi0 from the cached moments), S2 and S6 (two sweeps sharing H0),
// and the moments of psi1 at point 2 (S3) and of psi3 at point 1 (S7).
template <int GEOM>
__global__ void __launch_bounds__(256) k_phaseA(Dev d)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const double* __restrict__ psi0 = ctl->psi0;
    const double hm = ctl->hm[0];
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + (threadIdx.x >> 5), tw = gridDim.x * nw;
    const int epad = d.epad;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.;
    const int myv = lane >> 2;  // value slot owned after an 8-way reduce-scatter
    for (int b = gw; b < d.nbeams; b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        const BeamH h = beam_offsets<GEOM>(d, ctl->J0, 0, hm, bi);
        const double dl1 = geo(d, 3, 1, bi.ang), dl0 = geo(d, 3, 0, bi.ang);
        const double* in = psi0 + (size_t)b * 4 * epad;
        double* o1 = d.psi1 + (size_t)b * 4 * epad;
        double* o3 = d.psi3 + (size_t)b * 4 * epad;
        const double* fvp = d.fv + bi.p * epad;
        double v[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
        for (int e = lane; e < epad; e += 32) {
            const double h00 = d.hvac[e] + h.h00b;
            const double h01r = d.hvac[epad + e] + h.h01rb;
            const Psi x = load_psi(in, epad, e);
            double C1, S1, C0, S0;
            if (GEOM == 0) {
                // MA: dl0 = dl1/2 exactly, so U(dl1) coefficients follow from
                // the half-length ones by the double-angle identities.
                su2_coeffs(h00, h01r, h.h01i, dl0, C0, S0);
                C1 = fma(C0 + C0, C0, -1.0);
                S1 = (C0 + C0) * S0;
            } else {
                su2_coeffs(h00, h01r, h.h01i, dl1, C1, S1);
                su2_coeffs(h00, h01r, h.h01i, dl0, C0, S0);
            }
            const Psi y1 = su2_apply(C1, S1, h00, h01r, h.h01i, x);
            const Psi y3 = su2_apply(C0, S0, h00, h01r, h.h01i, x);
            store_psi(o1, epad, e, y1);
            store_psi(o3, epad, e, y3);
            const double f = fvp[e];
            acc_rho(y1, f, v[0], v[1], v[2]);
            acc_rho(y3, f, v[3], v[4], v[5]);
        }
        v[0] *= .5;
        v[3] *= .5;
        warp_reduce_scatter<8>(v, lane);
        if (myv < 3) add_moment<GEOM>(d, v[0], comp_of(myv), 2, bi, acc);
        else if (myv < 6) add_moment<GEOM>(d, v[0], comp_of(myv - 3), 1, bi, acc);
    }
    if (!block_and_grid_reduce<K>(d, PH_A, 4, 6, acc, 0., false, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) {
        ctl->JA1[threadIdx.x] = 0.;
        ctl->JA3[threadIdx.x] = 0.;
    }
    __syncthreads();
    if ((int)threadIdx.x < 6 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        double* J = v < 3 ? ctl->JA1 : ctl->JA3;
        J[k * 4 + comp_of(v % 3)] = s_out[threadIdx.x];
    }
}

// ------------------------------------------------------------------ phase B

// S4/S5 (psi4' = U(h1, dl1, hm(r+dr)) psi0 averaged into psi1) and S8
// (psi4 = U(h3, dl1, hm(r+dr/2)) psi0) with the moments of psi4 at point 2 (S9).
template <int GEOM>
__global__ void __launch_bounds__(256) k_phaseB(Dev d)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const double* __restrict__ psi0 = ctl->psi0;
    double* __restrict__ psi4 = ctl->psi4;
    const double hm_rdr = ctl->hm[2], hm_rdr2 = ctl->hm[1];
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + (threadIdx.x >> 5), tw = gridDim.x * nw;
    const int epad = d.epad;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.;
    const int myv = lane >> 3;
    for (int b = gw; b < d.nbeams; b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        const BeamH g1 = beam_offsets<GEOM>(d, ctl->JA1, 2, hm_rdr, bi);
        const BeamH g3 = beam_offsets<GEOM>(d, ctl->JA3, 1, hm_rdr2, bi);
        const double dl1 = geo(d, 3, 1, bi.ang);
        const double* in = psi0 + (size_t)b * 4 * epad;
        double* io1 = d.psi1 + (size_t)b * 4 * epad;
        double* o4 = psi4 + (size_t)b * 4 * epad;
        const double* fvp = d.fv + bi.p * epad;
        double v[4] = {0., 0., 0., 0.};
        for (int e = lane; e < epad; e += 32) {
            const double hv0 = d.hvac[e], hv1 = d.hvac[epad + e];
            const Psi x = load_psi(in, epad, e);
            double C, S;
            const double a00 = hv0 + g1.h00b, a01 = hv1 + g1.h01rb;
            su2_coeffs(a00, a01, g1.h01i, dl1, C, S);
            const Psi ya = su2_apply(C, S, a00, a01, g1.h01i, x);
            const Psi p1 = load_psi(io1, epad, e);
            Psi avg;
            avg.ar = (ya.ar + p1.ar) * .5;
            avg.ai = (ya.ai + p1.ai) * .5;
            avg.br = (ya.br + p1.br) * .5;
            avg.bi = (ya.bi + p1.bi) * .5;
            store_psi(io1, epad, e, avg);
            const double b00 = hv0 + g3.h00b, b01 = hv1 + g3.h01rb;
            su2_coeffs(b00, b01, g3.h01i, dl1, C, S);
            const Psi y4 = su2_apply(C, S, b00, b01, g3.h01i, x);
            store_psi(o4, epad, e, y4);
            acc_rho(y4, fvp[e], v[0], v[1], v[2]);
        }
        v[0] *= .5;
        warp_reduce_scatter<4>(v, lane);
        if (myv < 3) add_moment<GEOM>(d, v[0], comp_of(myv), 2, bi, acc);
    }
    if (!block_and_grid_reduce<K>(d, PH_B, 8, 3, acc, 0., false, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) ctl->JB4[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        ctl->JB4[k * 4 + comp_of(v)] = s_out[threadIdx.x];
    }
}

// ------------------------------------------------------------------ phase C

// S10/S11 (psi3' = U(h4, dl2, hm(r+dr)) psi3; psi4 <- (psi3' + psi4)/2), the
// error sweep NBeam::calcErrHvv against psi1 (src/NBeam.cpp:903-938) with the
// max over beams (src/Nmr.cpp:195-206), and the moments of the candidate.
// Under device control the last block also runs the step controller of
// src/Nmr.cpp:227-249.
template <int GEOM>
__global__ void __launch_bounds__(256) k_phaseC(Dev d)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    double* __restrict__ psi4 = ctl->psi4;
    double* __restrict__ S4 = ctl->S4;
    const double hm_rdr = ctl->hm[2];
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + (threadIdx.x >> 5), tw = gridDim.x * nw;
    const int epad = d.epad;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.;
    double mx = -1.0;
    const int myv = lane >> 3;  // 0: error, 1..3: density components 0, 2, 3
    for (int b = gw; b < d.nbeams; b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        const BeamH g = beam_offsets<GEOM>(d, ctl->JB4, 2, hm_rdr, bi);
        const double dl2 = geo(d, 3, 2, bi.ang);
        double* io3 = d.psi3 + (size_t)b * 4 * epad;
        double* io4 = psi4 + (size_t)b * 4 * epad;
        const double* p1b = d.psi1 + (size_t)b * 4 * epad;
        const double* fvp = d.fv + bi.p * epad;
        double v[4] = {0., 0., 0., 0.};
        for (int e = lane; e < epad; e += 32) {
            const double a00 = d.hvac[e] + g.h00b, a01 = d.hvac[epad + e] + g.h01rb;
            const Psi x3 = load_psi(io3, epad, e);
            double C, S;
            su2_coeffs(a00, a01, g.h01i, dl2, C, S);
            const Psi y3 = su2_apply(C, S, a00, a01, g.h01i, x3);
            if (d.debug_psi3) store_psi(io3, epad, e, y3);
            const Psi x4 = load_psi(io4, epad, e);
            Psi c;
            c.ar = (y3.ar + x4.ar) * .5;
            c.ai = (y3.ai + x4.ai) * .5;
            c.br = (y3.br + x4.br) * .5;
            c.bi = (y3.bi + x4.bi) * .5;
            store_psi(io4, epad, e, c);
            const Psi r1 = load_psi(p1b, epad, e);
            const double f = fvp[e];
            const double e0 = c.ar - r1.ar, e1 = c.ai - r1.ai, e2 = c.br - r1.br, e3 = c.bi - r1.bi;
            v[0] = fma((e0 * e0 + e1 * e1) + (e2 * e2 + e3 * e3), f, v[0]);
            acc_rho(c, f, v[1], v[2], v[3]);
        }
        v[1] *= .5;
        warp_reduce_scatter<4>(v, lane);
        if (myv == 0) mx = fmax(mx, v[0]);
        else add_moment<GEOM>(d, v[0], comp_of(myv - 1), 2, bi, acc);
        // per-beam moments of the candidate (the reference's hSumMat of psi4)
        if ((lane & 7) == 0) {
            if (myv == 0) S4[(size_t)b * 4 + 1] = 0.;
            else S4[(size_t)b * 4 + comp_of(myv - 1)] = v[0];
        }
    }
    // lanes 8..31 hold moments of slots 1..3; shift them to slots 0..2 for the block reduction
    double accs[K];
#pragma unroll
    for (int k = 0; k < K; ++k) accs[k] = __shfl_down_sync(kFull, acc[k], 8);
    if (!block_and_grid_reduce<K>(d, PH_C, 8, 3, accs, mx, true, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) ctl->JC[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        ctl->JC[k * 4 + comp_of(v)] = s_out[threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double me = sqrt(s_out[31]);
        ctl->max_err = me;
        if (d.device_control) step_control(d, ctl, me);
    }
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
        for (int e = lane; e < epad; e += 32) acc_rho(load_psi(in, epad, e), fvp[e], v[1], v[2], v[3]);
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
    constexpr int K = NK<GEOM>::K;
    // conditional: only after a renormalisation flagged by the step controller
    // (the mixed path refreshes J0 from the renormalised state); the last block
    // clears the flag once every block has passed this check.
    if (conditional && !d.ctl->renorm_due) return;
    const double* __restrict__ S = Sarg ? Sarg : d.ctl->S0;  // null: the cached sums of psi0
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    // lane owns beams gtid, gtid + nthreads, ...; every lane accumulates all 3*K slots
    double acc3[3][K];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < K; ++k) acc3[i][k] = 0.;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.nbeams; b += gridDim.x * blockDim.x) {
        const BeamIdx bi = decode_beam(d, b);
#pragma unroll
        for (int i = 0; i < 3; ++i) add_moment<GEOM>(d, S[(size_t)b * 4 + comp_of(i)], comp_of(i), pt, bi, acc3[i]);
    }
    // reduce 3*K values over the warp: lane l ends with slot l / (32/16)
    double v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = 0.;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < K; ++k) v[i * K + k] = acc3[i][k];
    const int lane = threadIdx.x & 31;
    warp_reduce_scatter<16>(v, lane);
    // slot s = lane/2 = i*K + k; present as a K-vector per slot i via the generic reducer
    double one[K];
#pragma unroll
    for (int k = 0; k < K; ++k) one[k] = 0.;
    // lanes with (lane % 2 == 0) own slot lane/2; re-pack as value v=i (<3) with K moments
    // by having lane 2*(i*K) gather its K neighbours' slots.
#pragma unroll
    for (int k = 0; k < K; ++k) one[k] = __shfl_sync(kFull, v[0], (lane & ~((2 * K) - 1)) + 2 * k);
    // group leaders are lanes 2*K*i, i.e. G = 2K lanes per value
    if (!block_and_grid_reduce<K>(d, PH_MOM, 2 * K, 3, one, 0., false, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) Jout[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int i = threadIdx.x / K, k = threadIdx.x % K;
        Jout[k * 4 + comp_of(i)] = s_out[threadIdx.x];
    }
    if (conditional && threadIdx.x == 0) d.ctl->renorm_due = 0;
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

}  // namespace

int max_phase_blocks(int nbeams, int threads)
{
    const int warps = threads / 32;
    const int need = (nbeams + warps - 1) / warps;
    return std::max(1, std::min(need, 152 * 16));
}

Shape default_shape(int nbeams, int epad)
{
    (void)epad;
    Shape s;
    s.threads = 256;
    s.blocks = max_phase_blocks(nbeams, s.threads);
    return s;
}

void launch_geometry(const Dev& d, cudaStream_t st)
{
    const int t = 128;
    k_geometry<<<(d.A + t - 1) / t, t, 0, st>>>(d);
}

void launch_esum(const Dev& d, const double* psi, double* S, cudaStream_t st)
{
    k_esum<<<max_phase_blocks(d.nbeams, 256), 256, 0, st>>>(d, psi, S);
}

void launch_moments(const Dev& d, const double* S, int pt, double* Jout, cudaStream_t st, int conditional)
{
    const int t = 256;
    const int blocks = std::max(1, std::min((d.nbeams + t - 1) / t, 152 * 4));
    if (d.geom == 0) k_moments<0><<<blocks, t, 0, st>>>(d, S, pt, Jout, conditional);
    else k_moments<1><<<blocks, t, 0, st>>>(d, S, pt, Jout, conditional);
}

void launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st)
{
    if (d.geom == 0) {
        if (phase == PH_A) k_phaseA<0><<<sh.blocks, sh.threads, 0, st>>>(d);
        else if (phase == PH_B) k_phaseB<0><<<sh.blocks, sh.threads, 0, st>>>(d);
        else k_phaseC<0><<<sh.blocks, sh.threads, 0, st>>>(d);
    } else {
        if (phase == PH_A) k_phaseA<1><<<sh.blocks, sh.threads, 0, st>>>(d);
        else if (phase == PH_B) k_phaseB<1><<<sh.blocks, sh.threads, 0, st>>>(d);
        else k_phaseC<1><<<sh.blocks, sh.threads, 0, st>>>(d);
    }
}

void launch_accept(const Dev& d, cudaStream_t st) { k_accept<<<1, 1, 0, st>>>(d); }

void launch_hvv_eval(const Dev& d, const double* J, int pt, double* hvv, cudaStream_t st)
{
    const int n = d.A * d.P, t = 128;
    if (d.geom == 0) k_hvv_eval<0><<<(n + t - 1) / t, t, 0, st>>>(d, J, pt, hvv);
    else k_hvv_eval<1><<<(n + t - 1) / t, t, 0, st>>>(d, J, pt, hvv);
}

}  // namespace xf
