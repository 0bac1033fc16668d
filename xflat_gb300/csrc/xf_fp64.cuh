// FP64 per-phase kernel bodies (MA and MAA), shared by the single-simulation
// kernels (xf_kernels.cu) and the batched kernels (xf_batch.cu).  A body
// processes beams first, first + stride, ... with one warp per beam and
// reduces its moments over the RedTarget group.
#pragma once
#include "xf_common.cuh"

namespace xf {
namespace fp64 {

using namespace detail;

constexpr double kSeriesT = 0.25;

// cos(sqrt(t)) and sin(sqrt(t))/sqrt(t) for 0 <= t <= kSeriesT, degree 7 in t
// (times Q, 1 or 1/2: see su2_coeffs).  Truncation error below 7.3e-19 (cos)
// and 4.3e-20 (sinc) at t = 0.25.
template <int Q2>
__device__ __forceinline__ void series_cs(double t, double& c, double& s)
{
    constexpr double q = Q2 ? 0.5 : 1.0;
    c = q * (-1.0 / 87178291200.0);
    c = fma(c, t, q * (1.0 / 479001600.0));
    c = fma(c, t, q * (-1.0 / 3628800.0));
    c = fma(c, t, q * (1.0 / 40320.0));
    c = fma(c, t, q * (-1.0 / 720.0));
    c = fma(c, t, q * (1.0 / 24.0));
    c = fma(c, t, q * -0.5);
    c = fma(c, t, q);
    s = q * (-1.0 / 1307674368000.0);
    s = fma(s, t, q * (1.0 / 6227020800.0));
    s = fma(s, t, q * (-1.0 / 39916800.0));
    s = fma(s, t, q * (1.0 / 362880.0));
    s = fma(s, t, q * (-1.0 / 5040.0));
    s = fma(s, t, q * (1.0 / 120.0));
    s = fma(s, t, q * (-1.0 / 6.0));
    s = fma(s, t, q);
}

// Coefficients (C, S) of U = C - i S H for H = [[h00, h01],[h01*, -h00]],
// h01 = h01r + i h01i, over the path length dl: C = cos(lambda dl),
// S = sin(lambda dl)/lambda, lambda = |H| (src/NBeam.cpp:366-369).
//
// The series degree is chosen per warp: when t is small in every lane (the
// common case, t <= 1e-3 along the whole bulb run) the truncation after t^2,
// t^3 or t^4 is already below a quarter ulp (t^3/6! <= 1.2e-17 for t <= 2e-5,
// t^4/8! <= 2.5e-17 for t <= 1e-3, t^5/10! <= 2.8e-17 for t <= 1e-2).  The
// thresholds are compared as bit patterns (t >= 0), on the integer pipe.
// Must be called by all 32 lanes of the warp.
//
// With Q2 set the coefficients come out halved, exactly (every constant of the
// series is halved, and binary scaling commutes with rounding): U/2 psi then
// costs nothing extra, and the averaging stages (S4/S5, S10/S11), which form
// (U psi + psi')/2, become a plain sum of halves with the same bits as before.
constexpr long long kT2 = 0x3EF4F8B588E368F1LL;  // 2e-5
constexpr long long kT3 = 0x3F50624DD2F1A9FCLL;  // 1e-3
constexpr long long kT4 = 0x3F847AE147AE147BLL;  // 1e-2

// Per-beam constants of one propagator: h01i (not energy dependent) squared,
// dl^2, and the sinc polynomial's first coefficients times dl, so that the
// degree-2 and degree-3 branches of su2_coeffs need no multiplication by dl
// per bin (2 + 1 + 2 + 2 and 2 + 1 + 3 + 3 FP64 operations).
struct PropK {
    double dl, dl2, h01i2;
    double s0, s1, s2, s3;  // q dl (1, -1/6, 1/120, -1/5040)
};

template <int Q2 = 0>
__device__ __forceinline__ PropK prop_k(double h01i, double dl)
{
    constexpr double q = Q2 ? 0.5 : 1.0;
    PropK p;
    p.dl = dl;
    p.dl2 = dl * dl;
    p.h01i2 = h01i * h01i;
    p.s0 = q * dl;
    p.s1 = (q * (-1.0 / 6.0)) * dl;
    p.s2 = (q * (1.0 / 120.0)) * dl;
    p.s3 = (q * (-1.0 / 5040.0)) * dl;
    return p;
}

template <int Q2 = 0>
__device__ __forceinline__ void su2_coeffs(double h00, double h01r, const PropK& pk, double& C, double& S)
{
    constexpr double q = Q2 ? 0.5 : 1.0;
    const double dl = pk.dl;
    const double lam2 = fma(h00, h00, fma(h01r, h01r, pk.h01i2));
    const double t = lam2 * pk.dl2;
    const long long tb = __double_as_longlong(t);
    if (__all_sync(kFull, tb <= kT2)) {
        C = fma(fma(t, q * (1.0 / 24.0), q * -0.5), t, q);
        S = fma(fma(t, pk.s2, pk.s1), t, pk.s0);
    } else if (__all_sync(kFull, tb <= kT3)) {
        C = fma(fma(fma(t, q * (-1.0 / 720.0), q * (1.0 / 24.0)), t, q * -0.5), t, q);
        S = fma(fma(fma(t, pk.s3, pk.s2), t, pk.s1), t, pk.s0);
    } else if (__all_sync(kFull, tb <= kT4)) {
        C = fma(fma(fma(fma(t, q * (1.0 / 40320.0), q * (-1.0 / 720.0)), t, q * (1.0 / 24.0)), t, q * -0.5), t, q);
        S = fma(fma(fma(fma(t, q * (1.0 / 362880.0), q * (-1.0 / 5040.0)), t, q * (1.0 / 120.0)), t, q * (-1.0 / 6.0)),
                t, q) * dl;
    } else if (t <= kSeriesT) {
        double s;
        series_cs<Q2>(t, C, s);
        S = s * dl;
    } else {
        const double lam = sqrt(lam2);
        double sn, cs;
        sincos(lam * dl, &sn, &cs);
        C = cs * q;
        S = (sn / lam) * q;
    }
}

// A bin of a beam state: psi = (a, b) = (ar + i ai, br + i bi).
struct Psi {
    double ar, ai, br, bi;
};

// psi' = U psi with the matrix entries of src/NBeam.cpp:371-392, written
// U psi = C psi + S w with w = -i sigma(h) psi: w costs 12 FP64 operations
// (products fused into FMAs) and U psi then 8, against 23 for the entries
// grouped as in the reference, and two propagators sharing h (phase A's two
// path lengths) share w.
__device__ __forceinline__ Psi su2_w(double h00, double h01r, double h01i, const Psi& x)
{
    Psi w;
    w.ar = fma(h00, x.ai, fma(h01i, x.br, h01r * x.bi));
    w.ai = fma(-h00, x.ar, fma(h01i, x.bi, -h01r * x.br));
    w.br = fma(-h01i, x.ar, fma(h01r, x.ai, -h00 * x.bi));
    w.bi = fma(-h01i, x.ai, fma(-h01r, x.ar, h00 * x.br));
    return w;
}

// C x + S w + a in one FMA chain per component (the averages of S4/S5 and
// S10/S11 without a separate addition; other rounding than su2_apply_w + a).
__device__ __forceinline__ Psi su2_apply_w_add(double C, double S, const Psi& x, const Psi& w, const Psi& a)
{
    Psi y;
    y.ar = fma(C, x.ar, fma(S, w.ar, a.ar));
    y.ai = fma(C, x.ai, fma(S, w.ai, a.ai));
    y.br = fma(C, x.br, fma(S, w.br, a.br));
    y.bi = fma(C, x.bi, fma(S, w.bi, a.bi));
    return y;
}

__device__ __forceinline__ Psi su2_apply_w(double C, double S, const Psi& x, const Psi& w)
{
    Psi y;
    y.ar = fma(C, x.ar, S * w.ar);
    y.ai = fma(C, x.ai, S * w.ai);
    y.br = fma(C, x.br, S * w.br);
    y.bi = fma(C, x.bi, S * w.bi);
    return y;
}

// Accumulates fv * rho(psi) (first row of the density matrix, src/NBeam.cpp:314-322);
// component 0 is accumulated without the factor 1/2, applied once per beam.
template <int FUSE = 0>
__device__ __forceinline__ void acc_rho(const Psi& x, double fv, double& s0, double& s2, double& s3)
{
    // FUSE: the four squares in one FMA chain (one operation fewer, other rounding)
    const double d0 = FUSE ? fma(x.ar, x.ar, fma(x.ai, x.ai, -fma(x.br, x.br, x.bi * x.bi)))
                           : (x.ar * x.ar + x.ai * x.ai) - (x.br * x.br + x.bi * x.bi);
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

// ------------------------------------------------------------------ phase A

// S1 (H of psi0 from the cached moments), S2 and S6 (two sweeps sharing H0),
// and the moments of psi1 at point 2 (S3) and of psi3 at point 1 (S7).
template <int GEOM>
__device__ inline void phaseA_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const double* __restrict__ psi0 = ctl->psi0;
    const double hm = ctl->hm[0];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    double acc = 0.;  // lane-split moment accumulator (add_moment_lane)
    const int myv = lane >> 2;  // value slot owned after an 8-way reduce-scatter
    const int stage = ctl->stage_kind;  // an output record waits for psi0 (device control with files)
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        if (stage) stage_beam(d, ctl, stage, b, lane, psi0, nullptr, nullptr);
        // lane-parallel set-up: lanes 0-2 the offsets of H0, lanes 3-4 dl0, dl1
        double sv = 0.;
        if (lane < 3) sv = beam_offset_k<GEOM>(d, ctl->J0, 0, hm, bi, lane);
        else if (lane < 5) sv = geo(d, 3, lane - 3, bi.ang);
        const BeamH h = shfl_beamh(sv, 0);
        const double dl0 = __shfl_sync(kFull, sv, 3), dl1 = __shfl_sync(kFull, sv, 4);
        const PropK pk0 = prop_k(h.h01i, dl0);
        const PropK pk1 = prop_k<1>(h.h01i, dl1);  // MAA only
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
                su2_coeffs(h00, h01r, pk0, C0, S0);
                // the halved U(dl1) (psi1 is stored halved, see su2_coeffs):
                // C1/2 = C0^2 - 1/2 and S1/2 = C0 S0, exactly half of 2C0^2 - 1 and 2 C0 S0
                C1 = fma(C0, C0, -0.5);
                S1 = C0 * S0;
            } else {
                su2_coeffs<1>(h00, h01r, pk1, C1, S1);
                su2_coeffs(h00, h01r, pk0, C0, S0);
            }
            const Psi w = su2_w(h00, h01r, h.h01i, x);
            const Psi y1 = su2_apply_w(C1, S1, x, w);
            const Psi y3 = su2_apply_w(C0, S0, x, w);
            store_psi(o1, epad, e, y1);
            store_psi(o3, epad, e, y3);
            const double f = fvp[e];
            acc_rho(y1, f, v[0], v[1], v[2]);
            acc_rho(y3, f, v[3], v[4], v[5]);
        }
        // psi1 was accumulated halved: its sums are a quarter (exactly) of psi1's
        v[0] *= 2.;
        v[1] *= 4.;
        v[2] *= 4.;
        v[3] *= .5;
        warp_reduce_scatter<8>(v, lane);
        if (myv < 3) add_moment_lane<GEOM>(d, v[0], comp_of(myv), 2, bi, lane & 3, acc);
        else if (myv < 6) add_moment_lane<GEOM>(d, v[0], comp_of(myv - 3), 1, bi, lane & 3, acc);
    }
    if (!group_reduce_split<K>(rt, 4, 6, acc, 0., false, s_warp, s_out)) return;
    stage_done(ctl);
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
template <int GEOM, int FUSE = 1>
__device__ inline void phaseB_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const double* __restrict__ psi0 = ctl->psi0;
    double* __restrict__ psi4 = ctl->psi4;
    const double hm_rdr = ctl->hm[2], hm_rdr2 = ctl->hm[1];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    double acc = 0.;  // lane-split moment accumulator (add_moment_lane)
    const int myv = lane >> 3;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up: lanes 0-2 the offsets of H1, 3-5 those of H3, lane 6 dl1
        double sv = 0.;
        if (lane < 3) sv = beam_offset_k<GEOM>(d, ctl->JA1, 2, hm_rdr, bi, lane);
        else if (lane < 6) sv = beam_offset_k<GEOM>(d, ctl->JA3, 1, hm_rdr2, bi, lane - 3);
        else if (lane == 6) sv = geo(d, 3, 1, bi.ang);
        const BeamH g1 = shfl_beamh(sv, 0), g3 = shfl_beamh(sv, 3);
        const double dl1 = __shfl_sync(kFull, sv, 6);
        const PropK pka = prop_k<1>(g1.h01i, dl1), pkb = prop_k<1>(g3.h01i, dl1);
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
            // S4/S5: (U psi0 + psi1)/2 as U/2 psi0 + psi1/2 (psi1 stored halved by phase A)
            su2_coeffs<1>(a00, a01, pka, C, S);
            const Psi p1 = load_psi(io1, epad, e);
            Psi avg;
            if (FUSE) {
                avg = su2_apply_w_add(C, S, x, su2_w(a00, a01, g1.h01i, x), p1);
            } else {
                const Psi ya = su2_apply_w(C, S, x, su2_w(a00, a01, g1.h01i, x));
                avg.ar = ya.ar + p1.ar;
                avg.ai = ya.ai + p1.ai;
                avg.br = ya.br + p1.br;
                avg.bi = ya.bi + p1.bi;
            }
            store_psi(io1, epad, e, avg);
            const double b00 = hv0 + g3.h00b, b01 = hv1 + g3.h01rb;
            // S8, stored halved for the average of S10/S11
            su2_coeffs<1>(b00, b01, pkb, C, S);
            const Psi y4 = su2_apply_w(C, S, x, su2_w(b00, b01, g3.h01i, x));
            store_psi(o4, epad, e, y4);
            acc_rho<FUSE>(y4, fvp[e], v[0], v[1], v[2]);
        }
        // psi4 was accumulated halved: its sums are a quarter (exactly) of psi4's
        v[0] *= 2.;
        v[1] *= 4.;
        v[2] *= 4.;
        warp_reduce_scatter<4>(v, lane);
        if (myv < 3) add_moment_lane<GEOM>(d, v[0], comp_of(myv), 2, bi, lane & 7, acc);
    }
    if (!group_reduce_split<K>(rt, 8, 3, acc, 0., false, s_warp, s_out)) return;
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
template <int GEOM, int FUSE = 1>
__device__ inline void phaseC_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    double* __restrict__ psi4 = ctl->psi4;
    double* __restrict__ S4 = ctl->S4;
    const double hm_rdr = ctl->hm[2];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    double acc = 0.;  // lane-split moment accumulator (add_moment_lane)
    double mx = -1.0;
    const int myv = lane >> 3;  // 0: error, 1..3: density components 0, 2, 3
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up: lanes 0-2 the offsets of H4, lane 3 dl2
        double sv = 0.;
        if (lane < 3) sv = beam_offset_k<GEOM>(d, ctl->JB4, 2, hm_rdr, bi, lane);
        else if (lane == 3) sv = geo(d, 3, 2, bi.ang);
        const BeamH g = shfl_beamh(sv, 0);
        const double dl2 = __shfl_sync(kFull, sv, 3);
        const PropK pk = prop_k<1>(g.h01i, dl2);
        double* io3 = d.psi3 + (size_t)b * 4 * epad;
        double* io4 = psi4 + (size_t)b * 4 * epad;
        const double* p1b = d.psi1 + (size_t)b * 4 * epad;
        const double* fvp = d.fv + bi.p * epad;
        double v[4] = {0., 0., 0., 0.};
        for (int e = lane; e < epad; e += 32) {
            const double a00 = d.hvac[e] + g.h00b, a01 = d.hvac[epad + e] + g.h01rb;
            const Psi x3 = load_psi(io3, epad, e);
            double C, S;
            // S10/S11: (U psi3 + psi4)/2 as U/2 psi3 + psi4/2 (psi4 stored halved by phase B)
            su2_coeffs<1>(a00, a01, pk, C, S);
            const Psi w3 = su2_w(a00, a01, g.h01i, x3);
            const Psi x4 = load_psi(io4, epad, e);
            Psi c;
            if (FUSE && !d.debug_psi3) {
                c = su2_apply_w_add(C, S, x3, w3, x4);
            } else {
                const Psi y3 = su2_apply_w(C, S, x3, w3);
                if (d.debug_psi3) {
                    Psi full;
                    full.ar = 2. * y3.ar;
                    full.ai = 2. * y3.ai;
                    full.br = 2. * y3.br;
                    full.bi = 2. * y3.bi;
                    store_psi(io3, epad, e, full);
                }
                c.ar = y3.ar + x4.ar;
                c.ai = y3.ai + x4.ai;
                c.br = y3.br + x4.br;
                c.bi = y3.bi + x4.bi;
            }
            store_psi(io4, epad, e, c);
            const Psi r1 = load_psi(p1b, epad, e);
            const double f = fvp[e];
            const double e0 = c.ar - r1.ar, e1 = c.ai - r1.ai, e2 = c.br - r1.br, e3 = c.bi - r1.bi;
            v[0] = fma((e0 * e0 + e1 * e1) + (e2 * e2 + e3 * e3), f, v[0]);
            acc_rho<FUSE>(c, f, v[1], v[2], v[3]);
        }
        v[1] *= .5;
        warp_reduce_scatter<4>(v, lane);
        if (myv == 0) mx = fmax(mx, v[0]);
        else add_moment_lane<GEOM>(d, v[0], comp_of(myv - 1), 2, bi, lane & 7, acc);
        // per-beam moments of the candidate (the reference's hSumMat of psi4)
        if ((lane & 7) == 0) {
            if (myv == 0) S4[(size_t)b * 4 + 1] = 0.;
            else S4[(size_t)b * 4 + comp_of(myv - 1)] = v[0];
        }
    }
    // lanes 8..31 hold moments of slots 1..3; shift them to slots 0..2 for the block reduction
    const double accs = __shfl_down_sync(kFull, acc, 8);
    if (!group_reduce_split<K>(rt, 8, 3, accs, mx, true, s_warp, s_out)) return;
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

}  // namespace fp64
}  // namespace xf
