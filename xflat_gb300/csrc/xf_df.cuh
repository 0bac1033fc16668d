// Double-float per-phase kernel bodies (MA, MAA and SA geometry): the FP64
// path's stages, with every state, propagator, average and moment carried as
// a pair of FP32 numbers (hi + lo, about 48 significant bits) and computed
// with FP32 error-free transformations instead of on the FP64 pipe, which runs
// at 1/64 of the FP32 rate on this GPU.
//
// The stages, buffers and reductions are those of xf_fp64.cuh: phase A forms
// psi1 = U(h0, dl1) psi0 (stored halved) and psi3 = U(h0, dl0) psi0 with their
// moments, phase B the average of S4/S5 into psi1 and psi4 = U(h3, dl1) psi0
// (halved) with its moments, phase C the average of S10/S11 into the
// candidate, the step error against psi1, the candidate's moments and the
// step controller (src/Nmr.cpp:153-249, src/NBeam.cpp:360-393, 462-514,
// 588-646, 690-736, 903-938).  Each propagator is U = q + (C - 1) - i S
// sigma(h) (q = 1, or 1/2 for the halved forms): C - 1 = t c1(t) and
// S = dl (1 + t s1(t)) with t = |h|^2 dl^2, whose leading constants are
// pairs; when t <= 1e-3 in the whole warp (the bulb run's steps) the rest of
// c1 and s1 is an FP32 tail, which with the FP32 rounding of t in it changes
// C and S by less than 5e-15 (3.1e-15 at t = 1e-3), otherwise the series is
// a pair Horner up to t = 0.25; beyond, the angle |h| dl is reduced by
// multiples of pi/2 in pairs and the remainder's series rotated by the
// quadrant (no FP64 sincos: the first step of a run from 10 km, dl = 1e-3
// km across a matter potential up to 1e4 /km, takes this branch in most bins).
//
// Arithmetic.  Intermediate values are "loose" pairs: the hi parts of
// products and sums are exact error-free transformations (TwoProduct with
// FMA, TwoSum), the lo parts collect the rounding errors and cross terms in
// plain FP32, and a pair is renormalised (Fast2Sum) only where it is stored.
// A lo part is then not necessarily below half an ulp of its hi part, but it
// stays below about 2^-22 of the magnitudes of the operands that formed it,
// so every value keeps an absolute error near 2^-47 of its natural scale (the
// state is O(1), an increment |h| dl); stored states are renormalised and
// exact to 2^-48.  The error-free steps use the _rn intrinsics, which the
// compiler never contracts into FMAs.
//
// The per-beam Hamiltonian offsets are formed in FP64 (a few operations per
// offset, once per beam, lane-parallel) and split into pairs; the vacuum
// term, energy weights and path lengths come from pair tables.  Moments are
// accumulated in pairs, scaled by kappa (add_moment_df), and reduced across
// blocks in FP64.  Every state is stored bin by bin ([beam][ebin][8] floats:
// the four components' hi parts, then their lo parts), psi0 and the candidate
// in the pair buffers the mixed path uses for its rows (sbin_ptr), psi1 and
// psi3 in the FP64 path's buffers (bin_ptr).
#pragma once
#include "xf_mixed.cuh"

namespace xf {
namespace dfp {

using namespace detail;
using mixed::DF;
using mixed::df_add;
using mixed::df_mul;
using mixed::df_value;

// ------------------------------------------------------------------ loose pair arithmetic

__device__ __forceinline__ DF two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return DF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ DF two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}

// Renormalisation (Fast2Sum): exact when |h| >= |l| or h = 0.
__device__ __forceinline__ DF norm(const DF& a)
{
    const float s = __fadd_rn(a.h, a.l);
    return DF{s, __fsub_rn(a.l, __fsub_rn(s, a.h))};
}

__device__ __forceinline__ DF neg(const DF& a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF dscale(float s, const DF& a) { return DF{s * a.h, s * a.l}; }  // s a power of two

// a b (the lo*lo product, 2^-48 of the result, is dropped).
__device__ __forceinline__ DF lmul(const DF& a, const DF& b)
{
    const DF p = two_prod(a.h, b.h);
    return DF{p.h, fmaf(a.h, b.l, fmaf(a.l, b.h, p.l))};
}

// a a.
__device__ __forceinline__ DF lsq(const DF& a)
{
    const DF p = two_prod(a.h, a.h);
    return DF{p.h, fmaf(a.h + a.h, a.l, p.l)};
}

__device__ __forceinline__ DF ladd(const DF& a, const DF& b)
{
    const DF s = two_sum(a.h, b.h);
    return DF{s.h, s.l + (a.l + b.l)};
}

__device__ __forceinline__ DF lsub(const DF& a, const DF& b) { return ladd(a, neg(b)); }

// a + b for |a| >= |b| (Fast2Sum on the hi parts).
__device__ __forceinline__ DF ladd_big(const DF& a, const DF& b)
{
    const float s = __fadd_rn(a.h, b.h);
    return DF{s, __fsub_rn(b.h, __fsub_rn(s, a.h)) + (a.l + b.l)};
}

// a0 b0 + a1 b1.
__device__ __forceinline__ DF ldot2(const DF& a0, const DF& b0, const DF& a1, const DF& b1)
{
    const DF p = two_prod(a0.h, b0.h), q = two_prod(a1.h, b1.h);
    const DF s = two_sum(p.h, q.h);
    const float lo = fmaf(a0.h, b0.l, fmaf(a0.l, b0.h, p.l)) + fmaf(a1.h, b1.l, fmaf(a1.l, b1.h, q.l));
    return DF{s.h, s.l + lo};
}

// a0 b0 + a1 b1 + a2 b2.
__device__ __forceinline__ DF ldot3(const DF& a0, const DF& b0, const DF& a1, const DF& b1, const DF& a2, const DF& b2)
{
    const DF p = two_prod(a0.h, b0.h), q = two_prod(a1.h, b1.h), r = two_prod(a2.h, b2.h);
    const DF s = two_sum(p.h, q.h);
    const DF u = two_sum(s.h, r.h);
    const float lo = fmaf(a0.h, b0.l, fmaf(a0.l, b0.h, p.l)) + fmaf(a1.h, b1.l, fmaf(a1.l, b1.h, q.l)) +
                     fmaf(a2.h, b2.l, fmaf(a2.l, b2.h, r.l));
    return DF{u.h, (s.l + u.l) + lo};
}

__device__ __forceinline__ DF dsplit(double x)
{
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}

struct DF4 {
    DF ar, ai, br, bi;
};

__device__ __forceinline__ DF4 norm4(const DF4& x)
{
    DF4 y;
    y.ar = norm(x.ar);
    y.ai = norm(x.ai);
    y.br = norm(x.br);
    y.bi = norm(x.bi);
    return y;
}

// ------------------------------------------------------------------ propagators

// Propagator coefficients: U = q + cm - i S sigma(h), cm = q (C - 1).
struct DK {
    DF cm, S;
};

// Per-beam constants of a propagator: the path length dl and dl^2, and the
// square of the beam's h01i (pairs).
struct DLen {
    DF dl, dl2;
};

__device__ __forceinline__ DLen dlen(const DF& dl) { return DLen{dl, norm(lsq(dl))}; }
__device__ __forceinline__ DF dsq(const DF& h01i) { return norm(lsq(h01i)); }

// c1 = (cos(sqrt t) - 1)/t and s1 = (sin(sqrt t)/sqrt t - 1)/t: the Taylor
// coefficients from k = 1 on (c: (-1)^k / (2k)!, s: (-1)^k / (2k+1)!), each
// as a pair.
struct DConst {
    float h, l;
};
#define XF_DFC(v) DConst{(float)(v), (float)((v) - (double)(float)(v))}
__constant__ DConst kDC[8] = {XF_DFC(-1.0 / 2.0),      XF_DFC(1.0 / 24.0),        XF_DFC(-1.0 / 720.0),
                              XF_DFC(1.0 / 40320.0),   XF_DFC(-1.0 / 3628800.0),  XF_DFC(1.0 / 479001600.0),
                              XF_DFC(-1.0 / 87178291200.0), XF_DFC(1.0 / 20922789888000.0)};
__constant__ DConst kDS[8] = {XF_DFC(-1.0 / 6.0),         XF_DFC(1.0 / 120.0),          XF_DFC(-1.0 / 5040.0),
                              XF_DFC(1.0 / 362880.0),     XF_DFC(-1.0 / 39916800.0),    XF_DFC(1.0 / 6227020800.0),
                              XF_DFC(-1.0 / 1307674368000.0), XF_DFC(1.0 / 355687428096000.0)};
#undef XF_DFC
constexpr float kS1h = (float)(-1.0 / 6.0);
constexpr float kS1l = (float)(-1.0 / 6.0 - (double)(float)(-1.0 / 6.0));

__device__ __forceinline__ DF dconst(const DConst& c) { return DF{c.h, c.l}; }

// pi/2 as three floats (their sum is pi/2 to 1.1e-23; each product with an
// integer n < 2^24 is an exact pair), and 2/pi rounded to FP32.
constexpr float kPio2a = 0x1.921fb6p+0f, kPio2b = -0x1.777a5cp-25f, kPio2c = -0x1.ee59dap-50f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;

// Square root of a normalised pair a > 0: the FP32 root s and one correction
// (a - s^2) / 2s from the residual, whose leading term an FMA forms exactly
// (Dekker's double-length square root, 1971).
__device__ __forceinline__ DF dsqrt(const DF& a)
{
    const float s = __fsqrt_rn(a.h);
    const float e = fmaf(-s, s, a.h) + a.l;
    return norm(DF{s, __fdividef(e, s + s)});
}

// 1/a for a normalised pair a != 0: the FP32 reciprocal r and one Newton
// correction r (1 - a r), the residual formed with FMAs.
__device__ __forceinline__ DF drcp(const DF& a)
{
    const float r = __frcp_rn(a.h);
    const float e = fmaf(-a.l, r, fmaf(-a.h, r, 1.f));
    return norm(DF{r, r * e});
}

// Coefficients of U over dl for the bin Hamiltonian (h00, h01r, beam h01i).
// Must be called by all 32 lanes of the warp (warp-uniform series choice).
template <int Q2>
__device__ __forceinline__ DK dcoeffs(const DF& h00, const DF& h01r, const DF& h01i2, const DLen& bm)
{
    constexpr float q = Q2 ? 0.5f : 1.f;
    const DF lam2 = ladd(ladd(lsq(h00), lsq(h01r)), h01i2);
    const DF t = lmul(lam2, bm.dl2);
    DK k;
    if (__all_sync(kFull, t.h <= 1e-3f)) {
        // c1 = -1/2 + th (1/24 - th/720) and s1 = -1/6 + th (1/120 - th/5040):
        // the tails are below 4.2e-5 and 8.4e-6, rounded to 2^-24 of that and
        // computed from t rounded to FP32; the next terms, t^3/40320 and
        // t^3/362880, are below 2.5e-14 and 2.8e-15 of c1 and s1; all of it
        // enters C and S times t
        const float th = t.h;
        const float ct = th * fmaf(th, -1.f / 720.f, 1.f / 24.f);
        const float st = th * fmaf(th, -1.f / 5040.f, 1.f / 120.f);
        // cm = q t c1 = -q t / 2 + q t ct, renormalised: its lo part (up to
        // 8e-5 of the hi part before) enters FP32 products with the state
        k.cm = norm(DF{-0.5f * q * t.h, fmaf(q * t.h, ct, q * fmaf(t.l, ct, -0.5f * t.l))});
        // S = q dl (1 + t s1), |t s1| <= 1.7e-4; s1 = -1/6 + st renormalised
        const DF s1 = two_sum(kS1h, st);
        const DF u = lmul(t, DF{s1.h, s1.l + kS1l});
        k.S = dscale(q, ladd_big(bm.dl, lmul(bm.dl, u)));
    } else if (t.h <= 0.25f) {
        // pair Horner to degree 7 in t (truncation below 1e-18 at t = 0.25)
        const DF tn = norm(t);
        DF c1 = dconst(kDC[6]), s1 = dconst(kDS[6]);
#pragma unroll
        for (int i = 5; i >= 0; --i) {
            c1 = df_add(dconst(kDC[i]), df_mul(c1, tn));
            s1 = df_add(dconst(kDS[i]), df_mul(s1, tn));
        }
        k.cm = dscale(q, df_mul(tn, c1));
        const DF dl = norm(bm.dl);
        k.S = dscale(q, df_add(dl, df_mul(dl, df_mul(tn, s1))));
    } else {
        // theta = sqrt(t) = |h| dl less the nearest multiple n pi/2 (Cody and
        // Waite's reduction with the three-float pi/2, in pairs: the remainder
        // keeps theta's own absolute precision, 2^-47 theta), |r| <= pi/4 +
        // 1e-3; cos r - 1 and sin r from the pair series to degree 8 in r^2
        // (truncation below 4e-18), rotated by the quadrant n mod 4:
        // cos(theta) - 1 and sin(theta), and S = q sin(theta) dl / theta
        const DF th = dsqrt(norm(t));
        const float n = rintf(th.h * kTwoOverPi);
        DF r = df_add(th, neg(two_prod(n, kPio2a)));
        r = df_add(r, neg(two_prod(n, kPio2b)));
        r = df_add(r, DF{-n * kPio2c, 0.f});
        const DF u = df_mul(r, r);
        DF c1 = dconst(kDC[7]), s1 = dconst(kDS[7]);
#pragma unroll
        for (int i = 6; i >= 0; --i) {
            c1 = df_add(dconst(kDC[i]), df_mul(c1, u));
            s1 = df_add(dconst(kDS[i]), df_mul(s1, u));
        }
        const DF cr = df_mul(u, c1);                          // cos r - 1
        const DF sr = df_add(r, df_mul(r, df_mul(u, s1)));  // sin r
        const int quad = (int)n & 3;
        DF cm, sn;
        if (quad == 0) {
            cm = cr;
            sn = sr;
        } else if (quad == 1) {
            cm = df_add(DF{-1.f, 0.f}, neg(sr));
            sn = df_add(DF{1.f, 0.f}, cr);
        } else if (quad == 2) {
            cm = df_add(DF{-2.f, 0.f}, neg(cr));
            sn = neg(sr);
        } else {
            cm = df_add(DF{-1.f, 0.f}, sr);
            sn = neg(df_add(DF{1.f, 0.f}, cr));
        }
        k.cm = dscale(q, cm);
        k.S = dscale(q, df_mul(df_mul(sn, norm(bm.dl)), drcp(th)));
    }
    return k;
}

// w = -i sigma(h) x (the form of su2_w in xf_fp64.cuh).
__device__ __forceinline__ DF4 dsig_w(const DF& h00, const DF& h01r, const DF& h01i, const DF4& x)
{
    DF4 w;
    w.ar = ldot3(h00, x.ai, h01i, x.br, h01r, x.bi);
    w.ai = ldot3(neg(h00), x.ar, h01i, x.bi, neg(h01r), x.br);
    w.br = ldot3(neg(h01i), x.ar, h01r, x.ai, neg(h00), x.bi);
    w.bi = ldot3(neg(h01i), x.ai, neg(h01r), x.ar, h00, x.br);
    return w;
}

// y = U x = q x + cm x + S w (loose; the stores renormalise).
__device__ __forceinline__ DF4 dapply(float q, const DK& k, const DF4& x, const DF4& w)
{
    DF4 y;
    y.ar = ladd(dscale(q, x.ar), ldot2(k.cm, x.ar, k.S, w.ar));
    y.ai = ladd(dscale(q, x.ai), ldot2(k.cm, x.ai, k.S, w.ai));
    y.br = ladd(dscale(q, x.br), ldot2(k.cm, x.br, k.S, w.br));
    y.bi = ladd(dscale(q, x.bi), ldot2(k.cm, x.bi, k.S, w.bi));
    return y;
}

// a0 b0 + a1 b1 + a2 b2 + a3 b3.
__device__ __forceinline__ DF ldot4(const DF& a0, const DF& b0, const DF& a1, const DF& b1, const DF& a2, const DF& b2,
                                   const DF& a3, const DF& b3)
{
    const DF p = two_prod(a0.h, b0.h), q = two_prod(a1.h, b1.h), r = two_prod(a2.h, b2.h), u = two_prod(a3.h, b3.h);
    const DF s1 = two_sum(p.h, q.h);
    const DF s2 = two_sum(r.h, u.h);
    const DF s = two_sum(s1.h, s2.h);
    const float lo = (fmaf(a0.h, b0.l, fmaf(a0.l, b0.h, p.l)) + fmaf(a1.h, b1.l, fmaf(a1.l, b1.h, q.l))) +
                     (fmaf(a2.h, b2.l, fmaf(a2.l, b2.h, r.l)) + fmaf(a3.h, b3.l, fmaf(a3.l, b3.h, u.l)));
    return DF{s.h, ((s1.l + s2.l) + s.l) + lo};
}

// y = U x = (q + cm) x - i S sigma(h) x as one four-term sum per component,
// with S folded into the Hamiltonian (z = S h, three products per bin): the
// form for a propagator that shares nothing with another.
__device__ __forceinline__ DF4 dapply_z(float q, const DK& k, const DF& h00, const DF& h01r, const DF& h01i,
                                        const DF4& x)
{
    const DF c = ladd_big(DF{q, 0.f}, k.cm);
    const DF z0 = lmul(k.S, h00), zr = lmul(k.S, h01r), zi = lmul(k.S, h01i);
    DF4 y;
    y.ar = ldot4(c, x.ar, z0, x.ai, zi, x.br, zr, x.bi);
    y.ai = ldot4(c, x.ai, neg(z0), x.ar, zi, x.bi, neg(zr), x.br);
    y.br = ldot4(c, x.br, neg(zi), x.ar, zr, x.ai, neg(z0), x.bi);
    y.bi = ldot4(c, x.bi, neg(zi), x.ai, neg(zr), x.ar, z0, x.br);
    return y;
}

__device__ __forceinline__ DF4 dadd4(const DF4& a, const DF4& b)
{
    DF4 c;
    c.ar = ladd(a.ar, b.ar);
    c.ai = ladd(a.ai, b.ai);
    c.br = ladd(a.br, b.br);
    c.bi = ladd(a.bi, b.bi);
    return c;
}

// Accumulates fv * rho(x) (acc_rho of xf_fp64.cuh: component 0 without the 1/2).
__device__ __forceinline__ void dacc_rho(const DF4& x, const DF& fv, DF& s0, DF& s2, DF& s3)
{
    const DF d0 = lsub(ladd(lsq(x.ar), lsq(x.ai)), ladd(lsq(x.br), lsq(x.bi)));
    const DF d2 = ldot2(x.ar, x.br, x.ai, x.bi);
    const DF d3 = ldot2(x.ai, x.br, neg(x.ar), x.bi);
    // the sums stay normalised, so their lo parts round at 2^-48 of the sums
    s0 = norm(ladd(s0, lmul(d0, fv)));
    s2 = norm(ladd(s2, lmul(d2, fv)));
    s3 = norm(ladd(s3, lmul(d3, fv)));
}

__device__ __forceinline__ DF shfl_df(const DF& v, int src)
{
    return DF{__shfl_sync(kFull, v.h, src), __shfl_sync(kFull, v.l, src)};
}

__device__ __forceinline__ DF hv_df(const Dev& d, int k, int e)
{
    return DF{d.hvf[k * d.epad + e], d.hvf_lo[k * d.epad + e]};
}

__device__ __forceinline__ DF fv_df(const Dev& d, int p, int e)
{
    return DF{d.fvf[p * d.epad + e], d.fvf_lo[p * d.epad + e]};
}

// Per-beam sums of a warp, renormalised, then reduce-scattered (each group of
// 32/NV lanes holds the warp total of one value).
template <int NV>
__device__ __forceinline__ void reduce_sums(DF (&v)[NV], int lane)
{
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = norm(v[i]);
    mixed::df_reduce_scatter<NV>(v, lane);
}

// psi1 / psi3, which only this path reads, in the FP64 path's buffers laid
// out bin by bin: [beam][ebin][8] floats, the four components' hi parts then
// their lo parts, so a lane moves a bin with two 16-byte accesses and a warp
// 1 KB of contiguous memory.
__device__ __forceinline__ float* bin_ptr(double* buf, int epad, int b, int e)
{
    return reinterpret_cast<float*>(buf) + ((size_t)b * epad + e) * 8;
}

__device__ __forceinline__ DF4 load_bin(const float* __restrict__ p)
{
    const float4 h = *reinterpret_cast<const float4*>(p), l = *reinterpret_cast<const float4*>(p + 4);
    DF4 x;
    x.ar = DF{h.x, l.x};
    x.ai = DF{h.y, l.y};
    x.br = DF{h.z, l.z};
    x.bi = DF{h.w, l.w};
    return x;
}

// Stores a renormalised x.
__device__ __forceinline__ void store_bin_raw(float* __restrict__ p, const DF4& x)
{
    *reinterpret_cast<float4*>(p) = make_float4(x.ar.h, x.ai.h, x.br.h, x.bi.h);
    *reinterpret_cast<float4*>(p + 4) = make_float4(x.ar.l, x.ai.l, x.br.l, x.bi.l);
}

__device__ __forceinline__ void store_bin(float* __restrict__ p, const DF4& x) { store_bin_raw(p, norm4(x)); }

// Intermediate states (psi1, psi3 and the halved psi4, read within the same
// iteration) are stored renormalised as well: storing them as computed saved
// 0.6 % on GB300, not worth the looser pairs.
__device__ __forceinline__ void store_mid_bin(float* __restrict__ p, const DF4& x) { store_bin(p, x); }

// psi0 and the candidate: the same bin layout in their own buffers
// (pair_at in xf_common.cuh reads it for the output and sum kernels).
__device__ __forceinline__ float* sbin_ptr(float* buf, int epad, int b, int e)
{
    return buf + ((size_t)b * epad + e) * 8;
}
__device__ __forceinline__ const float* sbin_ptr(const float* buf, int epad, int b, int e)
{
    return buf + ((size_t)b * epad + e) * 8;
}

__device__ __forceinline__ void prefetch_bin(const float* p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// ------------------------------------------------------------------ phase A

template <int GEOM>
__device__ inline void phaseA_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const float* __restrict__ s0 = ctl->m0hi;
    const double hm = ctl->hm[0];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};  // lane-split moment accumulator (add_moment_df)
    const int myv = lane >> 2;
    const int pf = 32 * d.prefetch;
    const int stage = ctl->stage_kind;  // an output record waits for psi0 (device control with files)
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        if (stage) stage_beam(d, ctl, stage, b, lane, nullptr, ctl->m0hi, ctl->m0lo);
        // lane-parallel set-up: lanes 0-2 the offsets of H0 (FP64, split), lanes 3-4 dl0, dl1
        DF sv{0.f, 0.f};
        if (lane < 3) sv = dsplit(beam_offset_k<GEOM>(d, ctl->J0, 0, hm, bi, lane));
        else if (lane < 5) sv = mixed::dfg(d, 3, lane - 3, bi.ang);
        const DF g00 = shfl_df(sv, 0), g01r = shfl_df(sv, 1), g01i = shfl_df(sv, 2);
        const DF g01i2 = dsq(g01i);
        const DLen bm0 = dlen(shfl_df(sv, 3));
        DLen bm1;
        if (GEOM == 1) bm1 = dlen(shfl_df(sv, 4));
        DF v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = DF{0.f, 0.f};
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) {
                prefetch_bin(sbin_ptr(s0, epad, b, e + pf));
            }
            const DF a00 = ladd(hv_df(d, 0, e), g00), a01 = ladd(hv_df(d, 1, e), g01r);
            const DF4 x = load_bin(sbin_ptr(s0, epad, b, e));
            const DK k0 = dcoeffs<0>(a00, a01, g01i2, bm0);
            DK k1;
            if (GEOM == 0) {
                // MA: dl1 = 2 dl0, so the halved U(dl1) has C1/2 - 1/2 = C0^2 - 1 =
                // 2 cm0 + cm0^2 and S1/2 = C0 S0 = S0 + cm0 S0
                k1.cm = ladd(dscale(2.f, k0.cm), lsq(k0.cm));
                k1.S = ladd_big(k0.S, lmul(k0.cm, k0.S));
            } else {
                k1 = dcoeffs<1>(a00, a01, g01i2, bm1);
            }
            const DF4 w = dsig_w(a00, a01, g01i, x);
            const DF4 y1 = dapply(.5f, k1, x, w);
            const DF4 y3 = dapply(1.f, k0, x, w);
            store_mid_bin(bin_ptr(d.psi1, epad, b, e), y1);
            store_mid_bin(bin_ptr(d.psi3, epad, b, e), y3);
            const DF f = fv_df(d, bi.p, e);
            dacc_rho(y1, f, v[0], v[1], v[2]);
            dacc_rho(y3, f, v[3], v[4], v[5]);
        }
        // psi1 was accumulated halved: its sums are a quarter (exactly) of psi1's
        v[0] = dscale(2.f, v[0]);
        v[1] = dscale(4.f, v[1]);
        v[2] = dscale(4.f, v[2]);
        v[3] = dscale(.5f, v[3]);
        reduce_sums<8>(v, lane);
        if (myv < 3) mixed::add_moment_df<GEOM>(d, v[0], comp_of(myv), 2, bi, lane & 3, acc);
        else if (myv < 6) mixed::add_moment_df<GEOM>(d, v[0], comp_of(myv - 3), 1, bi, lane & 3, acc);
    }
    if (!group_reduce_split<K>(rt, 4, 6, df_value(acc), 0., false, s_warp, s_out)) return;
    stage_done(ctl);
    if (threadIdx.x < kNJ) {
        ctl->JA1[threadIdx.x] = 0.;
        ctl->JA3[threadIdx.x] = 0.;
    }
    __syncthreads();
    if ((int)threadIdx.x < 6 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        double* J = v < 3 ? ctl->JA1 : ctl->JA3;
        J[k * 4 + comp_of(v % 3)] = s_out[threadIdx.x] / d.kappa;
    }
}

// ------------------------------------------------------------------ phase B

template <int GEOM>
__device__ inline void phaseB_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    const float* __restrict__ s0 = ctl->m0hi;
    float* s4 = ctl->m4hi;
    const double hm_rdr = ctl->hm[2], hm_rdr2 = ctl->hm[1];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};
    const int myv = lane >> 3;
    const int pf = 32 * d.prefetch;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up: lanes 0-2 the offsets of H1, 3-5 those of H3, lane 6 dl1
        DF sv{0.f, 0.f};
        if (lane < 3) sv = dsplit(beam_offset_k<GEOM>(d, ctl->JA1, 2, hm_rdr, bi, lane));
        else if (lane < 6) sv = dsplit(beam_offset_k<GEOM>(d, ctl->JA3, 1, hm_rdr2, bi, lane - 3));
        else if (lane == 6) sv = mixed::dfg(d, 3, 1, bi.ang);
        const DF g100 = shfl_df(sv, 0), g101r = shfl_df(sv, 1), g101i = shfl_df(sv, 2);
        const DF g300 = shfl_df(sv, 3), g301r = shfl_df(sv, 4), g301i = shfl_df(sv, 5);
        const DLen bl = dlen(shfl_df(sv, 6));
        const DF ga2 = dsq(g101i), gb2 = dsq(g301i);
        DF v[4] = {DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}};
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) {
                prefetch_bin(sbin_ptr(s0, epad, b, e + pf));
                prefetch_bin(bin_ptr(d.psi1, epad, b, e + pf));
            }
            const DF hv0 = hv_df(d, 0, e), hv1 = hv_df(d, 1, e);
            const DF4 x = load_bin(sbin_ptr(s0, epad, b, e));
            // S4/S5: (U psi0 + psi1)/2 as U/2 psi0 + psi1/2 (psi1 stored halved by phase A)
            const DF a00 = ladd(hv0, g100), a01 = ladd(hv1, g101r);
            const DK ka = dcoeffs<1>(a00, a01, ga2, bl);
            const DF4 ya = dapply_z(.5f, ka, a00, a01, g101i, x);
            float* p1p = bin_ptr(d.psi1, epad, b, e);
            store_mid_bin(p1p, dadd4(ya, load_bin(p1p)));
            // S8, stored halved for the average of S10/S11
            const DF b00 = ladd(hv0, g300), b01 = ladd(hv1, g301r);
            const DK kb = dcoeffs<1>(b00, b01, gb2, bl);
            const DF4 y4 = dapply_z(.5f, kb, b00, b01, g301i, x);
            store_mid_bin(sbin_ptr(s4, epad, b, e), y4);
            dacc_rho(y4, fv_df(d, bi.p, e), v[0], v[1], v[2]);
        }
        // psi4 was accumulated halved: its sums are a quarter (exactly) of psi4's
        v[0] = dscale(2.f, v[0]);
        v[1] = dscale(4.f, v[1]);
        v[2] = dscale(4.f, v[2]);
        reduce_sums<4>(v, lane);
        if (myv < 3) mixed::add_moment_df<GEOM>(d, v[0], comp_of(myv), 2, bi, lane & 7, acc);
    }
    if (!group_reduce_split<K>(rt, 8, 3, df_value(acc), 0., false, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) ctl->JB4[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        ctl->JB4[k * 4 + comp_of(v)] = s_out[threadIdx.x] / d.kappa;
    }
}

// ------------------------------------------------------------------ phase C

template <int GEOM>
__device__ inline void phaseC_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    float* s4 = ctl->m4hi;
    double* __restrict__ S4 = ctl->S4;
    float2* __restrict__ S4f = ctl->S4f;
    const double hm_rdr = ctl->hm[2];
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};
    float mx = -1.f;
    const int myv = lane >> 3;  // 0: error, 1..3: density components 0, 2, 3
    const int pf = 32 * d.prefetch;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up: lanes 0-2 the offsets of H4, lane 3 dl2
        DF sv{0.f, 0.f};
        if (lane < 3) sv = dsplit(beam_offset_k<GEOM>(d, ctl->JB4, 2, hm_rdr, bi, lane));
        else if (lane == 3) sv = mixed::dfg(d, 3, 2, bi.ang);
        const DF g00 = shfl_df(sv, 0), g01r = shfl_df(sv, 1), g01i = shfl_df(sv, 2);
        const DLen bm = dlen(shfl_df(sv, 3));
        const DF g01i2 = dsq(g01i);
        DF v[4] = {DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}};
        float err = 0.f;
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) {
                prefetch_bin(bin_ptr(d.psi3, epad, b, e + pf));
                prefetch_bin(sbin_ptr(s4, epad, b, e + pf));
                prefetch_bin(bin_ptr(d.psi1, epad, b, e + pf));
            }
            const DF a00 = ladd(hv_df(d, 0, e), g00), a01 = ladd(hv_df(d, 1, e), g01r);
            const DF4 x3 = load_bin(bin_ptr(d.psi3, epad, b, e));
            // S10/S11: (U psi3 + psi4)/2 as U/2 psi3 + psi4/2 (psi4 stored halved by phase B)
            const DK k = dcoeffs<1>(a00, a01, g01i2, bm);
            const DF4 y3 = dapply_z(.5f, k, a00, a01, g01i, x3);
            float* cp = sbin_ptr(s4, epad, b, e);
            const DF4 c = norm4(dadd4(y3, load_bin(cp)));
            store_bin_raw(cp, c);
            // calcErrHvv against psi1: the hi parts of two states this close
            // differ exactly (Sterbenz), so the difference is exact to 2^-48
            // of the state, far below the error's own size
            const DF4 r1 = load_bin(bin_ptr(d.psi1, epad, b, e));
            const float e0 = (c.ar.h - r1.ar.h) + (c.ar.l - r1.ar.l), e1 = (c.ai.h - r1.ai.h) + (c.ai.l - r1.ai.l);
            const float e2 = (c.br.h - r1.br.h) + (c.br.l - r1.br.l), e3 = (c.bi.h - r1.bi.h) + (c.bi.l - r1.bi.l);
            const DF f = fv_df(d, bi.p, e);
            err = fmaf((e0 * e0 + e1 * e1) + (e2 * e2 + e3 * e3), f.h, err);
            dacc_rho(c, f, v[1], v[2], v[3]);
        }
        v[0] = DF{err, 0.f};
        v[1] = dscale(.5f, v[1]);
        reduce_sums<4>(v, lane);
        if (myv == 0) {
            mx = fmaxf(mx, v[0].h + v[0].l);
            if ((lane & 7) == 0) {
                S4[(size_t)b * 4 + 1] = 0.;
                S4f[(size_t)b * 4 + 1] = make_float2(0.f, 0.f);
            }
        } else {
            const int comp = comp_of(myv - 1);
            mixed::add_moment_df<GEOM>(d, v[0], comp, 2, bi, lane & 7, acc);
            // per-beam moments of the candidate (the reference's hSumMat of psi4)
            if ((lane & 7) == 0) {
                S4[(size_t)b * 4 + comp] = df_value(v[0]);
                S4f[(size_t)b * 4 + comp] = make_float2(v[0].h, v[0].l);
            }
        }
    }
    const double accs = __shfl_down_sync(kFull, df_value(acc), 8);
    if (!group_reduce_split<K>(rt, 8, 3, accs, (double)mx, true, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) ctl->JC[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int v = threadIdx.x / K, k = threadIdx.x % K;
        ctl->JC[k * 4 + comp_of(v)] = s_out[threadIdx.x] / d.kappa;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double me = sqrt(s_out[31]);
        ctl->max_err = me;
        if (d.device_control && step_control(d, ctl, me)) {
            float* t = ctl->m0hi;
            ctl->m0hi = ctl->m4hi;
            ctl->m4hi = t;
            t = ctl->m0lo;
            ctl->m0lo = ctl->m4lo;
            ctl->m4lo = t;
        }
    }
}

}  // namespace dfp
}  // namespace xf
