// Mixed-precision per-phase kernel bodies, shared by the single-simulation
// kernels (xf_mixed.cu) and the batched kernels (xf_batch.cu).  The numerical
// method is described at the top of xf_mixed.cu.
#pragma once
#include "xf_common.cuh"

namespace xf {
namespace mixed {

using namespace detail;

constexpr float kSeriesTF = 1.0f;

// Taylor coefficients of cos(x) - 1 = sum_{k>=1} c_k t^k and
// sin(x)/x = sum_{k>=0} s_k t^k, t = x^2.  Degree 5 keeps the truncation below
// 4e-9 relative for t <= 1 (beyond, sqrt/sincos).  Degree 2 is used when every
// lane of a warp has t <= kSmallT: the dropped terms are then below t^2/360 =
// 2.5e-8 relative for the values and t^2/120 = 7.5e-8 for the divided
// differences, under FP32's rounding; the workloads' accepted steps have t
// around 1e-5 to 1e-3.
constexpr float kSmallT = 3e-3f;
__constant__ float kC[6] = {0.f, -0.5f, 1.f / 24.f, -1.f / 720.f, 1.f / 40320.f, -1.f / 3628800.f};
__constant__ float kS[6] = {1.f, -1.f / 6.f, 1.f / 120.f, -1.f / 5040.f, 1.f / 362880.f, -1.f / 39916800.f};
template <int DEG>
__device__ __forceinline__ float horner(const float* c, float t)
{
    float p = c[DEG];
#pragma unroll
    for (int k = DEG - 1; k >= 0; --k) p = fmaf(p, t, c[k]);
    return p;
}

// p(tB) and the divided difference p[tA, tB] = (p(tA) - p(tB)) / (tA - tB)
// of the degree-DEG truncation.
template <int DEG>
__device__ __forceinline__ void divdiff(const float* c, float tA, float tB, float& pB, float& dd)
{
    float P = c[DEG], D = 0.f;
#pragma unroll
    for (int k = DEG - 1; k >= 0; --k) {
        D = fmaf(D, tA, P);
        P = fmaf(P, tB, c[k]);
    }
    pB = P;
    dd = D;
}

// Series degree for a warp whose largest t is tmax: 2 when every lane is
// below kSmallT, else 5 (warp-uniform, so the branch does not diverge).
__device__ __forceinline__ bool warp_small_t(float tmax) { return __all_sync(0xffffffffu, tmax <= kSmallT); }

struct H3f {
    float h00, h01r, h01i;
};

struct F4 {
    float ar, ai, br, bi;
};

__device__ __forceinline__ float norm2(const H3f& h) { return h.h00 * h.h00 + (h.h01r * h.h01r + h.h01i * h.h01i); }

// u = sigma(h) psi for sigma(h) = [[h00, h01r + i h01i], [h01r - i h01i, -h00]]
// (the Hamiltonian matrix of src/NBeam.cpp:371-392).
__device__ __forceinline__ F4 sig_apply(const H3f& h, const F4& x)
{
    F4 u;
    u.ar = h.h00 * x.ar + h.h01r * x.br - h.h01i * x.bi;
    u.ai = h.h00 * x.ai + h.h01r * x.bi + h.h01i * x.br;
    u.br = h.h01r * x.ar + h.h01i * x.ai - h.h00 * x.br;
    u.bi = h.h01r * x.ai - h.h01i * x.ar - h.h00 * x.bi;
    return u;
}

// c psi - i v  with v given as the complex vector (v.ar + i v.ai, v.br + i v.bi)
__device__ __forceinline__ F4 combine(float c, const F4& x, const F4& v)
{
    F4 y;
    y.ar = c * x.ar + v.ai;
    y.ai = c * x.ai - v.ar;
    y.br = c * x.br + v.bi;
    y.bi = c * x.bi - v.br;
    return y;
}

__device__ __forceinline__ F4 scale(float s, const F4& u)
{
    F4 v;
    v.ar = s * u.ar;
    v.ai = s * u.ai;
    v.br = s * u.br;
    v.bi = s * u.bi;
    return v;
}

__device__ __forceinline__ F4 add(const F4& a, const F4& b)
{
    F4 c;
    c.ar = a.ar + b.ar;
    c.ai = a.ai + b.ai;
    c.br = a.br + b.br;
    c.bi = a.bi + b.bi;
    return c;
}

// K = (C - 1) - i S sigma(h) over the path length l.
struct KC {
    float cm1, S;
};

template <int DEG>
__device__ __forceinline__ KC kcoef(const H3f& h, float l)
{
    const float t = norm2(h) * (l * l);
    KC k;
    if (DEG < 5 || t <= kSeriesTF) {
        k.cm1 = horner<DEG>(kC, t);
        k.S = l * horner<DEG>(kS, t);
    } else {
        const float x = sqrtf(t);
        float s, c;
        sincosf(x, &s, &c);
        k.cm1 = c - 1.f;
        k.S = l * (s / x);
    }
    return k;
}

__device__ __forceinline__ F4 k_apply(const KC& k, const H3f& h, const F4& x)
{
    return combine(k.cm1, x, scale(k.S, sig_apply(h, x)));
}

__device__ __forceinline__ F4 sub(const F4& a, const F4& b)
{
    F4 c;
    c.ar = a.ar - b.ar;
    c.ai = a.ai - b.ai;
    c.br = a.br - b.br;
    c.bi = a.bi - b.bi;
    return c;
}

// [K(hA, l) - K(hB, l)] x given the accurate difference dh = hA - hB and the
// products sd = sigma(dh) x and sb = sigma(hB) x (sigma is linear in h, so
// callers form sb from a product they already hold).
template <int DEG>
__device__ __forceinline__ F4 diff_h(const H3f& hA, const H3f& hB, const H3f& dh, float l, const F4& x, const F4& sd,
                                     const F4& sb)
{
    const float l2 = l * l;
    const float tA = norm2(hA) * l2, tB = norm2(hB) * l2;
    if (DEG == 5 && (tA > kSeriesTF || tB > kSeriesTF)) {
        const KC ka = kcoef<DEG>(hA, l), kb = kcoef<DEG>(hB, l);
        return sub(combine(ka.cm1, x, scale(ka.S, add(sd, sb))), combine(kb.cm1, x, scale(kb.S, sb)));
    }
    const float dt = l2 * (dh.h00 * (hA.h00 + hB.h00) + dh.h01r * (hA.h01r + hB.h01r) + dh.h01i * (hA.h01i + hB.h01i));
    float cB, dc, sB, ds;
    divdiff<DEG>(kC, tA, tB, cB, dc);
    divdiff<DEG>(kS, tA, tB, sB, ds);
    const float SA = l * fmaf(dt, ds, sB);
    const float dS = l * (dt * ds);
    const F4 v = add(scale(SA, sd), scale(dS, sb));
    return combine(dt * dc, x, v);
}

// [K(h, lA) - K(h, lB)] x given the accurate difference dl = lA - lB and the
// product sh = sigma(h) x.
template <int DEG>
__device__ __forceinline__ F4 diff_l(const H3f& h, float lA, float lB, float dl, const F4& x, const F4& sh)
{
    const float n2 = norm2(h);
    const float tA = n2 * lA * lA, tB = n2 * lB * lB;
    if (DEG == 5 && (tA > kSeriesTF || tB > kSeriesTF)) {
        const KC ka = kcoef<DEG>(h, lA), kb = kcoef<DEG>(h, lB);
        return sub(combine(ka.cm1, x, scale(ka.S, sh)), combine(kb.cm1, x, scale(kb.S, sh)));
    }
    const float dt = n2 * dl * (lA + lB);
    float cB, dc, sB, ds;
    divdiff<DEG>(kC, tA, tB, cB, dc);
    divdiff<DEG>(kS, tA, tB, sB, ds);
    const float sA = fmaf(dt, ds, sB);
    const float dS = fmaf(dl, sA, lB * (dt * ds));
    return combine(dt * dc, x, scale(dS, sh));
}

// Kahan-compensated FP32 accumulation (per thread, over its energies).
struct KSum {
    float s, c;
    __device__ __forceinline__ void add(float v)
    {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// fv * [rho(x + d) - rho(x)] (first row of the density matrix, src/NBeam.cpp:314-322;
// component 0 without the factor 1/2): only the cross and quadratic terms in
// the increment d, so the FP32 result is precise relative to the increment.
__device__ __forceinline__ void acc_drho(const F4& x, const F4& dd, float fv, KSum& s0, KSum& s2, KSum& s3)
{
    const F4 y = add(x, dd);
    const float r0 = (dd.ar * (x.ar + y.ar) + dd.ai * (x.ai + y.ai)) - (dd.br * (x.br + y.br) + dd.bi * (x.bi + y.bi));
    const float r2 = (dd.ar * y.br + dd.ai * y.bi) + (x.ar * dd.br + x.ai * dd.bi);
    const float r3 = (dd.ai * y.br - dd.ar * y.bi) + (x.ai * dd.br - x.ar * dd.bi);
    s0.add(r0 * fv);
    s2.add(r2 * fv);
    s3.add(r3 * fv);
}

__device__ __forceinline__ F4 load_f(const float* __restrict__ b, int epad, int e)
{
    F4 x;
    x.ar = b[e];
    x.ai = b[epad + e];
    x.br = b[2 * epad + e];
    x.bi = b[3 * epad + e];
    return x;
}

// L1 prefetch of the four component rows of bin e: the load of a later
// energy-loop iteration starts without holding registers.
__device__ __forceinline__ void prefetch_f(const float* b, int epad, int e)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(b + e));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(b + epad + e));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(b + 2 * epad + e));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(b + 3 * epad + e));
}

__device__ __forceinline__ void store_f(float* __restrict__ b, int epad, int e, const F4& x)
{
    b[e] = x.ar;
    b[epad + e] = x.ai;
    b[2 * epad + e] = x.br;
    b[3 * epad + e] = x.bi;
}

// (hi, lo) + d as an FP32 pair: TwoSum of hi and d, then a renormalising
// Fast2Sum of the result with the accumulated low parts.
__device__ __forceinline__ void ff_add(float hi, float lo, float d, float& nhi, float& nlo)
{
    const float s = hi + d;
    const float bp = s - hi;
    const float e = ((hi - (s - bp)) + (d - bp)) + lo;
    nhi = s + e;
    nlo = e - (nhi - s);
}

// Offset k of the beam Hamiltonian at stage s of phase C: s = 0 the start
// (J0, point 0), 1 the A1 stage (point 2), 2 the A3 stage (point 1), 3 the B4
// stage (point 2).  Selected with conditionals so no local array is formed.
template <int GEOM>
__device__ __forceinline__ double stage_offset(const Dev& d, const Ctl* ctl, int s, const BeamIdx& bi, int k)
{
    const double* J = s == 0 ? ctl->J0 : s == 1 ? ctl->JA1 : s == 2 ? ctl->JA3 : ctl->JB4;
    const int pt = s == 0 ? 0 : s == 2 ? 1 : 2;
    const double hm = ctl->hm[pt];
    return beam_offset_k<GEOM>(d, J, pt, hm, bi, k);
}

__device__ __forceinline__ H3f bin_hf(const H3f& g, float hv0, float hv1)
{
    H3f h;
    h.h00 = hv0 + g.h00;
    h.h01r = hv1 + g.h01r;
    h.h01i = g.h01i;
    return h;
}

__device__ __forceinline__ H3f shfl_h3(float v, int first)
{
    H3f h;
    h.h00 = __shfl_sync(kFull, v, first);
    h.h01r = __shfl_sync(kFull, v, first + 1);
    h.h01i = __shfl_sync(kFull, v, first + 2);
    return h;
}

// ------------------------------------------------------------------ double-float

// Error-free transformations on FP32 (the compensated pairs' arithmetic):
// TwoSum (Knuth), Fast2Sum (Dekker, |a| >= |b|) and the FMA-based TwoProduct.
struct DF {
    float h, l;
};

__device__ __forceinline__ DF two_sum(float a, float b)
{
    const float s = a + b;
    const float bp = s - a;
    return DF{s, (a - (s - bp)) + (b - bp)};
}

__device__ __forceinline__ DF fast_two_sum(float a, float b)
{
    const float s = a + b;
    return DF{s, b - (s - a)};
}

__device__ __forceinline__ DF two_prod(float a, float b)
{
    const float p = a * b;
    return DF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ DF df_add(const DF& a, const DF& b)
{
    const DF s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, s.l + (a.l + b.l));
}

__device__ __forceinline__ DF df_mul(const DF& a, const DF& b)
{
    const DF p = two_prod(a.h, b.h);
    return fast_two_sum(p.h, fmaf(a.h, b.l, fmaf(a.l, b.h, p.l)));
}

// x0 x1 + y0 y1 for compensated pairs x = (x0 + xl0), ... (the lo*lo terms,
// 2^-48 of the result, are dropped).
__device__ __forceinline__ DF df_dot2(float x0, float xl0, float x1, float xl1, float y0, float yl0, float y1,
                                      float yl1)
{
    const DF p = two_prod(x0, x1), q = two_prod(y0, y1);
    const DF t = two_sum(p.h, q.h);
    const float cross = fmaf(x0, xl1, fmaf(xl0, x1, fmaf(y0, yl1, yl0 * y1)));
    return fast_two_sum(t.h, t.l + (p.l + q.l + cross));
}

// Warp reduce-scatter of NV double-float values (the FP32 counterpart of
// warp_reduce_scatter, same exchange pattern): afterwards each group of
// 32/NV lanes holds the warp total of one value.  Per-lane Kahan sums enter
// as (s, -c); the totals keep about 2^-44 of their size, far below the FP32
// precision of the increments they sum.
template <int NV>
__device__ __forceinline__ void df_reduce_scatter(DF (&v)[NV], int lane)
{
    int off = 16;
#pragma unroll
    for (int half = NV / 2; half >= 1; half >>= 1, off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const DF keep = upper ? v[i + half] : v[i];
            const DF send = upper ? v[i] : v[i + half];
            v[i] = df_add(keep, DF{__shfl_xor_sync(kFull, send.h, off), __shfl_xor_sync(kFull, send.l, off)});
        }
    }
#pragma unroll
    for (; off >= 1; off >>= 1)
        v[0] = df_add(v[0], DF{__shfl_xor_sync(kFull, v[0].h, off), __shfl_xor_sync(kFull, v[0].l, off)});
}

__device__ __forceinline__ double df_value(const DF& x) { return (double)x.h + (double)x.l; }

__device__ __forceinline__ DF df_neg(const DF& a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_sub(const DF& a, const DF& b) { return df_add(a, df_neg(b)); }

// ------------------------------------------------------------------ per-beam set-up and moments in double-float
//
// The per-beam work around the energy loop (the Hamiltonian offsets from the
// stage moments, the path lengths and their differences, the weighted angular
// moments) needs more than FP32 precision but not the FP64 pipe, which runs at
// 1/64 of the FP32 rate on this GPU: it is done in double-float arithmetic on
// tables the geometry kernel and the set-up provide as (hi, lo) pairs.  The
// moments J and matter terms a phase reads are converted once per block.

// Entry (q, pt, ang) of the geometry table as a double-float.
__device__ __forceinline__ DF dfg(const Dev& d, int q, int pt, int ang)
{
    const int i = geo_idx(q, pt, ang, d.A);
    return DF{d.geof[i], d.geof[12 * d.A + i]};
}

// The stage moments scaled by kappa (up to four sets of kNJ) and the three
// matter terms, per block.  kappa J is the Hamiltonian's scale (J itself, of
// order 1e50 in these units, and kappa, 1e-45, are outside FP32's range).
struct SharedJ {
    float h[4][kNJ], l[4][kNJ];
    float hmh[3], hml[3];
};

__device__ __forceinline__ void split_store(double x, float& h, float& l)
{
    h = (float)x;
    l = (float)(x - (double)h);
}

__device__ inline void load_shared_j(SharedJ& sj, const Ctl* ctl, double d_kappa, const double* J0, const double* J1,
                                     const double* J2, const double* J3)
{
    for (int i = threadIdx.x; i < 4 * kNJ; i += blockDim.x) {
        const int st = i / kNJ, k = i % kNJ;
        const double* J = st == 0 ? J0 : st == 1 ? J1 : st == 2 ? J2 : J3;
        if (J) split_store(d_kappa * J[k], sj.h[st][k], sj.l[st][k]);
    }
    if (threadIdx.x < 3) split_store(ctl->hm[threadIdx.x], sj.hmh[threadIdx.x], sj.hml[threadIdx.x]);
    __syncthreads();
}

__device__ __forceinline__ DF sj_get(const SharedJ& sj, int st, int i) { return DF{sj.h[st][i], sj.l[st][i]}; }

// Component k of the beam Hamiltonian offsets (beam_offset_k) at stage point
// pt from the kappa-scaled moments of shared stage st, in double-float:
// kJ0 - c kJ1 (MA) or kJ0 - (s cos(phi) kJx + s sin(phi) kJy + c kJz) (MAA),
// plus the matter term on component 0, with the particle sign.
template <int GEOM>
__device__ __forceinline__ DF beam_offset_df(const Dev& d, const SharedJ& sj, int st, int pt, const BeamIdx& bi, int k)
{
    const int z = k == 0 ? 0 : (k == 1 ? 2 : 3);
    const DF c = dfg(d, 0, pt, bi.ang);
    DF u;
    if (GEOM == 0) {
        u = df_sub(sj_get(sj, st, z), df_mul(sj_get(sj, st, 4 + z), c));
    } else {
        const DF s = dfg(d, 1, pt, bi.ang);
        const DF cp{d.cosphif[bi.phi], d.cosphif[d.P + bi.phi]}, sp{d.sinphif[bi.phi], d.sinphif[d.P + bi.phi]};
        const DF t = df_add(df_add(df_mul(df_mul(s, cp), sj_get(sj, st, 4 + z)), df_mul(df_mul(s, sp), sj_get(sj, st, 8 + z))),
                            df_mul(c, sj_get(sj, st, 12 + z)));
        u = df_sub(sj_get(sj, st, z), t);
    }
    DF H = u;
    if (k == 0) H = df_add(H, DF{sj.hmh[pt], sj.hml[pt]});
    return (k < 2 && (bi.p & 1)) ? df_neg(H) : H;
}

// add_moment_lane in double-float, scaled by kappa (the weight kappa L/<E>):
// lane k of a value group accumulates kappa times moment k; the block totals
// are divided by kappa in FP64 when the moments are written.
template <int GEOM>
__device__ __forceinline__ void add_moment_df(const Dev& d, const DF& val, int z, int pt, const BeamIdx& bi, int k, DF& acc)
{
    if (k >= NK<GEOM>::K) return;
    DF c = df_mul(val, DF{d.LEkf[bi.p], d.LEkf[4 + bi.p]});
    if (!(z == 3 || (bi.p & 1) == 0)) c = df_neg(c);
    const DF dc = dfg(d, 2, pt, bi.ang);
    DF m;
    if (GEOM == 0 || k == 0 || k == 3) {
        m = df_mul(c, dc);
        if (k != 0) m = df_mul(m, dfg(d, 0, pt, bi.ang));
    } else {
        const DF a = k == 1 ? DF{d.cosphif[bi.phi], d.cosphif[d.P + bi.phi]} : DF{d.sinphif[bi.phi], d.sinphif[d.P + bi.phi]};
        m = df_mul(df_mul(df_mul(c, a), dfg(d, 1, pt, bi.ang)), dc);
    }
    acc = df_add(acc, m);
}

// psi0's sum of density component comp for beam b, as a double-float.
__device__ __forceinline__ DF s0_df(const Ctl* ctl, int b, int comp)
{
    const float2 v = ctl->S0f[(size_t)b * 4 + comp];
    return DF{v.x, v.y};
}

// ------------------------------------------------------------------ phase A

// Moments of psi1 = U(h0, dl1) psi0 at point 2 and of psi3 = U(h0, dl0) psi0 at point 1.
template <int GEOM>
__device__ inline void phaseA_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    __shared__ SharedJ sj;
    if (GEOM == 1) load_shared_j(sj, ctl, d.kappa, ctl->J0, nullptr, nullptr, nullptr);
    const float* __restrict__ p0 = ctl->m0hi;
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};  // lane-split moment accumulator (add_moment_df)
    const int myv = lane >> 2;
    const int stage = ctl->stage_kind;  // an output record waits for psi0 (device control with files)
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        if (stage) stage_beam(d, ctl, stage, b, lane, nullptr, ctl->m0hi, ctl->m0lo);
        // lane-parallel set-up: lanes 0-2 the offsets of H0, lanes 3-4 dl0, dl1
        float sv = 0.f;
        if (lane < 3)
            sv = GEOM == 0 ? (float)beam_offset_k<GEOM>(d, ctl->J0, 0, ctl->hm[0], bi, lane)
                           : beam_offset_df<GEOM>(d, sj, 0, 0, bi, lane).h;
        else if (lane < 5) sv = d.geof[geo_idx(3, lane - 3, bi.ang, d.A)];
        const H3f g0 = shfl_h3(sv, 0);
        const float l0 = __shfl_sync(kFull, sv, 3), l1 = __shfl_sync(kFull, sv, 4);
        const float* in = p0 + (size_t)b * 4 * epad;
        const float* fvp = d.fvf + bi.p * epad;
        KSum s[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) s[i] = KSum{0.f, 0.f};
        const int pf = 32 * d.prefetch;
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) prefetch_f(in, epad, e + pf);
            const H3f h = bin_hf(g0, d.hvf[e], d.hvf[epad + e]);
            const F4 x = load_f(in, epad, e);
            const float lm = GEOM == 0 ? l0 : fmaxf(l0, l1);
            KC k0, k1;
            if (warp_small_t(norm2(h) * (lm * lm))) {
                k0 = kcoef<2>(h, l0);
                if (GEOM == 1) k1 = kcoef<2>(h, l1);
            } else {
                k0 = kcoef<5>(h, l0);
                if (GEOM == 1) k1 = kcoef<5>(h, l1);
            }
            if (GEOM == 0) {
                // MA: dl1 = 2 dl0, so C1 - 1 = 2 (C0 - 1)(C0 + 1) and S1 = 2 C0 S0
                k1.cm1 = 2.f * k0.cm1 * (k0.cm1 + 2.f);
                k1.S = 2.f * (1.f + k0.cm1) * k0.S;
            }
            const F4 u = sig_apply(h, x);
            const F4 d1 = combine(k1.cm1, x, scale(k1.S, u));
            const F4 d3 = combine(k0.cm1, x, scale(k0.S, u));
            const float f = fvp[e];
            acc_drho(x, d1, f, s[0], s[1], s[2]);
            acc_drho(x, d3, f, s[3], s[4], s[5]);
        }
        DF v[8];
#pragma unroll
        for (int i = 0; i < 6; ++i) v[i] = DF{s[i].s, -s[i].c};
        v[6] = v[7] = DF{0.f, 0.f};
        v[0] = DF{.5f * v[0].h, .5f * v[0].l};
        v[3] = DF{.5f * v[3].h, .5f * v[3].l};
        df_reduce_scatter<8>(v, lane);
        if (myv < 3) add_moment_df<GEOM>(d, df_add(s0_df(ctl, b, comp_of(myv)), v[0]), comp_of(myv), 2, bi, lane & 3, acc);
        else if (myv < 6)
            add_moment_df<GEOM>(d, df_add(s0_df(ctl, b, comp_of(myv - 3)), v[0]), comp_of(myv - 3), 1, bi, lane & 3, acc);
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

// Moments of psi4 = U(h3, dl1) psi0 at point 2.
template <int GEOM>
__device__ inline void phaseB_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    __shared__ SharedJ sj;
    if (GEOM == 1) load_shared_j(sj, ctl, d.kappa, ctl->JA3, nullptr, nullptr, nullptr);
    const float* __restrict__ p0 = ctl->m0hi;
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};  // lane-split moment accumulator (add_moment_df)
    const int myv = lane >> 3;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up: lanes 0-2 the offsets of H3, lane 3 dl1
        float sv = 0.f;
        if (lane < 3)
            sv = GEOM == 0 ? (float)beam_offset_k<GEOM>(d, ctl->JA3, 1, ctl->hm[1], bi, lane)
                           : beam_offset_df<GEOM>(d, sj, 0, 1, bi, lane).h;
        else if (lane == 3) sv = d.geof[geo_idx(3, 1, bi.ang, d.A)];
        const H3f g3 = shfl_h3(sv, 0);
        const float l1 = __shfl_sync(kFull, sv, 3);
        const float* in = p0 + (size_t)b * 4 * epad;
        const float* fvp = d.fvf + bi.p * epad;
        KSum s0{0.f, 0.f}, s2{0.f, 0.f}, s3{0.f, 0.f};
        const int pf = 32 * d.prefetch;
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) prefetch_f(in, epad, e + pf);
            const H3f h = bin_hf(g3, d.hvf[e], d.hvf[epad + e]);
            const F4 x = load_f(in, epad, e);
            const KC k = warp_small_t(norm2(h) * (l1 * l1)) ? kcoef<2>(h, l1) : kcoef<5>(h, l1);
            acc_drho(x, k_apply(k, h, x), fvp[e], s0, s2, s3);
        }
        DF v[4] = {DF{.5f * s0.s, -.5f * s0.c}, DF{s2.s, -s2.c}, DF{s3.s, -s3.c}, DF{0.f, 0.f}};
        df_reduce_scatter<4>(v, lane);
        if (myv < 3) add_moment_df<GEOM>(d, df_add(s0_df(ctl, b, comp_of(myv)), v[0]), comp_of(myv), 2, bi, lane & 7, acc);
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

// One bin of phase C: the candidate increment inc = (d3' + d4m)/2 with
// d3 = K(h0,l0) psi0, d3' = d3 + K(h4,l2)(psi0 + d3), d4m = K(h3,l1) psi0, and
// t2 = 2 delta = psi4 - psi1 in difference form (see the file header).  The
// sigma products of h1 and of h0 on psi3 follow from those of h3 and h4 by
// linearity (sigma(h1) x = sigma(h3) x - sigma(h3 - h1) x).
template <int DEG, int GEOM>
__device__ __forceinline__ void c_bin(const H3f& h0, const H3f& h1, const H3f& h3, const H3f& h4, const H3f& d31,
                                      const H3f& d40, float l0, float l1, float l2, float dl20, float dl01, const F4& x,
                                      F4& inc, F4& t2)
{
    const KC k0 = kcoef<DEG>(h0, l0), k4 = kcoef<DEG>(h4, l2), k3 = kcoef<DEG>(h3, l1);
    const F4 u0 = sig_apply(h0, x);
    const F4 d3 = combine(k0.cm1, x, scale(k0.S, u0));
    const F4 x3 = add(x, d3);
    const F4 u4 = sig_apply(h4, x3);
    const F4 d3p = add(d3, combine(k4.cm1, x3, scale(k4.S, u4)));
    const F4 u3 = sig_apply(h3, x);
    const F4 d4m = combine(k3.cm1, x, scale(k3.S, u3));
    inc.ar = .5f * (d3p.ar + d4m.ar);
    inc.ai = .5f * (d3p.ai + d4m.ai);
    inc.br = .5f * (d3p.br + d4m.br);
    inc.bi = .5f * (d3p.bi + d4m.bi);
    const F4 sd31 = sig_apply(d31, x);
    const F4 sd40 = sig_apply(d40, x3);
    const F4 s0x3 = sub(u4, sd40);  // sigma(h0) psi3
    t2 = diff_h<DEG>(h3, h1, d31, l1, x, sd31, sub(u3, sd31));
    t2 = add(t2, diff_h<DEG>(h4, h0, d40, l2, x3, sd40, s0x3));
    t2 = add(t2, diff_l<DEG>(h0, l2, l0, dl20, x3, s0x3));
    if (GEOM == 1) t2 = add(t2, diff_l<DEG>(h0, 2.f * l0, l1, dl01, x, u0));
}

// Candidate psi4 = psi0 + (d3' + d4m)/2 with d3 = K(h0,l0) psi0,
// d3' = d3 + K(h4,l2)(psi0 + d3), d4m = K(h3,l1) psi0; the error estimate in
// difference form; moments of the candidate; the step controller.
template <int GEOM>
__device__ inline void phaseC_body(const Dev& d, int first, int stride, const RedTarget& rt, int end = -1)
{
    constexpr int K = NK<GEOM>::K;
    Ctl* ctl = d.ctl;
    if (ctl->done) return;
    __shared__ double s_warp[8 * 32];
    __shared__ double s_out[32];
    __shared__ SharedJ sj;
    if (GEOM == 1) load_shared_j(sj, ctl, d.kappa, ctl->J0, ctl->JA1, ctl->JA3, ctl->JB4);
    const float* __restrict__ hi0 = ctl->m0hi;
    const float* __restrict__ lo0 = ctl->m0lo;
    float* __restrict__ hi4 = ctl->m4hi;
    float* __restrict__ lo4 = ctl->m4lo;
    double* __restrict__ S4 = ctl->S4;
    float2* __restrict__ S4f = ctl->S4f;
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    DF acc{0.f, 0.f};  // lane-split moment accumulator (add_moment_df)
    float mx = -1.f;
    const int myv = lane >> 3;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        const BeamIdx bi = decode_beam(d, b);
        // lane-parallel set-up, one scalar per lane: offsets of H0, H1, H3, H4
        // (lanes 0-11), the differences H3 - H1 and H4 - H0 in FP64 (12-17),
        // dl0, dl1, dl2, dl2 - dl0 and 2 dl0 - dl1 (18-22)
        float su = 0.f;  // this lane's scalar
        if (lane < 18) {
            // stage s: 0 the start (J0, point 0), 1 A1 (point 2), 2 A3 (point 1), 3 B4 (point 2)
            const int k = lane % 3;
            const int sa = lane < 12 ? lane / 3 : (lane < 15 ? 2 : 3);
            const int sb = lane < 12 ? sa : (lane < 15 ? 1 : 0);
            if (GEOM == 0) {
                // MA: two FP64 operations per offset, cheaper than the double-float route
                const double va = stage_offset<GEOM>(d, ctl, sa, bi, k);
                const double vb = stage_offset<GEOM>(d, ctl, sb, bi, k);
                su = (float)(lane < 12 ? va : va - vb);
            } else {
                const DF va = beam_offset_df<GEOM>(d, sj, sa, sa == 0 ? 0 : sa == 2 ? 1 : 2, bi, k);
                const DF vb = beam_offset_df<GEOM>(d, sj, sb, sb == 0 ? 0 : sb == 2 ? 1 : 2, bi, k);
                su = lane < 12 ? va.h : df_sub(va, vb).h;
            }
        } else if (lane < 23) {
            const DF L0 = dfg(d, 3, 0, bi.ang), L1 = dfg(d, 3, 1, bi.ang), L2 = dfg(d, 3, 2, bi.ang);
            const int j = lane - 18;
            // the last, 2 dl0 - dl1, is zero in MA
            su = j == 0 ? L0.h : j == 1 ? L1.h : j == 2 ? L2.h : j == 3 ? df_sub(L2, L0).h : df_sub(df_add(L0, L0), L1).h;
        }
        const H3f g0 = shfl_h3(su, 0), g1 = shfl_h3(su, 3), g3 = shfl_h3(su, 6), g4 = shfl_h3(su, 9);
        const H3f d31 = shfl_h3(su, 12), d40 = shfl_h3(su, 15);
        const float l0 = __shfl_sync(kFull, su, 18), l1 = __shfl_sync(kFull, su, 19), l2 = __shfl_sync(kFull, su, 20);
        const float dl20 = __shfl_sync(kFull, su, 21), dl01 = __shfl_sync(kFull, su, 22);
        const size_t base = (size_t)b * 4 * epad;
        const float* fvp = d.fvf + bi.p * epad;
        KSum s0{0.f, 0.f}, s2{0.f, 0.f}, s3{0.f, 0.f};
        float err = 0.f;
        const int pf = 32 * d.prefetch;
        for (int e = lane; e < epad; e += 32) {
            if (pf && e + pf < epad) {
                prefetch_f(hi0 + base, epad, e + pf);
                prefetch_f(lo0 + base, epad, e + pf);
            }
            const float hv0 = d.hvf[e], hv1 = d.hvf[epad + e];
            const H3f h0 = bin_hf(g0, hv0, hv1), h1 = bin_hf(g1, hv0, hv1);
            const H3f h3 = bin_hf(g3, hv0, hv1), h4 = bin_hf(g4, hv0, hv1);
            const F4 x = load_f(hi0 + base, epad, e);
            float lm = fmaxf(l0, l2);
            if (GEOM == 1) lm = fmaxf(lm, fmaxf(2.f * l0, l1));
            const float tmax = fmaxf(norm2(h0) * (lm * lm),
                                     fmaxf(norm2(h4) * (l2 * l2), fmaxf(norm2(h3), norm2(h1)) * (l1 * l1)));
            F4 inc, t2;
            if (warp_small_t(tmax)) c_bin<2, GEOM>(h0, h1, h3, h4, d31, d40, l0, l1, l2, dl20, dl01, x, inc, t2);
            else c_bin<5, GEOM>(h0, h1, h3, h4, d31, d40, l0, l1, l2, dl20, dl01, x, inc, t2);
            // candidate as a compensated pair
            const F4 xl = load_f(lo0 + base, epad, e);
            F4 ch, cl;
            ff_add(x.ar, xl.ar, inc.ar, ch.ar, cl.ar);
            ff_add(x.ai, xl.ai, inc.ai, ch.ai, cl.ai);
            ff_add(x.br, xl.br, inc.br, ch.br, cl.br);
            ff_add(x.bi, xl.bi, inc.bi, ch.bi, cl.bi);
            store_f(hi4 + base, epad, e, ch);
            store_f(lo4 + base, epad, e, cl);
            const float f = fvp[e];
            err = fmaf(.25f * ((t2.ar * t2.ar + t2.ai * t2.ai) + (t2.br * t2.br + t2.bi * t2.bi)), f, err);
            acc_drho(x, inc, f, s0, s2, s3);
        }
        DF v[4] = {DF{err, 0.f}, DF{.5f * s0.s, -.5f * s0.c}, DF{s2.s, -s2.c}, DF{s3.s, -s3.c}};
        df_reduce_scatter<4>(v, lane);
        if (myv == 0) {
            mx = fmaxf(mx, v[0].h + v[0].l);
            if ((lane & 7) == 0) {
                S4[(size_t)b * 4 + 1] = 0.;
                S4f[(size_t)b * 4 + 1] = make_float2(0.f, 0.f);
            }
        } else {
            const int comp = comp_of(myv - 1);
            const DF sv = df_add(s0_df(ctl, b, comp), v[0]);
            add_moment_df<GEOM>(d, sv, comp, 2, bi, lane & 7, acc);
            if ((lane & 7) == 0) {
                S4[(size_t)b * 4 + comp] = df_value(sv);
                S4f[(size_t)b * 4 + comp] = make_float2(sv.h, sv.l);
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

// ------------------------------------------------------------------ esum / renormalisation

// Energy sums of psi0 from its compensated pairs (NBeam::calcESum,
// src/NBeam.cpp:812-840), optionally after the unitarity renormalisation of
// every bin (|a|^2 + |b|^2 = 1, written back as compensated pairs); with
// `conditional` only when the step controller flagged a renormalisation.
//
// Without renormalisation (a state handed in by the host) the sums are FP64.
// The renormalisation, which runs every few accepted steps inside the
// stepping loop, stays off the FP64 pipe: n - 1 of a bin is formed in
// double-float arithmetic (the pairs carry 48 bits), the bin is scaled by
// 1 + dn (-1/2 + 3 dn/8) = 1/sqrt(n) to rounding for |dn| < 1e-6 (next term
// 5|dn|^3/16), and the density moments are accumulated in double-float per
// thread (weights fv as double-float pairs) and in FP64 across threads.  A
// bin whose norm has drifted further is renormalised in FP64.
__device__ __forceinline__ void renorm_bin_fp64(float* ph, float* pl, int epad, int e, double fe, DF* acc)
{
    double a[4];
    double n = 0.;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] = (double)ph[k * epad + e] + (double)pl[k * epad + e];
        n = fma(a[k], a[k], n);
    }
    const double f = 1. / sqrt(n);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] *= f;
        const float ah = (float)a[k];
        ph[k * epad + e] = ah;
        pl[k * epad + e] = (float)(a[k] - (double)ah);
    }
    const double r[3] = {((a[0] * a[0] + a[1] * a[1]) - (a[2] * a[2] + a[3] * a[3])) * fe,
                         (a[0] * a[2] + a[1] * a[3]) * fe, (a[1] * a[2] - a[0] * a[3]) * fe};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float rh = (float)r[k];
        acc[k] = df_add(acc[k], DF{rh, (float)(r[k] - (double)rh)});
    }
}

__device__ inline void esum_body(const Dev& d, int first, int stride, int renorm, int conditional, int end = -1)
{
    Ctl* ctl = d.ctl;
    if (conditional && !ctl->renorm_due) return;
    const int lane = threadIdx.x & 31;
    const int gw = first + (threadIdx.x >> 5), tw = stride;
    const int epad = d.epad;
    float* hi = ctl->m0hi;
    float* lo = ctl->m0lo;
    double* S = ctl->S0;
    for (int b = gw; b < (end < 0 ? d.nbeams : end); b += tw) {
        float* ph = hi + (size_t)b * 4 * epad;
        float* pl = lo + (size_t)b * 4 * epad;
        double v[4] = {0., 0., 0., 0.};
        if (!renorm) {
            const double* fvp = d.fv + (b & 3) * epad;
            for (int e = lane; e < epad; e += 32) {
                double a[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) a[k] = pair_at(d, hi, lo, b, k, e);
                const double fe = fvp[e];
                v[1] = fma((a[0] * a[0] + a[1] * a[1]) - (a[2] * a[2] + a[3] * a[3]), fe, v[1]);
                v[2] = fma(a[0] * a[2] + a[1] * a[3], fe, v[2]);
                v[3] = fma(a[1] * a[2] - a[0] * a[3], fe, v[3]);
            }
        } else {
            const float* fh = d.fvf + (b & 3) * epad;
            const float* fl = d.fvf_lo + (b & 3) * epad;
            DF acc[3] = {DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}};
            for (int e = lane; e < epad; e += 32) {
                float h[4], l[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    h[k] = ph[k * epad + e];
                    l[k] = pl[k * epad + e];
                }
                // n = sum (h + l)^2 as s + c: squares by TwoProduct, summed by TwoSum
                const DF q0 = two_prod(h[0], h[0]), q1 = two_prod(h[1], h[1]);
                const DF q2 = two_prod(h[2], h[2]), q3 = two_prod(h[3], h[3]);
                const DF s01 = two_sum(q0.h, q1.h), s23 = two_sum(q2.h, q3.h);
                const DF sn = two_sum(s01.h, s23.h);
                if (sn.h == 0.f) continue;  // padding bin
                const float cross = 2.f * fmaf(h[0], l[0], fmaf(h[1], l[1], fmaf(h[2], l[2], h[3] * l[3])));
                const float c = sn.l + (s01.l + s23.l) + ((q0.l + q1.l) + (q2.l + q3.l)) + cross;
                const float dn = (sn.h - 1.f) + c;  // sn.h - 1 is exact for sn.h in [1/2, 2]
                if (!(fabsf(dn) < 1e-6f)) {
                    renorm_bin_fp64(ph, pl, epad, e, (double)fh[e] + (double)fl[e], acc);
                    continue;
                }
                const float corr = dn * fmaf(dn, .375f, -.5f);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const DF x = fast_two_sum(h[k], fmaf(h[k], corr, l[k]));
                    h[k] = x.h;
                    l[k] = x.l;
                    ph[k * epad + e] = x.h;
                    pl[k * epad + e] = x.l;
                }
                // density moments of the renormalised bin, weighted by fv
                const DF a2 = df_dot2(h[0], l[0], h[0], l[0], h[1], l[1], h[1], l[1]);
                const DF b2 = df_dot2(h[2], l[2], h[2], l[2], h[3], l[3], h[3], l[3]);
                const DF r0 = df_add(a2, DF{-b2.h, -b2.l});
                const DF r2 = df_dot2(h[0], l[0], h[2], l[2], h[1], l[1], h[3], l[3]);
                const DF r3 = df_dot2(h[1], l[1], h[2], l[2], -h[0], -l[0], h[3], l[3]);
                const DF fe{fh[e], fl[e]};
                acc[0] = df_add(acc[0], df_mul(r0, fe));
                acc[1] = df_add(acc[1], df_mul(r2, fe));
                acc[2] = df_add(acc[2], df_mul(r3, fe));
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) v[k + 1] = (double)acc[k].h + (double)acc[k].l;
        }
        v[1] *= .5;
        warp_reduce_scatter<4>(v, lane);
        const int myv = lane >> 3;
        if ((lane & 7) == 0) {
            const size_t i = (size_t)b * 4 + (myv == 0 ? 1 : comp_of(myv - 1));
            const double x = (myv == 0) ? 0. : v[0];
            S[i] = x;
            const float xh = (float)x;
            ctl->S0f[i] = make_float2(xh, (float)(x - (double)xh));
        }
    }
}
}  // namespace mixed
}  // namespace xf
