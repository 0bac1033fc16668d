// Device helpers shared by the FP64 and mixed-precision kernels: warp
// reductions, beam indexing, per-beam Hamiltonian offsets from the angular
// moments, the weights of the moment reduction and the deterministic
// block + last-block grid reduction.
#pragma once
#include <cuda_runtime.h>

#include "xf_device.cuh"

namespace xf {
namespace detail {

constexpr unsigned kFull = 0xffffffffu;

// Warp reduce-scatter of NV values (NV a power of two, <= 32): after the call
// v[0] in lane l holds the warp total of value l / (32 / NV).  Costs NV-1 +
// log2(32/NV) additions per lane instead of 5*NV for independent reductions.
template <int NV>
__device__ __forceinline__ void warp_reduce_scatter(double (&v)[NV], int lane)
{
    int off = 16;
#pragma unroll
    for (int half = NV / 2; half >= 1; half >>= 1, off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const double keep = upper ? v[i + half] : v[i];
            const double send = upper ? v[i] : v[i + half];
            v[i] = keep + __shfl_xor_sync(kFull, send, off);
        }
    }
#pragma unroll
    for (; off >= 1; off >>= 1) v[0] += __shfl_xor_sync(kFull, v[0], off);
}

struct BeamIdx {
    int ang, phi, p;
};

__device__ __forceinline__ BeamIdx decode_beam(const Dev& d, int b)
{
    BeamIdx bi;
    bi.p = b & 3;
    const int ap = b >> 2;
    bi.ang = ap / d.P;
    bi.phi = ap - bi.ang * d.P;
    return bi;
}

__device__ __forceinline__ double geo(const Dev& d, int q, int pt, int ang)
{
    return d.geo[geo_idx(q, pt, ang, d.A)];
}

// Hamiltonian components 0, 2, 3 of one beam at stage point pt from the angular
// moments J: MA  H = kappa (J0 - cos J1)          (src/Phy_MA.cpp:372-377)
//            MAA H = kappa' dphi (J0 - sin cosphi Jx - sin sinphi Jy - cos Jz)
//                                                  (src/Phy_MAA.cpp:445-461)
template <int GEOM>
__device__ __forceinline__ void beam_hvv(const Dev& d, const double* J, int pt, const BeamIdx& bi, double H[3])
{
    const int zs[3] = {0, 2, 3};
    const double c = geo(d, 0, pt, bi.ang);
    if (GEOM == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) H[k] = (J[zs[k]] - (J[4 + zs[k]] * c)) * d.kappa;
    } else {
        const double s = geo(d, 1, pt, bi.ang);
        const double cp = d.cosphi[bi.phi], sp = d.sinphi[bi.phi];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            H[k] = (J[zs[k]] - (s * cp * J[4 + zs[k]] + s * sp * J[8 + zs[k]] + c * J[12 + zs[k]])) * d.kappa;
    }
}

// Per-beam Hamiltonian offsets with the particle sign and the matter term
// (src/NBeam.cpp:602-607): h00 = hvac0 + s (H0 + hm), h01r = hvac1 + s H2,
// h01i = H3 (not sign-flipped), s = -1 for anti-neutrinos.
struct BeamH {
    double h00b, h01rb, h01i;
};

template <int GEOM>
__device__ __forceinline__ BeamH beam_offsets(const Dev& d, const double* J, int pt, double hm, const BeamIdx& bi)
{
    double H[3];
    beam_hvv<GEOM>(d, J, pt, bi, H);
    BeamH h;
    const double a = H[0] + hm;
    h.h00b = (bi.p & 1) ? -a : a;
    h.h01rb = (bi.p & 1) ? -H[1] : H[1];
    h.h01i = H[2];
    return h;
}

// L/<E> of particle p without a dynamic index into the kernel parameters
// (which would copy the array to local memory).
__device__ __forceinline__ double le_of(const Dev& d, int p)
{
    return p == 0 ? d.LE[0] : (p == 1 ? d.LE[1] : (p == 2 ? d.LE[2] : d.LE[3]));
}

// Number of moment outputs per summed quantity: MA (J0, J1), MAA (J0, Jx, Jy, Jz).
template <int GEOM>
struct NK {
    static constexpr int K = GEOM == 0 ? 2 : 4;
};

// Adds the weighted contribution of one per-beam energy sum `val` (density
// component z in {0,2,3}) at stage point pt into acc[K].  The weights restate
// the flavor combination of include/NBeam.h:47-53 (nu minus anti-nu on
// components 0-2, plus on component 3) and the angular weights of
// src/Phy_MA.cpp:418-426 / src/Phy_MAA.cpp:513-536.
template <int GEOM>
__device__ __forceinline__ void add_moment(const Dev& d, double val, int z, int pt, const BeamIdx& bi,
                                           double (&acc)[NK<GEOM>::K])
{
    const double sgn = (z == 3 || (bi.p & 1) == 0) ? 1.0 : -1.0;
    const double c = (val * le_of(d, bi.p)) * sgn;
    const double dc = geo(d, 2, pt, bi.ang);
    const double w = c * dc;
    acc[0] += w;
    if (GEOM == 0) {
        acc[1] += w * geo(d, 0, pt, bi.ang);
    } else {
        const double s = geo(d, 1, pt, bi.ang);
        acc[1] += c * d.cosphi[bi.phi] * s * dc;
        acc[2] += c * d.sinphi[bi.phi] * s * dc;
        acc[3] += w * geo(d, 0, pt, bi.ang);
    }
}

// Value slot v of a phase -> (stage point, density component) of the moment it feeds.
__device__ __forceinline__ int comp_of(int k) { return k == 0 ? 0 : (k == 1 ? 2 : 3); }

// Block-level combination of per-lane moment accumulators followed by the
// last-block reduction over blocks.  Lanes l with l % G == 0 (G = 32/NV) own
// value v = l / G; values v < nused feed moments.  Returns true in the last
// block, with s_out[0..nused*K) holding the grid totals and s_out[31] the grid
// maximum of `mx` (ignored unless with_max).
template <int K>
__device__ inline bool block_and_grid_reduce(const Dev& d, int phase, int G, int nused, const double (&acc)[K], double mx,
                                      bool with_max, double* s_warp, double* s_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nout = nused * K;
    const int v = lane / G;
    if ((lane % G) == 0 && v < nused) {
#pragma unroll
        for (int k = 0; k < K; ++k) s_warp[warp * 32 + v * K + k] = acc[k];
    }
    if (with_max && lane == 0) s_warp[warp * 32 + 31] = mx;
    __syncthreads();
    double* part = d.partials + (size_t)blockIdx.x * kPartStride;
    if ((int)threadIdx.x < nout) {
        double t = 0.;
        for (int w = 0; w < nw; ++w) t += s_warp[w * 32 + threadIdx.x];
        part[threadIdx.x] = t;
    }
    if (with_max && threadIdx.x == 31) {
        double m = s_warp[31];
        for (int w = 1; w < nw; ++w) m = fmax(m, s_warp[w * 32 + 31]);
        part[31] = m;
    }
    __threadfence();
    __syncthreads();
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(&d.ctl->ticket[phase], 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    // Last block: thread t sums blocks t, t+bs, ... for every slot, then the
    // block reduces the 32 slots with a reduce-scatter per warp.
    double vals[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) vals[k] = 0.;
    double m = -1.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const double* pb = d.partials + (size_t)b * kPartStride;
#pragma unroll
        for (int k = 0; k < 31; ++k)
            if (k < nout) vals[k] += __ldcg(pb + k);
        if (with_max) m = fmax(m, __ldcg(pb + 31));
    }
    warp_reduce_scatter<32>(vals, lane);
    __syncthreads();
    s_warp[warp * 32 + lane] = vals[0];
    if (with_max) {
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) m = fmax(m, __shfl_xor_sync(kFull, m, off));
    }
    __syncthreads();
    if ((int)threadIdx.x < nout) {
        double t = 0.;
        for (int w = 0; w < nw; ++w) t += s_warp[w * 32 + threadIdx.x];
        s_out[threadIdx.x] = t;
    }
    if (with_max) {
        __shared__ double s_m[32];
        if (lane == 0) s_m[warp] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            double mm = s_m[0];
            for (int w = 1; w < nw; ++w) mm = fmax(mm, s_m[w]);
            s_out[31] = mm;
        }
    }
    if (threadIdx.x == 0) d.ctl->ticket[phase] = 0u;
    __syncthreads();
    return true;
}

// The step controller of src/Nmr.cpp:227-249 under device control, run by one
// thread after Max_err is known: accept (r += dr, psi0 <-> psi4, S0 <-> S4,
// J0 <- JC, record the step), count the iteration, update dr with the
// reference's formula and clamps, and decide whether the loop ends.  Returns
// true when the step was accepted.
__device__ inline bool step_control(const Dev& d, Ctl* ctl, double me)
{
    double r = ctl->r, dr = ctl->dr;
    bool acc = false;
    if (me != me) ctl->nan_seen = 1;
    if (me < d.eps0) {
        r += dr;
        double* t = ctl->psi0;
        ctl->psi0 = ctl->psi4;
        ctl->psi4 = t;
        double* ts = ctl->S0;
        ctl->S0 = ctl->S4;
        ctl->S4 = ts;
        for (int i = 0; i < kNJ; ++i) ctl->J0[i] = ctl->JC[i];
        if (d.log && ctl->log_len < d.log_cap) {
            double* rec = d.log + 3 * ctl->log_len;
            rec[0] = (double)ctl->iters;
            rec[1] = r;
            rec[2] = dr;
            ctl->log_len++;
        }
        ctl->accepted++;
        acc = true;
    }
    ctl->iters++;
    dr *= d.ksi * sqrt(d.eps0 / me);
    dr = (dr > d.maxdr) ? d.maxdr : dr;
    dr = (r + dr > d.Rn) ? d.Rn - r : dr;
    ctl->r = r;
    ctl->dr = dr;
    ctl->renorm_due = (acc && d.renorm_every > 0 && ctl->accepted % d.renorm_every == 0) ? 1 : 0;
    if (!(r < d.Rn) || ctl->iters >= ctl->max_iters || ctl->nan_seen) ctl->done = 1;
    return acc;
}

}  // namespace detail
}  // namespace xf
