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


// Component k of the beam Hamiltonian offsets (0: the h00 part s (H0 + hm),
// 1: the h01r part s H2, 2: the h01i part H3) from the moments J at stage
// point pt (beam_hvv's formula), for lane-parallel per-beam set-up: a warp
// evaluates one scalar per lane and broadcasts them, instead of every lane
// evaluating every scalar on the (slow) FP64 pipe.
__device__ __forceinline__ BeamH shfl_beamh(double v, int first)
{
    BeamH h;
    h.h00b = __shfl_sync(kFull, v, first);
    h.h01rb = __shfl_sync(kFull, v, first + 1);
    h.h01i = __shfl_sync(kFull, v, first + 2);
    return h;
}

template <int GEOM>
__device__ __forceinline__ double beam_offset_k(const Dev& d, const double* J, int pt, double hm, const BeamIdx& bi,
                                                int k)
{
    const int z = k == 0 ? 0 : (k == 1 ? 2 : 3);
    const double c = d.geo[geo_idx(0, pt, bi.ang, d.A)];
    double H;
    if (GEOM == 0) {
        H = (J[z] - (J[4 + z] * c)) * d.kappa;
    } else {
        const double s = d.geo[geo_idx(1, pt, bi.ang, d.A)];
        const double cp = d.cosphi[bi.phi], sp = d.sinphi[bi.phi];
        H = (J[z] - (s * cp * J[4 + z] + s * sp * J[8 + z] + c * J[12 + z])) * d.kappa;
    }
    if (k == 0) H = H + hm;
    return (k < 2 && (bi.p & 1)) ? -H : H;
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

// The same contribution split over lanes: after a reduce-scatter the G lanes
// of a value slot hold the same value, and lane k of the group accumulates
// moment k alone (k < K; MA has 2 moments, MAA 4).  Each moment is formed as
// ((c A) B) C with the factors chosen per lane, which repeats the operations
// of add_moment exactly (the unused factors are 1), so the sums are the same
// bits while the FP64 work per lane drops from all K moments to one.
template <int GEOM>
__device__ __forceinline__ void add_moment_lane(const Dev& d, double val, int z, int pt, const BeamIdx& bi, int k,
                                                double& acc)
{
    if (k >= NK<GEOM>::K) return;
    const double sgn = (z == 3 || (bi.p & 1) == 0) ? 1.0 : -1.0;
    const double c = (val * le_of(d, bi.p)) * sgn;
    const double dc = geo(d, 2, pt, bi.ang);
    double A, B, C;
    if (GEOM == 0 || k == 0 || k == 3) {
        // c dc, or (c dc) cos
        A = dc;
        B = k == 0 ? 1.0 : geo(d, 0, pt, bi.ang);
        C = 1.0;
    } else {
        // ((c cos(phi)) sin(theta)) dc and ((c sin(phi)) sin(theta)) dc
        A = k == 1 ? d.cosphi[bi.phi] : d.sinphi[bi.phi];
        B = geo(d, 1, pt, bi.ang);
        C = dc;
    }
    acc += ((c * A) * B) * C;
}

// Value slot v of a phase -> (stage point, density component) of the moment it feeds.
__device__ __forceinline__ int comp_of(int k) { return k == 0 ? 0 : (k == 1 ? 2 : 3); }

// Where a group of blocks reduces its per-block partials: the block's slot
// `idx` of `count` slots at `partials` (followed by room for the group sums,
// red_rows(count) rows in all), the tickets that elect the last block of each
// group of kRedGroup slots (`gticket`, one per group) and the last group
// (`ticket`).  Single simulation: the grid; batch: one instance's tiles.
struct RedTarget {
    double* partials;
    int idx;
    int count;
    unsigned int* ticket;
    unsigned int* gticket;
};

template <int K>
__device__ inline bool group_reduce_tail(const RedTarget& rt, int nused, double mx, bool with_max, double* s_warp,
                                         double* s_out);

// Block-level combination of per-lane moment accumulators followed by the
// last-block reduction over the group's blocks.  Lanes l with l % G == 0 (G = 32/NV) own
// value v = l / G; values v < nused feed moments.  Returns true in the last
// block, with s_out[0..nused*K) holding the grid totals and s_out[31] the grid
// maximum of `mx` (ignored unless with_max).
template <int K>
__device__ inline bool group_reduce(const RedTarget& rt, int G, int nused, const double (&acc)[K], double mx,
                                    bool with_max, double* s_warp, double* s_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int v = lane / G;
    if ((lane % G) == 0 && v < nused) {
#pragma unroll
        for (int k = 0; k < K; ++k) s_warp[warp * 32 + v * K + k] = acc[k];
    }
    return group_reduce_tail<K>(rt, nused, mx, with_max, s_warp, s_out);
}

// group_reduce for lane-split accumulators (add_moment_lane): lane v G + k
// holds moment k of value slot v.
template <int K>
__device__ inline bool group_reduce_split(const RedTarget& rt, int G, int nused, double acc, double mx, bool with_max,
                                          double* s_warp, double* s_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int v = lane / G, k = lane % G;
    if (k < K && v < nused) s_warp[warp * 32 + v * K + k] = acc;
    return group_reduce_tail<K>(rt, nused, mx, with_max, s_warp, s_out);
}

// Sums rows [0, n) of `rows` (row stride kPartStride) slot by slot: slots
// [0, nout) by addition and, with with_max, slot 31 by maximum.  Warp w takes
// rows w, w + nw, ... (lane = slot), then the warps' sums are combined in warp
// order, so the result depends only on n and the block size.  Leaves the
// totals in s_out[0..32).
__device__ inline void sum_rows(const double* rows, int n, int nout, bool with_max, double* s_warp, double* s_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const bool is_max = with_max && lane == 31;
    double t = is_max ? -1.0 : 0.;
    if (lane < nout || is_max) {
        for (int j = warp; j < n; j += nw) {
            const double x = __ldcg(rows + (size_t)j * kPartStride + lane);
            t = is_max ? fmax(t, x) : t + x;
        }
    }
    __syncthreads();  // s_warp may still be read by the caller's block-partial pass
    s_warp[warp * 32 + lane] = t;
    __syncthreads();
    if (warp == 0) {
        double a = s_warp[lane];
        for (int w = 1; w < nw; ++w) a = is_max ? fmax(a, s_warp[w * 32 + lane]) : a + s_warp[w * 32 + lane];
        s_out[lane] = a;
    }
    __syncthreads();
}

template <int K>
__device__ inline bool group_reduce_tail(const RedTarget& rt, int nused, double mx, bool with_max, double* s_warp,
                                         double* s_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nout = nused * K;
    if (with_max && lane == 0) s_warp[warp * 32 + 31] = mx;
    __syncthreads();
    double* part = rt.partials + (size_t)rt.idx * kPartStride;
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
    // level 1: the last block of this group of kRedGroup partials sums the group
    const int g = rt.idx / kRedGroup, ng = (rt.count + kRedGroup - 1) / kRedGroup;
    const int g0 = g * kRedGroup, gsize = min(kRedGroup, rt.count - g0);
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(&rt.gticket[g], 1u);
        s_last = (t == (unsigned)gsize - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    if (threadIdx.x == 0) rt.gticket[g] = 0u;
    sum_rows(rt.partials + (size_t)g0 * kPartStride, gsize, nout, with_max, s_warp, s_out);
    if (ng == 1) return true;
    // level 2: the group sum goes after the block partials; the last group sums them
    double* gpart = rt.partials + (size_t)rt.count * kPartStride;
    if ((int)threadIdx.x < 32 && ((int)threadIdx.x < nout || (with_max && threadIdx.x == 31)))
        gpart[(size_t)g * kPartStride + threadIdx.x] = s_out[threadIdx.x];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(rt.ticket, 1u);
        s_last = (t == (unsigned)ng - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    if (threadIdx.x == 0) *rt.ticket = 0u;
    sum_rows(gpart, ng, nout, with_max, s_warp, s_out);
    return true;
}

// The 8 bytes of v in reverse order: the halves swapped, each byte-reversed
// (a double in the NetCDF file's big-endian encoding on a little-endian GPU).
__device__ __forceinline__ double byte_reversed(double v)
{
    const unsigned lo = (unsigned)__double2loint(v), hi = (unsigned)__double2hiint(v);
    return __hiloint2double((int)__byte_perm(lo, 0, 0x0123), (int)__byte_perm(hi, 0, 0x0123));
}

// Component k of energy bin e of beam b of a compensated-pair state (hi, lo)
// as a double: the mixed path's rows ([beam][comp][epad] hi and lo arrays)
// or, for the double-float path (d.df), its bin layout ([beam][epad][8]
// floats in the buffer at hi: the four hi parts, then the four lo parts).
__device__ __forceinline__ double pair_at(const Dev& d, const float* hi, const float* lo, int b, int k, int e)
{
    if (d.df) {
        const float* p = hi + ((size_t)b * d.epad + e) * 8;
        return (double)p[k] + (double)p[4 + k];
    }
    const size_t i = ((size_t)b * 4 + k) * d.epad + e;
    return (double)hi[i] + (double)lo[i];
}

// Staging of one beam of psi0 for a record decided by the step controller
// (one warp): the Snapshot slot receives the beam's four components, unpadded
// and big-endian; the Probability slot its survival sum_e fv (ar^2 + ai^2)
// with the spectrum of particle p % 2 (src/IO_f.cpp:341-351), reduced in the
// order of the stand-alone output kernels so both routes write the same
// bits.  psi is the FP64 state, or null for the compensated pair (hi, lo).
__device__ inline void stage_beam(const Dev& d, const Ctl* ctl, int kind, int b, int lane, const double* psi,
                                  const float* hi, const float* lo)
{
    const int epad = d.epad, ne = d.ne;
    const size_t base = (size_t)b * 4 * epad;
    if (kind & 1) {
        double* dst = ctl->io_snap + (size_t)ctl->stage_snap_slot * ((size_t)d.nbeams * 4 * ne) + (size_t)b * 4 * ne;
        for (int k = 0; k < 4; ++k)
            for (int e = lane; e < ne; e += 32) {
                const double v = psi ? psi[base + (size_t)k * epad + e] : pair_at(d, hi, lo, b, k, e);
                dst[(size_t)k * ne + e] = byte_reversed(v);
            }
    }
    if (kind & 2) {
        const double* fv = d.fv + (size_t)((b & 3) % 2) * epad;
        double s = 0.;
        for (int e = lane; e < epad; e += 32) {
            double ar, ai;
            if (psi) {
                ar = psi[base + e];
                ai = psi[base + epad + e];
            } else {
                ar = pair_at(d, hi, lo, b, 0, e);
                ai = pair_at(d, hi, lo, b, 1, e);
            }
            s = fma(ar * ar + ai * ai, fv[e], s);
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
        if (lane == 0) ctl->io_prob[(size_t)ctl->stage_prob_slot * d.nbeams + b] = s;
    }
}

// After the last block of a phase A that staged a record: the record's slots
// are complete.
__device__ __forceinline__ void stage_done(Ctl* ctl)
{
    if (threadIdx.x == 0 && ctl->stage_kind) {
        ctl->io_staged = ctl->io_count;
        ctl->stage_kind = 0;
    }
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The dump triggers of io_f::dumpToFile (src/IO_f.cpp:387-424) at an accepted
// step (itr = counter_tot, r after the step, dr used), on the device.  The
// radius and iteration triggers are exact; the wall-time triggers use the GPU
// global timer in whole seconds since the last record, as the reference's
// tv_sec differences do.  File rotation (src/IO_f.cpp:275-279) resets the
// radius and time triggers to R0 and now, as io_f::init does.  A fired dump
// becomes an IoRec and a staging request for the next phase A.
__device__ inline void io_triggers(const Dev& d, Ctl* ctl, double r, double dr, long long itr)
{
    const unsigned long long now = globaltimer_ns();
    if (!ctl->io_tinit) {
        ctl->io_t1 = now - (unsigned long long)ctl->io_age1 * 1000000000ull;
        ctl->io_t2 = now - (unsigned long long)ctl->io_age2 * 1000000000ull;
        ctl->io_tinit = 1;
    }
    ctl->io_gt = now;
    IoRec rec;
    rec.r = r;
    rec.dr = dr;
    rec.itr = itr;
    rec.kind = 0;
    rec.snap_slot = rec.prob_slot = -1;
    rec.rotate = rec.sync_snap = rec.sync_prob = 0;
    if (ctl->io_mode & 1) {
        const long long el = (long long)((now - ctl->io_t1) / 1000000000ull);
        if (r == d.Rn || r - ctl->io_last_r1 > ctl->io_rstep1 || el > ctl->io_tstep1 ||
            (ctl->io_itrstep1 > 0 && !(itr % ctl->io_itrstep1))) {
            ctl->io_last_r1 = r;
            ctl->io_t1 = now;
            if (ctl->io_file_itr >= ctl->io_new_file_step) {
                rec.rotate = 1;
                ctl->io_file_itr = 0;
                ctl->io_last_r1 = ctl->io_R0;
                ctl->io_t1 = now;
                if (ctl->io_mode & 2) {
                    ctl->io_last_r2 = ctl->io_R0;
                    ctl->io_t2 = now;
                }
            }
            ctl->io_file_itr++;
            rec.kind |= 1;
            rec.snap_slot = (int)(ctl->io_snaps++ % ctl->io_nslots);
            rec.sync_snap = ctl->io_sync_step > 0 && ctl->io_file_itr % ctl->io_sync_step == 0;
        }
    }
    if (ctl->io_mode & 2) {
        const long long el = (long long)((now - ctl->io_t2) / 1000000000ull);
        if (r == d.Rn || r - ctl->io_last_r2 > ctl->io_rstep2 || el > ctl->io_tstep2 ||
            (ctl->io_itrstep2 > 0 && !(itr % ctl->io_itrstep2))) {
            ctl->io_last_r2 = r;
            ctl->io_t2 = now;
            rec.kind |= 2;
            rec.prob_slot = (int)(ctl->io_probs++ % ctl->io_nslots);
            rec.sync_prob = ctl->io_sync_step > 0 && ctl->io_file_itr % ctl->io_sync_step == 0;
        }
    }
    if (rec.kind) {
        ctl->io_log[ctl->io_count % ctl->io_log_cap] = rec;
        ctl->io_count++;
        ctl->stage_kind = rec.kind;
        ctl->stage_snap_slot = rec.snap_slot;
        ctl->stage_prob_slot = rec.prob_slot;
    }
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
        float2* tf = ctl->S0f;  // null outside the mixed path
        ctl->S0f = ctl->S4f;
        ctl->S4f = tf;
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
        if (ctl->io_mode) io_triggers(d, ctl, r, dr, ctl->iters);
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

namespace xf {
namespace detail {
// The whole grid as one reduction group (single simulation).
__device__ __forceinline__ RedTarget grid_target(const Dev& d, int phase)
{
    RedTarget rt;
    rt.partials = d.partials;
    rt.idx = blockIdx.x;
    rt.count = gridDim.x;
    rt.ticket = &d.ctl->ticket[phase];
    rt.gticket = d.gticket + phase * kMaxRedGroups;
    return rt;
}
}  // namespace detail
}  // namespace xf

namespace xf {
namespace detail {

// Mirrors entry i of the geometry table as a double-float pair (mixed path).
__device__ __forceinline__ void geo_store(const Dev& d, int i, double v)
{
    d.geo[i] = v;
    if (d.geof) {
        const float h = (float)v;
        d.geof[i] = h;
        d.geof[12 * d.A + i] = (float)(v - (double)h);
    }
}

// phy::calcAngleBins at r, r+dr/2, r+dr and phy::calcDeltaLs for the three
// path segments (src/Nmr.cpp:153-173, src/Phy_MA.cpp:172-227,
// src/Phy_MAA.cpp:194-241), one thread per (angle bin, stage point): the
// thread of point pt evaluates cos, sin and the weight at r_pt and the path
// length of segment pt, which needs the cosines of two points; the block
// exchanges them through s_c[3][nslots] (slot = the angle's place in the
// block).  Every thread of the block must call it (it synchronises the
// block); ang < 0 marks a thread without an angle.  Under device control the
// threads of angle 0 also evaluate the matter term at their point
// (src/Matt.cpp:31-64).
__device__ inline void geometry_point(const Dev& d, int ang, int pt, int slot, int nslots, double* s_c)
{
    const bool live = ang >= 0 && !d.ctl->done;
    double dr = 0., dr2 = 0.;
    if (live) {
        Ctl* ctl = d.ctl;
        const double r = ctl->r;
        dr = ctl->dr;
        dr2 = .5 * dr;
        const double rp = pt == 0 ? r : (pt == 1 ? r + dr2 : r + dr);
        if (d.device_control && ang == 0) {
            double hm = 0.;
            if (d.has_matter) {
                const double R = 10. / rp;
                const double far = d.nbfar * (R * R * R);
                const double near = d.nb0 * exp((d.Rv - rp) / d.hNS);
                hm = d.mat_coeff * (far + near) * .5;
            }
            ctl->hm[pt] = hm;
        }
        if (d.sa) {
            // SA (src/Phy_SA.cpp:121-147, 250-256): no angular dependence, dl =
            // dr/2, dr, dr/2, and H = kappa D(r) N.  Stored in the MA layout as
            // cos = 0 and weight D(r), so the MA moment J0 = sum_b w N_b gives
            // H = kappa (J0 - cos J1) = kappa D(r) N.
            const double R = d.Rv / rp;
            const double tm = 1. - sqrt(1. - (R * R));
            geo_store(d, geo_idx(0, pt, ang, d.A), 0.);
            geo_store(d, geo_idx(1, pt, ang, d.A), 0.);
            geo_store(d, geo_idx(2, pt, ang, d.A), .5 * (tm * tm));
            geo_store(d, geo_idx(3, pt, ang, d.A), pt == 1 ? dr : dr2);
        } else {
            const double ra = d.Rv / rp;
            const double r2 = ra * ra;
            const double c = sqrt(1. - r2 * (1. - d.cos2R[ang]));
            geo_store(d, geo_idx(0, pt, ang, d.A), c);
            geo_store(d, geo_idx(1, pt, ang, d.A), ra * d.sinR[ang]);
            geo_store(d, geo_idx(2, pt, ang, d.A), .5 * (1. / c) * r2 * d.dcos2R[ang]);
            s_c[pt * nslots + slot] = c;
        }
    }
    __syncthreads();
    if (live && !d.sa) {
        const double c0 = s_c[slot], c1 = s_c[nslots + slot], c2 = s_c[2 * nslots + slot];
        double dl;
        if (d.geom == 0) dl = pt == 0 ? dr2 / (c0) : (pt == 1 ? dr / (c0) : dr2 / (c1));
        else dl = pt == 0 ? dr2 / ((c0 + c1) * .5) : (pt == 1 ? dr / ((c0 + c2) * .5) : dr2 / ((c1 + c2) * .5));
        geo_store(d, geo_idx(3, pt, ang, d.A), dl);
    }
}

// Angular moments from per-beam energy sums at stage point pt: the reduction of
// phy::getHvv_partial (src/Phy_MA.cpp:388-446, src/Phy_MAA.cpp:468-562); one
// thread per beam over beams first + threadIdx.x, + stride, ...
template <int GEOM>
__device__ inline void moments_body(const Dev& d, int first, int stride, const RedTarget& rt,
                                    const double* __restrict__ Sarg, int pt, double* Jout, int conditional)
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
    for (int b = first + threadIdx.x; b < d.nbeams; b += stride) {
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
    if (!group_reduce<K>(rt, 2 * K, 3, one, 0., false, s_warp, s_out)) return;
    if (threadIdx.x < kNJ) Jout[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        const int i = threadIdx.x / K, k = threadIdx.x % K;
        Jout[k * 4 + comp_of(i)] = s_out[threadIdx.x];
    }
    if (conditional && threadIdx.x == 0) d.ctl->renorm_due = 0;
}

}  // namespace detail
}  // namespace xf
