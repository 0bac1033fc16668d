// Handle-based engine behind the C ABI (include/xflat_gpu.h): owns the device
// state of one simulation, runs single iterations for a host-driven loop
// (the reference's nmr::evolutionLoop, src/Nmr.cpp:89-262) and whole loops
// under device control, where CUDA graphs of several iterations run with the
// accept/reject and dr controller on the GPU and the host only polls.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "xf_device.cuh"
#include "xf_engine.h"
#include "xf_kernels.h"
#include "xf_mixed.h"
#include "xf_physics.h"
#include "xflat_gpu.h"

using xf::Ctl;
using xf::Dev;

#define XF_CUDA(h, call)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return (h)->fail(XF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int xf_handle::fail(int code, const std::string& msg)
{
    err = msg;
    return code;
}

namespace {

constexpr int kDefaultItersPerLaunch = 16;

int check_config(const xf_config& c, std::string& why)
{
    if (c.geometry != XF_GEOM_MA && c.geometry != XF_GEOM_MAA && c.geometry != XF_GEOM_SA) {
        why = "geometry must be MA, MAA or SA";
        return XF_EINVAL;
    }
    if (c.precision != XF_PREC_FP64 && c.precision != XF_PREC_MIXED && c.precision != XF_PREC_DF) {
        why = "precision must be fp64, mixed or df";
        return XF_EINVAL;
    }
    if (c.flvs != 2) { why = "only two flavors are supported (Flvs= 2), as by the MA/MAA modules"; return XF_EUNSUPPORTED; }
    if ((c.geometry != XF_GEOM_SA && c.abins <= 0) || c.ebins <= 0) { why = "Abins and Ebins must be positive"; return XF_EINVAL; }
    if (c.geometry == XF_GEOM_MAA && c.pbins <= 0) { why = "Pbins must be positive for MAA"; return XF_EINVAL; }
    if (c.E1 <= c.E0) { why = "E1 must exceed E0"; return XF_EINVAL; }
    if (c.Rv <= 0.) { why = "Rv must be positive"; return XF_EINVAL; }
    int A, P;
    xf::beam_dims(c, A, P);
    const double nb = (double)A * P * 4.;
    if (nb > 2147483647.0 / 4) { why = "too many beams"; return XF_EINVAL; }
    return XF_OK;
}

template <typename T>
int dalloc(xf_handle* h, T** p, size_t n)
{
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return h->fail(XF_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemset(*p, 0, n * sizeof(T));
    if (e != cudaSuccess) return h->fail(XF_ECUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
    return XF_OK;
}

template <typename T>
int upload(xf_handle* h, T* dst, const std::vector<T>& src)
{
    if (src.empty()) return XF_OK;
    XF_CUDA(h, cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return XF_OK;
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ------------------------------------------------------------------ internals

int xf_handle::init(const xf_config& c)
{
    cfg = c;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(XF_ECUDA, "no usable GPU");
    XF_CUDA(this, cudaGetDevice(&device));
    xf::build_tables(cfg, tab);
    xf::beam_dims(cfg, A, P);
    ne = cfg.ebins;
    epad = (ne + 31) / 32 * 32;
    nbeams = A * P * 4;
    shape = xf::default_shape(nbeams, epad, cfg.precision == XF_PREC_MIXED);
    if (cfg.precision == XF_PREC_DF) {
        renorm_every = 0;  // pair arithmetic keeps |a|^2 + |b|^2 = 1 to 2^-48
        xf::df_default_shape(nbeams, shape);
    }
    XF_CUDA(this, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (int i = 0; i < 7; ++i) XF_CUDA(this, cudaEventCreate(&ev[i]));

    // energy tables padded to epad
    std::vector<double> fvp(4 * (size_t)epad, 0.), hv(2 * (size_t)epad, 0.);
    for (int p = 0; p < 4; ++p)
        for (int e = 0; e < ne; ++e) fvp[(size_t)p * epad + e] = tab.fv[(size_t)p * ne + e];
    for (int e = 0; e < ne; ++e) {
        hv[e] = tab.hvac[2 * (size_t)e];
        hv[epad + e] = tab.hvac[2 * (size_t)e + 1];
    }
    std::vector<double> cphi = tab.cosphi, sphi = tab.sinphi;
    if (cphi.empty()) { cphi.assign(1, 1.); sphi.assign(1, 0.); }
    int rc;
    if ((rc = dalloc(this, &d_fv, fvp.size())) || (rc = upload(this, d_fv, fvp))) return rc;
    if ((rc = dalloc(this, &d_hvac, hv.size())) || (rc = upload(this, d_hvac, hv))) return rc;
    if ((rc = dalloc(this, &d_cos2R, A)) || (rc = upload(this, d_cos2R, tab.cos2R))) return rc;
    if ((rc = dalloc(this, &d_dcos2R, A)) || (rc = upload(this, d_dcos2R, tab.dcos2R))) return rc;
    if ((rc = dalloc(this, &d_sinR, A)) || (rc = upload(this, d_sinR, tab.sinR))) return rc;
    if ((rc = dalloc(this, &d_cosphi, cphi.size())) || (rc = upload(this, d_cosphi, cphi))) return rc;
    if ((rc = dalloc(this, &d_sinphi, sphi.size())) || (rc = upload(this, d_sinphi, sphi))) return rc;
    if ((rc = dalloc(this, &d_geo, 12 * (size_t)A))) return rc;
    if ((rc = dalloc(this, &d_geof, 24 * (size_t)A))) return rc;
    {
        // azimuth tables as double-float pairs for the mixed-precision kernels
        const int np = (int)cphi.size();
        std::vector<float> pf(4 * (size_t)np);
        for (int i = 0; i < np; ++i) {
            pf[i] = (float)cphi[i];
            pf[np + i] = (float)(cphi[i] - (double)pf[i]);
            pf[2 * np + i] = (float)sphi[i];
            pf[3 * np + i] = (float)(sphi[i] - (double)pf[2 * np + i]);
        }
        if ((rc = dalloc(this, &d_phif, pf.size())) || (rc = upload(this, d_phif, pf))) return rc;
    }
    const int maxblk = std::max(xf::max_phase_blocks(nbeams, 256), 152 * 4);
    if ((rc = dalloc(this, &d_partials, (size_t)xf::red_rows(maxblk) * xf::kPartStride))) return rc;
    if ((rc = dalloc(this, &d_gticket, 4 * (size_t)xf::kMaxRedGroups))) return rc;
    if ((rc = dalloc(this, &d_ctl, 1))) return rc;
    if ((rc = dalloc(this, &d_hvv, 4 * (size_t)A * P))) return rc;
    if ((rc = dalloc(this, &d_Sscratch, 4 * (size_t)nbeams))) return rc;
    XF_CUDA(this, cudaMallocHost((void**)&h_ctl, sizeof(Ctl)));
    XF_CUDA(this, cudaMallocHost((void**)&h_in, 8 * sizeof(double)));
    std::memset(h_ctl, 0, sizeof(Ctl));

    dev = Dev{};
    dev.geom = cfg.geometry == XF_GEOM_MAA ? 1 : 0;
    dev.sa = cfg.geometry == XF_GEOM_SA;
    dev.nbeams = nbeams;
    dev.A = A;
    dev.P = P;
    dev.ne = ne;
    dev.epad = epad;
    dev.fv = d_fv;
    dev.hvac = d_hvac;
    dev.cos2R = d_cos2R;
    dev.dcos2R = d_dcos2R;
    dev.sinR = d_sinR;
    dev.cosphi = d_cosphi;
    dev.sinphi = d_sinphi;
    dev.geo = d_geo;
    dev.geof = cfg.precision != XF_PREC_FP64 ? d_geof : nullptr;  // the FP64 path reads only geo
    dev.cosphif = d_phif;
    dev.sinphif = d_phif + 2 * cphi.size();
    dev.partials = d_partials;
    dev.gticket = d_gticket;
    // mixed phases: state rows prefetched into L1 one energy-loop iteration
    // ahead (GB300: 0.221 -> 0.216 ms per iteration at 4.19M MA bins, results
    // unchanged)
    dev.prefetch = 1;
    dev.ctl = d_ctl;
    for (int p = 0; p < 4; ++p) dev.LE[p] = tab.LE[p];
    dev.kappa = tab.integ_coef;
    for (int p = 0; p < 4; ++p) {
        const double lk = tab.LE[p] * tab.integ_coef;
        dev.LEkf[p] = (float)lk;
        dev.LEkf[4 + p] = (float)(lk - (double)dev.LEkf[p]);
    }
    dev.Rv = cfg.Rv;
    dev.eps0 = cfg.eps0;
    dev.ksi = cfg.ksi;
    dev.maxdr = cfg.max_dr;
    dev.Rn = cfg.Rn;
    dev.has_matter = cfg.has_matter;
    dev.mat_coeff = tab.mat_coeff;
    dev.nbfar = tab.nbfar_coeff;
    dev.nb0 = cfg.nb0;
    dev.hNS = cfg.hNS;

    if (cfg.precision != XF_PREC_FP64) {
        mixed = xf::mixed_create(this);
        if (!mixed) return err.empty() ? fail(XF_ENOMEM, "mixed-precision state allocation failed") : XF_ENOMEM;
        if (cfg.precision == XF_PREC_DF) {
            // psi1 and psi3 as compensated pairs, hi then lo, in FP64-sized buffers
            const size_t nst = (size_t)nbeams * 4 * epad;
            if ((rc = dalloc(this, &d_psi[1], nst)) || (rc = dalloc(this, &d_psi[2], nst))) return rc;
            dev.psi1 = d_psi[1];
            dev.psi3 = d_psi[2];
            dev.df = 1;
        }
    } else {
        const size_t nst = (size_t)nbeams * 4 * epad;
        for (int i = 0; i < 4; ++i)
            if ((rc = dalloc(this, &d_psi[i], nst))) return rc;
        for (int i = 0; i < 2; ++i)
            if ((rc = dalloc(this, &d_S[i], 4 * (size_t)nbeams))) return rc;
        dev.psi1 = d_psi[1];
        dev.psi3 = d_psi[2];
        h_ctl->psi0 = d_psi[0];
        h_ctl->psi4 = d_psi[3];
        h_ctl->S0 = d_S[0];
        h_ctl->S4 = d_S[1];
        XF_CUDA(this, cudaMemcpy(d_ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice));
    }
    std::vector<double> psi;
    xf::initial_state(nbeams, ne, cfg.seed, cfg.noise_amp, psi);
    return set_state(psi.data());
}

void xf_handle::release()
{
    xf_io_close(this);
    if (mixed) xf::mixed_destroy(mixed);
    mixed = nullptr;
    for (auto& g : graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    graphs.clear();
    if (step_exec) cudaGraphExecDestroy(step_exec);
    step_exec = nullptr;
    double* bufs[] = {d_fv, d_hvac, d_cos2R, d_dcos2R, d_sinR, d_cosphi, d_sinphi, d_geo, d_partials, d_hvv,
                      d_Sscratch, d_psi[0], d_psi[1], d_psi[2], d_psi[3], d_S[0], d_S[1], d_log};
    for (double* b : bufs)
        if (b) cudaFree(b);
    if (d_geof) cudaFree(d_geof);
    if (d_gticket) cudaFree(d_gticket);
    if (d_phif) cudaFree(d_phif);
    if (d_ctl) cudaFree(d_ctl);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_in) cudaFreeHost(h_in);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : tev)
        if (e) cudaEventDestroy(e);
    tev.clear();
    if (st) cudaStreamDestroy(st);
}

void xf_handle::launch_ph(int phase, const Dev& d)
{
    if (mixed) xf::mixed_launch_phase(phase, d, shape, st);
    else xf::launch_phase(phase, d, shape, st);
}

int xf_handle::pull_ctl()
{
    XF_CUDA(this, cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    d2h_bytes += sizeof(Ctl);
    return XF_OK;
}

int xf_handle::set_state(const double* psi)
{
    if (mixed) return xf::mixed_set_state(this, mixed, psi);
    int rc;
    if ((rc = pull_ctl())) return rc;
    XF_CUDA(this, cudaMemcpy2DAsync(h_ctl->psi0, epad * sizeof(double), psi, ne * sizeof(double),
                                    ne * sizeof(double), (size_t)nbeams * 4, cudaMemcpyHostToDevice, st));
    xf::launch_esum(dev, h_ctl->psi0, h_ctl->S0, st);
    XF_CUDA(this, cudaGetLastError());
    XF_CUDA(this, cudaStreamSynchronize(st));
    j0_valid = false;
    return XF_OK;
}

int xf_handle::get_state(int which, double* psi)
{
    if (mixed) return xf::mixed_get_state(this, mixed, which, psi);
    int rc;
    if ((rc = pull_ctl())) return rc;
    const double* src = nullptr;
    switch (which) {
    case 0: src = h_ctl->psi0; break;
    case 1: src = d_psi[1]; break;
    case 3: src = d_psi[2]; break;
    case 4: src = h_ctl->psi4; break;
    default: return fail(XF_EINVAL, "which must be 0, 1, 3 or 4");
    }
    XF_CUDA(this, cudaMemcpy2DAsync(psi, ne * sizeof(double), src, epad * sizeof(double), ne * sizeof(double),
                                    (size_t)nbeams * 4, cudaMemcpyDeviceToHost, st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    return XF_OK;
}

// Writes r, dr and the host matter terms (matt::getHm at the three stage
// points, src/Nmr.cpp:162-165) into the control block.
int xf_handle::push_inputs(double r, double dr)
{
    const double dr2 = .5 * dr;
    h_in[0] = r;
    h_in[1] = dr;
    h_in[2] = xf::matter_hm(cfg, tab, r);
    h_in[3] = xf::matter_hm(cfg, tab, r + dr2);
    h_in[4] = xf::matter_hm(cfg, tab, r + dr);
    XF_CUDA(this, cudaMemcpyAsync(&d_ctl->r, h_in, 5 * sizeof(double), cudaMemcpyHostToDevice, st));
    h2d_bytes += 5 * sizeof(double);
    return XF_OK;
}

// Recomputes the cached moments J0 of psi0 at stage point 0 of radius r, from
// the per-beam sums S0 (the reference's calc_Hvv(psi0, 0) uses the cached
// hSumMat with the angle tables of the current r, src/Phy_MA.cpp:455-474).
int xf_handle::refresh_j0(double r)
{
    if (j0_valid && j0_r == r) return XF_OK;
    Dev d = dev;
    d.device_control = 0;
    xf::launch_moments(d, nullptr, 0, &d_ctl->J0[0], st);
    XF_CUDA(this, cudaGetLastError());
    j0_valid = true;
    j0_r = r;
    launches++;
    return XF_OK;
}

int xf_handle::step(double r, double dr, double* max_err)
{
    int rc;
    if ((rc = push_inputs(r, dr))) return rc;
    Dev d = dev;
    d.device_control = 0;
    d.debug_psi3 = debug_psi3;
    xf::launch_geometry(d, st);
    if ((rc = refresh_j0(r))) return rc;
    if (time_phases) XF_CUDA(this, cudaEventRecord(ev[0], st));
    launch_ph(xf::PH_A, d);
    if (time_phases) XF_CUDA(this, cudaEventRecord(ev[1], st));
    launch_ph(xf::PH_B, d);
    if (time_phases) XF_CUDA(this, cudaEventRecord(ev[2], st));
    launch_ph(xf::PH_C, d);
    if (time_phases) XF_CUDA(this, cudaEventRecord(ev[3], st));
    XF_CUDA(this, cudaGetLastError());
    launches += 4;
    XF_CUDA(this, cudaMemcpyAsync(&h_ctl->max_err, &d_ctl->max_err, sizeof(double), cudaMemcpyDeviceToHost, st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    d2h_bytes += sizeof(double);
    if (time_phases) {
        float ms;
        for (int i = 0; i < 3; ++i) {
            XF_CUDA(this, cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            phase_ms[i] += ms;
            phase_n[i]++;
        }
    }
    last_r = r;
    last_dr = dr;
    *max_err = h_ctl->max_err;
    if (*max_err != *max_err) return fail(XF_ENAN, "step error is NaN");
    return XF_OK;
}

int xf_handle::accept()
{
    Dev d = dev;
    bool renormed = false;
    if (mixed) {
        xf::mixed_launch_accept(d, st);
        // unitarity renormalisation of the accepted FP32 state every renorm_every steps
        if (renorm_every > 0 && ++accepts_since_renorm >= renorm_every) {
            xf::mixed_launch_renorm(d, 0, st);
            accepts_since_renorm = 0;
            renormed = true;
            launches++;
        }
    } else {
        xf::launch_accept(d, st);
    }
    XF_CUDA(this, cudaGetLastError());
    XF_CUDA(this, cudaStreamSynchronize(st));
    launches++;
    // J0 now holds the candidate's moments at point 2 of the last step, which
    // is point 0 of radius r + dr; after a renormalisation it is recomputed
    // from the renormalised state at the next step.
    j0_valid = !renormed;
    j0_r = last_r + last_dr;
    return XF_OK;
}

int xf_handle::run_host(const xf_run_opts& o, xf_step_cb cb, void* user, xf_run_stats& s)
{
    double r = std::isnan(o.r0) ? cfg.R0 : o.r0;
    double dr = std::isnan(o.dr0) ? cfg.dr : o.dr0;
    const long Ts = o.max_iters >= 0 ? o.max_iters : cfg.Ts;
    long it = 0, acc = 0;
    const double t0 = now_s();
    double me = 0.;
    int rc = XF_OK;
    XF_CUDA(this, cudaEventRecord(ev[4], st));
    while (true) {
        const double el = now_s() - t0;
        if (!((r < cfg.Rn) && ((long)el < cfg.Tn) && (it < Ts))) break;
        rc = step(r, dr, &me);
        if (rc == XF_ENAN) break;
        if (rc) return rc;
        if (me < cfg.eps0) {
            r += dr;
            if ((rc = accept())) return rc;
            if (o.log && acc < o.log_cap) {
                o.log[3 * acc + 0] = (double)it;
                o.log[3 * acc + 1] = r;
                o.log[3 * acc + 2] = dr;
                s.log_len = acc + 1;
            }
            if (o.write_files && (rc = dump_files(it, r, dr))) {
                flush_files();
                return rc;
            }
            acc++;
            if (cb && cb(user, it, r, dr)) {
                it++;
                break;
            }
        }
        it++;
        dr *= cfg.ksi * std::sqrt(cfg.eps0 / me);
        dr = (dr > cfg.max_dr) ? cfg.max_dr : dr;
        dr = (r + dr > cfg.Rn) ? cfg.Rn - r : dr;
    }
    XF_CUDA(this, cudaEventRecord(ev[5], st));
    XF_CUDA(this, cudaEventSynchronize(ev[5]));
    float ms = 0.f;
    XF_CUDA(this, cudaEventElapsedTime(&ms, ev[4], ev[5]));
    // the run's output records are complete when xf_run returns
    if (o.write_files) {
        const int frc = flush_files();
        if (!rc) rc = frc;
    }
    s.device_ms = ms;
    s.iterations = it;
    s.accepted = acc;
    s.r_end = r;
    s.dr_end = dr;
    s.seconds = now_s() - t0;
    s.last_max_err = me;
    return rc;
}

// Builds (once per iteration count) a CUDA graph of `k` device-controlled
// iterations, each geometry + phases A, B, C, followed by a copy of the control
// block to pinned host memory.  With timing enabled, external event records
// bracket every phase kernel.
int xf_handle::get_graph(int k, bool timed, cudaGraphExec_t* out)
{
    for (auto& g : graphs)
        if (g.k == k && g.timed == timed) {
            *out = g.exec;
            return XF_OK;
        }
    Dev d = dev;
    d.device_control = 1;
    d.log = d_log;
    d.log_cap = log_cap_dev;
    d.renorm_every = mixed ? renorm_every : 0;
    if (timed) {
        const size_t need = (size_t)k * 6;
        while (tev.size() < need) {
            cudaEvent_t e;
            XF_CUDA(this, cudaEventCreate(&e));
            tev.push_back(e);
        }
    }
    cudaGraph_t g;
    XF_CUDA(this, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < k; ++i) {
        xf::launch_geometry(d, st);
        if (mixed && !dev.df) {
            // after a flagged accepted step: renormalise psi0, refresh its exact
            // sums and its moments at stage point 0 of the new radius
            xf::mixed_launch_renorm(d, 1, st);
            xf::launch_moments(d, nullptr, 0, &d_ctl->J0[0], st, 1);
        }
        for (int ph = 0; ph < 3; ++ph) {
            if (timed) cudaEventRecordWithFlags(tev[6 * i + 2 * ph], st, cudaEventRecordExternal);
            launch_ph(ph, d);
            if (timed) cudaEventRecordWithFlags(tev[6 * i + 2 * ph + 1], st, cudaEventRecordExternal);
        }
    }
    cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (ce != cudaSuccess) return fail(XF_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    cudaGraphExec_t ex;
    ce = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(XF_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    graphs.push_back(GraphEntry{k, timed, ex});
    *out = ex;
    return XF_OK;
}

// One cooperative launch of up to k device-controlled iterations (the
// persistent loop, xf_persist.cu) followed by the copy of the control block,
// as one launch of a k-iteration graph does.  A barrier wait that ran out
// leaves the reduction tickets of an unfinished phase behind: they are
// cleared, and the call reports XF_ETIMEOUT.
int xf_handle::launch_persistent(int k)
{
    Dev d = dev;
    d.device_control = 1;
    d.log = d_log;
    d.log_cap = log_cap_dev;
    d.renorm_every = 0;
    const int blocks = xf::persist_blocks(d);
    if (blocks <= 0) return fail(XF_ECUDA, "persistent loop: the kernel cannot be resident");
    XF_CUDA(this, cudaMemsetAsync(&d_ctl->bar, 0, sizeof(unsigned int), st));
    const unsigned long long limit = (unsigned long long)(barrier_timeout_ms * 1e6);
    XF_CUDA(this, xf::launch_persist(d, blocks, k, (unsigned)barrier_extra, limit, st));
    XF_CUDA(this, cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    if (h_ctl->bar_timeout) {
        XF_CUDA(this, cudaMemsetAsync(d_gticket, 0, 4 * (size_t)xf::kMaxRedGroups * sizeof(unsigned int), st));
        XF_CUDA(this, cudaMemsetAsync(&d_ctl->ticket[0], 0, sizeof(h_ctl->ticket), st));
        XF_CUDA(this, cudaMemsetAsync(&d_ctl->bar_timeout, 0, sizeof(int), st));
        XF_CUDA(this, cudaStreamSynchronize(st));
        j0_valid = false;
        return fail(XF_ETIMEOUT, "persistent loop: a grid-barrier wait ran out");
    }
    return XF_OK;
}

// Prepares the control block for a device-controlled loop from (r, dr) with
// an iteration budget Ts: moments of psi0 at stage point 0 of r, counters
// reset, done set if there is nothing to do.  Synchronous.
int xf_handle::start_device_run(double r, double dr, long Ts, bool files)
{
    int rc;
    if ((rc = push_inputs(r, dr))) return rc;
    {
        Dev d = dev;
        xf::launch_geometry(d, st);
        if ((rc = refresh_j0(r))) return rc;
    }
    if ((rc = pull_ctl())) return rc;
    h_ctl->r = r;
    h_ctl->dr = dr;
    h_ctl->iters = 0;
    h_ctl->accepted = 0;
    h_ctl->max_iters = Ts;
    h_ctl->nan_seen = 0;
    h_ctl->log_len = 0;
    h_ctl->renorm_due = 0;
    h_ctl->done = (r < cfg.Rn && Ts > 0) ? 0 : 1;
    for (int i = 0; i < 4; ++i) h_ctl->ticket[i] = 0;
    h_ctl->bar = 0;
    h_ctl->bar_timeout = 0;
    h_ctl->io_mode = 0;
    h_ctl->stage_kind = 0;
    if (files) io_dev_fill(h_ctl);
    XF_CUDA(this, cudaMemcpyAsync(d_ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    h2d_bytes += sizeof(Ctl);
    return XF_OK;
}

int xf_handle::run_device(const xf_run_opts& o, xf_run_stats& s)
{
    double r = std::isnan(o.r0) ? cfg.R0 : o.r0;
    double dr = std::isnan(o.dr0) ? cfg.dr : o.dr0;
    const long Ts = o.max_iters >= 0 ? o.max_iters : cfg.Ts;
    const int k = o.iters_per_launch > 0 ? o.iters_per_launch : kDefaultItersPerLaunch;
    int rc;
    // device log buffer for accepted steps
    if (o.log && o.log_cap > 0 && o.log_cap > log_cap_dev) {
        for (auto& g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        graphs.clear();
        if (d_log) cudaFree(d_log);
        d_log = nullptr;
        if ((rc = dalloc(this, &d_log, 3 * (size_t)o.log_cap))) return rc;
        log_cap_dev = o.log_cap;
    }
    const bool files = o.write_files && cfg.dump_mode != 0;
    // the persistent loop serves FP64 and double-float; per-phase timing needs the graphs' events.
    // The default takes it when one wave of two 8-warp blocks per SM covers every beam: there it
    // wins (GB300, ms per iteration, graphs -> persistent, 65 K bins: FP64 0.0734 -> 0.0679,
    // double-float 0.0512 -> 0.0500), while at 4.19 M bins the phase kernels' own grids are
    // better balanced (FP64 1.70 -> 1.91, double-float 0.442 -> 0.465).
    const bool auto_pers = (!mixed || dev.df) && nbeams <= 2 * 152 * 8;
    // (the persistent kernel has the FP64 averages folded; fp64_fused = 0 runs the graphs)
    const bool pers = (persistent > 0 || (persistent < 0 && auto_pers)) && (!mixed || dev.df) && !o.time_phases &&
                      (dev.df || shape.fp64_fused);
    if (files && (rc = io_dev_prepare(k))) return rc;
    if ((rc = start_device_run(r, dr, Ts, files))) return rc;
    // instantiate the graph sizes this run needs before the timed region starts
    if (!pers) {
        cudaGraphExec_t ex;
        if (Ts > 0 && (rc = get_graph((int)std::min<long>(k, Ts), o.time_phases != 0, &ex))) return rc;
        if (Ts > k && Ts % k && (rc = get_graph((int)(Ts % k), o.time_phases != 0, &ex))) return rc;
    }
    const double t0 = now_s();
    XF_CUDA(this, cudaEventRecord(ev[4], st));
    long long prev_iters = 0;
    long long io_count = 0, io_staged = 0;  // records of the previous launch, drained during the next
    bool io_pending = false;
    while (!h_ctl->done) {
        if ((long)(now_s() - t0) >= cfg.Tn) break;
        // the last launch is sized to the remaining iteration budget, so that no
        // graph node runs only to find the loop finished
        const long long left = Ts - prev_iters;
        const int kk = (int)std::min<long long>(k, std::max<long long>(1, left));
        cudaGraphExec_t ex = nullptr;
        if (!pers && (rc = get_graph(kk, o.time_phases != 0, &ex))) return rc;
        // every iteration of the launch may decide an output record: their slots must be free
        if (files && (rc = io_dev_reserve(kk))) return rc;
        if (pers) {
            // the previous launch's records go to the writer before this one
            if (io_pending && (rc = io_dev_drain(io_count, io_staged, false))) return rc;
            io_pending = false;
            if ((rc = launch_persistent(kk))) return rc;
        } else {
            XF_CUDA(this, cudaGraphLaunch(ex, st));
            // the previous launch's records go to the writer while this launch runs
            if (io_pending && (rc = io_dev_drain(io_count, io_staged, false))) return rc;
            io_pending = false;
            XF_CUDA(this, cudaStreamSynchronize(st));
        }
        if (files) {
            io_count = h_ctl->io_count;
            io_staged = h_ctl->io_staged;
            io_pending = true;
        }
        const long long ran = h_ctl->iters - prev_iters;
        launches += pers ? 1 : 4 * ran;
        d2h_bytes += sizeof(Ctl);  // the graph's copy of the control block
        if (o.time_phases) {
            for (long long i = 0; i < ran && i < kk; ++i)
                for (int ph = 0; ph < 3; ++ph) {
                    float ms;
                    XF_CUDA(this, cudaEventElapsedTime(&ms, tev[6 * i + 2 * ph], tev[6 * i + 2 * ph + 1]));
                    phase_ms[ph] += ms;
                    phase_n[ph]++;
                }
        }
        prev_iters = h_ctl->iters;
        if (ran == 0) break;
    }
    XF_CUDA(this, cudaEventRecord(ev[5], st));
    XF_CUDA(this, cudaEventSynchronize(ev[5]));
    float ms = 0.f;
    XF_CUDA(this, cudaEventElapsedTime(&ms, ev[4], ev[5]));
    if (files) {
        // the record of the last accepted step (if any) is staged here; then
        // the trigger state returns to the host and the files are flushed
        if ((rc = io_dev_drain(h_ctl->io_count, h_ctl->io_staged, true))) return rc;
        if ((rc = io_dev_end())) return rc;
    }
    s.device_ms = ms;
    s.seconds = now_s() - t0;
    s.iterations = (long)h_ctl->iters;
    s.accepted = (long)h_ctl->accepted;
    s.r_end = h_ctl->r;
    s.dr_end = h_ctl->dr;
    s.last_max_err = h_ctl->max_err;
    if (o.log && h_ctl->log_len > 0) {
        const long n = (long)std::min<long long>(h_ctl->log_len, o.log_cap);
        XF_CUDA(this, cudaMemcpy(o.log, d_log, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
        d2h_bytes += 3 * (long long)n * sizeof(double);
        s.log_len = n;
    }
    j0_valid = true;
    j0_r = h_ctl->r;
    // hand the control block back to host-driven use: kernels skip work while done is set
    XF_CUDA(this, cudaMemsetAsync(&d_ctl->done, 0, sizeof(int), st));
    XF_CUDA(this, cudaStreamSynchronize(st));
    if (h_ctl->nan_seen) return fail(XF_ENAN, "step error is NaN");
    return XF_OK;
}


// ------------------------------------------------------------------ C ABI

extern "C" {

int xf_run_opts_default(xf_run_opts* o)
{
    if (!o) return XF_EINVAL;
    std::memset(o, 0, sizeof(*o));
    o->max_iters = -1;
    o->iters_per_launch = kDefaultItersPerLaunch;
    o->r0 = NAN;
    o->dr0 = NAN;
    return XF_OK;
}

int xf_create(const xf_config* cfg, xf_handle** out)
{
    if (!cfg || !out) return XF_EINVAL;
    *out = nullptr;
    std::string why;
    int rc = check_config(*cfg, why);
    if (rc) {
        std::fprintf(stderr, "xf_create: %s\n", why.c_str());
        return rc;
    }
    xf_handle* h = new (std::nothrow) xf_handle();
    if (!h) return XF_ENOMEM;
    rc = h->init(*cfg);
    if (rc) {
        std::fprintf(stderr, "xf_create: %s\n", h->err.c_str());
        h->release();
        delete h;
        return rc;
    }
    *out = h;
    return XF_OK;
}

int xf_destroy(xf_handle* h)
{
    if (!h) return XF_EINVAL;
    h->release();
    delete h;
    return XF_OK;
}

const char* xf_last_error(const xf_handle* h) { return h ? h->err.c_str() : "null handle"; }

int xf_dims(const xf_handle* h, int* nbeams, int* ebins, int* abins, int* pbins)
{
    if (!h) return XF_EINVAL;
    if (nbeams) *nbeams = h->nbeams;
    if (ebins) *ebins = h->ne;
    if (abins) *abins = h->A;
    if (pbins) *pbins = h->P;
    return XF_OK;
}

int xf_set_option(xf_handle* h, const char* name, double value)
{
    if (!h || !name) return XF_EINVAL;
    const std::string n = name;
    if (n == "debug_psi3") {
        h->debug_psi3 = value != 0.;
    } else if (n == "renorm_every") {
        if (value < 0.) return h->fail(XF_EINVAL, "renorm_every must be >= 0");
        if (h->dev.df && value > 0.)
            return h->fail(XF_EUNSUPPORTED, "the double-float path keeps |a|^2 + |b|^2 = 1 without renormalisation");
        h->renorm_every = (int)value;
    } else if (n == "prefetch") {
        if (value < 0. || value > 8.) return h->fail(XF_EINVAL, "prefetch must be in [0, 8]");
        h->dev.prefetch = (int)value;
    } else if (n == "threads") {
        const int t = (int)value;
        if (t != 0 && (t < 32 || t > 256 || t % 32)) return h->fail(XF_EINVAL, "threads must be a multiple of 32 in [32, 256]");
        h->shape.threads = t ? t : 256;
        const int cap = xf::max_phase_blocks(h->nbeams, 32);
        h->shape.blocks = std::min(h->shape.blocks, std::max(1, cap));
        h->shape.blocks_ab = std::min(h->shape.blocks_ab, std::max(1, cap));
        for (int& pb : h->shape.phase_blocks) pb = std::min(pb, std::max(1, cap));
    } else if (n == "blocks") {
        const int b = (int)value;
        const int cap = std::max(xf::max_phase_blocks(h->nbeams, 256), 152 * 4);
        if (b < 0 || b > cap) return h->fail(XF_EINVAL, "blocks out of range");
        xf::Shape def = h->shape;
        if (h->dev.df) xf::df_default_shape(h->nbeams, def);
        else def = xf::default_shape(h->nbeams, h->epad, h->mixed != nullptr);
        h->shape.blocks = b ? b : def.blocks;
        h->shape.blocks_ab = b ? b : def.blocks_ab;
        for (int p = 0; p < 3; ++p) h->shape.phase_blocks[p] = b ? b : def.phase_blocks[p];
    } else if (n == "fp64_fused") {
        h->shape.fp64_fused = value != 0.;
    } else if (n == "persistent") {
        if (value != -1. && value != 0. && value != 1.) return h->fail(XF_EINVAL, "persistent must be -1, 0 or 1");
        h->persistent = (int)value;
    } else if (n == "barrier_timeout_ms") {
        if (!(value > 0.) || value > 60000.) return h->fail(XF_EINVAL, "barrier_timeout_ms must be in (0, 60000]");
        h->barrier_timeout_ms = value;
    } else if (n == "debug_barrier_extra") {
        if (value < 0. || value > 1024.) return h->fail(XF_EINVAL, "debug_barrier_extra must be in [0, 1024]");
        h->barrier_extra = (int)value;
    } else if (n == "df_b_occupancy") {
        const int o = (int)value;
        if (!h->dev.df) return h->fail(XF_EUNSUPPORTED, "df_b_occupancy applies to the double-float path");
        if (o != 2 && o != 3) return h->fail(XF_EINVAL, "df_b_occupancy must be 2 or 3");
        h->shape.df_b_occ = o;
        xf::df_default_shape(h->nbeams, h->shape);
    } else {
        return h->fail(XF_EINVAL, "unknown option " + n);
    }
    for (auto& g : h->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
    return XF_OK;
}

int xf_set_state(xf_handle* h, const double* psi)
{
    if (!h || !psi) return XF_EINVAL;
    return h->set_state(psi);
}

int xf_get_state(xf_handle* h, int which, double* psi)
{
    if (!h || !psi) return XF_EINVAL;
    return h->get_state(which, psi);
}

int xf_set_noise(xf_handle* h, uint64_t seed, double amp)
{
    if (!h) return XF_EINVAL;
    std::vector<double> psi;
    xf::initial_state(h->nbeams, h->ne, seed, amp, psi);
    return h->set_state(psi.data());
}

int xf_tables(const xf_handle* h, double* fv, double* hvac, double* LE, double* Ev)
{
    if (!h) return XF_EINVAL;
    if (fv) std::memcpy(fv, h->tab.fv.data(), h->tab.fv.size() * sizeof(double));
    if (hvac) std::memcpy(hvac, h->tab.hvac.data(), h->tab.hvac.size() * sizeof(double));
    if (LE) std::memcpy(LE, h->tab.LE, 4 * sizeof(double));
    if (Ev) std::memcpy(Ev, h->tab.Ev, 4 * sizeof(double));
    return XF_OK;
}

int xf_matter(const xf_handle* h, double r, double* hm)
{
    if (!h || !hm) return XF_EINVAL;
    *hm = xf::matter_hm(h->cfg, h->tab, r);
    return XF_OK;
}

int xf_angle_bins(xf_handle* h, double r, double dr, double* cosb, double* sinb, double* dcosb, double* dl)
{
    if (!h) return XF_EINVAL;
    int rc;
    if ((rc = h->push_inputs(r, dr))) return rc;
    Dev d = h->dev;
    d.device_control = 0;
    xf::launch_geometry(d, h->st);
    XF_CUDA(h, cudaGetLastError());
    std::vector<double> g(12 * (size_t)h->A);
    XF_CUDA(h, cudaMemcpyAsync(g.data(), h->d_geo, g.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    XF_CUDA(h, cudaStreamSynchronize(h->st));
    const size_t n = 3 * (size_t)h->A;
    if (cosb) std::memcpy(cosb, &g[0], n * sizeof(double));
    if (sinb) std::memcpy(sinb, &g[n], n * sizeof(double));
    if (dcosb) std::memcpy(dcosb, &g[2 * n], n * sizeof(double));
    if (dl) std::memcpy(dl, &g[3 * n], n * sizeof(double));
    return XF_OK;
}

int xf_calc_hvv(xf_handle* h, int which, int pt, double r, double dr, double* hvv)
{
    if (!h || !hvv || pt < 0 || pt > 2) return XF_EINVAL;
    if (h->mixed && which != 0) return h->fail(XF_EUNSUPPORTED, "the mixed path keeps only psi0's energy sums");
    int rc;
    if ((rc = h->pull_ctl())) return rc;
    if ((rc = h->push_inputs(r, dr))) return rc;
    Dev d = h->dev;
    d.device_control = 0;
    xf::launch_geometry(d, h->st);
    const double* S;
    if (which == 0) {
        S = h->h_ctl->S0;
    } else {
        const double* src = which == 1 ? h->d_psi[1] : which == 3 ? h->d_psi[2] : which == 4 ? h->h_ctl->psi4 : nullptr;
        if (!src) return h->fail(XF_EINVAL, "which must be 0, 1, 3 or 4");
        xf::launch_esum(d, src, h->d_Sscratch, h->st);
        S = h->d_Sscratch;
    }
    xf::launch_moments(d, S, pt, &h->d_ctl->JM[0], h->st);
    xf::launch_hvv_eval(d, &h->d_ctl->JM[0], pt, h->d_hvv, h->st);
    XF_CUDA(h, cudaGetLastError());
    XF_CUDA(h, cudaMemcpyAsync(hvv, h->d_hvv, 4 * (size_t)h->A * h->P * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    XF_CUDA(h, cudaStreamSynchronize(h->st));
    return XF_OK;
}

int xf_step(xf_handle* h, double r, double dr, double* max_err)
{
    if (!h || !max_err) return XF_EINVAL;
    return h->step(r, dr, max_err);
}

int xf_accept(xf_handle* h)
{
    if (!h) return XF_EINVAL;
    return h->accept();
}

int xf_run(xf_handle* h, const xf_run_opts* opts, xf_step_cb cb, void* user, xf_run_stats* stats)
{
    if (!h) return XF_EINVAL;
    xf_run_opts o;
    if (opts) o = *opts;
    else xf_run_opts_default(&o);
    xf_run_stats s;
    std::memset(&s, 0, sizeof(s));
    h->launches = 0;
    h->h2d_bytes = h->d2h_bytes = 0;
    h->time_phases = o.time_phases;
    // xf_phase_times reports the last run that timed its phases
    if (o.time_phases)
        for (int i = 0; i < 3; ++i) {
            h->phase_ms[i] = 0.;
            h->phase_n[i] = 0;
        }
    int rc;
    if (o.device_control) {
        if (cb) return h->fail(XF_EUNSUPPORTED, "per-step callbacks need the host-driven loop");
        rc = h->run_device(o, s);
    } else {
        rc = h->run_host(o, cb, user, s);
    }
    h->time_phases = 0;
    s.kernel_launches = h->launches;
    s.h2d_bytes = h->h2d_bytes;
    s.d2h_bytes = h->d2h_bytes;
    if (stats) *stats = s;
    return rc;
}

int xf_replay(xf_handle* h, const double* r_before, const double* dr, long n)
{
    if (!h || (n > 0 && (!r_before || !dr))) return XF_EINVAL;
    for (long i = 0; i < n; ++i) {
        double me;
        int rc = h->step(r_before[i], dr[i], &me);
        if (rc) return rc;
        if ((rc = h->accept())) return rc;
    }
    return XF_OK;
}

int xf_phase_times(const xf_handle* h, double* out, long* counts)
{
    if (!h || !out) return XF_EINVAL;
    for (int i = 0; i < 3; ++i) {
        out[i] = h->phase_n[i] ? h->phase_ms[i] / h->phase_n[i] : 0.;
        if (counts) counts[i] = h->phase_n[i];
    }
    return XF_OK;
}

// Per-beam survival of psi0 (src/IO_f.cpp:341-351), computed on the device.
int xf_survival(xf_handle* h, double* out)
{
    if (!h || !out) return XF_EINVAL;
    xf::launch_survival(h->dev, h->mixed != nullptr, h->d_Sscratch, h->st);
    XF_CUDA(h, cudaGetLastError());
    h->launches++;
    XF_CUDA(h, cudaMemcpyAsync(out, h->d_Sscratch, (size_t)h->nbeams * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    XF_CUDA(h, cudaStreamSynchronize(h->st));
    return XF_OK;
}

}  // extern "C"
