// Batched path: many independent MA simulations of uneven angle and energy
// counts, each with its own adaptive step control, advanced together.
//
// Every instance keeps its own tables, state, control block and partial-sum
// buffer (an xf_handle).  One iteration of the batch is one launch per stage
// kernel over a work list of tiles: a tile is warps x beams-per-warp
// consecutive beams of one instance, each warp striding over its beams.  The
// blocks of an instance form that instance's
// reduction group: the last of its tiles to finish reduces the instance's
// moments in fixed order and, in the last phase, runs the instance's step
// controller (accept/reject, dr, termination; src/Nmr.cpp:227-249).  An
// instance that has finished skips its tiles, so instances with different step
// counts share the launches.  Iterations are captured in CUDA graphs and the
// host only polls a compact status array between graph launches.  The tile
// shape (warps per block, which sets the block size, and beams per warp,
// which sets the number of blocks per phase) is chosen at creation by timing
// the candidates on the batch itself (xf_batch_create's autotuner).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xf_common.cuh"
#include "xf_launch.cuh"
#include "xf_engine.h"
#include "xf_df.cuh"
#include "xf_fp64.cuh"
#include "xf_mixed.cuh"
#include "xf_persist.cuh"
#include "xflat_gpu.h"

using xf::Ctl;
using xf::Dev;

namespace {

using namespace xf::detail;

struct Tile {
    int inst, first, idx, count;  // instance, first beam, tile index and tile count within the instance
    int end;                      // one past the tile's last beam
};

struct Status {
    double r, dr;
    long long iters, accepted;
    int done, nan_seen;
};

__device__ __forceinline__ RedTarget tile_target(const Dev& d, const Tile& t, int phase)
{
    RedTarget rt;
    rt.partials = d.partials;
    rt.idx = t.idx;
    rt.count = t.count;
    rt.ticket = &d.ctl->ticket[phase];
    rt.gticket = d.gticket + phase * xf::kMaxRedGroups;
    return rt;
}

// Blocks of 32 work-list angles x 3 stage points (geometry_point); the
// angles of one block may belong to different instances.
__global__ void __launch_bounds__(96) k_batch_geometry(const Dev* __restrict__ devs, const int2* __restrict__ angles, int n)
{
    xf::pdl_enter();
    __shared__ double s_c[96];
    const int slot = threadIdx.x % 32, pt = threadIdx.x / 32;
    const int i = blockIdx.x * 32 + slot;
    const int2 a = i < n ? angles[i] : make_int2(0, -1);
    geometry_point(devs[a.x], a.y, pt, slot, 32, s_c);
}

// The batched phases take the single-simulation kernels' register caps for
// MA (resident warps per SM over spills; see xf_kernels.cu, xf_mixed.cu and
// xf_df.cu).
template <int PREC, int PH>
constexpr int batch_min_blocks()
{
    return PREC == XF_PREC_FP64    ? (PH == xf::PH_C ? 3 : 1)
           : PREC == XF_PREC_MIXED ? (PH == xf::PH_A ? 5 : (PH == xf::PH_B ? 6 : 4))
                                   : 3;
}

template <int PREC, int PH>
__global__ void __launch_bounds__(256, batch_min_blocks<PREC, PH>()) k_batch_phase(const Dev* __restrict__ devs,
                                                                                     const Tile* __restrict__ tiles)
{
    xf::pdl_enter();
    const Tile t = tiles[blockIdx.x];
    const Dev& d = devs[t.inst];
    const RedTarget rt = tile_target(d, t, PH);
    const int nw = blockDim.x >> 5;
    if (PREC == XF_PREC_FP64) {
        if (PH == xf::PH_A) xf::fp64::phaseA_body<0>(d, t.first, nw, rt, t.end);
        else if (PH == xf::PH_B) xf::fp64::phaseB_body<0>(d, t.first, nw, rt, t.end);
        else xf::fp64::phaseC_body<0>(d, t.first, nw, rt, t.end);
    } else if (PREC == XF_PREC_MIXED) {
        if (PH == xf::PH_A) xf::mixed::phaseA_body<0>(d, t.first, nw, rt, t.end);
        else if (PH == xf::PH_B) xf::mixed::phaseB_body<0>(d, t.first, nw, rt, t.end);
        else xf::mixed::phaseC_body<0>(d, t.first, nw, rt, t.end);
    } else {
        if (PH == xf::PH_A) xf::dfp::phaseA_body<0>(d, t.first, nw, rt, t.end);
        else if (PH == xf::PH_B) xf::dfp::phaseB_body<0>(d, t.first, nw, rt, t.end);
        else xf::dfp::phaseC_body<0>(d, t.first, nw, rt, t.end);
    }
}

template <int PREC, int PH>
__device__ __forceinline__ void tile_phase(const Dev* __restrict__ devs, const Tile& t)
{
    const Dev& d = devs[t.inst];
    const RedTarget rt = tile_target(d, t, PH);
    const int nw = blockDim.x >> 5;
    if (PREC == XF_PREC_FP64) {
        if (PH == xf::PH_A) xf::fp64::phaseA_body<0>(d, t.first, nw, rt, t.end);
        else if (PH == xf::PH_B) xf::fp64::phaseB_body<0>(d, t.first, nw, rt, t.end);
        else xf::fp64::phaseC_body<0>(d, t.first, nw, rt, t.end);
    } else {
        if (PH == xf::PH_A) xf::dfp::phaseA_body<0>(d, t.first, nw, rt, t.end);
        else if (PH == xf::PH_B) xf::dfp::phaseB_body<0>(d, t.first, nw, rt, t.end);
        else xf::dfp::phaseC_body<0>(d, t.first, nw, rt, t.end);
    }
}

// Persistent form of `iters` batch iterations (FP64 and double-float): one
// cooperative launch whose blocks stride over the angle list and then over
// the tile list of each phase, the stages separated by bounded grid barriers
// (xf_persist.cuh) on the batch's own counter and timeout flag.
template <int PREC>
__global__ void __launch_bounds__(256, 2) k_batch_persist(const Dev* __restrict__ devs, const Tile* __restrict__ tiles,
                                                          int ntiles, const int2* __restrict__ angles, int nang,
                                                          int iters, unsigned int* bar, int* timeout, unsigned extra,
                                                          unsigned long long limit_ns)
{
    unsigned gen = 0;
    const auto at = [&](int i, int& ang) {
        const int2 a = angles[i];
        ang = a.y;
        return &devs[a.x];
    };
    for (int i = 0; i < iters; ++i) {
        geometry_pass(nang, at);
        if (!grid_barrier(bar, timeout, gen, extra, limit_ns)) return;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) tile_phase<PREC, xf::PH_A>(devs, tiles[t]);
        if (!grid_barrier(bar, timeout, gen, extra, limit_ns)) return;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) tile_phase<PREC, xf::PH_B>(devs, tiles[t]);
        if (!grid_barrier(bar, timeout, gen, extra, limit_ns)) return;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) tile_phase<PREC, xf::PH_C>(devs, tiles[t]);
        if (!grid_barrier(bar, timeout, gen, extra, limit_ns)) return;
    }
}

// Mixed precision: flagged renormalisation with exact energy sums (warp tiles)
// and the refreshed moments of psi0 (thread tiles of 256 beams).
__global__ void __launch_bounds__(256) k_batch_renorm(const Dev* __restrict__ devs, const Tile* __restrict__ tiles)
{
    xf::pdl_enter();
    const Tile t = tiles[blockIdx.x];
    xf::mixed::esum_body(devs[t.inst], t.first, blockDim.x >> 5, 1, 1, t.end);
}

__global__ void __launch_bounds__(256) k_batch_moments(const Dev* __restrict__ devs, const Tile* __restrict__ tiles)
{
    xf::pdl_enter();
    const Tile t = tiles[blockIdx.x];
    const Dev& d = devs[t.inst];
    moments_body<0>(d, t.first, d.nbeams, tile_target(d, t, xf::PH_MOM), nullptr, 0, &d.ctl->J0[0], 1);
}

__global__ void k_batch_status(const Dev* __restrict__ devs, int n, Status* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Ctl* c = devs[i].ctl;
    Status s;
    s.r = c->r;
    s.dr = c->dr;
    s.iters = c->iters;
    s.accepted = c->accepted;
    s.done = c->done;
    s.nan_seen = c->nan_seen;
    out[i] = s;
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct xf_batch {
    std::vector<xf_handle*> h;
    int prec = XF_PREC_FP64;
    int persistent = 0;             // iterations as one cooperative launch (FP64, df; 8-warp tiles)
    unsigned int* d_bar = nullptr;  // persistent form: [0] barrier arrivals, [1] timeout flag
    int pblocks = 0;                // persistent form: resident blocks
    int warps = 8;                  // warps per block
    int bpw = 1;                    // beams per warp (a tile holds warps x bpw beams)
    cudaStream_t st = nullptr;
    Dev* d_devs = nullptr;
    Tile* d_wtiles = nullptr;       // warp tiles for the stage kernels
    Tile* d_ttiles = nullptr;       // thread tiles for the moment kernel
    int2* d_angles = nullptr;
    double* d_part = nullptr;       // partial sums of every instance
    Status* d_status = nullptr;
    Status* h_status = nullptr;     // pinned
    int nwt = 0, ntt = 0, nang = 0;
    struct G {
        int k;
        cudaGraphExec_t ex;
    };
    std::vector<G> graphs;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    static constexpr int kMaxCand = 16;
    int ncand = 0;
    int cand_warps[kMaxCand] = {}, cand_bpw[kMaxCand] = {}, cand_pers[kMaxCand] = {};
    double cand_ms[kMaxCand] = {};
    std::string err;

    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
};

#define XB_CUDA(b, call)                                                                             \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return (b)->fail(XF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

void drop_graphs(xf_batch* b)
{
    for (auto& g : b->graphs)
        if (g.ex) cudaGraphExecDestroy(g.ex);
    b->graphs.clear();
}

// Work lists and per-instance device parameter blocks for a tile shape.
int build_lists(xf_batch* b, int warps, int bpw)
{
    drop_graphs(b);
    b->warps = warps;
    b->bpw = bpw;
    const int n = (int)b->h.size();
    std::vector<Tile> wt, tt;
    std::vector<int2> ang;
    std::vector<Dev> devs(n);
    std::vector<size_t> part_off(n);
    size_t part_total = 0;
    for (int i = 0; i < n; ++i) {
        const xf_handle* h = b->h[i];
        const int span = warps * bpw;
        const int nwti = (h->nbeams + span - 1) / span;
        const int ntti = (h->nbeams + 255) / 256;
        for (int t = 0; t < nwti; ++t) wt.push_back(Tile{i, t * span, t, nwti, std::min(h->nbeams, (t + 1) * span)});
        for (int t = 0; t < ntti; ++t) tt.push_back(Tile{i, t * 256, t, ntti, std::min(h->nbeams, (t + 1) * 256)});
        for (int a = 0; a < h->A; ++a) ang.push_back(make_int2(i, a));
        part_off[i] = part_total;
        if (std::max(nwti, ntti) > xf::kRedGroup * xf::kMaxRedGroups)
            return b->fail(XF_EUNSUPPORTED, "instance " + std::to_string(i) + ": too many tiles for the reduction");
        part_total += (size_t)xf::red_rows(std::max(nwti, ntti)) * xf::kPartStride;
    }
    if (b->d_part) cudaFree(b->d_part);
    if (b->d_wtiles) cudaFree(b->d_wtiles);
    if (b->d_ttiles) cudaFree(b->d_ttiles);
    if (b->d_angles) cudaFree(b->d_angles);
    if (b->d_devs) cudaFree(b->d_devs);
    b->d_part = nullptr;
    b->d_wtiles = b->d_ttiles = nullptr;
    b->d_angles = nullptr;
    b->d_devs = nullptr;
    XB_CUDA(b, cudaMalloc(&b->d_part, part_total * sizeof(double)));
    XB_CUDA(b, cudaMemset(b->d_part, 0, part_total * sizeof(double)));
    for (int i = 0; i < n; ++i) {
        devs[i] = b->h[i]->dev;
        devs[i].device_control = 1;
        devs[i].log = nullptr;
        devs[i].log_cap = 0;
        devs[i].renorm_every = b->prec == XF_PREC_MIXED ? b->h[i]->renorm_every : 0;
        devs[i].partials = b->d_part + part_off[i];
    }
    XB_CUDA(b, cudaMalloc(&b->d_devs, n * sizeof(Dev)));
    XB_CUDA(b, cudaMemcpy(b->d_devs, devs.data(), n * sizeof(Dev), cudaMemcpyHostToDevice));
    XB_CUDA(b, cudaMalloc(&b->d_wtiles, wt.size() * sizeof(Tile)));
    XB_CUDA(b, cudaMemcpy(b->d_wtiles, wt.data(), wt.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    XB_CUDA(b, cudaMalloc(&b->d_ttiles, tt.size() * sizeof(Tile)));
    XB_CUDA(b, cudaMemcpy(b->d_ttiles, tt.data(), tt.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    XB_CUDA(b, cudaMalloc(&b->d_angles, ang.size() * sizeof(int2)));
    XB_CUDA(b, cudaMemcpy(b->d_angles, ang.data(), ang.size() * sizeof(int2), cudaMemcpyHostToDevice));
    b->nwt = (int)wt.size();
    b->ntt = (int)tt.size();
    b->nang = (int)ang.size();
    return XF_OK;
}

void launch_iteration(xf_batch* b)
{
    const int threads = 32 * b->warps;
    const Dev* dv = b->d_devs;
    const Tile* wt = b->d_wtiles;
    xf::launch_pdl(k_batch_geometry, (b->nang + 31) / 32, 96, b->st, dv, (const int2*)b->d_angles, b->nang);
    if (b->prec == XF_PREC_MIXED) {
        xf::launch_pdl(k_batch_renorm, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_moments, b->ntt, 256, b->st, dv, (const Tile*)b->d_ttiles);
        xf::launch_pdl(k_batch_phase<XF_PREC_MIXED, xf::PH_A>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_MIXED, xf::PH_B>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_MIXED, xf::PH_C>, b->nwt, threads, b->st, dv, wt);
    } else if (b->prec == XF_PREC_DF) {
        xf::launch_pdl(k_batch_phase<XF_PREC_DF, xf::PH_A>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_DF, xf::PH_B>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_DF, xf::PH_C>, b->nwt, threads, b->st, dv, wt);
    } else {
        xf::launch_pdl(k_batch_phase<XF_PREC_FP64, xf::PH_A>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_FP64, xf::PH_B>, b->nwt, threads, b->st, dv, wt);
        xf::launch_pdl(k_batch_phase<XF_PREC_FP64, xf::PH_C>, b->nwt, threads, b->st, dv, wt);
    }
}

// One cooperative launch of k iterations and the status copy (the persistent
// counterpart of a k-iteration graph launch).
int launch_persistent(xf_batch* b, int k)
{
    const int n = (int)b->h.size();
    void* fn = b->prec == XF_PREC_DF ? reinterpret_cast<void*>(k_batch_persist<XF_PREC_DF>)
                                     : reinterpret_cast<void*>(k_batch_persist<XF_PREC_FP64>);
    if (!b->pblocks) {
        int dev = 0, sms = 152, occ = 0;
        XB_CUDA(b, cudaGetDevice(&dev));
        XB_CUDA(b, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        XB_CUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 256, 0));
        if (occ < 1) return b->fail(XF_ECUDA, "persistent batch kernel cannot be resident");
        b->pblocks = std::min(occ * sms, std::max(b->nwt, (b->nang + 63) / 64));
    }
    if (!b->d_bar) XB_CUDA(b, cudaMalloc(&b->d_bar, 2 * sizeof(unsigned int)));
    XB_CUDA(b, cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned int), b->st));
    const Dev* dv = b->d_devs;
    const Tile* wt = b->d_wtiles;
    const int2* an = b->d_angles;
    int nt = b->nwt, na = b->nang, it = k;
    unsigned int* bar = b->d_bar;
    int* tmo = reinterpret_cast<int*>(b->d_bar + 1);
    unsigned extra = 0;
    unsigned long long limit = 2000000000ull;
    void* args[] = {&dv, &wt, &nt, &an, &na, &it, &bar, &tmo, &extra, &limit};
    XB_CUDA(b, cudaLaunchCooperativeKernel(fn, dim3(b->pblocks), dim3(256), args, 0, b->st));
    k_batch_status<<<(n + 63) / 64, 64, 0, b->st>>>(b->d_devs, n, b->d_status);
    XB_CUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, n * sizeof(Status), cudaMemcpyDeviceToHost, b->st));
    unsigned int flag[2] = {0, 0};
    XB_CUDA(b, cudaMemcpyAsync(flag, b->d_bar, sizeof(flag), cudaMemcpyDeviceToHost, b->st));
    XB_CUDA(b, cudaStreamSynchronize(b->st));
    if (flag[1]) return b->fail(XF_ETIMEOUT, "persistent batch: a grid-barrier wait ran out");
    return XF_OK;
}

int get_graph(xf_batch* b, int k, cudaGraphExec_t* out)
{
    for (auto& g : b->graphs)
        if (g.k == k) {
            *out = g.ex;
            return XF_OK;
        }
    cudaGraph_t g;
    XB_CUDA(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < k; ++i) launch_iteration(b);
    const int n = (int)b->h.size();
    k_batch_status<<<(n + 63) / 64, 64, 0, b->st>>>(b->d_devs, n, b->d_status);
    cudaMemcpyAsync(b->h_status, b->d_status, n * sizeof(Status), cudaMemcpyDeviceToHost, b->st);
    cudaError_t ce = cudaStreamEndCapture(b->st, &g);
    if (ce != cudaSuccess) return b->fail(XF_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    cudaGraphExec_t ex;
    ce = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return b->fail(XF_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    b->graphs.push_back(xf_batch::G{k, ex});
    *out = ex;
    return XF_OK;
}

// Device-controlled run of every instance from its config's R0/dr (or from
// where a previous run stopped when `resume`), max_iters iterations each.
int run(xf_batch* b, long max_iters, bool resume, double* device_ms)
{
    const int n = (int)b->h.size();
    long budget = max_iters;
    for (int i = 0; i < n; ++i) {
        xf_handle* h = b->h[i];
        const long Ts = max_iters >= 0 ? max_iters : h->cfg.Ts;
        budget = std::max(budget, Ts);
        double r = h->cfg.R0, dr = h->cfg.dr;
        if (resume) {
            r = b->h_status[i].r;
            dr = b->h_status[i].dr;
        }
        int rc = h->start_device_run(r, dr, Ts);
        if (rc) return b->fail(rc, "instance " + std::to_string(i) + ": " + h->err);
    }
    const int k = 8;
    cudaGraphExec_t ex = nullptr;
    int rc;
    const bool pers = b->persistent && b->prec != XF_PREC_MIXED;
    if (!pers && (rc = get_graph(b, k, &ex))) return rc;
    XB_CUDA(b, cudaEventRecord(b->e0, b->st));
    long done_iters = 0;
    while (true) {
        if (pers) {
            if ((rc = launch_persistent(b, k))) return rc;
        } else {
            XB_CUDA(b, cudaGraphLaunch(ex, b->st));
            XB_CUDA(b, cudaStreamSynchronize(b->st));
        }
        done_iters += k;
        bool all = true;
        for (int i = 0; i < n; ++i) all = all && b->h_status[i].done;
        if (all || done_iters >= budget + k) break;
    }
    XB_CUDA(b, cudaEventRecord(b->e1, b->st));
    XB_CUDA(b, cudaEventSynchronize(b->e1));
    float ms = 0.f;
    XB_CUDA(b, cudaEventElapsedTime(&ms, b->e0, b->e1));
    if (device_ms) *device_ms = ms;
    // hand the control blocks back to host-driven use
    for (int i = 0; i < n; ++i) {
        xf_handle* h = b->h[i];
        XB_CUDA(b, cudaMemsetAsync(&h->d_ctl->done, 0, sizeof(int), b->st));
        h->j0_valid = true;
        h->j0_r = b->h_status[i].r;
    }
    XB_CUDA(b, cudaStreamSynchronize(b->st));
    for (int i = 0; i < n; ++i)
        if (b->h_status[i].nan_seen) return b->fail(XF_ENAN, "instance " + std::to_string(i) + ": step error is NaN");
    return XF_OK;
}

}  // namespace

extern "C" {

int xf_batch_create(const xf_config* cfgs, int n, xf_batch** out)
{
    if (!cfgs || n <= 0 || !out) return XF_EINVAL;
    *out = nullptr;
    for (int i = 0; i < n; ++i)
        if ((cfgs[i].geometry != XF_GEOM_MA && cfgs[i].geometry != XF_GEOM_SA) || cfgs[i].precision != cfgs[0].precision)
            return XF_EUNSUPPORTED;
    xf_batch* b = new xf_batch();
    b->prec = cfgs[0].precision;
    int rc = XF_OK;
    for (int i = 0; i < n && rc == XF_OK; ++i) {
        xf_handle* h = nullptr;
        rc = xf_create(&cfgs[i], &h);
        if (rc == XF_OK) b->h.push_back(h);
    }
    if (rc == XF_OK && cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) rc = XF_ECUDA;
    if (rc == XF_OK && (cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess)) rc = XF_ECUDA;
    if (rc == XF_OK && cudaMalloc(&b->d_status, n * sizeof(Status)) != cudaSuccess) rc = XF_ENOMEM;
    if (rc == XF_OK && cudaMallocHost(&b->h_status, n * sizeof(Status)) != cudaSuccess) rc = XF_ENOMEM;
    // autotune the launch form on the batch itself: a few iterations per
    // candidate from the initial states, which are restored afterwards.  The
    // candidates are the graph-launched stages with warps per block x beams
    // per warp in {2, 4, 8} x {1, 2, 4}, and (FP64, df) the persistent form
    // with 8-warp tiles of 1, 2 or 4 beams per warp.
    if (rc == XF_OK) {
        const int cw[3] = {2, 4, 8}, cb[3] = {1, 2, 4};
        double best = 1e300;
        int best_w = 8, best_b = 1, best_p = 0;
        b->ncand = 0;
        const int nforms = b->prec == XF_PREC_MIXED ? 1 : 2;
        for (int f = 0; f < nforms && rc == XF_OK; ++f)
            for (int i = 0; i < 3 && rc == XF_OK; ++i)
                for (int j = 0; j < 3 && rc == XF_OK; ++j) {
                    if (f == 1 && cw[i] != 8) continue;
                    b->persistent = f;
                    b->pblocks = 0;
                    rc = build_lists(b, cw[i], cb[j]);
                    double ms = 0.;
                    if (rc == XF_OK) rc = run(b, 2, false, nullptr);  // the first launch instantiates the graph
                    if (rc == XF_OK) rc = run(b, 8, false, &ms);
                    const int c = b->ncand++;
                    b->cand_warps[c] = cw[i];
                    b->cand_bpw[c] = cb[j];
                    b->cand_pers[c] = f;
                    b->cand_ms[c] = ms;
                    if (rc == XF_OK && ms < best) {
                        best = ms;
                        best_w = cw[i];
                        best_b = cb[j];
                        best_p = f;
                    }
                }
        b->persistent = best_p;
        b->pblocks = 0;
        if (rc == XF_OK) rc = build_lists(b, best_w, best_b);
        for (int i = 0; i < n && rc == XF_OK; ++i) {
            std::vector<double> psi;
            xf::initial_state(b->h[i]->nbeams, b->h[i]->ne, cfgs[i].seed, cfgs[i].noise_amp, psi);
            rc = b->h[i]->set_state(psi.data());
        }
    }
    if (rc != XF_OK) {
        xf_batch_destroy(b);
        return rc;
    }
    *out = b;
    return XF_OK;
}

int xf_batch_destroy(xf_batch* b)
{
    if (!b) return XF_EINVAL;
    drop_graphs(b);
    for (auto* h : b->h) xf_destroy(h);
    if (b->d_devs) cudaFree(b->d_devs);
    if (b->d_wtiles) cudaFree(b->d_wtiles);
    if (b->d_ttiles) cudaFree(b->d_ttiles);
    if (b->d_angles) cudaFree(b->d_angles);
    if (b->d_part) cudaFree(b->d_part);
    if (b->d_status) cudaFree(b->d_status);
    if (b->h_status) cudaFreeHost(b->h_status);
    if (b->d_bar) cudaFree(b->d_bar);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return XF_OK;
}

const char* xf_batch_last_error(const xf_batch* b) { return b ? b->err.c_str() : "null batch"; }

int xf_batch_dims(const xf_batch* b, int inst, int* nbeams, int* ebins)
{
    if (!b || inst < 0 || inst >= (int)b->h.size()) return XF_EINVAL;
    if (nbeams) *nbeams = b->h[inst]->nbeams;
    if (ebins) *ebins = b->h[inst]->ne;
    return XF_OK;
}

int xf_batch_set_state(xf_batch* b, int inst, const double* psi)
{
    if (!b || !psi || inst < 0 || inst >= (int)b->h.size()) return XF_EINVAL;
    const int rc = b->h[inst]->set_state(psi);
    if (rc) b->err = b->h[inst]->err;
    return rc;
}

int xf_batch_get_state(xf_batch* b, int inst, double* psi)
{
    if (!b || !psi || inst < 0 || inst >= (int)b->h.size()) return XF_EINVAL;
    const int rc = b->h[inst]->get_state(0, psi);
    if (rc) b->err = b->h[inst]->err;
    return rc;
}

int xf_batch_run(xf_batch* b, long max_iters, long* iters, long* accepted, double* r_end, double* seconds)
{
    if (!b) return XF_EINVAL;
    const double t0 = now_s();
    double ms = 0.;
    const int rc = run(b, max_iters, false, &ms);
    const int n = (int)b->h.size();
    for (int i = 0; i < n; ++i) {
        if (iters) iters[i] = (long)b->h_status[i].iters;
        if (accepted) accepted[i] = (long)b->h_status[i].accepted;
        if (r_end) r_end[i] = b->h_status[i].r;
    }
    if (seconds) *seconds = ms > 0. ? ms * 1e-3 : now_s() - t0;
    return rc;
}

int xf_batch_tile_shape(const xf_batch* b, int* warps, double* tuned_ms)
{
    if (!b) return XF_EINVAL;
    if (warps) *warps = b->warps;
    // the graph-launched one-beam-per-warp candidates {2, 4, 8} warps
    if (tuned_ms)
        for (int i = 0, k = 0; i < b->ncand && k < 3; ++i)
            if (b->cand_bpw[i] == 1 && !b->cand_pers[i]) tuned_ms[k++] = b->cand_ms[i];
    return XF_OK;
}

int xf_batch_set_shape(xf_batch* b, int warps, int beams_per_warp)
{
    if (!b || warps < 1 || warps > 8 || beams_per_warp < 1 || beams_per_warp > 64) return XF_EINVAL;
    if (b->persistent && warps != 8) return b->fail(XF_EINVAL, "the persistent batch runs 8-warp tiles");
    return build_lists(b, warps, beams_per_warp);
}

int xf_batch_set_persistent(xf_batch* b, int on, int beams_per_warp)
{
    if (!b || beams_per_warp < 1 || beams_per_warp > 64) return XF_EINVAL;
    if (on && b->prec == XF_PREC_MIXED) return b->fail(XF_EUNSUPPORTED, "the persistent batch serves FP64 and df");
    b->persistent = on ? 1 : 0;
    b->pblocks = 0;
    return on ? build_lists(b, 8, beams_per_warp) : XF_OK;
}

int xf_batch_tuning(const xf_batch* b, int* warps, int* beams_per_warp, int* persistent, int* ncand, int* cand_warps,
                    int* cand_bpw, int* cand_persistent, double* cand_ms)
{
    if (!b) return XF_EINVAL;
    if (warps) *warps = b->warps;
    if (beams_per_warp) *beams_per_warp = b->bpw;
    if (persistent) *persistent = b->persistent;
    if (ncand) *ncand = b->ncand;
    for (int i = 0; i < b->ncand; ++i) {
        if (cand_warps) cand_warps[i] = b->cand_warps[i];
        if (cand_bpw) cand_bpw[i] = b->cand_bpw[i];
        if (cand_persistent) cand_persistent[i] = b->cand_pers[i];
        if (cand_ms) cand_ms[i] = b->cand_ms[i];
    }
    return XF_OK;
}

}  // extern "C"
