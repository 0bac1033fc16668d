// Snapshot / Probability files and resume: the reference's NetCDF IO module
// (src/IO_f.cpp) on top of the project's classic-format writer and reader.
// Files, dimension and variable names, attribute names and values, dump
// triggers, file rotation and sync follow src/IO_f.cpp:90-424 so existing
// post-processing reads them unchanged.
//
// Output is asynchronous.  A dump decides its triggers on the calling thread
// (as the reference does), then enqueues on the compute stream a kernel that
// stages psi0 (or the per-beam survival) into a device buffer, and on a copy
// stream the device-to-host copy of that buffer into one of two pinned host
// buffers.  A writer thread waits for each copy and appends the record.  The
// stepper therefore continues while a record is copied and written; it only
// waits when both host buffers of a kind are still being written (disk slower
// than the dumps) or when a device staging buffer is reused before its copy
// has finished.  File creation and rotation drain the writer first and stay
// synchronous, so their errors are reported by the dump that triggers them;
// an append error is reported by the next dump, xf_io_close or the end of
// xf_run.
//
// Under device control the step controller itself evaluates the triggers at
// every accepted step and logs a record; the next phase A stages psi0 and the
// survival into a ring of device slots while it reads psi0 anyway.  Between
// graph launches the host hands the staged records to the same copy stream
// and writer thread, and before each launch it makes sure that the slots the
// launch may fill have been copied out.  Records, their order, rotation and
// sync are those of the host-driven loop.
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "xf_engine.h"
#include "xf_kernels.h"
#include "xf_netcdf.h"
#include "xf_physics.h"
#include "xflat_gpu.h"

namespace {

enum { JOB_SNAP = 0, JOB_PROB = 1 };

// Pinned host buffers per record kind: two for the (large) Snapshot records,
// many for the (small) Probability records, so that a burst of the latter does
// not wait for the writer.
constexpr int kStateBufs = 2, kSurvBufs = 32;

struct Job {
    int kind;
    int buf;
    double r, dr;
    bool sync;
};

}  // namespace

struct xf_io {
    xf::nc::Writer snap, prob;
    int ctr = 0;               // files created so far (rotation counter)
    uint64_t itr = 0;          // records in the current snapshot file
    double last_r0 = 0., last_r1 = 0., last_r2 = 0.;
    long t1 = 0, t2 = 0;       // wall seconds of the last time-triggered dumps
    bool inited = false;
    int verbose = 0;

    // asynchronous pipeline (allocated at the first dump)
    bool pipe = false;
    int nbeams = 0;
    cudaStream_t cs = nullptr;                // copy stream
    double* d_state = nullptr;                // staged psi0, padded layout, big-endian
    double* d_surv = nullptr;                 // staged survival, [nbeams]
    double* h_state[kStateBufs] = {};         // pinned, unpadded [beam][comp][ebin], big-endian
    double* h_surv[kSurvBufs] = {};
    cudaEvent_t staged = nullptr;             // compute stream: staging kernel done
    cudaEvent_t state_copied[kStateBufs] = {}, surv_copied[kSurvBufs] = {};
    cudaEvent_t state_d2h = nullptr, surv_d2h = nullptr;  // last copy out of each staging buffer
    bool state_d2h_pending = false, surv_d2h_pending = false;
    int next_state = 0, next_surv = 0;

    std::thread writer;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job> q;
    bool busy_state[kStateBufs] = {}, busy_surv[kSurvBufs] = {};
    bool working = false, stop = false;
    int werr = 0;
    std::string werr_msg;

    // device-controlled runs: slots the next phase A stages records into
    int nslots = 0;
    double* d_snapslots = nullptr;   // [nslots][nbeams][4][ne], big-endian
    double* d_probslots = nullptr;   // [nslots][nbeams]
    xf::IoRec* d_log = nullptr;      // [nslots] ring of records
    std::vector<cudaEvent_t> snap_evt, prob_evt;  // last copy out of each slot
    std::vector<char> snap_pend, prob_pend;
    long long dev_done = 0;          // records of the current run handed to the writer
};

namespace {

long wall_s()
{
    return (long)std::chrono::duration_cast<std::chrono::seconds>(std::chrono::system_clock::now().time_since_epoch()).count();
}

std::string file_name(const xf_config& c, const char* kind, int ctr)
{
    // <prefix><kind><ctr>_<rank>_.nc with rank 0 (src/IO_f.cpp:119, 162)
    return std::string(c.file_prefix) + kind + std::to_string(ctr) + "_0_.nc";
}

// Dimensions, variables and attributes of the Snapshot file (src/IO_f.cpp:116-144);
// the dimensions are the module's getDimInfo/countDim: MA r, theta, prtcl,
// comp, ebin (src/Phy_MA.cpp), MAA adds phi (src/Phy_MAA.cpp), SA has no
// angle (src/Phy_SA.cpp:67-96).
void snapshot_schema(const xf_config& c, std::vector<xf::nc::Dim>& dims, std::vector<xf::nc::Var>& vars)
{
    using xf::nc::Attr;
    using xf::nc::Dim;
    using xf::nc::Var;
    int A, P;
    xf::beam_dims(c, A, P);
    dims.clear();
    dims.push_back(Dim{"r", 0});
    if (c.geometry != XF_GEOM_SA) dims.push_back(Dim{"theta", (uint64_t)A});
    if (c.geometry == XF_GEOM_MAA) dims.push_back(Dim{"phi", (uint64_t)P});
    dims.push_back(Dim{"prtcl", 4});
    dims.push_back(Dim{"comp", 4});
    dims.push_back(Dim{"ebin", (uint64_t)c.ebins});
    Var r{"r", {0}, {}}, dr{"dr", {0}, {}}, psi{"psi", {}, {}};
    for (int i = 0; i < (int)dims.size(); ++i) psi.dims.push_back(i);
    psi.atts.push_back(Attr{"E0", {c.E0}});
    psi.atts.push_back(Attr{"E1", {c.E1}});
    // src/IO_f.cpp:136-143 names the attributes string("..."+i): the literal
    // advanced by i characters, with the values Tv(i), Tv(i+1), eta(i),
    // eta(i+1).  Kept as written so readers of existing files match.
    const char* tp = "Teprature for particle";
    const char* ta = "Teprature for anti-particle";
    const char* ep = "eta for particle";
    const char* ea = "eta for anti-particle";
    for (int i = 0; i < c.flvs; ++i) {
        psi.atts.push_back(Attr{tp + i, {c.Tv[i]}});
        psi.atts.push_back(Attr{ta + i, {c.Tv[i + 1]}});
        psi.atts.push_back(Attr{ep + i, {c.eta[i]}});
        psi.atts.push_back(Attr{ea + i, {c.eta[i + 1]}});
    }
    vars = {r, dr, psi};
}

// ---------------------------------------------------------------- writer thread

// Appends queued records in order.  A record's host buffer is filled by a
// copy on the copy stream; the writer waits for that copy's event first.
void writer_main(xf_io* io, int device)
{
    cudaSetDevice(device);  // the handle's device, current in this thread too
    std::vector<double> cols;
    for (;;) {
        Job j;
        {
            std::unique_lock<std::mutex> lk(io->mu);
            io->cv.wait(lk, [io] { return io->stop || !io->q.empty(); });
            if (io->q.empty()) return;  // stop requested and nothing left
            j = io->q.front();
            io->q.pop_front();
            io->working = true;
        }
        bool ok = true;
        std::string msg;
        if (j.kind == JOB_SNAP) {
            if (cudaEventSynchronize(io->state_copied[j.buf]) != cudaSuccess) {
                ok = false;
                msg = "snapshot copy failed";
            } else if (!io->snap.append({&j.r, &j.dr, io->h_state[j.buf]}, {false, false, true})) {
                ok = false;
                msg = "snapshot write failed";
            } else if (j.sync) {
                io->snap.sync();
            }
        } else {
            if (cudaEventSynchronize(io->surv_copied[j.buf]) != cudaSuccess) {
                ok = false;
                msg = "probability copy failed";
            } else {
                // per-particle columns prtcl0..3 over (theta, phi) (src/IO_f.cpp:341-384)
                const int n = io->nbeams / 4;
                cols.resize((size_t)4 * n);
                const double* sv = io->h_surv[j.buf];
                for (int i = 0; i < n; ++i)
                    for (int p = 0; p < 4; ++p) cols[(size_t)p * n + i] = sv[(size_t)i * 4 + p];
                if (!io->prob.append({&j.r, &cols[0], &cols[(size_t)n], &cols[2 * (size_t)n], &cols[3 * (size_t)n]})) {
                    ok = false;
                    msg = "probability write failed";
                } else if (j.sync) {
                    io->prob.sync();
                }
            }
        }
        {
            std::lock_guard<std::mutex> lk(io->mu);
            if (j.kind == JOB_SNAP) io->busy_state[j.buf] = false;
            else io->busy_surv[j.buf] = false;
            if (!ok && !io->werr) {
                io->werr = XF_EIO;
                io->werr_msg = msg;
            }
            io->working = false;
        }
        io->cv.notify_all();
    }
}

// Waits until every queued record is written; returns the first writer error.
int drain(xf_handle* h)
{
    xf_io& io = *h->io;
    if (!io.pipe) return XF_OK;
    std::unique_lock<std::mutex> lk(io.mu);
    io.cv.wait(lk, [&io] { return io.q.empty() && !io.working; });
    if (io.werr) return h->fail(io.werr, io.werr_msg);
    return XF_OK;
}

int pipe_open(xf_handle* h)
{
    xf_io& io = *h->io;
    if (io.pipe) return XF_OK;
    io.nbeams = h->nbeams;
    const size_t padded = (size_t)h->nbeams * 4 * h->epad, plain = (size_t)h->nbeams * 4 * h->ne;
    auto ck = [h](cudaError_t e, const char* what) {
        return e == cudaSuccess ? XF_OK : h->fail(XF_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    int rc;
    if ((rc = ck(cudaStreamCreateWithFlags(&io.cs, cudaStreamNonBlocking), "copy stream"))) return rc;
    if ((rc = ck(cudaMalloc((void**)&io.d_state, padded * sizeof(double)), "cudaMalloc"))) return rc;
    if ((rc = ck(cudaMalloc((void**)&io.d_surv, (size_t)h->nbeams * sizeof(double)), "cudaMalloc"))) return rc;
    for (int i = 0; i < kStateBufs; ++i) {
        if ((rc = ck(cudaMallocHost((void**)&io.h_state[i], plain * sizeof(double)), "cudaMallocHost"))) return rc;
        if ((rc = ck(cudaEventCreateWithFlags(&io.state_copied[i], cudaEventDisableTiming), "event"))) return rc;
    }
    for (int i = 0; i < kSurvBufs; ++i) {
        if ((rc = ck(cudaMallocHost((void**)&io.h_surv[i], (size_t)h->nbeams * sizeof(double)), "cudaMallocHost")))
            return rc;
        if ((rc = ck(cudaEventCreateWithFlags(&io.surv_copied[i], cudaEventDisableTiming), "event"))) return rc;
    }
    if ((rc = ck(cudaEventCreateWithFlags(&io.staged, cudaEventDisableTiming), "event"))) return rc;
    if ((rc = ck(cudaEventCreateWithFlags(&io.state_d2h, cudaEventDisableTiming), "event"))) return rc;
    if ((rc = ck(cudaEventCreateWithFlags(&io.surv_d2h, cudaEventDisableTiming), "event"))) return rc;
    io.stop = false;
    io.writer = std::thread(writer_main, &io, h->device);
    io.pipe = true;
    return XF_OK;
}

void slots_free(xf_io& io)
{
    if (io.d_snapslots) cudaFree(io.d_snapslots);
    if (io.d_probslots) cudaFree(io.d_probslots);
    if (io.d_log) cudaFree(io.d_log);
    for (auto e : io.snap_evt)
        if (e) cudaEventDestroy(e);
    for (auto e : io.prob_evt)
        if (e) cudaEventDestroy(e);
    io.d_snapslots = io.d_probslots = nullptr;
    io.d_log = nullptr;
    io.snap_evt.clear();
    io.prob_evt.clear();
    io.snap_pend.clear();
    io.prob_pend.clear();
    io.nslots = 0;
}

void pipe_close(xf_io& io)
{
    if (io.writer.joinable()) {
        {
            std::lock_guard<std::mutex> lk(io.mu);
            io.stop = true;
        }
        io.cv.notify_all();
        io.writer.join();
    }
    if (io.cs) cudaStreamSynchronize(io.cs);
    slots_free(io);
    for (int i = 0; i < kStateBufs; ++i) {
        if (io.h_state[i]) cudaFreeHost(io.h_state[i]);
        if (io.state_copied[i]) cudaEventDestroy(io.state_copied[i]);
        io.h_state[i] = nullptr;
        io.state_copied[i] = nullptr;
    }
    for (int i = 0; i < kSurvBufs; ++i) {
        if (io.h_surv[i]) cudaFreeHost(io.h_surv[i]);
        if (io.surv_copied[i]) cudaEventDestroy(io.surv_copied[i]);
        io.h_surv[i] = nullptr;
        io.surv_copied[i] = nullptr;
    }
    if (io.d_state) cudaFree(io.d_state);
    if (io.d_surv) cudaFree(io.d_surv);
    if (io.staged) cudaEventDestroy(io.staged);
    if (io.state_d2h) cudaEventDestroy(io.state_d2h);
    if (io.surv_d2h) cudaEventDestroy(io.surv_d2h);
    if (io.cs) cudaStreamDestroy(io.cs);
    io.d_state = io.d_surv = nullptr;
    io.staged = io.state_d2h = io.surv_d2h = nullptr;
    io.cs = nullptr;
    io.pipe = false;
}

// Claims host buffer `b` of a kind, waiting while the writer still uses it.
int claim(xf_handle* h, bool* busy, int b)
{
    xf_io& io = *h->io;
    std::unique_lock<std::mutex> lk(io.mu);
    io.cv.wait(lk, [&] { return !busy[b] || io.werr; });
    if (io.werr) return h->fail(io.werr, io.werr_msg);
    busy[b] = true;
    return XF_OK;
}

// Returns a claimed buffer when its copy could not be enqueued.
void unclaim(xf_io& io, bool* busy, int b)
{
    std::lock_guard<std::mutex> lk(io.mu);
    busy[b] = false;
}

void enqueue(xf_io& io, const Job& j)
{
    {
        std::lock_guard<std::mutex> lk(io.mu);
        io.q.push_back(j);
    }
    io.cv.notify_all();
}

// io_f::init (src/IO_f.cpp:90-194).  Drains the writer before touching files.
int io_init(xf_handle* h, int ctr)
{
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    int rc;
    if ((rc = drain(h))) return rc;
    io.snap.close();
    io.prob.close();
    io.ctr = ctr;
    io.itr = 0;
    io.last_r0 = c.R0;
    using xf::nc::Dim;
    using xf::nc::Var;
    if (c.dump_mode & 1) {
        std::vector<Dim> dims;
        std::vector<Var> vars;
        snapshot_schema(c, dims, vars);
        if (!io.snap.create(file_name(c, "Snapshot", ctr), dims, vars))
            return h->fail(XF_EIO, "cannot create " + file_name(c, "Snapshot", ctr));
        io.last_r1 = c.R0;
        io.t1 = wall_s();
    }
    if (c.dump_mode & 2) {
        std::vector<Dim> dims = {Dim{"r", 0}, Dim{"theta", (uint64_t)h->A}, Dim{"phi", (uint64_t)h->P}};
        std::vector<Var> vars = {Var{"r", {0}, {}}};
        for (int p = 0; p < 4; ++p) vars.push_back(Var{"prtcl" + std::to_string(p), {0, 1, 2}, {}});
        if (!io.prob.create(file_name(c, "Probability", ctr), dims, vars))
            return h->fail(XF_EIO, "cannot create " + file_name(c, "Probability", ctr));
        io.last_r2 = c.R0;
        io.t2 = wall_s();
    }
    io.inited = true;
    return XF_OK;
}

// Stream-ordered staging of one record: `stage` fills the device buffer on the
// compute stream after the step that produced the state; the copy stream then
// moves it to the claimed host buffer.  The compute stream first waits for the
// previous copy out of the same device buffer.
template <typename Stage, typename Copy>
int stage_and_copy(xf_handle* h, cudaEvent_t d2h, bool& d2h_pending, cudaEvent_t copied, Stage stage, Copy copy)
{
    xf_io& io = *h->io;
    cudaError_t e = cudaSuccess;
    if (d2h_pending) e = cudaStreamWaitEvent(h->st, d2h, 0);
    if (e == cudaSuccess) {
        stage();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(io.staged, h->st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(io.cs, io.staged, 0);
    if (e == cudaSuccess) e = copy();
    if (e == cudaSuccess) e = cudaEventRecord(copied, io.cs);
    if (e == cudaSuccess) e = cudaEventRecord(d2h, io.cs);
    if (e != cudaSuccess) return h->fail(XF_ECUDA, std::string("output staging: ") + cudaGetErrorString(e));
    d2h_pending = true;
    h->launches++;
    return XF_OK;
}

// io_f::writeToFile for the snapshot (src/IO_f.cpp:266-328), asynchronous.
int write_snapshot(xf_handle* h, double r, double dr)
{
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    int rc;
    if ((int64_t)io.itr >= c.new_file_step && (rc = io_init(h, io.ctr + 1))) return rc;
    if ((rc = pipe_open(h))) return rc;
    const int b = io.next_state;
    if ((rc = claim(h, io.busy_state, b))) return rc;
    rc = stage_and_copy(
        h, io.state_d2h, io.state_d2h_pending, io.state_copied[b],
        [&] { xf::launch_stage_state(h->dev, h->mixed != nullptr, 1, io.d_state, h->st); },
        [&] {
            return cudaMemcpy2DAsync(io.h_state[b], h->ne * sizeof(double), io.d_state, h->epad * sizeof(double),
                                     h->ne * sizeof(double), (size_t)h->nbeams * 4, cudaMemcpyDeviceToHost, io.cs);
        });
    if (rc) {
        unclaim(io, io.busy_state, b);
        return rc;
    }
    h->d2h_bytes += (long long)h->nbeams * 4 * h->ne * sizeof(double);
    io.itr++;
    enqueue(io, Job{JOB_SNAP, b, r, dr, c.sync_step > 0 && io.itr % c.sync_step == 0});
    io.next_state = (io.next_state + 1) % kStateBufs;
    return XF_OK;
}

// io_f::writeToFile for the probability file (src/IO_f.cpp:331-384), asynchronous.
int write_probability(xf_handle* h, double r)
{
    xf_io& io = *h->io;
    int rc;
    if ((rc = pipe_open(h))) return rc;
    const int b = io.next_surv;
    if ((rc = claim(h, io.busy_surv, b))) return rc;
    rc = stage_and_copy(
        h, io.surv_d2h, io.surv_d2h_pending, io.surv_copied[b],
        [&] { xf::launch_survival(h->dev, h->mixed != nullptr, io.d_surv, h->st); },
        [&] {
            return cudaMemcpyAsync(io.h_surv[b], io.d_surv, (size_t)h->nbeams * sizeof(double), cudaMemcpyDeviceToHost,
                                   io.cs);
        });
    if (rc) {
        unclaim(io, io.busy_surv, b);
        return rc;
    }
    h->d2h_bytes += (long long)h->nbeams * sizeof(double);
    const int64_t ss = h->cfg.sync_step;
    enqueue(io, Job{JOB_PROB, b, r, 0., ss > 0 && io.itr % ss == 0});
    io.next_surv = (io.next_surv + 1) % kSurvBufs;
    return XF_OK;
}

}  // namespace

int xf_handle::dump_files(long it, double r, double dr) { return xf_dump(this, it, r, dr); }

// ---------------------------------------------------------------- device-controlled runs

int xf_handle::io_dev_prepare(int k)
{
    if (!io) io = new xf_io();
    int rc;
    if (!io->inited && (rc = io_init(this, 0))) return rc;
    if ((rc = pipe_open(this))) return rc;
    // records of two launches (one being written while the next runs), the
    // record still waiting for its phase A, one spare
    const int ns = 2 * k + 2;
    if (io->nslots != ns) {
        if ((rc = drain(this))) return rc;
        cudaStreamSynchronize(io->cs);
        slots_free(*io);
        const size_t snap = (size_t)nbeams * 4 * ne;
        cudaError_t e = cudaSuccess;
        if (cfg.dump_mode & 1) e = cudaMalloc((void**)&io->d_snapslots, ns * snap * sizeof(double));
        if (e == cudaSuccess && (cfg.dump_mode & 2))
            e = cudaMalloc((void**)&io->d_probslots, ns * (size_t)nbeams * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc((void**)&io->d_log, ns * sizeof(xf::IoRec));
        io->snap_evt.assign(ns, nullptr);
        io->prob_evt.assign(ns, nullptr);
        for (int i = 0; i < ns && e == cudaSuccess; ++i) {
            e = cudaEventCreateWithFlags(&io->snap_evt[i], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&io->prob_evt[i], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            slots_free(*io);
            return fail(XF_ENOMEM, std::string("output slots: ") + cudaGetErrorString(e));
        }
        io->snap_pend.assign(ns, 0);
        io->prob_pend.assign(ns, 0);
        io->nslots = ns;
    }
    io->dev_done = 0;
    return XF_OK;
}

void xf_handle::io_dev_fill(xf::Ctl* hc)
{
    const xf_config& c = cfg;
    const long now = wall_s();
    hc->io_mode = c.dump_mode;
    hc->io_nslots = io->nslots;
    hc->io_R0 = c.R0;
    hc->io_rstep1 = c.rstep1;
    hc->io_rstep2 = c.rstep2;
    hc->io_tstep1 = c.tstep1;
    hc->io_tstep2 = c.tstep2;
    hc->io_itrstep1 = c.itrstep1;
    hc->io_itrstep2 = c.itrstep2;
    hc->io_new_file_step = c.new_file_step;
    hc->io_sync_step = c.sync_step;
    hc->io_snap = io->d_snapslots;
    hc->io_prob = io->d_probslots;
    hc->io_log = io->d_log;
    hc->io_log_cap = io->nslots;
    hc->io_last_r1 = io->last_r1;
    hc->io_last_r2 = io->last_r2;
    hc->io_age1 = std::max(0L, now - io->t1);
    hc->io_age2 = std::max(0L, now - io->t2);
    hc->io_tinit = 0;
    hc->io_file_itr = (long long)io->itr;
    hc->io_count = hc->io_staged = hc->io_snaps = hc->io_probs = 0;
    hc->stage_kind = 0;
}

int xf_handle::io_dev_reserve(int k)
{
    for (int i = 0; i < k; ++i) {
        const int s = (int)((h_ctl->io_snaps + i) % io->nslots), p = (int)((h_ctl->io_probs + i) % io->nslots);
        if (io->snap_pend[s]) {
            if (cudaEventSynchronize(io->snap_evt[s]) != cudaSuccess) return fail(XF_ECUDA, "output slot copy failed");
            io->snap_pend[s] = 0;
        }
        if (io->prob_pend[p]) {
            if (cudaEventSynchronize(io->prob_evt[p]) != cudaSuccess) return fail(XF_ECUDA, "output slot copy failed");
            io->prob_pend[p] = 0;
        }
    }
    return XF_OK;
}

int xf_handle::io_dev_drain(long long count, long long staged_in, bool final)
{
    int rc;
    if (final && staged_in < count) {
        // the run ended with the step that decided this record
        xf::launch_stage_pending(dev, mixed != nullptr, st);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
            return fail(XF_ECUDA, "staging the last output record failed");
        launches++;
    }
    const long long staged = final ? count : staged_in;
    if (staged <= io->dev_done) return XF_OK;
    std::vector<xf::IoRec> ring(io->nslots);
    if (cudaMemcpy(ring.data(), io->d_log, ring.size() * sizeof(xf::IoRec), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(XF_ECUDA, "reading the output records failed");
    d2h_bytes += (long long)ring.size() * sizeof(xf::IoRec);
    const size_t snap = (size_t)nbeams * 4 * ne;
    for (long long n = io->dev_done; n < staged; ++n) {
        const xf::IoRec& rec = ring[n % io->nslots];
        if (rec.rotate && (rc = io_init(this, io->ctr + 1))) return rc;
        if (rec.kind & 1) {
            if (io->verbose) std::printf("%f\n", rec.r);
            const int b = io->next_state;
            if ((rc = claim(this, io->busy_state, b))) return rc;
            cudaError_t e = cudaMemcpyAsync(io->h_state[b], io->d_snapslots + rec.snap_slot * snap, snap * sizeof(double),
                                            cudaMemcpyDeviceToHost, io->cs);
            if (e == cudaSuccess) e = cudaEventRecord(io->state_copied[b], io->cs);
            if (e == cudaSuccess) e = cudaEventRecord(io->snap_evt[rec.snap_slot], io->cs);
            if (e != cudaSuccess) {
                unclaim(*io, io->busy_state, b);
                return fail(XF_ECUDA, std::string("output copy: ") + cudaGetErrorString(e));
            }
            io->snap_pend[rec.snap_slot] = 1;
            d2h_bytes += (long long)snap * sizeof(double);
            io->itr++;
            enqueue(*io, Job{JOB_SNAP, b, rec.r, rec.dr, rec.sync_snap != 0});
            io->next_state = (io->next_state + 1) % kStateBufs;
        }
        if (rec.kind & 2) {
            if (io->verbose) std::printf("%f\n", rec.r);
            const int b = io->next_surv;
            if ((rc = claim(this, io->busy_surv, b))) return rc;
            cudaError_t e = cudaMemcpyAsync(io->h_surv[b], io->d_probslots + (size_t)rec.prob_slot * nbeams,
                                            (size_t)nbeams * sizeof(double), cudaMemcpyDeviceToHost, io->cs);
            if (e == cudaSuccess) e = cudaEventRecord(io->surv_copied[b], io->cs);
            if (e == cudaSuccess) e = cudaEventRecord(io->prob_evt[rec.prob_slot], io->cs);
            if (e != cudaSuccess) {
                unclaim(*io, io->busy_surv, b);
                return fail(XF_ECUDA, std::string("output copy: ") + cudaGetErrorString(e));
            }
            io->prob_pend[rec.prob_slot] = 1;
            d2h_bytes += (long long)nbeams * sizeof(double);
            enqueue(*io, Job{JOB_PROB, b, rec.r, 0., rec.sync_prob != 0});
            io->next_surv = (io->next_surv + 1) % kSurvBufs;
        }
    }
    io->dev_done = staged;
    return XF_OK;
}

int xf_handle::io_dev_end()
{
    int rc;
    if ((rc = pull_ctl())) return rc;
    // the trigger state continues on the host (a later host-driven run or xf_dump)
    io->last_r1 = h_ctl->io_last_r1;
    io->last_r2 = h_ctl->io_last_r2;
    if (h_ctl->io_tinit) {
        const long now = wall_s();
        io->t1 = now - (long)((h_ctl->io_gt - h_ctl->io_t1) / 1000000000ull);
        io->t2 = now - (long)((h_ctl->io_gt - h_ctl->io_t2) / 1000000000ull);
    }
    h_ctl->io_mode = 0;
    h_ctl->stage_kind = 0;
    if (cudaMemcpyAsync(d_ctl, h_ctl, sizeof(xf::Ctl), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(XF_ECUDA, "control block upload failed");
    h2d_bytes += sizeof(xf::Ctl);
    return flush_files();
}

// Drains the writer and flushes both files (records and the header's record
// count), so another reader sees every record written so far.
int xf_handle::flush_files()
{
    if (!io) return XF_OK;
    const int rc = drain(this);
    io->snap.sync();
    io->prob.sync();
    return rc;
}

extern "C" {

// io_f::dumpToFile (src/IO_f.cpp:387-424)
int xf_dump(xf_handle* h, long it, double r, double dr)
{
    if (!h) return XF_EINVAL;
    if (!h->io) h->io = new xf_io();
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    int rc;
    if (!io.inited && (rc = io_init(h, 0))) return rc;
    {
        std::lock_guard<std::mutex> lk(io.mu);
        if (io.werr) return h->fail(io.werr, io.werr_msg);
    }
    const long now = wall_s();
    if (!c.dump_mode) {
        if (r - io.last_r0 > 1.0) {
            io.last_r0 = r;
            if (io.verbose) std::printf("%f\n", r);
        }
    }
    if (c.dump_mode & 1) {
        if (r == c.Rn || r - io.last_r1 > c.rstep1 || (now - io.t1) > c.tstep1 || (c.itrstep1 > 0 && !(it % c.itrstep1))) {
            if (io.verbose) std::printf("%f\n", r);
            io.last_r1 = r;
            io.t1 = now;
            if ((rc = write_snapshot(h, r, dr))) return rc;
        }
    }
    if (c.dump_mode & 2) {
        if (r == c.Rn || r - io.last_r2 > c.rstep2 || (now - io.t2) > c.tstep2 || (c.itrstep2 > 0 && !(it % c.itrstep2))) {
            if (io.verbose) std::printf("%f\n", r);
            io.last_r2 = r;
            io.t2 = now;
            if ((rc = write_probability(h, r))) return rc;
        }
    }
    return XF_OK;
}

int xf_snapshot_write(const char* path, const xf_config* c, long nrec, const double* r, const double* dr,
                      const double* psi)
{
    int A = 0, P = 0;
    if (c) xf::beam_dims(*c, A, P);
    if (!path || !c || nrec < 0 || (nrec > 0 && (!r || !dr || !psi)) || A <= 0 || P <= 0 || c->ebins <= 0)
        return XF_EINVAL;
    std::vector<xf::nc::Dim> dims;
    std::vector<xf::nc::Var> vars;
    snapshot_schema(*c, dims, vars);
    xf::nc::Writer w;
    if (!w.create(path, dims, vars)) return XF_EIO;
    const size_t n = (size_t)A * P * 4 * 4 * c->ebins;
    for (long i = 0; i < nrec; ++i)
        if (!w.append({&r[i], &dr[i], psi + (size_t)i * n})) return XF_EIO;
    w.close();
    return XF_OK;
}

int xf_snapshot_read(const char* path, long rec, double* r, double* dr, double* psi, long* nrec)
{
    if (!path) return XF_EINVAL;
    xf::nc::Reader rd;
    if (!rd.open(path)) return XF_EIO;
    const int vpsi = rd.find_var("psi"), vr = rd.find_var("r"), vdr = rd.find_var("dr");
    if (vpsi < 0 || vr < 0 || vdr < 0) return XF_EIO;
    if (nrec) *nrec = (long)rd.records();
    if (rd.records() == 0) return (r || dr || psi) ? XF_EIO : XF_OK;
    const uint64_t k = rec < 0 ? rd.records() - 1 : (uint64_t)rec;
    if (k >= rd.records()) return XF_EINVAL;
    std::vector<double> v;
    if (r) {
        if (!rd.read(vr, k, v)) return XF_EIO;
        *r = v[0];
    }
    if (dr) {
        if (!rd.read(vdr, k, v)) return XF_EIO;
        *dr = v[0];
    }
    if (psi) {
        if (!rd.read(vpsi, k, v)) return XF_EIO;
        std::memcpy(psi, v.data(), v.size() * sizeof(double));
    }
    return XF_OK;
}

int xf_io_close(xf_handle* h)
{
    if (!h) return XF_EINVAL;
    int rc = XF_OK;
    if (h->io) {
        rc = drain(h);
        pipe_close(*h->io);
        h->io->snap.close();
        h->io->prob.close();
        delete h->io;
        h->io = nullptr;
    }
    return rc;
}

int xf_io_verbose(xf_handle* h, int on)
{
    if (!h) return XF_EINVAL;
    if (!h->io) h->io = new xf_io();
    h->io->verbose = on;
    return XF_OK;
}

// io_f::fillInitData (src/IO_f.cpp:197-250): the last record of psi, r and dr.
int xf_resume(xf_handle* h, const char* path, double* r, double* dr)
{
    if (!h || !path) return XF_EINVAL;
    xf::nc::Reader rd;
    if (!rd.open(path)) return h->fail(XF_EIO, std::string("cannot read NetCDF file ") + path);
    const int vpsi = rd.find_var("psi"), vr = rd.find_var("r"), vdr = rd.find_var("dr");
    if (vpsi < 0 || vr < 0 || vdr < 0 || rd.records() == 0)
        return h->fail(XF_EIO, std::string("no psi/r/dr records in ") + path);
    if (rd.count(vpsi) != (uint64_t)h->nbeams * 4 * h->ne)
        return h->fail(XF_EINVAL, std::string("psi in ") + path + " does not match this configuration's shape");
    const uint64_t last = rd.records() - 1;
    std::vector<double> psi, rv, drv;
    if (!rd.read(vpsi, last, psi) || !rd.read(vr, last, rv) || !rd.read(vdr, last, drv))
        return h->fail(XF_EIO, std::string("short read from ") + path);
    int rc = h->set_state(psi.data());
    if (rc) return rc;
    if (r) *r = rv[0];
    if (dr) *dr = drv[0];
    return XF_OK;
}

}  // extern "C"
