// The handle behind the C ABI.  Internal to the library.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "xf_device.cuh"
#include "xf_kernels.h"
#include "xf_physics.h"
#include "xflat_gpu.h"

namespace xf {
struct Mixed;  // mixed-precision state (xf_mixed.cu)
}
struct xf_io;  // Snapshot / Probability files (xf_io.cpp)

struct xf_handle {
    xf_config cfg{};
    xf::Tables tab;
    int device = 0;
    int A = 0, P = 1, ne = 0, epad = 0, nbeams = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[7] = {};
    std::vector<cudaEvent_t> tev;  // timing events captured into graphs

    // device memory
    double* d_fv = nullptr;
    double* d_hvac = nullptr;
    double* d_cos2R = nullptr;
    double* d_dcos2R = nullptr;
    double* d_sinR = nullptr;
    double* d_cosphi = nullptr;
    double* d_sinphi = nullptr;
    double* d_geo = nullptr;
    float* d_geof = nullptr;     // geometry table as double-float (mixed path)
    float* d_phif = nullptr;     // [4][P]: cos(phi) hi, lo, sin(phi) hi, lo
    double* d_partials = nullptr;
    unsigned int* d_gticket = nullptr;  // [4][kMaxRedGroups]
    double* d_hvv = nullptr;
    double* d_Sscratch = nullptr;
    double* d_psi[4] = {};  // storage for psi0, psi1, psi3, psi4 (roles of 0 and 3 swap)
    double* d_S[2] = {};    // per-beam energy sums of psi0 / candidate
    double* d_log = nullptr;
    long log_cap_dev = 0;
    xf::Ctl* d_ctl = nullptr;
    xf::Ctl* h_ctl = nullptr;  // pinned mirror
    double* h_in = nullptr;    // pinned r, dr, hm[3]

    xf::Dev dev{};
    xf::Shape shape;
    xf::Mixed* mixed = nullptr;
    xf_io* io = nullptr;

    // host bookkeeping
    bool j0_valid = false;
    double j0_r = 0.;
    double last_r = 0., last_dr = 0.;
    int debug_psi3 = 0;
    int renorm_every = 16;        // mixed precision: accepted steps between renormalisations
    int accepts_since_renorm = 0;
    int time_phases = 0;
    int persistent = -1;          // device control as one cooperative launch per k iterations (FP64, df);
                                  // -1: chosen by size and precision (persistent_default)
    double barrier_timeout_ms = 2000.;  // limit of each grid-barrier wait of the persistent loop
    int barrier_extra = 0;        // test hook: arrivals each barrier waits for beyond the grid (never come)
    double phase_ms[3] = {0., 0., 0.};
    long phase_n[3] = {0, 0, 0};
    long launches = 0;
    long long h2d_bytes = 0, d2h_bytes = 0;  // host<->device bytes copied by the current xf_run
    std::string err;

    struct GraphEntry {
        int k;
        bool timed;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs;
    cudaGraphExec_t step_exec = nullptr;

    int fail(int code, const std::string& msg);
    int init(const xf_config& c);
    void release();
    int pull_ctl();
    void launch_ph(int phase, const xf::Dev& d);
    int set_state(const double* psi);
    int get_state(int which, double* psi);
    int push_inputs(double r, double dr);
    int refresh_j0(double r);
    int step(double r, double dr, double* max_err);
    int accept();
    int run_host(const xf_run_opts& o, xf_step_cb cb, void* user, xf_run_stats& s);
    int run_device(const xf_run_opts& o, xf_run_stats& s);
    int start_device_run(double r, double dr, long Ts, bool files = false);
    int get_graph(int k, bool timed, cudaGraphExec_t* out);
    int launch_persistent(int k);
    int dump_files(long itr, double r, double dr);
    int flush_files();  // waits until every queued output record is written
    // Device-controlled runs with files (xf_io.cpp): slots and files before the
    // run, the per-run output fields of the control block, slot reservation
    // before each graph launch, the records of each launch, and the end of the run.
    int io_dev_prepare(int k);
    void io_dev_fill(xf::Ctl* hc);
    int io_dev_reserve(int k);
    int io_dev_drain(long long count, long long staged, bool final);
    int io_dev_end();
};
