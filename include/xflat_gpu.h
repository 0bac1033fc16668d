/*
 * xflat_gpu.h -- C ABI of the GB300 implementation of XFLAT's per-radius-step
 * hot path (bulb-model MA/MAA neutrino-neutrino Hamiltonian moment integral and
 * the SU(2) evolution of every beam, driven by the reference's adaptive
 * three-point stepper).
 *
 * The reference selects its physics and numerics modules at compile time
 * (include/global.h:5-28) and binds them as free functions:
 *   include/Phy.h:24-159   phy::init, calcAngleBins, calcDeltaLs, calc_Hvv,
 *                          evolveHvv, evolveAvg, initBeam, freemem ...
 *   include/Nmr.h:20-31    nmr::init, evolutionLoop, freemem
 *   include/Fio.h:22-38    fio::init, fillInitData, dumpToFile, freemem
 *   include/Matt.h:22-36   matt::init, getHm
 *   include/Parser.h:9-28  Parser(configFile)
 * This header replaces that contract with handle-based entry points.  The
 * buffers crossing the ABI are host memory in the reference's NetCDF psi
 * layout [theta][phi][prtcl][comp][ebin] (src/IO_f.cpp:280-288), copied
 * synchronously, with one exception: xf_calc_hvv_static takes caller-owned
 * device pointers and a CUDA stream.  No C++ types cross the ABI.  Every entry
 * point returns an xf_status; none exits or traps.  Calls on one handle must
 * come from one thread at a time; handles are independent.
 */
#ifndef XFLAT_GPU_H_
#define XFLAT_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference has none: its hot functions are throw() and IO
 * failures call exit(-10) (src/IO_f.cpp:88). */
enum {
    XF_OK = 0,
    XF_EINVAL = 1,       /* bad argument or configuration */
    XF_ECUDA = 2,        /* CUDA runtime error, or no usable GPU */
    XF_ETIMEOUT = 3,     /* a bounded device-side wait ran out */
    XF_ENAN = 4,         /* the step error became NaN (the reference would spin until Ts) */
    XF_EIO = 5,          /* file could not be read or written */
    XF_ENOMEM = 6,       /* device or host allocation failed */
    XF_EUNSUPPORTED = 7  /* option not supported for this geometry/precision */
};

/* MA and MAA: bulb model with polar (and azimuthal) angle bins; SA: the
 * single-angle bulb model (src/Phy_SA.cpp), one beam per particle, Abins and
 * Pbins ignored. */
enum { XF_GEOM_MA = 0, XF_GEOM_MAA = 1, XF_GEOM_SA = 2 };
enum { XF_PREC_FP64 = 0, XF_PREC_MIXED = 1, XF_PREC_DF = 2 };

/* Run configuration.  Fields carry the reference's Util:: values in the same
 * internal units after the same parse-time conversions (src/Parser.cpp:40-123:
 * energies in km^-1, dm2 in km^-2, luminosities in km^-2, nb0 x 1e15).
 * Keys missing from a config file keep the xf_config_default() value (the
 * reference leaves them uninitialized). */
typedef struct xf_config {
    int geometry;        /* XF_GEOM_*  (extension key "geometry= MA|MAA|SA") */
    int precision;       /* XF_PREC_*  (extension key "precision= fp64|mixed|df") */
    int abins, pbins, ebins, flvs;
    int has_matter;      /* hasMatter= */
    int dump_mode;       /* dumpMode= (bit 1 snapshot file, bit 2 probability file) */
    int Ts;              /* max iterations */
    int Tn;              /* max wall seconds */
    int new_file_step, sync_step;
    int tstep1, itrstep1, tstep2, itrstep2;
    int start_beam, end_beam;
    double rstep1, rstep2;
    double eps0, ksi, mu;
    double R0, Rn, dr, max_dr;
    double E0, E1;
    double Ye, Rv, Mns, gs, S, hNS, nb0;
    double theta, theta2, dm2;
    double Lv[4], Tv[4], eta[4];
    uint64_t seed;       /* extension key "seed=" */
    double noise_amp;    /* extension key "noise_amp=" (0 = pure flavor states) */
    char file_prefix[256];
} xf_config;

typedef struct xf_handle xf_handle;

/* Options and results of xf_run (the replacement of nmr::evolutionLoop,
 * src/Nmr.cpp:89-262). */
typedef struct xf_run_opts {
    long max_iters;        /* < 0: use cfg.Ts */
    int device_control;    /* 1: accept/reject and dr control run on the GPU, no per-step host sync */
    int iters_per_launch;  /* device_control: iterations captured per CUDA graph launch (default 16) */
    int write_files;       /* 1: honour dump_mode through the NetCDF writer; under device_control the
                              dump triggers run on the GPU and the state is staged there (same files) */
    int time_phases;       /* 1: time every phase kernel with CUDA events (see xf_phase_times) */
    double r0, dr0;        /* starting radius and step; NaN -> cfg.R0 / cfg.dr */
    double* log;           /* optional host buffer for accepted steps (itr, r_after, dr_used) */
    long log_cap;          /* capacity of log in records */
} xf_run_opts;

typedef struct xf_run_stats {
    long iterations;       /* counter_tot (src/Nmr.cpp:246) */
    long accepted;         /* counter (src/Nmr.cpp:244) */
    double r_end, dr_end;
    double seconds;        /* wall time of the loop */
    double last_max_err;
    double device_ms;      /* CUDA-event time of the loop on the handle's stream */
    long kernel_launches;  /* device kernels launched by this call */
    long log_len;          /* accepted-step records written to opts->log */
    long h2d_bytes;        /* host-to-device bytes this call copied (inputs, control block) */
    long d2h_bytes;        /* device-to-host bytes this call copied (control, Max_err, log, output records) */
} xf_run_stats;

/* Defaults: max_iters -1, device_control 0, iters_per_launch 16, r0/dr0 NaN. */
int xf_run_opts_default(xf_run_opts* o);

/* Called on every accepted step of a host-driven xf_run, in the place of
 * fio::dumpToFile (src/Nmr.cpp:238): (user, itr, r_after, dr_used).  Return
 * nonzero to stop the loop. */
typedef int (*xf_step_cb)(void* user, long itr, double r, double dr);

/* ---------------------------------------------------------------- config */
/* Parser(configFile) (src/Parser.cpp:13-127). */
int xf_config_default(xf_config* cfg);
int xf_config_load(const char* path, xf_config* cfg);
int xf_config_parse(const char* text, xf_config* cfg);
const char* xf_strerror(int status);

/* Host-only (no GPU needed): the tables of xf_tables, the matter term of
 * xf_matter and the initial state of xf_create computed from a configuration
 * (src/NBeam.cpp:138-209, src/Matt.cpp:58-64, src/NBeam.cpp:246-276). */
int xf_host_tables(const xf_config* cfg, double* fv, double* hvac, double* LE, double* Ev);
int xf_host_matter(const xf_config* cfg, double r, double* hm);
int xf_host_initial_state(const xf_config* cfg, uint64_t seed, double amp, double* psi);

/* ---------------------------------------------------------------- lifecycle */
/* nbm::init + phy::init + nmr::init + matt::init (src/NBGroup.cpp:129-139;
 * src/NBeam.cpp:138-209; src/Phy_MA.cpp:233-284; src/Phy_MAA.cpp:247-304;
 * src/Nmr.cpp:48-70; src/Matt.cpp:22-29).  Beams start in pure flavor states
 * (src/NBeam.cpp:246-276), plus seeded noise when cfg->noise_amp > 0. */
int xf_create(const xf_config* cfg, xf_handle** out);
/* phy::freemem / nmr::freemem / nbm::freemem (src/Phy_MA.cpp:290-302). */
int xf_destroy(xf_handle* h);
/* Message of the last failing call on this handle. */
const char* xf_last_error(const xf_handle* h);
/* nbeams = theta*phi*4 (phy::beamLen, src/Phy_MA.cpp:78). */
int xf_dims(const xf_handle* h, int* nbeams, int* ebins, int* abins, int* pbins);
/* Tuning and diagnostics, no reference counterpart: "threads" / "blocks" set
 * the launch shape of the phase kernels (0 = default; the double-float
 * default is one wave of resident blocks per phase); "renorm_every" sets the
 * accepted steps between the mixed path's unitarity renormalisations
 * (default 16, 0 = never; the double-float path takes 0 only); "prefetch"
 * sets how many energy-loop iterations ahead the mixed and double-float phase
 * kernels prefetch the state rows into L1 (default 1, 0 = none);
 * "df_b_occupancy" (2 or 3, default 3) picks the double-float phase-B kernel
 * built for that many resident blocks per SM; "persistent" (1, 0, or -1 for
 * the default choice by size and precision) runs a device-controlled xf_run
 * of FP64 or double-float as one cooperative launch per iters_per_launch
 * iterations, the stages separated by grid barriers whose waits are bounded
 * by "barrier_timeout_ms" (default 2000; XF_ETIMEOUT when one runs out;
 * "debug_barrier_extra" > 0 makes every wait run out, for tests), not when
 * time_phases is set; "fp64_fused" (default 1) folds the FP64 averages of
 * phases B and C into their FMA chains, 0 keeps them as separate additions
 * (other rounding; graph-launched only); "debug_psi3" = 1 makes the last
 * phase also store U(h4, dl2) psi3 into psi3, as the reference's in-place
 * stage S10 does (src/Nmr.cpp:191). */
int xf_set_option(xf_handle* h, const char* name, double value);

/* ---------------------------------------------------------------- state */
/* fio::fillInitData / phy::initBeam (src/IO_f.cpp:197-250): psi0 <- psi and
 * the cached energy moments S(psi0) are recomputed (src/Nmr.cpp:117-121). */
int xf_set_state(xf_handle* h, const double* psi);
/* Reads buffer `which` (0 = psi0, 1 = psi1, 3 = psi3, 4 = psi4) into psi. */
int xf_get_state(xf_handle* h, int which, double* psi);
/* Seeded initial noise (a,b) = (sqrt(1-e^2-n^2), e+i n) on psi0, the form of
 * src/NBeam.cpp:260-275 with a counter-based generator. */
int xf_set_noise(xf_handle* h, uint64_t seed, double amp);

/* ---------------------------------------------------------------- tables */
/* Energy tables fv[4][ebins], hvac[2*ebins], L/<E> per particle and <E>
 * (src/NBeam.cpp:138-209, src/Fenergy.cpp:16-47, src/Phy_MA.cpp:280-282). */
int xf_tables(const xf_handle* h, double* fv, double* hvac, double* LE, double* Ev);
/* matt::getHm (src/Matt.cpp:58-64). */
int xf_matter(const xf_handle* h, double r, double* hm);
/* phy::calcAngleBins(r,0..2) + calcDeltaLs (src/Nmr.cpp:167-173) on the GPU;
 * outputs [3][abins] each (sinb unused for MA). */
int xf_angle_bins(xf_handle* h, double r, double dr, double* cosb, double* sinb, double* dcosb, double* dl);
/* phy::calc_Hvv on buffer `which` at stage point pt after xf_angle_bins(r, dr)
 * (src/Phy_MA.cpp:455-474, src/Phy_MAA.cpp:571-621); hvv[abins*pbins][4]. */
int xf_calc_hvv(xf_handle* h, int which, int pt, double r, double dr, double* hvv);

/* ---------------------------------------------------------------- stepping */
/* One stepper iteration at (r, dr): stages S1..S11 and the error sweep of
 * src/Nmr.cpp:153-206.  The candidate stays on the device; *max_err receives
 * Max_err.  Returns XF_ENAN if Max_err is NaN. */
int xf_step(xf_handle* h, double r, double dr, double* max_err);
/* Accept the candidate: psi0 <-> psi4 (src/Nmr.cpp:227-233). */
int xf_accept(xf_handle* h);
/* Full loop with the reference's termination, accept/reject and dr control
 * (src/Nmr.cpp:89-262).  cb may be NULL.  opts may be NULL (defaults). */
int xf_run(xf_handle* h, const xf_run_opts* opts, xf_step_cb cb, void* user, xf_run_stats* stats);
/* Forced steps: applies n accepted steps (r_before[i], dr[i]) in order, as
 * the reference's loop did; used to replay a recorded step sequence. */
int xf_replay(xf_handle* h, const double* r_before, const double* dr, long n);
/* Average CUDA-event time per launch (ms) of the three phase kernels over the
 * last xf_run with time_phases = 1: out[0..2]; counts[0..2] launches timed. */
int xf_phase_times(const xf_handle* h, double* out, long* counts);

/* ---------------------------------------------------------------- output */
/* Per-beam survival probabilities written to the reference's Probability file:
 * sum_e fv*(ar^2+ai^2), with the fv of beam i*4 + p%2 (src/IO_f.cpp:341-351);
 * out[theta*phi][4]. */
int xf_survival(xf_handle* h, double* out);

/* No counterpart in the reference.  phy::calc_Hvv for callers that cannot
 * allocate device memory (their device memory is owned and budgeted up front
 * by another allocator, or their per-step loop must not pay cudaMalloc's
 * implicit device synchronisation).  Every pointer except LE (host, 4
 * doubles) is device memory the caller owns: psi [abins*pbins*4][4][epad]
 * (epad >= ebins), fv [4][epad], cosb/sinb/dcosb [abins] at the stage point
 * (sinb, cosphi, sinphi [pbins] only for MAA), hvv [abins*pbins][4] out;
 * kappa is the Hamiltonian coefficient.  Allocates nothing: its scratch is a
 * fixed 2.06 MiB device array inside the library, which limits it to
 * abins*pbins*4 <= 65536 beams (larger sizes return XF_EINVAL).  The first call
 * on a device looks that array up (make it before any stream capture); calls
 * that overlap on the GPU race on the shared array.  Work is queued on
 * `stream` (a cudaStream_t of the current device, NULL for the default
 * stream; a stream of another device returns XF_EINVAL).  A CUDA error
 * already pending on entry returns XF_ECUDA and stays pending. */
int xf_calc_hvv_static(int geometry, int abins, int pbins, int ebins, int epad, const double* psi,
                       const double* fv, const double* cosb, const double* sinb, const double* dcosb,
                       const double* cosphi, const double* sinphi, const double* LE, double kappa,
                       double* hvv, void* stream);

/* ---------------------------------------------------------------- measurement */
/* No reference counterpart.  Measures this GPU's FP64 FMA throughput with a
 * register-resident DFMA loop (8 independent chains per thread, grid of 8
 * blocks per SM) for about `ms` milliseconds: *tflops = 2 flops per FMA. */
int xf_probe_fp64_peak(double ms, double* tflops);

/* No reference counterpart.  The double-float propagator coefficients of
 * NBeam::U (src/NBeam.cpp:360-393) for n bin Hamiltonians: h[3i..3i+2] =
 * (h00, h01r, h01i) and path length dl[i] (host arrays), each split into FP32
 * pairs, evaluated on the device by the double-float kernels' own code, with
 * q = 1/2 when `half` is set, else 1.  Returns cm[i] = q (cos(|h| dl) - 1)
 * and S[i] = q sin(|h| dl) / |h| (host arrays).  The series branch is chosen
 * per warp of 32 consecutive inputs, as in the kernels.  1 <= n <= 2^26. */
int xf_probe_df_propagator(int n, const double* h, const double* dl, int half, double* cm, double* S);

/* ---------------------------------------------------------------- files */
/* The reference's NetCDF IO module (src/IO_f.cpp), written without libnetcdf
 * in the classic format (64-bit offsets): file names <prefix>Snapshot<n>_0_.nc
 * (dims r[unlimited], theta (not for SA), [phi], prtcl, comp, ebin; variables
 * r, dr, psi) and <prefix>Probability<n>_0_.nc (dims r, theta, phi; variables
 * r, prtcl0..prtcl3).
 * xf_dump: fio::dumpToFile (src/IO_f.cpp:387-424) with the same radius, time
 *   and iteration triggers, file rotation every new_file_step records and
 *   sync every sync_step; files are created on the first call.  The record is
 *   the state at the call, stream-ordered; it is staged on the device, copied
 *   to pinned host memory on a copy stream and appended by a writer thread,
 *   so the call returns without waiting for the copy or the write.  A failed
 *   append is reported by the next xf_dump, xf_io_close or the end of xf_run;
 *   xf_run (write_files) returns with every record written and flushed.
 * xf_resume: fio::fillInitData (src/IO_f.cpp:197-250): psi0 and the last r
 *   and dr from the last record of a Snapshot file.
 * xf_io_close: fio::freemem (src/IO_f.cpp:252-263); waits for pending records.
 * xf_io_verbose: print the radius on dumps, as the reference does (default off). */
int xf_dump(xf_handle* h, long itr, double r, double dr);
int xf_resume(xf_handle* h, const char* path, double* r, double* dr);
int xf_io_close(xf_handle* h);
int xf_io_verbose(xf_handle* h, int on);
/* Host-only (no GPU): write a Snapshot file with nrec records from host arrays
 * (psi: nrec x [beam][comp][ebin]) for configuration cfg, and read record rec
 * (< 0: the last) of one; *nrec receives the record count.  Any output may be
 * NULL. */
int xf_snapshot_write(const char* path, const xf_config* cfg, long nrec, const double* r, const double* dr,
                      const double* psi);
int xf_snapshot_read(const char* path, long rec, double* r, double* dr, double* psi, long* nrec);

/* ---------------------------------------------------------------- batch */
/* Many independent simulations with per-instance adaptive steps, advanced
 * together by the same phase kernels (one launch per phase covers every
 * instance), captured in CUDA graphs.  Configs may be MA or SA (they share
 * the MA-shaped kernels) and must share precision (fp64, mixed or df). */
typedef struct xf_batch xf_batch;
int xf_batch_create(const xf_config* cfgs, int n, xf_batch** out);
int xf_batch_destroy(xf_batch* b);
const char* xf_batch_last_error(const xf_batch* b);
int xf_batch_dims(const xf_batch* b, int inst, int* nbeams, int* ebins);
int xf_batch_set_state(xf_batch* b, int inst, const double* psi);
int xf_batch_get_state(xf_batch* b, int inst, double* psi);
/* Advance every unfinished instance by up to max_iters iterations (< 0: each
 * instance's Ts); per-instance results in iters/accepted/r_end (may be NULL). */
int xf_batch_run(xf_batch* b, long max_iters, long* iters, long* accepted, double* r_end, double* seconds);
/* Warps per block chosen by the autotuner at creation, and the measured time
 * (ms, 8 iterations) of the candidates {2, 4, 8} warps with one beam per warp
 * (may be NULL). */
int xf_batch_tile_shape(const xf_batch* b, int* warps, double* tuned_ms);
/* The autotuner's full table: the chosen warps per block (block size 32 x
 * warps), beams per warp (blocks per phase = beams / (warps x beams per
 * warp)) and launch form (persistent 1: one cooperative launch per 8
 * iterations, 0: graphs of per-stage launches), and for each of the *ncand
 * (<= 16) candidates its shape, form and measured time (ms, 8 iterations of
 * the whole batch).  Any output may be NULL. */
int xf_batch_tuning(const xf_batch* b, int* warps, int* beams_per_warp, int* persistent, int* ncand, int* cand_warps,
                    int* cand_bpw, int* cand_persistent, double* cand_ms);
/* Replaces the tuned tile shape: warps per block in [1, 8], beams per warp in
 * [1, 64]. */
int xf_batch_set_shape(xf_batch* b, int warps, int beams_per_warp);
/* on = 1: run the batch's iterations as one cooperative launch per 8
 * iterations (FP64 and df), the stages separated by grid barriers whose waits
 * are bounded (XF_ETIMEOUT when one runs out), over 8-warp tiles of
 * beams_per_warp beams per warp; on = 0: CUDA graphs of the per-stage
 * launches.  Overrides the autotuner's choice. */
int xf_batch_set_persistent(xf_batch* b, int on, int beams_per_warp);

#ifdef __cplusplus
}
#endif
#endif /* XFLAT_GPU_H_ */
