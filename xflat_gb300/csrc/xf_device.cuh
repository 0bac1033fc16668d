// Device-side types shared by the kernels and the host engine.
//
// Data layout in HBM (one handle = one simulation):
//   state buffers  psi0, psi1, psi3, psi4: [beam][comp][epad] (comp = ar, ai,
//                  br, bi; epad = ebins rounded up to a multiple of 32; padding
//                  bins hold zeros and have zero weight).  This is the
//                  reference's NetCDF psi layout with the energy axis padded,
//                  so a warp reads 32 consecutive energies of one component.
//   per-beam sums  S0, S4: [beam][4] energy moments sum_e fv*rho(psi) of psi0
//                  and of the candidate (the reference's NBeam::hSumMat).
//   tables         fv[4][epad], hvac[2][epad], angle grids [abins], azimuth
//                  grids [pbins], geometry at the three stage points
//                  geo[4][3][abins] (cos, sin, dcos, dl).
//   control block  Ctl: radius, step, matter terms, the angular moments J of
//                  every stage, the step error and the loop counters.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace xf {

constexpr int kNJ = 16;        // moment slots: MA uses J0[4], J1[4]; MAA J0, Jx, Jy, Jz [4] each
constexpr int kPartStride = 32;  // doubles per block in the partial-sum buffer
// Block partials are reduced in two levels: the last block of each group of
// kRedGroup consecutive partials sums the group, and the last group sums the
// group sums (stored after the block partials).
constexpr int kRedGroup = 32;
constexpr int kMaxRedGroups = 1024;  // groups per reduction (group tickets per phase)
// Rows of the partial-sum buffer for `count` block partials and their group sums.
__host__ __device__ constexpr int red_rows(int count) { return count + (count + kRedGroup - 1) / kRedGroup; }

enum Phase { PH_A = 0, PH_B = 1, PH_C = 2, PH_MOM = 3 };

// One output record decided on the device by the step controller (the dump
// triggers of src/IO_f.cpp:387-424 evaluated at an accepted step); the host
// writes it once the following phase A has staged the state into its slots.
struct IoRec {
    double r, dr;
    long long itr;
    int kind;             // bit 1: Snapshot record, bit 2: Probability record
    int snap_slot, prob_slot;
    int rotate;           // the Snapshot record starts a new pair of files (src/IO_f.cpp:275-279)
    int sync_snap, sync_prob;
};

struct Ctl {
    double r, dr;         // current iteration
    double hm[3];         // matter term at r, r+dr/2, r+dr
    double J0[kNJ];       // moments of psi0 at stage point 0
    double JA1[kNJ];      // psi1 = U(h0, dl1) psi0 at point 2   (S2 -> S3)
    double JA3[kNJ];      // psi3 = U(h0, dl0) psi0 at point 1   (S6 -> S7)
    double JB4[kNJ];      // psi4 = U(h3, dl1) psi0 at point 2   (S8 -> S9)
    double JC[kNJ];       // candidate at point 2 (J0 of the next iteration if accepted)
    double JM[kNJ];       // scratch result of the standalone moment kernel
    double max_err;       // Max_err = sqrt(max_b err_b)   (src/Nmr.cpp:195-206)
    double* psi0;         // roles swapped on accept (src/Nmr.cpp:231-233)
    double* psi4;
    double* S0;
    double* S4;
    float2* S0f;          // mixed precision: the sums S0 / S4 also as double-float (hi, lo) pairs
    float2* S4f;
    float* m0hi;          // mixed precision: psi0 and candidate as FP32 value + FP32 compensation
    float* m0lo;
    float* m4hi;
    float* m4lo;
    unsigned int ticket[4];  // last-block tickets per phase
    unsigned int bar;     // persistent loop: grid-barrier arrivals of the current launch
    int bar_timeout;      // persistent loop: a barrier wait ran out
    int done;             // device control: no further iterations
    int nan_seen;
    long long iters;      // counter_tot
    long long accepted;   // counter
    long long max_iters;  // Ts
    long long log_len;    // accepted-step records written to the log
    int renorm_due;       // mixed precision: the last accepted step calls for a renormalisation
    // device-side output (device control with files): trigger state of
    // src/IO_f.cpp:387-424, record counters and the staging request
    double io_last_r1, io_last_r2;
    unsigned long long io_t1, io_t2;  // globaltimer (ns) of the last Snapshot / Probability record
    long long io_age1, io_age2;       // seconds since those records when the run started
    long long io_file_itr;            // records in the current Snapshot file
    long long io_count;               // records decided
    long long io_staged;              // records whose slots are filled
    long long io_snaps, io_probs;     // slots handed out per kind (ring positions)
    unsigned long long io_gt;         // globaltimer at the last evaluation
    int io_tinit;                     // io_t1/io_t2 set from the ages
    int stage_kind;                   // phase A stages psi0 (bit 1) / the survival (bit 2)
    int stage_snap_slot, stage_prob_slot;
    // device-side output configuration for the current run (io_mode 0: none);
    // a per-run setting, kept here rather than in the kernel parameters so the
    // cached CUDA graphs serve runs with and without files
    int io_mode;                      // dumpMode bits
    int io_nslots;
    double io_R0, io_rstep1, io_rstep2;
    long long io_tstep1, io_tstep2;   // seconds
    long long io_itrstep1, io_itrstep2, io_new_file_step, io_sync_step;
    double* io_snap;                  // [nslots][nbeams][4][ne] big-endian doubles (the file's encoding)
    double* io_prob;                  // [nslots][nbeams] survival
    IoRec* io_log;                    // [io_log_cap] ring of records
    long long io_log_cap;
};

// Kernel parameters (passed by value).
struct Dev {
    int geom;             // kernel family: 0 MA-shaped moments (MA and SA), 1 MAA
    int sa;               // SA geometry table (single angle, dilution factor D(r))
    int nbeams, A, P, ne, epad;
    const double* fv;     // [4][epad]
    const double* hvac;   // [2][epad]: h00 part, then h01 real part
    const float* fvf;     // FP32 copies for the mixed-precision kernels
    const float* fvf_lo;  // fv - fvf rounded to FP32: (fvf, fvf_lo) is fv as a double-float
    const float* hvf;
    const double* cos2R;  // [A]
    const double* dcos2R; // [A]
    const double* sinR;   // [A]
    const double* cosphi; // [P]
    const double* sinphi; // [P]
    double* geo;          // [4][3][A]
    float* geof;          // [2][4][3][A]: the geometry table as double-float, hi block then lo block
    const float* cosphif; // [2][P] azimuth tables as double-float (hi, then lo)
    const float* sinphif;
    float LEkf[8];        // kappa L/<E> per particle as double-float: hi[4], lo[4] (kappa ~ 1e-45 and
                          // J ~ 1e50 are outside FP32's range; kappa J, the Hamiltonian scale, is not)
    double* psi1;
    double* psi3;
    double* partials;     // [red_rows(grid)][kPartStride]
    unsigned int* gticket;  // [4 phases][kMaxRedGroups] group tickets of the two-level reduction
    double* log;          // accepted-step log [cap][3] (device control), may be null
    long long log_cap;
    Ctl* ctl;
    double LE[4];
    double kappa;
    double Rv;
    // step control (src/Nmr.cpp:227-249)
    double eps0, ksi, maxdr, Rn;
    // matter profile (src/Matt.cpp:22-64)
    int has_matter;
    double mat_coeff, nbfar, nb0, hNS;
    int device_control;   // phase C runs the accept/reject/dr controller
    int renorm_every;     // mixed precision: renormalise psi0 every this many accepted steps
    int debug_psi3;       // phase C also stores U(h4, dl2) psi3 into psi3 (the reference's S10 result)
    int prefetch;         // mixed precision: L1 prefetch distance of the state rows, in energy-loop iterations
    int df;               // double-float path (phase kernels of xf_df.cu on the compensated-pair state)
    const float* hvf_lo;  // hvac - hvf rounded to FP32: (hvf, hvf_lo) is hvac as a double-float
};

// Geometry table accessors: q = 0 cos, 1 sin, 2 dcos, 3 dl.
__host__ __device__ inline int geo_idx(int q, int pt, int ang, int A) { return (q * 3 + pt) * A + ang; }

}  // namespace xf
