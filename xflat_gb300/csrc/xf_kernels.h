// Launch wrappers for the FP64 kernels (xf_kernels.cu).  Every wrapper only
// enqueues work on `st`; errors surface through cudaGetLastError().
#pragma once
#include <cuda_runtime.h>

#include "xf_device.cuh"

namespace xf {

struct Shape {
    int threads = 256;   // threads per block (multiple of 32)
    int blocks = 0;      // grid size of the phase kernels
    int blocks_ab = 0;   // mixed precision: grid size of phases A and B (0: blocks)
    int phase_blocks[3] = {0, 0, 0};  // double-float: grid size of phases A, B, C (0: blocks)
    int df_b_occ = 3;    // double-float: resident blocks per SM of the phase-B kernel (2 or 3)
    int fp64_fused = 1;  // FP64: averages folded into the FMA chains of phases B and C (0: separate additions)
};

// Grid-size limit used to size the partial-sum buffer.
int max_phase_blocks(int nbeams, int threads);
Shape default_shape(int nbeams, int epad, bool mixed = false);

void launch_geometry(const Dev& d, cudaStream_t st);
void launch_esum(const Dev& d, const double* psi, double* S, cudaStream_t st);
void launch_moments(const Dev& d, const double* S, int pt, double* Jout, cudaStream_t st, int conditional = 0);
void launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st);
void launch_accept(const Dev& d, cudaStream_t st);
void launch_hvv_eval(const Dev& d, const double* J, int pt, double* hvv, cudaStream_t st);
// FP64 copy of the accepted state psi0 (the mixed path's compensated pair
// summed) in the padded [beam][comp][epad] layout, for output; with
// big_endian set each double is stored byte-reversed (the NetCDF file
// encoding on a little-endian host).
void launch_stage_state(const Dev& d, int mixed, int big_endian, double* dst, cudaStream_t st);
// Per-beam survival sum_e fv (ar^2 + ai^2) of psi0 (the Probability file's
// quantity, src/IO_f.cpp:341-351), out[nbeams].
void launch_survival(const Dev& d, int mixed, double* out, cudaStream_t st);
// Stages the output record the step controller decided last, if its phase A
// did not run (the run ended with that step).
void launch_stage_pending(const Dev& d, int mixed, cudaStream_t st);

}  // namespace xf
