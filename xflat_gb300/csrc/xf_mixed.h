// Mixed-precision path (xf_mixed.cu): FP32 beam state (value + compensation)
// and SU(2) rotations with FP64 moment reduction, error reduction, step
// control and renormalisation.
#pragma once
#include <cuda_runtime.h>

#include "xf_device.cuh"
#include "xf_kernels.h"
#include "xflat_gpu.h"

struct xf_handle;

namespace xf {
struct Mixed;
Mixed* mixed_create(xf_handle* h);
void mixed_destroy(Mixed* m);
int mixed_set_state(xf_handle* h, Mixed* m, const double* psi);
int mixed_get_state(xf_handle* h, Mixed* m, int which, double* psi);
void mixed_launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st);
// Phase kernels of the double-float path (xf_df.cu), on the same state buffers.
void df_launch_phase(int phase, const Dev& d, const Shape& sh, cudaStream_t st);
// Grid sizes of the double-float phase kernels (one wave of resident blocks
// each) for the shape's block size and phase-B variant.
void df_default_shape(int nbeams, Shape& sh);
// Persistent device-controlled loop (xf_persist.cu, FP64 and double-float):
// the grid size (0 if the kernel cannot be resident) and one cooperative
// launch of up to `iters` iterations.
int persist_blocks(const Dev& d);
cudaError_t launch_persist(const Dev& d, int blocks, int iters, unsigned extra, unsigned long long limit_ns,
                           cudaStream_t st);
void mixed_launch_accept(const Dev& d, cudaStream_t st);
// Renormalises psi0 and recomputes its exact FP64 energy sums; with
// `conditional` only when the step controller flagged it.
void mixed_launch_renorm(const Dev& d, int conditional, cudaStream_t st);
}  // namespace xf
