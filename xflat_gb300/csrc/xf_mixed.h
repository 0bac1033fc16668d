// Mixed-precision path (xf_mixed.cu): FP32 beam state and SU(2) rotations with
// FP64 moment reduction, error estimate, step control and renormalisation.
#pragma once
#include "xflat_gpu.h"

struct xf_handle;

namespace xf {
struct Mixed;
Mixed* mixed_create(xf_handle* h);
void mixed_destroy(Mixed* m);
int mixed_set_state(xf_handle* h, Mixed* m, const double* psi);
int mixed_get_state(xf_handle* h, Mixed* m, int which, double* psi);
int mixed_step(xf_handle* h, Mixed* m, double r, double dr, double* max_err);
int mixed_accept(xf_handle* h, Mixed* m, double r_new);
int mixed_run_device(xf_handle* h, Mixed* m, const xf_run_opts& o, xf_run_stats& s);
}  // namespace xf
