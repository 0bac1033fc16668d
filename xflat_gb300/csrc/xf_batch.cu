// Batched path: placeholder until the batched kernels land.
#include "xflat_gpu.h"

extern "C" {
int xf_batch_create(const xf_config*, int, xf_batch** out)
{
    if (out) *out = nullptr;
    return XF_EUNSUPPORTED;
}
int xf_batch_destroy(xf_batch*) { return XF_OK; }
const char* xf_batch_last_error(const xf_batch*) { return "batched path not available in this build"; }
int xf_batch_dims(const xf_batch*, int, int*, int*) { return XF_EUNSUPPORTED; }
int xf_batch_set_state(xf_batch*, int, const double*) { return XF_EUNSUPPORTED; }
int xf_batch_get_state(xf_batch*, int, double*) { return XF_EUNSUPPORTED; }
int xf_batch_run(xf_batch*, long, long*, long*, double*, double*) { return XF_EUNSUPPORTED; }
}
