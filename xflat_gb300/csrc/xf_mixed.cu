// Mixed-precision path: placeholder until the FP32 kernels land.
#include "xf_engine.h"
#include "xf_mixed.h"

namespace xf {
struct Mixed {
    int unused;
};
Mixed* mixed_create(xf_handle* h)
{
    h->fail(XF_EUNSUPPORTED, "mixed precision is not available in this build");
    return nullptr;
}
void mixed_destroy(Mixed* m) { delete m; }
int mixed_set_state(xf_handle*, Mixed*, const double*) { return XF_EUNSUPPORTED; }
int mixed_get_state(xf_handle*, Mixed*, int, double*) { return XF_EUNSUPPORTED; }
int mixed_step(xf_handle*, Mixed*, double, double, double*) { return XF_EUNSUPPORTED; }
int mixed_accept(xf_handle*, Mixed*, double) { return XF_EUNSUPPORTED; }
int mixed_run_device(xf_handle*, Mixed*, const xf_run_opts&, xf_run_stats&) { return XF_EUNSUPPORTED; }
}  // namespace xf
