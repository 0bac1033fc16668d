// Programmatic dependent launch (PDL) for the kernels of the stepping loop.
//
// A stepper iteration is a chain of short, grid-wide dependent kernels
// (geometry, the three phases and, in the mixed path, the conditional
// renormalisation).  Launched normally, each kernel starts only after its
// predecessor has drained, and the launch latency is paid in full at every
// boundary.  With the programmatic-serialization launch attribute the next
// kernel is scheduled while its predecessor is still finishing; it then waits
// in `griddepcontrol.wait`, which returns once every prerequisite grid has
// completed and its memory is visible.  Every kernel launched this way calls
// pdl_enter() before it reads or writes any memory, so the results are those
// of fully serialised launches.  Without a programmatic predecessor both
// instructions are no-ops.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace xf {

__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // this grid's own successor may now be scheduled (it waits for this grid in turn)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... P, typename... A>
inline cudaError_t launch_pdl(void (*kernel)(P...), unsigned grid, unsigned block, cudaStream_t st, A&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace xf
