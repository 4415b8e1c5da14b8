// pdl.cuh -- programmatic dependent launch (sm_90 and later) for the kernels of a step.
//
// A kernel launched by launch_pdl may be scheduled while the previous kernel of its stream
// is still draining: its blocks take the SM slots the previous grid's last blocks free, run
// what does not depend on earlier kernels (twiddle tables into shared memory, index set-up),
// then pdl_wait() until every earlier grid of the stream has completed and its writes are
// visible.  Everything a kernel reads from earlier kernels, and every global write, comes
// after its pdl_wait().  pdl_launch() lets the next kernel be scheduled once every block of
// this grid has started; called at the top of a kernel it only moves the next launch ahead,
// it does not publish any data (the next kernel's pdl_wait still waits for completion).
// Launched plainly (or after a copy or a host node), pdl_wait returns at once.
#pragma once
#include <cuda_runtime.h>

namespace cmm {

#ifdef __CUDACC__
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

}  // namespace cmm
