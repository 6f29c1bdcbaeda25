// Programmatic dependent launch, shared by the CG and flexible-CG iterations.
//
// The kernels of one solver iteration are launched with programmatic stream
// serialisation: a kernel's CTAs may become resident while the previous
// kernel's last wave still runs.  Before pdl_wait() a kernel reads only data
// that the previous kernel does not write (written two or more launches
// earlier, or static); pdl_wait() returns once the previous kernel has
// completed and its writes are visible.  Every kernel triggers its dependents
// right after its own wait, so the kernel two launches back has always
// completed when a kernel starts, and no dependent can hold SM resources that
// a not yet launched CTA of its predecessor needs.  Launched without the
// attribute, both calls are no-ops.
#pragma once

#include <cuda_runtime.h>

namespace ipfem {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static inline void launch_pdl(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t stream,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace ipfem
