// Grid-wide barrier of a cooperative grid (every CTA resident at once), used
// where one solver kernel runs two phases separated by a global reduction.
//
// Arrival: each CTA fences its writes and takes a ticket; the CTA with the
// last ticket runs the caller's epilogue (the final reduction and the scalar
// update) with all its threads, resets the ticket and publishes the next
// value of a generation word with release semantics.  The other CTAs read
// the generation before they arrive and wait, with acquire loads, until it
// changes.  The wait is bounded: after kGridSpinLimit polls it records an
// error in *err and gives up, so that no launch can hang the device; the
// caller then skips its remaining work and the host reports the error.
// Launched with cudaLaunchAttributeCooperative and a grid no larger than the
// resident capacity (grid_capacity()), the wait always ends well before the
// limit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ipfem_internal.h"

namespace ipfem {

constexpr long long kGridSpinLimit = 1LL << 23;   // polls of ~100 ns: about a second

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Every thread of the CTA calls it after the CTA's phase-1 writes; true in
// every thread of the CTA that arrived last.
__device__ __forceinline__ bool grid_arrive(unsigned *count)
{
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    return s_last != 0;
}

// The last CTA, after its epilogue: reset the ticket and release the others.
__device__ __forceinline__ void grid_release(unsigned *count, unsigned *gen, unsigned gen0)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        *count = 0u;
        __threadfence();
        st_release_gpu(gen, gen0 + 1u);
    }
    __syncthreads();
}

// The other CTAs: wait until the generation moves past gen0 (read before
// arriving).  False in every thread if the wait gave up (error recorded).
__device__ __forceinline__ bool grid_wait(const unsigned *gen, unsigned gen0, int *err)
{
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        long long n = 0;
        while (ld_acquire_gpu(gen) == gen0) {
            if (++n > kGridSpinLimit) {
                ok = 0;
                atomicExch(err, kErrGridWait);
                break;
            }
            __nanosleep(64);
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Largest cooperative grid of `kern` with `block` threads and `smem` bytes of
// dynamic shared memory on the current device (0 on error).
template <class K>
static inline int grid_capacity(K kern, int block, size_t smem)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem) != cudaSuccess) return 0;
    return sms * per_sm;
}

// cooperative launch (all CTAs resident together), with programmatic
// dependent launch when pdl is set
template <typename... KArgs, typename... Args>
static inline cudaError_t launch_coop(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t stream,
                                      bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace ipfem
