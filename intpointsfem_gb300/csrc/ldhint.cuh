// Loads with an L2 eviction-priority hint for the SpMV vector gathers.
//
// A block SpMV streams the tangent once (hundreds of MB, loaded evict-first)
// and gathers every vector entry once per block that couples to it, about 16
// times per SpMV.  The gathered vectors are a few MB; loading them with an
// evict_last policy (createpolicy + ld.global.nc.L2::cache_hint, PTX ISA 7.4,
// sm_80 and later) keeps their lines in L2 while the tangent streams past.
// The hint changes no value that is loaded.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ipfem {

__device__ __forceinline__ uint64_t l2_policy_keep()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ float2 ld_keep(const float2 *p, uint64_t pol)
{
    float2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                 : "=f"(v.x), "=f"(v.y)
                 : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ double2 ld_keep(const double2 *p, uint64_t pol)
{
    double2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                 : "=d"(v.x), "=d"(v.y)
                 : "l"(p), "l"(pol));
    return v;
}

}  // namespace ipfem
