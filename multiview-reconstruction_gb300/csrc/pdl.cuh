// Programmatic dependent launch.  A kernel launched with launch_pdl may be scheduled while
// its predecessor in the stream is still finishing (once every CTA of the predecessor has
// run pdl_trigger); it computes its prologue (twiddle and index tables, constants) and then
// waits in pdl_wait until the predecessor has completed and its writes are visible.  Only
// SMs the predecessor no longer fills take the early CTAs, so the launch gap and the table
// set-up overlap the predecessor's last wave.  MVR_PDL=0 launches without the attribute
// (pdl_wait and pdl_trigger are then no-ops).
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>
#include <utility>

namespace mvr {

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("MVR_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace mvr
