// ose_pdl.cuh - programmatic dependent launch for the plane-path kernels
// (ose_plane.cu), the Bluestein passes (ose_bluestein.cu) and the source
// injection; the generic path's register and Stockham passes measured slower
// with it and launch plainly.
//
// A kernel launched with launch_pdl may start its CTAs while the kernel
// before it in the stream still runs its last wave; griddep_wait() blocks
// until that kernel has completed and its writes are visible.  Every kernel
// launched this way calls griddep_wait() before it reads or writes any
// buffer an earlier kernel of the step touches (only constant tables are
// read before it).  Launched without the attribute, both instructions do
// nothing.  OSE3D_PDL=0 in the environment launches without it.
#pragma once

#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

namespace ose {

__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_enabled()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("OSE3D_PDL");
        v = (e && strcmp(e, "0") == 0) ? 0 : 1;
    }
    return v == 1;
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args)
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
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

}  // namespace ose
