// Programmatic dependent launch (sm_90 and later) for the chains of small
// kernels of an operator application and of an Arnoldi step: a kernel
// launched with launch_pdl may be scheduled while the previous kernel of its
// stream is finishing; its first statement, pdl_entry(), waits until every
// preceding grid has completed and its memory is visible (griddepcontrol.wait)
// and then lets the next kernel be scheduled (griddepcontrol.launch_dependents).
// A kernel that calls pdl_entry() but is launched without the attribute runs
// as before (both instructions have no effect then).  PIBEM_PDL=0 in the
// environment launches everything without the attribute.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <utility>

#include "pibem_internal.h"

namespace pibem
{
  __device__ __forceinline__ void pdl_entry()
  {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  }

  inline bool pdl_on()
  {
    static const bool on = [] {
      const char *e = std::getenv("PIBEM_PDL");
      return !e || std::atoi(e) != 0;
    }();
    return on;
  }

  template <typename... P, typename... A>
  inline void launch_pdl(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                         A &&...args)
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = grid;
    cfg.blockDim           = block;
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = s;
    cudaLaunchAttribute at[1];
    at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs                                        = at;
    cfg.numAttrs                                     = pdl_on() ? 1 : 0;
    PIBEM_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...));
  }
} // namespace pibem
