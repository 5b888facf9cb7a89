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

  // Launches of this host thread may use the attribute (cleared around the
  // operator applications of several columns: there the near field and the
  // tree passes run on two streams with multi-wave kernels, and a dependent
  // grid waiting on SMs for its predecessor holds slots the other stream's
  // kernels need -- measured 8 % slower at 16 columns, 0.3 % faster at one).
  inline thread_local bool t_pdl_allowed = true;
  struct PdlScope
  {
    bool prev;
    explicit PdlScope(bool on) : prev(t_pdl_allowed) { t_pdl_allowed = on && prev; }
    ~PdlScope() { t_pdl_allowed = prev; }
    PdlScope(const PdlScope &)            = delete;
    PdlScope &operator=(const PdlScope &) = delete;
  };

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
    cfg.numAttrs                                     = (pdl_on() && t_pdl_allowed) ? 1 : 0;
    PIBEM_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...));
  }
} // namespace pibem
