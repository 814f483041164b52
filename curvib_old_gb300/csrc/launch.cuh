// Launch helper of the per-solve kernels: programmatic dependent launch.
//
// A kernel launched through launch_dep() may be launched before the previous
// kernel of its stream has completed: each block of the previous grid lets it
// go when the block exits, so the new grid's blocks are scheduled onto SMs as
// the previous grid's tail drains, instead of after its completion and a full
// launch.  It must call dep_sync() before its first global-memory access;
// dep_sync() waits until the previous kernel has completed and its writes are
// visible, so the memory accesses of consecutive kernels stay ordered exactly
// as with plain launches.  The same holds inside captured CUDA graphs (the
// capture records programmatic edges).  No kernel releases its successor
// early (griddepcontrol.launch_dependents at its start): measured on the
// channel's FP64 zebra half-sweep that took 292 us against 212 us, the waiting
// successor blocks holding the shared memory the line solve needs.  Set
// CVB_NO_PDL=1 in the environment to launch plainly.
#pragma once
#include <cstdlib>
#include <utility>

#include "cvb_internal.h"

namespace cvb {

__device__ __forceinline__ void dep_sync() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_enabled() {
  static const int on = [] {
    const char *e = std::getenv("CVB_NO_PDL");
    return (e && e[0] && e[0] != '0') ? 0 : 1;
  }();
  return on != 0;
}

template <typename... P, typename... A>
inline void launch_dep(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A &&...a) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = s;
  c.attrs = at;
  c.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&c, k, std::forward<A>(a)...);
  count_launch();
}

}  // namespace cvb
