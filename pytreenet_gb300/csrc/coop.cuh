// Grid-wide barrier for cooperatively launched kernels (all CTAs resident).
// ctrl[0] counts arrivals, ctrl[1] is the generation, ctrl[2] the abort flag;
// the caller zeroes the words before the launch. Every wait is bounded: after
// `max_cycles` SM clocks the waiting CTA raises the abort flag, and every CTA
// that sees the flag leaves. Returns false when the kernel must leave.
// Data written before the barrier by other CTAs must be read with
// L2-coherent loads (__ldcg) after it.
#pragma once
#include <stdint.h>

__device__ __forceinline__ bool ptn_grid_barrier(unsigned* ctrl, long long max_cycles) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = ctrl + 1;
    volatile unsigned* vabort = ctrl + 2;
    const unsigned g = *vgen;
    __threadfence();
    int ok = 1;
    const unsigned arrived = atomicAdd(ctrl, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(ctrl, 0u);
      __threadfence();
      atomicAdd(ctrl + 1, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g) {
        if (*vabort != 0u) {
          ok = 0;
          break;
        }
        if (clock64() - t0 > max_cycles) {
          atomicExch(ctrl + 2, 1u);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}
