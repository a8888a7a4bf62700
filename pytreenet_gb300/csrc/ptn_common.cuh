// Shared helpers for the ptn_gb300 kernels (complex128 arithmetic, launch checks).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/ptn_gb300.h"

#define PTN_HD __host__ __device__ __forceinline__

PTN_HD double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * b + c
PTN_HD double2 cfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
// conj(a) * b + c
PTN_HD double2 cfmac(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
PTN_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
PTN_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
PTN_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
PTN_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
PTN_HD double cabs2(double2 a) { return fma(a.x, a.x, a.y * a.y); }

// Host-side count of kernel launches issued by this library (ptn_launch_counter);
// atomic because independent realisations may drive the library from several
// host threads.
#include <atomic>
extern std::atomic<unsigned long long> g_ptn_launches;
#define PTN_COUNT(n) (g_ptn_launches.fetch_add((unsigned long long)(n), std::memory_order_relaxed))

static inline int ptn_launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PTN_OK : PTN_ERR_LAUNCH;
}

static inline cudaStream_t ptn_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Warp-level sum of a double.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}
