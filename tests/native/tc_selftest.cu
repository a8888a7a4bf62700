// Self-test of the tcgen05 building blocks used by the mixed-precision
// contraction: shared-memory descriptors (K-major, 128-byte swizzle), the
// kind::f16 instruction descriptor, TMEM allocation and the 32x32b TMEM load
// layout. One CTA computes D = A * B^T for a 128 x 64 A and a 128 x 64 B
// (bf16, K contiguous) with four K=16 MMAs and writes the 128 x 128 FP32
// accumulator. Every wait is bounded; a timeout sets *status = 1.
//
// Test-only: built into its own library by tests/test_gpu_mixed.py, not part
// of libptn_gb300.
#include "ptn_common.cuh"
#include "tc_ptx.cuh"

std::atomic<unsigned long long> g_ptn_launches{0};

namespace {

__global__ void __launch_bounds__(128) tc_selftest_kernel(const uint16_t* __restrict__ A,
                                                          const uint16_t* __restrict__ B, float* __restrict__ D,
                                                          int32_t* status, int sw64) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = base;
  uint8_t* sB = base + 16384;
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x;
  // K = 64: one SW128 tile (sw64 = 0), two SW64 tiles of 32 (sw64 = 1,
  // second at +8 KB), or four SW32 tiles of 16 (sw64 = 2, at +4 KB each)
  for (int e = tid; e < 128 * 64; e += 128) {
    const int r = e >> 6, k = e & 63;
    const uint32_t off = sw64 == 2 ? (uint32_t)(k >> 4) * 4096u + tc::sw32_offset(r, k & 15)
                         : sw64 ? (uint32_t)(k >> 5) * 8192u + tc::sw64_offset(r, k & 31) : tc::sw128_offset(r, k);
    *reinterpret_cast<uint16_t*>(sA + off) = A[e];
    *reinterpret_cast<uint16_t*>(sB + off) = B[e];
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if (tid < 32) {
    tc::tmem_alloc(&tmem_base, 128);
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_base;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 128);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const uint32_t o = sw64 == 2 ? (uint32_t)kk * 4096u
                         : sw64 ? (uint32_t)(kk >> 1) * 8192u + (kk & 1) * 32u : kk * 32u;
      const uint64_t ad = sw64 == 2 ? tc::sdesc_sw32(tc::smem_u32(sA) + o)
                          : sw64 ? tc::sdesc_sw64(tc::smem_u32(sA) + o) : tc::sdesc_sw128(tc::smem_u32(sA) + o);
      const uint64_t bd = sw64 == 2 ? tc::sdesc_sw32(tc::smem_u32(sB) + o)
                          : sw64 ? tc::sdesc_sw64(tc::smem_u32(sB) + o) : tc::sdesc_sw128(tc::smem_u32(sB) + o);
      tc::mma_bf16(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
    }
    tc::mma_commit(&bar);
  }
  bool ok = tc::mbar_wait(&bar, 0, 2000000000LL);
  tc::fence_after();
  if (!ok) {
    if ((tid & 31) == 0) atomicExch(status, 1);
  } else {
    const int warp = tid >> 5, lane = tid & 31;
    const int row = warp * 32 + lane;
    for (int c0 = 0; c0 < 128; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[row * 128 + c0 + i] = v[i];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(tmem, 128);
}

}  // namespace

extern "C" int tc_selftest(const void* A, const void* B, void* D, int32_t* status, int32_t sw64,
                               void* stream) {
  if (!A || !B || !D || !status) return PTN_ERR_ARG;
  PTN_COUNT(1);
  tc_selftest_kernel<<<1, 128, 32768 + 1024, ptn_stream(stream)>>>(
      static_cast<const uint16_t*>(A), static_cast<const uint16_t*>(B), static_cast<float*>(D), status, sw64);
  return ptn_launch_status();
}
