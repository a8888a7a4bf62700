// Krylov (Lanczos/Arnoldi) vector kernels in complex128.
//
// The Krylov basis q_0..q_j is stored as rows of one matrix; the Gram-Schmidt
// projections of krylov_exp_action (time_evolution/time_evolution.py:721-821)
// become one multi-dot pass (every vector read once, j+1 sums in registers)
// and one multi-axpy pass. Reductions are deterministic: warp shuffles, then a
// shared-memory tree per CTA, then one CTA summing the per-CTA partials in a
// fixed order, so repeated runs give identical bits.
#include "ptn_common.cuh"
#include "coop.cuh"

#include <mutex>

namespace {

constexpr int RT = 256;        // threads per CTA
constexpr int MAXQ = 16;       // vectors per multi-dot launch
constexpr int64_t CHUNK = 4096;

inline int64_t nblocks_for(int64_t n) {
  int64_t b = (n + CHUNK - 1) / CHUNK;
  if (b < 1) b = 1;
  if (b > 1184) b = 1184;  // 8 CTAs per SM on 148+ SMs
  return b;
}

template <int NQ>
__global__ void __launch_bounds__(RT) zdot_partial_kernel(const double2* __restrict__ Q, int64_t ldq,
                                                          int nq, const double2* __restrict__ w,
                                                          int64_t n, double2* __restrict__ partial) {
  double2 acc[NQ];
#pragma unroll
  for (int i = 0; i < NQ; ++i) acc[i] = make_double2(0.0, 0.0);
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT) {
    double2 wv = w[x];
#pragma unroll
    for (int i = 0; i < NQ; ++i)
      if (i < nq) acc[i] = cfmac(Q[(int64_t)i * ldq + x], wv, acc[i]);
  }
  __shared__ double2 red[RT / 32][NQ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (i >= nq) break;
    double2 v = warp_sum2(acc[i]);
    if (lane == 0) red[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double2 s = make_double2(0.0, 0.0);
    for (int wi = 0; wi < RT / 32; ++wi) s = cadd(s, red[wi][threadIdx.x]);
    partial[(int64_t)blockIdx.x * MAXQ + threadIdx.x] = s;
  }
}

__global__ void zdot_finish_kernel(const double2* __restrict__ partial, int nb, int nq,
                                   double2* __restrict__ h, int accumulate) {
  // one warp per output, lanes stride over the partials in a fixed order
  const int i = blockIdx.x;
  double2 s = make_double2(0.0, 0.0);
  for (int b = threadIdx.x; b < nb; b += 32) s = cadd(s, partial[(int64_t)b * MAXQ + i]);
  s = warp_sum2(s);
  if (threadIdx.x == 0) h[i] = accumulate ? cadd(h[i], s) : s;
}

__global__ void __launch_bounds__(RT) zaxpy_multi_kernel(const double2* __restrict__ Q, int64_t ldq,
                                                         int nq, const double2* __restrict__ h,
                                                         double2* __restrict__ w, int64_t n) {
  __shared__ double2 hs[64];
  if (threadIdx.x < nq) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT) {
    double2 v = w[x];
    for (int i = 0; i < nq; ++i) {
      double2 q = Q[(int64_t)i * ldq + x];
      double2 hq = cmul(hs[i], q);
      v = csub(v, hq);
    }
    w[x] = v;
  }
}

__global__ void __launch_bounds__(RT) nrm2_partial_kernel(const double2* __restrict__ w, int64_t n,
                                                          double* __restrict__ partial) {
  double acc = 0.0;
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT)
    acc += cabs2(w[x]);
  __shared__ double red[RT / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < RT / 32; ++i) s += red[i];
    partial[blockIdx.x] = s;
  }
}

__global__ void nrm2_finish_kernel(const double* __restrict__ partial, int nb, double* out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) s += partial[b];
  s = warp_sum(s);
  if (threadIdx.x == 0) out[0] = sqrt(s);
}

__global__ void __launch_bounds__(RT) zscal_inv_kernel(const double2* __restrict__ w,
                                                       const double* __restrict__ scale,
                                                       double2* __restrict__ y, int64_t n) {
  const double inv = 1.0 / scale[0];
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT)
    y[x] = cscale(w[x], inv);
}

__global__ void __launch_bounds__(RT) zscal_ratio_kernel(const double2* __restrict__ w,
                                                         const double* __restrict__ num,
                                                         const double* __restrict__ den,
                                                         double2* __restrict__ y, int64_t n) {
  const double f = den[0] > 0.0 ? num[0] / den[0] : 1.0;
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT)
    y[x] = cscale(w[x], f);
}

__global__ void __launch_bounds__(RT) zcombine_kernel(const double2* __restrict__ Q, int64_t ldq,
                                                      int nq, const double2* __restrict__ c,
                                                      double2* __restrict__ out, int64_t n) {
  __shared__ double2 cs[64];
  if (threadIdx.x < nq) cs[threadIdx.x] = c[threadIdx.x];
  __syncthreads();
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT) {
    double2 v = make_double2(0.0, 0.0);
    for (int i = 0; i < nq; ++i) v = cfma(cs[i], Q[(int64_t)i * ldq + x], v);
    out[x] = v;
  }
}

__global__ void check_finite_kernel(const double* __restrict__ x, int64_t n2, int32_t* flag) {
  for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n2; i += (int64_t)gridDim.x * RT)
    if (!isfinite(x[i])) *flag = 1;
}

}  // namespace

unsigned long long g_ptn_launches = 0;

extern "C" unsigned long long ptn_launch_counter(void) { return g_ptn_launches; }

// ---- fused Gram-Schmidt step (one cooperative launch) ---------------------------------
// Phase 1: |w|^2 and d_i = Q_i^H w; phase 2: w -= sum d_i Q_i and, in the same
// pass, e_i = Q_i^H w; phase 3: w -= sum e_i Q_i and |w|^2; phase 4:
// qnext = w / |w|. Every CTA writes its partial sums for a phase to its own
// slot; after the grid barrier every CTA adds the slots in CTA order, so all
// CTAs hold bit-identical totals (deterministic, like the multi-kernel path).
// Consecutive phases use alternating slot sets: a CTA that runs ahead writes
// the next phase's partials while others still read this phase's.
constexpr int GS_MAXQ = 16;
constexpr long long GS_WAIT_CYCLES = 4000000000LL;

struct GsArgs {
  const double2* Q;
  int64_t ldq;
  int nq;
  double2* w;
  int64_t n;
  double2* h;        // [2 nq]
  double* norms;     // [2]
  double2* qnext;    // may be null
  double2* slots;    // [2][G][GS_MAXQ + 1]
  unsigned* ctrl;
};

// Block-reduce k complex values (thread-local v[0..k)) into out[0..k) (thread 0 writes).
template <int K>
__device__ __forceinline__ void block_reduce_store(double2 (&v)[K], int k, double2* out) {
  __shared__ double2 red[RT / 32][K];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    if (i < k) {
      const double2 r = warp_sum2(v[i]);
      if (lane == 0) red[wp][i] = r;
    }
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double2 t = make_double2(0.0, 0.0);
    for (int u = 0; u < RT / 32; ++u) t = cadd(t, red[u][threadIdx.x]);
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

__device__ __forceinline__ double2* slot_set(const GsArgs& a, int phase) {
  return a.slots + (int64_t)(phase & 1) * gridDim.x * (GS_MAXQ + 1);
}

// Sum entries [0, k) of one slot set over CTAs in order, into shared tot[].
__device__ __forceinline__ void gather_totals(const double2* set, int k, double2* tot) {
  if (threadIdx.x < k) {
    double2 t = make_double2(0.0, 0.0);
    for (unsigned b = 0; b < gridDim.x; ++b) t = cadd(t, __ldcg(set + (int64_t)b * (GS_MAXQ + 1) + threadIdx.x));
    tot[threadIdx.x] = t;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(RT) zgs_step_kernel(GsArgs a) {
  __shared__ double2 tot[GS_MAXQ + 1];
  const int nq = a.nq;
  const int64_t gt = (int64_t)blockIdx.x * RT + threadIdx.x, nt = (int64_t)gridDim.x * RT;
  double2 acc[GS_MAXQ + 1];
  // phase 1: slot[0..nq) = Q^H w, slot[nq] = (|w|^2, 0)
#pragma unroll
  for (int i = 0; i <= GS_MAXQ; ++i) acc[i] = make_double2(0.0, 0.0);
  for (int64_t x = gt; x < a.n; x += nt) {
    const double2 wx = a.w[x];
    acc[GS_MAXQ].x += cabs2(wx);
#pragma unroll
    for (int i = 0; i < GS_MAXQ; ++i)
      if (i < nq) acc[i] = cfmac(a.Q[(int64_t)i * a.ldq + x], wx, acc[i]);
  }
  acc[nq] = acc[GS_MAXQ];
  block_reduce_store<GS_MAXQ + 1>(acc, nq + 1, slot_set(a, 0) + (int64_t)blockIdx.x * (GS_MAXQ + 1));
  if (!ptn_grid_barrier(a.ctrl, GS_WAIT_CYCLES)) goto abort;
  gather_totals(slot_set(a, 0), nq + 1, tot);
  if (blockIdx.x == 0 && threadIdx.x < nq) a.h[threadIdx.x] = tot[threadIdx.x];
  if (blockIdx.x == 0 && threadIdx.x == 0) a.norms[0] = sqrt(tot[nq].x);
  // phase 2: w -= Q d, then slot[0..nq) = Q^H w
  {
    double2 d[GS_MAXQ];
#pragma unroll
    for (int i = 0; i < GS_MAXQ; ++i) d[i] = i < nq ? tot[i] : make_double2(0.0, 0.0);
    __syncthreads();
#pragma unroll
    for (int i = 0; i <= GS_MAXQ; ++i) acc[i] = make_double2(0.0, 0.0);
    for (int64_t x = gt; x < a.n; x += nt) {
      double2 wx = a.w[x];
      double2 qv[GS_MAXQ];
#pragma unroll
      for (int i = 0; i < GS_MAXQ; ++i)
        if (i < nq) {
          qv[i] = a.Q[(int64_t)i * a.ldq + x];
          wx = csub(wx, cmul(d[i], qv[i]));
        }
#pragma unroll
      for (int i = 0; i < GS_MAXQ; ++i)
        if (i < nq) acc[i] = cfmac(qv[i], wx, acc[i]);
      a.w[x] = wx;
    }
  }
  block_reduce_store<GS_MAXQ + 1>(acc, nq, slot_set(a, 1) + (int64_t)blockIdx.x * (GS_MAXQ + 1));
  if (!ptn_grid_barrier(a.ctrl, GS_WAIT_CYCLES)) goto abort;
  gather_totals(slot_set(a, 1), nq, tot);
  if (blockIdx.x == 0 && threadIdx.x < nq) a.h[nq + threadIdx.x] = tot[threadIdx.x];
  // phase 3: w -= Q e, |w|^2
  {
    double2 e[GS_MAXQ];
#pragma unroll
    for (int i = 0; i < GS_MAXQ; ++i) e[i] = i < nq ? tot[i] : make_double2(0.0, 0.0);
    __syncthreads();
    double2 nrm[1] = {make_double2(0.0, 0.0)};
    for (int64_t x = gt; x < a.n; x += nt) {
      double2 wx = a.w[x];
#pragma unroll
      for (int i = 0; i < GS_MAXQ; ++i)
        if (i < nq) wx = csub(wx, cmul(e[i], a.Q[(int64_t)i * a.ldq + x]));
      a.w[x] = wx;
      nrm[0].x += cabs2(wx);
    }
    block_reduce_store<1>(nrm, 1, slot_set(a, 2) + (int64_t)blockIdx.x * (GS_MAXQ + 1));
  }
  if (!ptn_grid_barrier(a.ctrl, GS_WAIT_CYCLES)) goto abort;
  gather_totals(slot_set(a, 2), 1, tot);
  {
    const double beta = sqrt(tot[0].x);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.norms[1] = beta;
    if (a.qnext) {
      const double inv = 1.0 / beta;
      for (int64_t x = gt; x < a.n; x += nt) a.qnext[x] = cscale(a.w[x], inv);
    }
  }
  return;
abort:
  if (threadIdx.x == 0) a.norms[1] = __longlong_as_double(0x7ff8000000000000LL);
}

extern "C" int64_t ptn_krylov_partials(int64_t n) { return nblocks_for(n) * 36 + 64; }

extern "C" int ptn_zdot_multi(const void* Q, int64_t ldq, int32_t nq, const void* w, int64_t n,
                              void* h, int32_t accumulate, void* partial, void* stream) {
  if (!Q || !w || !h || !partial || nq < 1 || n < 1 || ldq < n) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  const int nb = (int)nblocks_for(n);
  for (int i0 = 0; i0 < nq; i0 += MAXQ) {
    int cnt = nq - i0 < MAXQ ? nq - i0 : MAXQ;
    const double2* Qi = static_cast<const double2*>(Q) + (int64_t)i0 * ldq;
    double2* hp = static_cast<double2*>(h) + i0;
    double2* pp = static_cast<double2*>(partial);
    PTN_COUNT(2);
    if (cnt <= 4)
      zdot_partial_kernel<4><<<nb, RT, 0, s>>>(Qi, ldq, cnt, static_cast<const double2*>(w), n, pp);
    else if (cnt <= 8)
      zdot_partial_kernel<8><<<nb, RT, 0, s>>>(Qi, ldq, cnt, static_cast<const double2*>(w), n, pp);
    else
      zdot_partial_kernel<16><<<nb, RT, 0, s>>>(Qi, ldq, cnt, static_cast<const double2*>(w), n, pp);
    zdot_finish_kernel<<<cnt, 32, 0, s>>>(pp, nb, cnt, hp, accumulate);
  }
  return ptn_launch_status();
}

extern "C" int ptn_zaxpy_multi(const void* Q, int64_t ldq, int32_t nq, const void* h, void* w,
                               int64_t n, void* stream) {
  if (!Q || !w || !h || nq < 1 || n < 1 || ldq < n) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  const int nb = (int)nblocks_for(n);
  for (int i0 = 0; i0 < nq; i0 += 64) {
    int cnt = nq - i0 < 64 ? nq - i0 : 64;
    PTN_COUNT(1);
    zaxpy_multi_kernel<<<nb, RT, 0, s>>>(static_cast<const double2*>(Q) + (int64_t)i0 * ldq, ldq, cnt,
                                         static_cast<const double2*>(h) + i0,
                                         static_cast<double2*>(w), n);
  }
  return ptn_launch_status();
}

extern "C" int ptn_dznrm2(const void* w, int64_t n, void* out_norm, void* partial, void* stream) {
  if (!w || !out_norm || !partial || n < 1) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  const int nb = (int)nblocks_for(n);
  PTN_COUNT(1);
  nrm2_partial_kernel<<<nb, RT, 0, s>>>(static_cast<const double2*>(w), n, static_cast<double*>(partial));
  PTN_COUNT(1);
  nrm2_finish_kernel<<<1, 32, 0, s>>>(static_cast<const double*>(partial), nb, static_cast<double*>(out_norm));
  return ptn_launch_status();
}

extern "C" int ptn_zscal_inv(const void* w, const double* scale, void* y, int64_t n, void* stream) {
  if (!w || !scale || !y || n < 1) return PTN_ERR_ARG;
  PTN_COUNT(1);
  zscal_inv_kernel<<<(int)nblocks_for(n), RT, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(w), scale, static_cast<double2*>(y), n);
  return ptn_launch_status();
}

extern "C" int ptn_zscal_ratio(const void* w, const double* num, const double* den, void* y, int64_t n,
                               void* stream) {
  if (!w || !num || !den || !y || n < 1) return PTN_ERR_ARG;
  PTN_COUNT(1);
  zscal_ratio_kernel<<<(int)nblocks_for(n), RT, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(w), num, den, static_cast<double2*>(y), n);
  return ptn_launch_status();
}

extern "C" int ptn_zcombine(const void* Q, int64_t ldq, int32_t nq, const void* c, void* out,
                            int64_t n, void* stream) {
  if (!Q || !c || !out || nq < 1 || nq > 64 || n < 1 || ldq < n) return PTN_ERR_ARG;
  PTN_COUNT(1);
  zcombine_kernel<<<(int)nblocks_for(n), RT, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(Q), ldq, nq, static_cast<const double2*>(c),
      static_cast<double2*>(out), n);
  return ptn_launch_status();
}

extern "C" int ptn_check_finite(const void* x, int64_t n, int32_t* flag, void* stream) {
  if (!x || !flag || n < 0) return PTN_ERR_ARG;
  if (n == 0) return PTN_OK;
  PTN_COUNT(1);
  check_finite_kernel<<<(int)nblocks_for(n), RT, 0, ptn_stream(stream)>>>(
      static_cast<const double*>(x), 2 * n, flag);
  return ptn_launch_status();
}

// Fused Gram-Schmidt step for nq <= GS_MAXQ and n <= 2^21 (one cooperative launch); returns
// PTN_ERR_UNSUPPORTED when it does not apply, so the caller runs the kernels
// one by one.
int ptn_gs_step_fused(const void* Q, int64_t ldq, int32_t nq, void* w, int64_t n, void* h, void* partial,
                      double* norms, void* qnext, void* stream) {
  static int cached[64] = {0};
  static std::mutex mu;
  // Long vectors keep the multi-kernel path: it runs ~8 CTAs per SM for
  // bandwidth, this kernel one (its grid must be co-resident).
  if (nq > GS_MAXQ || n > (int64_t(1) << 21)) return PTN_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PTN_ERR_UNSUPPORTED;
  int maxb;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (cached[dev] == 0) {
      int per_sm = 0, sms = 0, coop = 0;
      if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) cached[dev] = -1;
      else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zgs_step_kernel, RT, 0) != cudaSuccess ||
               cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        cached[dev] = -1;
      else
        cached[dev] = per_sm * sms;
    }
    maxb = cached[dev];
  }
  if (maxb <= 0) return PTN_ERR_UNSUPPORTED;
  int64_t G = nblocks_for(n);
  if (G > maxb) G = maxb;
  if (G > 152) G = 152;
  GsArgs a;
  a.Q = static_cast<const double2*>(Q);
  a.ldq = ldq;
  a.nq = nq;
  a.w = static_cast<double2*>(w);
  a.n = n;
  a.h = static_cast<double2*>(h);
  a.norms = norms;
  a.qnext = static_cast<double2*>(qnext);
  a.slots = static_cast<double2*>(partial);
  a.ctrl = reinterpret_cast<unsigned*>(a.slots + 2 * G * (GS_MAXQ + 1));
  cudaStream_t s = ptn_stream(stream);
  if (cudaMemsetAsync(a.ctrl, 0, 256, s) != cudaSuccess) return PTN_ERR_LAUNCH;
  void* args[] = {&a};
  PTN_COUNT(1);
  if (cudaLaunchCooperativeKernel((const void*)zgs_step_kernel, dim3((unsigned)G), dim3(RT), args, 0, s) !=
      cudaSuccess) {
    cudaGetLastError();
    return PTN_ERR_LAUNCH;
  }
  return PTN_OK;
}
