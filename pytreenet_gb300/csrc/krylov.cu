// Krylov (Lanczos/Arnoldi) vector kernels in complex128.
//
// The Krylov basis q_0..q_j is stored as rows of one matrix; the Gram-Schmidt
// projections of krylov_exp_action (time_evolution/time_evolution.py:721-821)
// become one multi-dot pass (every vector read once, j+1 sums in registers)
// and one multi-axpy pass. Reductions are deterministic: warp shuffles, then a
// shared-memory tree per CTA, then one CTA summing the per-CTA partials in a
// fixed order, so repeated runs give identical bits.
#include "ptn_common.cuh"

namespace {

constexpr int RT = 256;        // threads per CTA
constexpr int MAXQ = 16;       // vectors per multi-dot launch
constexpr int64_t CHUNK = 1024;   // elements per CTA: enough CTAs to keep HBM busy on 131k-entry vectors

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

std::atomic<unsigned long long> g_ptn_launches{0};

extern "C" unsigned long long ptn_launch_counter(void) { return g_ptn_launches.load(); }

extern "C" int ptn_stream_synchronize(void* stream) {
  return cudaStreamSynchronize(ptn_stream(stream)) == cudaSuccess ? PTN_OK : PTN_ERR_LAUNCH;
}

// ---- Gram-Schmidt step in three passes ----------------------------------------------------
// One pass over w per kernel; each CTA writes fixed-order partial sums, and
// the last CTA to finish (atomic ticket, no waiting) adds them up in CTA
// order, so the totals are deterministic. The last CTA also re-arms the
// ticket for the next pass.
//   mode 0: (Q^H w, |w|^2)            -> h[0..nq), norms[0] = |w|
//   mode 1: w -= Q hin, then Q^H w    -> h[nq..2nq)
//   mode 2: w -= Q hin, then |w|^2    -> norms[1] = |w|
template <int NQ>
__global__ void __launch_bounds__(RT) gs_pass_kernel(const double2* __restrict__ Q, int64_t ldq, int nq,
                                                     double2* __restrict__ w, int64_t n,
                                                     const double2* __restrict__ hin, double2* __restrict__ hout,
                                                     double* __restrict__ nout, double2* __restrict__ partial,
                                                     unsigned* __restrict__ ticket, int mode) {
  __shared__ double2 hs[NQ];
  __shared__ double2 red[RT / 32][NQ + 1];
  __shared__ int last;
  if (mode != 0 && threadIdx.x < nq) hs[threadIdx.x] = hin[threadIdx.x];
  __syncthreads();
  double2 acc[NQ];
#pragma unroll
  for (int i = 0; i < NQ; ++i) acc[i] = make_double2(0.0, 0.0);
  double nacc = 0.0;
  for (int64_t x = blockIdx.x * (int64_t)RT + threadIdx.x; x < n; x += (int64_t)gridDim.x * RT) {
    double2 wv = w[x];
    if (mode != 0) {
      for (int i = 0; i < nq; ++i) wv = csub(wv, cmul(hs[i], Q[(int64_t)i * ldq + x]));
      w[x] = wv;
    }
    if (mode != 2) {
#pragma unroll
      for (int i = 0; i < NQ; ++i)
        if (i < nq) acc[i] = cfmac(Q[(int64_t)i * ldq + x], wv, acc[i]);
    }
    if (mode != 1) nacc += cabs2(wv);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (i >= nq) break;
    const double2 v = warp_sum2(acc[i]);
    if (lane == 0) red[warp][i] = v;
  }
  {
    const double v = warp_sum(nacc);
    if (lane == 0) red[warp][NQ] = make_double2(v, 0.0);
  }
  __syncthreads();
  double2* mine = partial + (int64_t)blockIdx.x * (NQ + 1);
  if (threadIdx.x < nq || threadIdx.x == NQ) {
    double2 t = make_double2(0.0, 0.0);
    for (int u = 0; u < RT / 32; ++u) t = cadd(t, red[u][threadIdx.x]);
    mine[threadIdx.x] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // The CTAs' partial sums, added in CTA order by one thread per value (the
  // order fixes the bits); they are staged through shared memory in chunks of
  // GS_STAGE CTAs, loaded by every thread at once, so the adds wait on shared
  // memory instead of one L2 round trip each.
  constexpr int GS_STAGE = 64;
  __shared__ double2 stage[GS_STAGE * (NQ + 1)];
  double2 t = make_double2(0.0, 0.0);
  const bool mine_v = threadIdx.x < nq || threadIdx.x == NQ;
  for (unsigned b0 = 0; b0 < gridDim.x; b0 += GS_STAGE) {
    const unsigned cnt = gridDim.x - b0 < GS_STAGE ? gridDim.x - b0 : GS_STAGE;
    for (unsigned e = threadIdx.x; e < cnt * (NQ + 1); e += RT)
      stage[e] = __ldcg(partial + (int64_t)b0 * (NQ + 1) + e);
    __syncthreads();
    if (mine_v)
      for (unsigned b = 0; b < cnt; ++b) t = cadd(t, stage[b * (NQ + 1) + threadIdx.x]);
    __syncthreads();
  }
  if (mine_v) {
    if (threadIdx.x == NQ) {
      if (mode != 1) nout[0] = sqrt(t.x);
    } else if (mode != 2) {
      hout[threadIdx.x] = t;
    }
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

template <int NQ>
static int gs_step_passes(const double2* Q, int64_t ldq, int nq, double2* w, int64_t n, double2* h,
                          double2* partial, double* norms, double2* qnext, cudaStream_t s) {
  const int nb = (int)nblocks_for(n);
  unsigned* ticket = reinterpret_cast<unsigned*>(partial + (int64_t)nb * (NQ + 1));
  if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), s) != cudaSuccess) return PTN_ERR_LAUNCH;
  PTN_COUNT(3);
  gs_pass_kernel<NQ><<<nb, RT, 0, s>>>(Q, ldq, nq, w, n, nullptr, h, norms, partial, ticket, 0);
  gs_pass_kernel<NQ><<<nb, RT, 0, s>>>(Q, ldq, nq, w, n, h, h + nq, nullptr, partial, ticket, 1);
  gs_pass_kernel<NQ><<<nb, RT, 0, s>>>(Q, ldq, nq, w, n, h + nq, nullptr, norms + 1, partial, ticket, 2);
  if (qnext) {
    PTN_COUNT(1);
    zscal_inv_kernel<<<(int)nblocks_for(n), RT, 0, s>>>(w, norms + 1, qnext, n);
  }
  return ptn_launch_status();
}

// The Gram-Schmidt step as three passes for nq <= MAXQ (PTN_ERR_UNSUPPORTED
// otherwise, and the caller runs the kernels one by one).
int ptn_gs_step_passes(const void* Q, int64_t ldq, int32_t nq, void* w, int64_t n, void* h, void* partial,
                       double* norms, void* qnext, void* stream) {
  const double2* q = static_cast<const double2*>(Q);
  double2* wv = static_cast<double2*>(w);
  double2* hv = static_cast<double2*>(h);
  double2* pv = static_cast<double2*>(partial);
  double2* qn = static_cast<double2*>(qnext);
  cudaStream_t s = ptn_stream(stream);
  if (nq <= 4) return gs_step_passes<4>(q, ldq, nq, wv, n, hv, pv, norms, qn, s);
  if (nq <= 8) return gs_step_passes<8>(q, ldq, nq, wv, n, hv, pv, norms, qn, s);
  if (nq <= MAXQ) return gs_step_passes<MAXQ>(q, ldq, nq, wv, n, hv, pv, norms, qn, s);
  return PTN_ERR_UNSUPPORTED;
}

extern "C" int64_t ptn_krylov_partials(int64_t n) { return nblocks_for(n) * (MAXQ + 1) + 16; }

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
