// Strided multi-mode complex128 tensor contraction (FP64 plain path).
//
// C[m, n] = alpha * sum_k opA(A)[m, k] opB(B)[k, n] + beta * C[m, n], where m, n
// and k are each a group of up to PTN_MAX_MODES tensor legs addressed through
// per-operand strides. Legs are never transposed in memory: the environment,
// TTNO and site tensors of a tree node are contracted where they lie.
//
// GB300 FP64 issues about two DFMA per clock per SM, so this kernel is bound by
// the FP64 pipe at modest tile sizes: 64 x 64 complex outputs per CTA, 256
// threads with a 4 x 4 register tile each, K staged through shared memory in
// steps of 8. Tile offsets of the M and N rows are decoded once per CTA; the K
// offsets once per K step.
//
// Skinny outputs over a long K (an environment, or the gradient of one, is
// chi x w x chi summed over everything else) would leave most SMs idle with
// one CTA per output tile, so when there are few tiles the K range is split
// over gridDim.y: a first kernel writes beta * C (or zero), and each split
// adds alpha times its partial sums with double-precision atomics. The
// summation order then varies between runs at the level of rounding.
#include "ptn_common.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 8;

struct ModeDev {
  int n;
  int64_t dim[PTN_MAX_MODES];
  int64_t s0[PTN_MAX_MODES];
  int64_t s1[PTN_MAX_MODES];
};

struct ContractArgs {
  const double2* A;
  const double2* B;
  double2* C;
  double2 alpha, beta;
  int conj_a, conj_b;
  int beta_zero;
  int64_t M, N, K;
  int64_t tiles_n;
  int64_t k_chunk;  // K indices per split (the whole K when not split)
  int split;        // accumulate with atomics into a pre-scaled C
  ModeDev m, n, k;  // m: (A, C) strides; n: (B, C); k: (A, B)
};

__device__ __forceinline__ void decode(const ModeDev& md, int64_t idx, int64_t& o0, int64_t& o1) {
  o0 = 0;
  o1 = 0;
  for (int d = md.n - 1; d >= 0; --d) {
    int64_t dd = md.dim[d];
    int64_t q = idx / dd;
    int64_t r = idx - q * dd;
    o0 += r * md.s0[d];
    o1 += r * md.s1[d];
    idx = q;
  }
}

__global__ void __launch_bounds__(256) zcontract_kernel(const ContractArgs a) {
  __shared__ double2 As[BK][BM];
  __shared__ double2 Bs[BK][BN];
  __shared__ int64_t offAm[BM], offCm[BM], offBn[BN], offCn[BN];
  __shared__ int64_t offAk[BK], offBk[BK];

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t tile = blockIdx.x;
  const int64_t tm = tile / a.tiles_n;
  const int64_t tn = tile - tm * a.tiles_n;
  const int64_t m0 = tm * BM, n0 = tn * BN;

  if (tid < BM) {
    int64_t mi = m0 + tid;
    int64_t oa = -1, oc = -1;
    if (mi < a.M) decode(a.m, mi, oa, oc);
    offAm[tid] = oa;
    offCm[tid] = oc;
  } else if (tid < BM + BN) {
    int t = tid - BM;
    int64_t ni = n0 + t;
    int64_t ob = -1, oc = -1;
    if (ni < a.N) decode(a.n, ni, ob, oc);
    offBn[t] = ob;
    offCn[t] = oc;
  }

  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);

  const int64_t kbeg = (int64_t)blockIdx.y * a.k_chunk;
  const int64_t kend = (kbeg + a.k_chunk < a.K) ? kbeg + a.k_chunk : a.K;
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
    __syncthreads();
    if (tid < BK) {
      int64_t ki = k0 + tid;
      int64_t oa = -1, ob = -1;
      if (ki < kend) decode(a.k, ki, oa, ob);
      offAk[tid] = oa;
      offBk[tid] = ob;
    }
    __syncthreads();
    // 512 elements of each tile, two per thread.
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      int e = tid + r * 256;
      int kk = e / BM, mm = e - kk * BM;
      double2 v = make_double2(0.0, 0.0);
      if (offAk[kk] >= 0 && offAm[mm] >= 0) {
        v = a.A[offAm[mm] + offAk[kk]];
        if (a.conj_a) v.y = -v.y;
      }
      As[kk][mm] = v;
      int nn = e - kk * BN;
      double2 w = make_double2(0.0, 0.0);
      if (offBk[kk] >= 0 && offBn[nn] >= 0) {
        w = a.B[offBk[kk] + offBn[nn]];
        if (a.conj_b) w.y = -w.y;
      }
      Bs[kk][nn] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double2 av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cfma(av[i], bv[j], acc[i][j]);
    }
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int mm = ty + 16 * i;
    if (offCm[mm] < 0) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int nn = tx + 16 * j;
      if (offCn[nn] < 0) continue;
      double2* p = a.C + offCm[mm] + offCn[nn];
      double2 v = cmul(a.alpha, acc[i][j]);
      if (a.split) {
        atomicAdd(&p->x, v.x);
        atomicAdd(&p->y, v.y);
        continue;
      }
      if (!a.beta_zero) v = cfma(a.beta, *p, v);
      *p = v;
    }
  }
}

// Few outputs over a long K (a reduced density matrix: 2 x 2 outputs summed
// over every bond index; the last step of a small environment update): the
// tiled kernel would walk K on one CTA in steps of BK. Here each output is
// summed by a group of G = SMALL_THREADS / P threads (P = the next power of two
// of M * N), lane g of the group taking k = g, g + G, ...; the group's partial
// sums are then added by a fixed tree, so the result does not vary between runs.
constexpr int SMALL_THREADS = 1024;
constexpr int64_t SMALL_MAX_OUT = 256;   // M * N up to this (G >= 4)
constexpr int64_t SMALL_MIN_K = 64;

__global__ void __launch_bounds__(SMALL_THREADS) zcontract_small_kernel(const ContractArgs a) {
  __shared__ double2 part[SMALL_THREADS];
  __shared__ int64_t offAk[SMALL_THREADS], offBk[SMALL_THREADS];
  const int tid = threadIdx.x;
  const int64_t outs = a.M * a.N;
  int P = 1;
  while (P < outs) P <<= 1;
  const int G = SMALL_THREADS / P;
  const int o = tid / G, g = tid - o * G;
  double2 acc = make_double2(0.0, 0.0);
  int64_t oa = 0, ob = 0, ocm = 0, ocn = 0;
  if (o < outs) {
    const int64_t mi = o / a.N, ni = o - mi * a.N;
    decode(a.m, mi, oa, ocm);
    decode(a.n, ni, ob, ocn);
  }
  // the K offsets of a chunk of SMALL_THREADS indices are decoded once, one
  // per thread; each lane still takes k = g, g + G, ... in increasing order
  // (G divides the chunk)
  for (int64_t k0 = 0; k0 < a.K; k0 += SMALL_THREADS) {
    {
      const int64_t k = k0 + tid;
      int64_t x = 0, y = 0;
      if (k < a.K) decode(a.k, k, x, y);
      offAk[tid] = x;
      offBk[tid] = y;
    }
    __syncthreads();
    if (o < outs) {
      const int cnt = (int)(a.K - k0 < SMALL_THREADS ? a.K - k0 : SMALL_THREADS);
      // eight operand pairs loaded ahead of their (in-order) accumulation, so
      // the loads overlap; the order of the additions is unchanged
      constexpr int AHEAD = 8;
      int kk = g;
      for (; kk + (AHEAD - 1) * G < cnt; kk += AHEAD * G) {
        double2 x[AHEAD], y[AHEAD];
#pragma unroll
        for (int u = 0; u < AHEAD; ++u) {
          x[u] = a.A[oa + offAk[kk + u * G]];
          y[u] = a.B[offBk[kk + u * G] + ob];
        }
#pragma unroll
        for (int u = 0; u < AHEAD; ++u) {
          if (a.conj_a) x[u].y = -x[u].y;
          if (a.conj_b) y[u].y = -y[u].y;
          acc = cfma(x[u], y[u], acc);
        }
      }
      for (; kk < cnt; kk += G) {
        double2 x = a.A[oa + offAk[kk]];
        double2 y = a.B[offBk[kk] + ob];
        if (a.conj_a) x.y = -x.y;
        if (a.conj_b) y.y = -y.y;
        acc = cfma(x, y, acc);
      }
    }
    __syncthreads();
  }
  part[tid] = acc;
  __syncthreads();
  for (int h = G / 2; h > 0; h >>= 1) {
    if (g < h) {
      const double2 u = part[tid + h];
      part[tid] = make_double2(part[tid].x + u.x, part[tid].y + u.y);
    }
    __syncthreads();
  }
  if (g == 0 && o < outs) {
    double2* p = a.C + ocm + ocn;
    double2 v = cmul(a.alpha, part[tid]);
    if (!a.beta_zero) v = cfma(a.beta, *p, v);
    *p = v;
  }
}

// Products with fewer output tiles than SMs (and no K split): the tiled
// kernel would put a whole 64 x 64 tile -- most of it padding when M or N is
// small -- on each of a few SMs, at ~2 FP64 FMAs per clock per SM. Here one
// thread owns one output and adds A[m, k] B[k, n] over k in increasing order
// with the same complex FMA as the tiled kernel, so the result has the same
// bits; the K offsets are decoded once per CTA into shared memory.
constexpr int ELEM_THREADS = 64;

__global__ void __launch_bounds__(ELEM_THREADS) zcontract_elem_kernel(const ContractArgs a) {
  __shared__ int64_t offAk[ELEM_THREADS], offBk[ELEM_THREADS];
  const int64_t o = blockIdx.x * (int64_t)ELEM_THREADS + threadIdx.x;
  const bool valid = o < a.M * a.N;
  int64_t oa = 0, ocm = 0, ob = 0, ocn = 0;
  if (valid) {
    const int64_t mi = o / a.N, ni = o - mi * a.N;
    decode(a.m, mi, oa, ocm);
    decode(a.n, ni, ob, ocn);
  }
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t k0 = 0; k0 < a.K; k0 += ELEM_THREADS) {
    __syncthreads();
    {
      const int64_t k = k0 + threadIdx.x;
      int64_t x = -1, y = -1;
      if (k < a.K) decode(a.k, k, x, y);
      offAk[threadIdx.x] = x;
      offBk[threadIdx.x] = y;
    }
    __syncthreads();
    const int cnt = (int)(a.K - k0 < ELEM_THREADS ? a.K - k0 : ELEM_THREADS);
    if (valid) {
      // operand pairs loaded four ahead of their in-order accumulation
      int kk = 0;
      for (; kk + 3 < cnt; kk += 4) {
        double2 av[4], bv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          av[u] = a.A[oa + offAk[kk + u]];
          bv[u] = a.B[offBk[kk + u] + ob];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (a.conj_a) av[u].y = -av[u].y;
          if (a.conj_b) bv[u].y = -bv[u].y;
          acc = cfma(av[u], bv[u], acc);
        }
      }
      for (; kk < cnt; ++kk) {
        double2 av = a.A[oa + offAk[kk]];
        double2 bv = a.B[offBk[kk] + ob];
        if (a.conj_a) av.y = -av.y;
        if (a.conj_b) bv.y = -bv.y;
        acc = cfma(av, bv, acc);
      }
    }
  }
  if (valid) {
    double2* p = a.C + ocm + ocn;
    double2 v = cmul(a.alpha, acc);
    if (!a.beta_zero) v = cfma(a.beta, *p, v);
    *p = v;
  }
}

// C <- beta * C (zero when beta == 0) over the M x N output positions.// C <- beta * C (zero when beta == 0) over the M x N output positions.
__global__ void __launch_bounds__(256) zcontract_scale_c(const ContractArgs a) {
  const int64_t total = a.M * a.N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t mi = i / a.N, ni = i - mi * a.N;
    int64_t oa, ocm, ob, ocn;
    decode(a.m, mi, oa, ocm);
    decode(a.n, ni, ob, ocn);
    double2* p = a.C + ocm + ocn;
    *p = a.beta_zero ? make_double2(0.0, 0.0) : cmul(a.beta, *p);
  }
}

int fill_modes(const ptn_modes& src, ModeDev& dst, int which, int64_t& total) {
  // which: 0 -> (a, c) strides, 1 -> (b, c), 2 -> (a, b)
  if (src.n < 0 || src.n > PTN_MAX_MODES) return PTN_ERR_ARG;
  dst.n = src.n;
  total = 1;
  for (int i = 0; i < src.n; ++i) {
    if (src.dim[i] <= 0) return PTN_ERR_ARG;
    dst.dim[i] = src.dim[i];
    total *= src.dim[i];
    switch (which) {
      case 0: dst.s0[i] = src.stride_a[i]; dst.s1[i] = src.stride_c[i]; break;
      case 1: dst.s0[i] = src.stride_b[i]; dst.s1[i] = src.stride_c[i]; break;
      default: dst.s0[i] = src.stride_a[i]; dst.s1[i] = src.stride_b[i]; break;
    }
  }
  return PTN_OK;
}

}  // namespace

// Split K when the output tiles cover at most a quarter of the 152 SMs: about
// 304 CTAs in all, each split at least 256 K indices long, chunks a multiple
// of the K step; the chunks cover [0, K) exactly once.
extern "C" int64_t ptn_zcontract_splits(int64_t tiles, int64_t K, int64_t* k_chunk) {
  *k_chunk = K;
  if (tiles > 38 || K < 2048) return 1;
  int64_t want = (304 + tiles - 1) / tiles;
  int64_t most = K / 256;
  int64_t splits = want < most ? want : most;
  if (splits < 2) return 1;
  *k_chunk = ((K + splits - 1) / splits + BK - 1) / BK * BK;
  return (K + *k_chunk - 1) / *k_chunk;
}

extern "C" int ptn_zcontract(const ptn_contract_desc* d, void* stream) {
  if (!d || !d->A || !d->B || !d->C) return PTN_ERR_ARG;
  ContractArgs a;
  int64_t M, N, K;
  if (fill_modes(d->m, a.m, 0, M) || fill_modes(d->n, a.n, 1, N) || fill_modes(d->k, a.k, 2, K))
    return PTN_ERR_ARG;
  a.A = static_cast<const double2*>(d->A);
  a.B = static_cast<const double2*>(d->B);
  a.C = static_cast<double2*>(d->C);
  a.alpha = make_double2(d->alpha_re, d->alpha_im);
  a.beta = make_double2(d->beta_re, d->beta_im);
  a.beta_zero = (d->beta_re == 0.0 && d->beta_im == 0.0);
  a.conj_a = d->conj_a;
  a.conj_b = d->conj_b;
  a.M = M;
  a.N = N;
  a.K = K;
  if (M == 0 || N == 0) return PTN_OK;
  cudaStream_t s = ptn_stream(stream);
  if (M * N <= SMALL_MAX_OUT && K >= SMALL_MIN_K) {
    a.tiles_n = 1;
    a.k_chunk = K;
    a.split = 0;
    PTN_COUNT(1);
    zcontract_small_kernel<<<1, SMALL_THREADS, 0, s>>>(a);
    return ptn_launch_status();
  }
  int64_t tm = (M + BM - 1) / BM, tn = (N + BN - 1) / BN;
  a.tiles_n = tn;
  int64_t tiles = tm * tn;
  if (tiles > 0x7fffffffLL) return PTN_ERR_UNSUPPORTED;
  int64_t splits = ptn_zcontract_splits(tiles, K, &a.k_chunk);
  a.split = splits > 1;
  if (!a.split && tiles < 152) {
    const int64_t blocks = (M * N + ELEM_THREADS - 1) / ELEM_THREADS;
    if (blocks <= 0x7fffffffLL) {
      PTN_COUNT(1);
      zcontract_elem_kernel<<<(unsigned)blocks, ELEM_THREADS, 0, s>>>(a);
      return ptn_launch_status();
    }
  }
  if (a.split) {
    int64_t total = M * N;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    PTN_COUNT(1);
    zcontract_scale_c<<<(unsigned)blocks, 256, 0, s>>>(a);
  }
  PTN_COUNT(1);
  zcontract_kernel<<<dim3((unsigned)tiles, (unsigned)splits), 256, 0, s>>>(a);
  return ptn_launch_status();
}
