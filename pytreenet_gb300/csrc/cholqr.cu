// Device-side pieces of CholeskyQR2 for the mixed-precision QR split, and the
// row scan that lets a Householder QR skip exactly-zero trailing rows.
//
// The QR split of a site tensor (tensor_qr_decomposition, util/tensor_splitting.py:60-107)
// is, for a tall matrix A (m x k) of full numerical rank, done as CholeskyQR2:
//   G1 = A^H A,   G1 = R1^H R1,   Q1 = A R1^{-1},
//   G2 = Q1^H Q1, G2 = R2^H R2,   Q  = Q1 R2^{-1},   R = R2 R1.
// The Gram matrices and the products with R^{-1} run on the tensor cores
// (BF16 splits, FP32 accumulation); this file holds the k x k factorisations
// (Cholesky, triangular inverse), done in FP32 on one CTA so that no host
// round trip sits between the Gram matrix and its use, and the product R2 R1.
// Q differs from the Householder Q by a diagonal phase only, which one-site
// TDVP absorbs as a gauge change on the bond.
//
// A matrix that is not of full numerical rank (a pivot below ratio * the
// largest, or not positive) is reported through *status; the caller then
// takes the Householder path, whose orthonormal complement the reference's
// results depend on.
#include <math.h>

#include "ptn_common.cuh"

namespace {

constexpr int CH_T = 1024;     // threads of the factorisation CTA
constexpr int CH_B = 32;       // panel width
constexpr int CH_MAXK = 256;   // largest k (the inverse phase stages ~211 KB of shared memory at k = 256)
constexpr int PLD = CH_B + 1;  // padded row of a smem block (float2 entries)

// acc += a * conj(b)
__device__ __forceinline__ void fma_cb(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(a.y, b.x, acc.y);
  acc.y = fmaf(-a.x, b.y, acc.y);
}
// acc += a * b
__device__ __forceinline__ void fma_c(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// (bi, bj), bj <= bi, from the row-wise index of a lower-triangular block list.
__device__ __forceinline__ void tri_decode(int idx, int& bi, int& bj) {
  int r = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
  while ((r + 1) * (r + 2) / 2 <= idx) ++r;
  while (r * (r + 1) / 2 > idx) --r;
  bi = r;
  bj = idx - r * (r + 1) / 2;
}

// G (k x k, row-major with leading dimension ldg, Hermitian up to rounding)
// = R^H R with R upper triangular. Writes R and R^{-1} (k x k row-major,
// zero below the diagonal). Work: L and T, kp x kp float2 each (kp = k
// rounded up to CH_B). series != 0 allows the first-order form for a Gram
// matrix close to the identity: with E = G - I and ||E||_F <= series_tol,
// R = I + U, R^{-1} = I - U where U is E's strict upper part plus half its
// diagonal (the neglected terms are O(||E||^2)).
__global__ void __launch_bounds__(CH_T, 1)
    chol_inv_kernel(const double2* __restrict__ G, int64_t ldg, int k, int kp, float2* __restrict__ L,
                    float2* __restrict__ T, double2* __restrict__ R, double2* __restrict__ Rinv, float ratio,
                    int series, float series_tol, int32_t* __restrict__ status) {
  extern __shared__ float2 sm[];
  __shared__ float piv_s[CH_B];
  __shared__ float red_s[CH_T / 32];
  __shared__ float dmin_s, dmax_s;
  __shared__ int bad_s, use_series_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = kp / CH_B;

  if (series) {
    // ||G - I||_F over the Hermitian part
    float acc = 0.f;
    for (int64_t e = tid; e < (int64_t)k * k; e += CH_T) {
      const int i = (int)(e / k), j = (int)(e - (int64_t)i * k);
      const double2 a = G[i * ldg + j], b = G[j * ldg + i];
      float ex = (float)(0.5 * (a.x + b.x)) - (i == j ? 1.f : 0.f);
      float ey = (float)(0.5 * (a.y - b.y));
      acc = fmaf(ex, ex, fmaf(ey, ey, acc));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red_s[warp] = acc;
    __syncthreads();
    if (tid == 0) {
      float s = 0.f;
      for (int w = 0; w < CH_T / 32; ++w) s += red_s[w];
      use_series_s = (sqrtf(s) <= series_tol) ? 1 : 0;
    }
    __syncthreads();
    if (use_series_s) {
      for (int64_t e = tid; e < (int64_t)k * k; e += CH_T) {
        const int i = (int)(e / k), j = (int)(e - (int64_t)i * k);
        double2 u = make_double2(0.0, 0.0);
        if (j > i) {
          const double2 a = G[i * ldg + j], b = G[j * ldg + i];
          u = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
        } else if (j == i) {
          u = make_double2(0.5 * (G[i * ldg + i].x - 1.0), 0.0);
        }
        const double one = (i == j) ? 1.0 : 0.0;
        R[e] = make_double2(one + u.x, u.y);
        Rinv[e] = make_double2(one - u.x, -u.y);
      }
      return;
    }
  }

  // ---- phase 0: L <- lower triangle of the Hermitian part of G, identity padding
  for (int64_t e = tid; e < (int64_t)kp * kp; e += CH_T) {
    const int i = (int)(e / kp), j = (int)(e - (int64_t)i * kp);
    float2 v = make_float2(0.f, 0.f);
    if (i >= j) {
      if (i < k) {
        const double2 a = G[i * ldg + j], b = G[j * ldg + i];
        v = make_float2((float)(0.5 * (a.x + b.x)), (float)(0.5 * (a.y - b.y)));
      } else if (i == j) {
        v = make_float2(1.f, 0.f);
      }
    }
    L[e] = v;
  }
  if (tid == 0) {
    bad_s = 0;
    dmin_s = INFINITY;
    dmax_s = 0.f;
  }
  __syncthreads();

  // ---- phase 1: blocked right-looking Cholesky, G = L L^H
  for (int p = 0; p < nb; ++p) {
    const int r0 = p * CH_B, rows = kp - r0;
    for (int e = tid; e < rows * CH_B; e += CH_T) {
      const int rr = e / CH_B, c = e - rr * CH_B;
      sm[rr * PLD + c] = L[(int64_t)(r0 + rr) * kp + r0 + c];
    }
    __syncthreads();
    // unblocked LDL^H elimination of the panel (pivot P[c][c] left unscaled)
    for (int c = 0; c < CH_B; ++c) {
      const float ip = 1.0f / sm[c * PLD + c].x;
      const int s = lane;
      if (s > c) {
        const float2 ps = sm[s * PLD + c];
        for (int rr = (warp >= s ? warp : warp + 32 * ((s - warp + 31) / 32)); rr < rows; rr += 32) {
          const float2 prc = sm[rr * PLD + c];
          float2 t = make_float2(0.f, 0.f);
          fma_cb(t, prc, ps);
          float2* q = &sm[rr * PLD + s];
          q->x = fmaf(-t.x, ip, q->x);
          q->y = fmaf(-t.y, ip, q->y);
        }
      }
      __syncthreads();
    }
    if (warp == 0) {
      const float pv = sm[lane * PLD + lane].x;
      const bool bad = !(pv > 0.f) || !isfinite(pv);
      const float d = bad ? 0.f : sqrtf(pv);
      piv_s[lane] = d;
      const unsigned anyb = __ballot_sync(0xffffffffu, bad);
      const bool real_col = r0 + lane < k;   // the identity padding takes no part in the ratio test
      const float mn = warp_minf(real_col ? d : INFINITY), mx = warp_maxf(real_col ? d : 0.f);
      if (lane == 0) {
        if (anyb) bad_s = 1;
        dmin_s = fminf(dmin_s, mn);
        dmax_s = fmaxf(dmax_s, mx);
      }
    }
    __syncthreads();
    if (bad_s) break;
    // scale the panel: L[rr][c] = P[rr][c] / d_c (rr > c), d_c on the diagonal
    for (int e = tid; e < rows * CH_B; e += CH_T) {
      const int rr = e / CH_B, c = e - rr * CH_B;
      const float d = piv_s[c];
      float2 v = sm[rr * PLD + c];
      if (rr == c) v = make_float2(d, 0.f);
      else if (rr > c) v = make_float2(v.x / d, v.y / d);
      else v = make_float2(0.f, 0.f);
      sm[rr * PLD + c] = v;
      L[(int64_t)(r0 + rr) * kp + r0 + c] = v;
    }
    __syncthreads();
    // trailing update of the lower triangle: L[i][j] -= sum_c L[i][c] conj(L[j][c])
    const int nt = nb - p - 1;
    const int nblk = nt * (nt + 1) / 2;
    for (int b = 0; b < nblk; ++b) {
      int bi, bj;
      tri_decode(b, bi, bj);
      const int r = warp, s = lane;
      if (bi == bj && r < s) continue;
      const int gi = (p + 1 + bi) * CH_B + r, gj = (p + 1 + bj) * CH_B + s;
      float2* dst = &L[(int64_t)gi * kp + gj];
      float2 cur = *dst;
      const float2* pi = &sm[(gi - r0) * PLD];
      const float2* pj = &sm[(gj - r0) * PLD];
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll 8
      for (int c = 0; c < CH_B; ++c) fma_cb(acc, pi[c], pj[c]);
      cur.x -= acc.x;
      cur.y -= acc.y;
      *dst = cur;
    }
    __syncthreads();
  }
  if (bad_s || !(dmin_s > ratio * dmax_s)) {
    if (tid == 0) atomicExch(status, PTN_ERR_NOCONVERGE);
    return;
  }

  // ---- phase 2: T = L^{-1} by blocks. Diagonal blocks first (warp w inverts
  // block w by forward substitution, lane = column), then block rows.
  const int lrow = (nb * CH_B * PLD > CH_B * (kp + 1)) ? nb * CH_B * PLD : CH_B * (kp + 1);
  float2* sL = sm;                          // [nb][32][PLD] diagonal blocks of L
  float2* sT = sm + lrow;                   // [nb][32][PLD] their inverses
  for (int e = tid; e < nb * CH_B * CH_B; e += CH_T) {
    const int b = e / (CH_B * CH_B), rr = (e / CH_B) % CH_B, c = e % CH_B;
    sL[(b * CH_B + rr) * PLD + c] = L[(int64_t)(b * CH_B + rr) * kp + b * CH_B + c];
  }
  __syncthreads();
  for (int b = warp; b < nb; b += 32) {
    const float2* Lb = sL + b * CH_B * PLD;
    float2* Tb = sT + b * CH_B * PLD;
    const int c = lane;
    for (int rr = 0; rr < CH_B; ++rr) {
      float2 v = make_float2(rr == c ? 1.f : 0.f, 0.f);
      if (rr >= c) {
        for (int l = c; l < rr; ++l) {
          const float2 a = Lb[rr * PLD + l], t = Tb[l * PLD + c];
          v.x -= a.x * t.x - a.y * t.y;
          v.y -= a.x * t.y + a.y * t.x;
        }
        const float d = Lb[rr * PLD + rr].x;
        v = make_float2(v.x / d, v.y / d);
      } else {
        v = make_float2(0.f, 0.f);
      }
      Tb[rr * PLD + c] = v;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int e = tid; e < nb * CH_B * CH_B; e += CH_T) {
    const int b = e / (CH_B * CH_B), rr = (e / CH_B) % CH_B, c = e % CH_B;
    T[(int64_t)(b * CH_B + rr) * kp + b * CH_B + c] = sT[(b * CH_B + rr) * PLD + c];
  }
  __syncthreads();
  // block row i: T_ip = -T_ii * sum_{j=p}^{i-1} L_ij T_jp, p < i
  float2* sRow = sm;                        // L block row i: [32][i*32] (ld = kp + 1), reuses sL
  float2* sCol = sT + nb * CH_B * PLD;      // T block column p, rows p*32 .. i*32-1: [(i-p)*32][PLD]
  float2* sO = sCol + kp * PLD;             // [32][PLD]
  const int RLD = kp + 1;
  for (int i = 1; i < nb; ++i) {
    for (int e = tid; e < CH_B * i * CH_B; e += CH_T) {
      const int rr = e / (i * CH_B), c = e - rr * (i * CH_B);
      sRow[rr * RLD + c] = L[(int64_t)(i * CH_B + rr) * kp + c];
    }
    for (int p = 0; p < i; ++p) {
      const int nr = (i - p) * CH_B;
      for (int e = tid; e < nr * CH_B; e += CH_T) {
        const int rr = e / CH_B, c = e - rr * CH_B;
        sCol[rr * PLD + c] = T[(int64_t)(p * CH_B + rr) * kp + p * CH_B + c];
      }
      __syncthreads();
      const int r = warp, s = lane;
      float2 acc = make_float2(0.f, 0.f);
      const float2* lr = sRow + r * RLD + p * CH_B;
#pragma unroll 8
      for (int l = 0; l < nr; ++l) fma_c(acc, lr[l], sCol[l * PLD + s]);
      sO[r * PLD + s] = acc;
      __syncthreads();
      const float2* ti = sT + (i * CH_B + r) * PLD;
      float2 out = make_float2(0.f, 0.f);
#pragma unroll 8
      for (int l = 0; l <= r; ++l) fma_c(out, ti[l], sO[l * PLD + s]);
      T[(int64_t)(i * CH_B + r) * kp + p * CH_B + s] = make_float2(-out.x, -out.y);
      __syncthreads();
    }
  }
  __syncthreads();
  // ---- outputs: R = L^H, R^{-1} = T^H (upper triangular, k x k, row-major)
  for (int64_t e = tid; e < (int64_t)k * k; e += CH_T) {
    const int i = (int)(e / k), j = (int)(e - (int64_t)i * k);
    if (j >= i) {
      const float2 l = L[(int64_t)j * kp + i], t = T[(int64_t)j * kp + i];
      R[e] = make_double2((double)l.x, -(double)l.y);
      Rinv[e] = make_double2((double)t.x, -(double)t.y);
    } else {
      R[e] = make_double2(0.0, 0.0);
      Rinv[e] = make_double2(0.0, 0.0);
    }
  }
}

// C = A B for upper-triangular A, B (k x k row-major); C[i][j] = sum_{l=i..j} A[i][l] B[l][j].
__global__ void tri_mul_kernel(const double2* __restrict__ A, const double2* __restrict__ B, double2* __restrict__ C,
                               int64_t k) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= k * k) return;
  const int64_t i = e / k, j = e - (e / k) * k;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t l = i; l <= j; ++l) acc = cfma(A[i * k + l], B[l * k + j], acc);
  C[e] = acc;
}

// R[i][j] = 2 R0[i][j] - sum_{l=i..j} R0[i][l] W[l][j] (upper triangular): the
// Newton step R = R0 (2I - W) with W = X R0.
__global__ void newton_inv_kernel(const double2* __restrict__ R0, const double2* __restrict__ W,
                                  double2* __restrict__ R, int64_t k) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= k * k) return;
  const int64_t i = e / k, j = e - (e / k) * k;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t l = i; l <= j; ++l) acc = cfma(R0[i * k + l], W[l * k + j], acc);
  const double2 r0 = (j >= i) ? R0[e] : make_double2(0.0, 0.0);
  R[e] = (j >= i) ? make_double2(2.0 * r0.x - acc.x, 2.0 * r0.y - acc.y) : make_double2(0.0, 0.0);
}

// out[0] = 1 + the largest row index i with a nonzero entry (0 when A is zero);
// out must start at 0.
__global__ void nonzero_rows_kernel(const double2* __restrict__ A, const int64_t* __restrict__ rowoff, int64_t m,
                                        int64_t k, int64_t cs, unsigned long long* __restrict__ out) {
  const int64_t total = m * k;
  int64_t best = -1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, c = e - (e / k) * k;
    const double2 v = A[rowoff[i] + c * cs];
    if ((v.x != 0.0 || v.y != 0.0) && i > best) best = i;
  }
  unsigned long long b = (unsigned long long)(best + 1);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  if ((threadIdx.x & 31) == 0 && b > 0) atomicMax(out, b);
}

__global__ void init_u64_kernel(unsigned long long* p) { *p = 0ull; }

inline int64_t kpad(int64_t k) { return (k + CH_B - 1) / CH_B * CH_B; }

inline size_t chol_smem_bytes(int64_t kp) {
  const int64_t nb = kp / CH_B;
  const int64_t panel = kp * PLD;                                            // phase 1
  const int64_t lrow = (nb * CH_B * PLD > CH_B * (kp + 1)) ? nb * CH_B * PLD : CH_B * (kp + 1);
  const int64_t inv = lrow + nb * CH_B * PLD + kp * PLD + CH_B * PLD;        // phase 2
  return sizeof(float2) * (size_t)(panel > inv ? panel : inv);
}

}  // namespace

extern "C" int64_t ptn_zchol_work_bytes(int64_t k) {
  if (k < 1) return 0;
  const int64_t kp = kpad(k);
  return 2 * kp * kp * (int64_t)sizeof(float2) + 256;
}

extern "C" int64_t ptn_zchol_max_k(void) { return CH_MAXK; }

extern "C" int ptn_zchol_upper(const void* G, int64_t ldg, int64_t k, void* R, void* Rinv, double pivot_ratio,
                               int32_t series, double series_tol, int32_t* status, void* work, void* stream) {
  if (!G || !R || !Rinv || !status || !work || k < 1 || ldg < k) return PTN_ERR_ARG;
  if (k > CH_MAXK) return PTN_ERR_UNSUPPORTED;
  if (reinterpret_cast<uintptr_t>(work) & 15) return PTN_ERR_ARG;
  const int64_t kp = kpad(k);
  const size_t smem = chol_smem_bytes(kp);
  if (smem > 227 * 1024) return PTN_ERR_UNSUPPORTED;
  // the largest dynamic size any k <= CH_MAXK needs (the kernel's static
  // shared memory comes on top, within the 227 KB opt-in limit)
  static const cudaError_t attr = cudaFuncSetAttribute(
      chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chol_smem_bytes(kpad(CH_MAXK)));
  if (attr != cudaSuccess) return PTN_ERR_LAUNCH;
  float2* L = static_cast<float2*>(work);
  float2* T = L + kp * kp;
  PTN_COUNT(1);
  chol_inv_kernel<<<1, CH_T, smem, ptn_stream(stream)>>>(static_cast<const double2*>(G), ldg, (int)k, (int)kp, L, T,
                                                          static_cast<double2*>(R), static_cast<double2*>(Rinv),
                                                          (float)pivot_ratio, series ? 1 : 0, (float)series_tol,
                                                          status);
  return ptn_launch_status();
}

extern "C" int ptn_ztri_mul_upper(const void* A, const void* B, void* C, int64_t k, void* stream) {
  if (!A || !B || !C || k < 1) return PTN_ERR_ARG;
  if (C == A || C == B) return PTN_ERR_ARG;
  const int64_t n = k * k;
  PTN_COUNT(1);
  tri_mul_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(A), static_cast<const double2*>(B), static_cast<double2*>(C), k);
  return ptn_launch_status();
}

extern "C" int ptn_ztri_inv_newton(const void* X, const void* R0, void* R, void* work, int64_t k, void* stream) {
  if (!X || !R0 || !R || !work || k < 1) return PTN_ERR_ARG;
  if (R == X || R == R0 || work == X || work == R0 || work == R) return PTN_ERR_ARG;
  const int64_t n = k * k;
  const unsigned g = (unsigned)((n + 255) / 256);
  cudaStream_t s = ptn_stream(stream);
  PTN_COUNT(2);
  tri_mul_kernel<<<g, 256, 0, s>>>(static_cast<const double2*>(X), static_cast<const double2*>(R0),
                                   static_cast<double2*>(work), k);
  newton_inv_kernel<<<g, 256, 0, s>>>(static_cast<const double2*>(R0), static_cast<const double2*>(work),
                                      static_cast<double2*>(R), k);
  return ptn_launch_status();
}

extern "C" int ptn_znonzero_rows(const void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                                     int64_t* out, void* stream) {
  if (!A || !rowoff || !out || m < 1 || k < 1 || colstride < 1) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
  PTN_COUNT(2);
  init_u64_kernel<<<1, 1, 0, s>>>(o);
  int64_t blocks = (m * k + 255) / 256;
  if (blocks > 1216) blocks = 1216;   // 8 CTAs per SM on 152 SMs
  nonzero_rows_kernel<<<(unsigned)blocks, 256, 0, s>>>(static_cast<const double2*>(A), rowoff, m, k, colstride,
                                                           o);
  return ptn_launch_status();
}
