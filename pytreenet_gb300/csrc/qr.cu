// Householder QR in complex128 with LAPACK's zgeqr2/zung2r conventions.
//
// PyTreeNet splits a site with np.linalg.qr (LAPACK zgeqrf + zungqr) inside
// tensor_qr_decomposition(mode=KEEP) (util/tensor_splitting.py:60-107). On the
// zero-padded, rank-deficient tensors that one-site TDVP starts from, the
// orthonormal complement that Householder QR produces decides the TDVP result,
// so this follows the same published reflector convention (zlarfg: beta real,
// beta = -sign(Re alpha) * ||(alpha, x)||, tau = (beta - alpha) / beta,
// v = x / (alpha - beta); H = I - tau v v^H applied as H^H during the
// factorisation and as H when Q is formed). Exact zeros stay exact zeros, so
// the complement is reproduced exactly.
//
// The matrix is addressed in place inside the site tensor: element (i, c) at
// A[rowoff[i] + c * colstride], where the row-offset table carries the
// reference's (logical) row order. Each Householder step is a short sequence
// of ordinary launches (column norm, reflector, column dots, dot reduction,
// trailing update); no kernel waits on another.
#include "ptn_common.cuh"

namespace {

constexpr int QT = 256;          // threads per CTA
constexpr int RB = 1024;         // rows per row-chunk
constexpr int CB = 8;            // columns per column-chunk (one warp each)

struct QRWork {
  // device layout of the work buffer
  double2* tau;       // [k]
  double2* scal;      // [k]
  double2* w;         // [k]
  double* npart;      // [nrb]
  double2* dpart;     // [nrb * k]
};

inline int64_t nrb_for(int64_t m) { return (m + RB - 1) / RB; }

inline QRWork carve(void* work, int64_t m, int64_t k) {
  QRWork q;
  char* p = static_cast<char*>(work);
  q.tau = reinterpret_cast<double2*>(p);
  p += 16 * k;
  q.scal = reinterpret_cast<double2*>(p);
  p += 16 * k;
  q.w = reinterpret_cast<double2*>(p);
  p += 16 * k;
  q.npart = reinterpret_cast<double*>(p);
  p += 16 * ((nrb_for(m) + 1) / 2 + 1);
  q.dpart = reinterpret_cast<double2*>(p);
  return q;
}

__device__ __forceinline__ double2 ld(const double2* A, const int64_t* rowoff, int64_t cs,
                                      int64_t i, int64_t c) {
  return A[rowoff[i] + c * cs];
}

// partial[b] = sum_{i in chunk b, i > j} |A[i, j]|^2
__global__ void __launch_bounds__(QT) colnorm_kernel(const double2* __restrict__ A,
                                                     const int64_t* __restrict__ rowoff, int64_t cs,
                                                     int64_t m, int64_t j, double* __restrict__ part) {
  const int64_t r0 = (j + 1) + (int64_t)blockIdx.x * RB;
  double acc = 0.0;
  for (int64_t i = r0 + threadIdx.x; i < m && i < r0 + RB; i += QT) acc += cabs2(ld(A, rowoff, cs, i, j));
  __shared__ double red[QT / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < QT / 32; ++i) s += red[i];
    part[blockIdx.x] = s;
  }
}

// One thread: zlarfg on (A[j, j], A[j+1:, j]).
__global__ void reflector_kernel(double2* __restrict__ A, const int64_t* __restrict__ rowoff, int64_t cs,
                                 int64_t j, const double* __restrict__ part, int nparts,
                                 double2* __restrict__ tau, double2* __restrict__ scal) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[b];
  const double xnorm = sqrt(s);
  double2* pa = A + rowoff[j] + j * cs;
  const double2 alpha = *pa;
  if (xnorm == 0.0 && alpha.y == 0.0) {
    tau[j] = make_double2(0.0, 0.0);
    scal[j] = make_double2(0.0, 0.0);
    return;
  }
  double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
  const double beta = (alpha.x >= 0.0) ? -nrm : nrm;
  tau[j] = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
  // scal = 1 / (alpha - beta)
  double2 d = make_double2(alpha.x - beta, alpha.y);
  double den = d.x * d.x + d.y * d.y;
  scal[j] = make_double2(d.x / den, -d.y / den);
  *pa = make_double2(beta, 0.0);
}

// Reflector component v_i (v_j = 1).
__device__ __forceinline__ double2 vcomp(const double2* A, const int64_t* rowoff, int64_t cs, int64_t i,
                                         int64_t j, double2 sc, bool stored) {
  if (i == j) return make_double2(1.0, 0.0);
  double2 a = ld(A, rowoff, cs, i, j);
  return stored ? a : cmul(a, sc);
}

// dpart[rb * k + c] = sum_{i in chunk rb, i >= j} conj(v_i) X[i, c], for c in [c_lo, k)
// grid: (row chunks, column chunks of CB); one warp per column.
// stored != 0: column j already holds v (Q formation); else v = scal * A[:, j].
__global__ void __launch_bounds__(QT) dots_kernel(const double2* __restrict__ A,
                                                  const int64_t* __restrict__ rowoff, int64_t cs,
                                                  int64_t m, int64_t k, int64_t j, int64_t c_lo,
                                                  const double2* __restrict__ scal, int stored,
                                                  double2* __restrict__ dpart) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c = c_lo + (int64_t)blockIdx.y * CB + warp;
  const int64_t r0 = j + (int64_t)blockIdx.x * RB;
  const double2 sc = scal[j];
  __shared__ double2 vs[RB];
  for (int64_t t = threadIdx.x; t < RB; t += QT) {
    int64_t i = r0 + t;
    vs[t] = (i < m) ? vcomp(A, rowoff, cs, i, j, sc, stored != 0) : make_double2(0.0, 0.0);
  }
  __syncthreads();
  if (c >= k) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t t = lane; t < RB; t += 32) {
    int64_t i = r0 + t;
    if (i >= m) break;
    acc = cfmac(vs[t], ld(A, rowoff, cs, i, c), acc);
  }
  acc = warp_sum2(acc);
  if (lane == 0) dpart[(int64_t)blockIdx.x * k + c] = acc;
}

__global__ void dots_finish_kernel(const double2* __restrict__ dpart, int nrb, int64_t k, int64_t c_lo,
                                   double2* __restrict__ w) {
  const int64_t c = c_lo + blockIdx.x;
  double2 s = make_double2(0.0, 0.0);
  for (int b = threadIdx.x; b < nrb; b += 32) s = cadd(s, dpart[(int64_t)b * k + c]);
  s = warp_sum2(s);
  if (threadIdx.x == 0) w[c] = s;
}

// X[i, c] -= f * v_i * w_c for i >= j, c in [c_lo, k); f = conj(tau) (factorisation)
// or tau (Q formation).
__global__ void __launch_bounds__(QT) update_kernel(double2* __restrict__ A,
                                                    const int64_t* __restrict__ rowoff, int64_t cs,
                                                    int64_t m, int64_t k, int64_t j, int64_t c_lo,
                                                    const double2* __restrict__ tau,
                                                    const double2* __restrict__ scal,
                                                    const double2* __restrict__ w, int stored,
                                                    int conj_tau) {
  const int64_t r0 = j + (int64_t)blockIdx.x * RB;
  const int64_t cbase = c_lo + (int64_t)blockIdx.y * CB;
  double2 f = tau[j];
  if (conj_tau) f.y = -f.y;
  const double2 sc = scal[j];
  for (int64_t t = threadIdx.x; t < RB; t += QT) {
    int64_t i = r0 + t;
    if (i >= m) break;
    double2 v = vcomp(A, rowoff, cs, i, j, sc, stored != 0);
    double2 fv = cmul(f, v);
    const int64_t ro = rowoff[i];
    for (int cc = 0; cc < CB; ++cc) {
      int64_t c = cbase + cc;
      if (c >= k) break;
      double2* p = A + ro + c * cs;
      *p = csub(*p, cmul(fv, w[c]));
    }
  }
}

// After the trailing update of step j: A[i, j] <- scal * A[i, j] (the stored v_i), i > j.
__global__ void __launch_bounds__(QT) store_v_kernel(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                     int64_t cs, int64_t m, int64_t j,
                                                     const double2* __restrict__ scal) {
  const double2 sc = scal[j];
  for (int64_t i = j + 1 + blockIdx.x * (int64_t)QT + threadIdx.x; i < m; i += (int64_t)gridDim.x * QT) {
    double2* p = A + rowoff[i] + j * cs;
    *p = cmul(*p, sc);
  }
}

// Copy the upper triangle of rows < p into R (k x k row-major), zero elsewhere.
__global__ void extract_r_kernel(const double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                 int64_t cs, int64_t k, int64_t p, double2* __restrict__ R) {
  for (int64_t e = blockIdx.x * (int64_t)QT + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * QT) {
    int64_t r = e / k, c = e - r * k;
    R[e] = (r < p && c >= r) ? ld(A, rowoff, cs, r, c) : make_double2(0.0, 0.0);
  }
}

// Column j of Q: Q[j, j] = 1 - tau, Q[i > j, j] = -tau v_i, Q[i < j, j] = 0.
__global__ void __launch_bounds__(QT) qcol_kernel(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                  int64_t cs, int64_t m, int64_t j,
                                                  const double2* __restrict__ tau) {
  const double2 t = tau[j];
  for (int64_t i = blockIdx.x * (int64_t)QT + threadIdx.x; i < m; i += (int64_t)gridDim.x * QT) {
    double2* p = A + rowoff[i] + j * cs;
    if (i < j) *p = make_double2(0.0, 0.0);
    else if (i == j) *p = make_double2(1.0 - t.x, -t.y);
    else *p = make_double2(-(t.x * p->x - t.y * p->y), -(t.x * p->y + t.y * p->x));
  }
}

// KEEP padding: zero the columns p..k-1 of Q.
__global__ void zero_cols_kernel(double2* __restrict__ A, const int64_t* __restrict__ rowoff, int64_t cs,
                                 int64_t m, int64_t k, int64_t p) {
  const int64_t nc = k - p;
  for (int64_t e = blockIdx.x * (int64_t)QT + threadIdx.x; e < m * nc; e += (int64_t)gridDim.x * QT) {
    int64_t i = e / nc, c = p + (e - (e / nc) * nc);
    A[rowoff[i] + c * cs] = make_double2(0.0, 0.0);
  }
}

// ---- small-m path: one launch per Householder step ------------------------------------
// For m <= QR_SMALL_M each step is one kernel: every CTA recomputes the
// reflector from column j (a few KB, identical arithmetic in every CTA, so the
// result is the same everywhere) and then owns one trailing column (dot and
// update). The reflectors go to a separate V buffer and the diagonal of R to
// `betas`, so no CTA writes what another reads in the same launch.
constexpr int64_t QR_SMALL_M = 2048;
constexpr int ST = 256;

template <int NTH>
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  if (NTH == 32) return v;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NTH / 32; ++i) s += red[i];
    red[NTH / 32] = s;
  }
  __syncthreads();
  s = red[NTH / 32];
  __syncthreads();
  return s;
}

template <int NTH>
__device__ __forceinline__ double2 block_sum2(double2 v, double* red) {
  double re = block_sum<NTH>(v.x, red);
  double im = block_sum<NTH>(v.y, red);
  return make_double2(re, im);
}

// block_sum2 in one pass: both parts reduced with block_sum's tree (same warp
// shuffles, warp partials added in warp order by thread 0), so the same bits,
// with half the barriers. red2: NTH / 32 + 1 entries.
template <int NTH>
__device__ __forceinline__ double2 block_sum2_fused(double2 v, double2* red2) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red2[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sx = 0.0, sy = 0.0;
    for (int i = 0; i < NTH / 32; ++i) {
      sx += red2[i].x;
      sy += red2[i].y;
    }
    red2[NTH / 32] = make_double2(sx, sy);
  }
  __syncthreads();
  const double2 s = red2[NTH / 32];
  __syncthreads();
  return s;
}

// Step j of the factorisation. grid = max(1, k - j - 1); CTA b owns column j+1+b.
template <int NTH>
__global__ void __launch_bounds__(NTH) hh_fact_small(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                    int64_t cs, int64_t m, int64_t k, int64_t j,
                                                    double2* __restrict__ tau, double2* __restrict__ betas,
                                                    double2* __restrict__ V) {
  __shared__ double2 vs[QR_SMALL_M];
  __shared__ double red[NTH / 32 + 1];
  __shared__ double2 sc[3];  // tau, scal, w
  const int64_t len = m - j;
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < len; t += NTH) {
    const double2 a = A[rowoff[j + t] + j * cs];
    vs[t] = a;
    if (t > 0) acc += cabs2(a);
  }
  const double xn2 = block_sum<NTH>(acc, red);
  if (threadIdx.x == 0) {
    const double2 alpha = vs[0];
    const double xnorm = sqrt(xn2);
    double2 t_, s_, b_;
    if (xnorm == 0.0 && alpha.y == 0.0) {
      t_ = make_double2(0.0, 0.0);
      s_ = make_double2(0.0, 0.0);
      b_ = alpha;
    } else {
      const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
      const double beta = (alpha.x >= 0.0) ? -nrm : nrm;
      t_ = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      const double2 d = make_double2(alpha.x - beta, alpha.y);
      const double den = d.x * d.x + d.y * d.y;
      s_ = make_double2(d.x / den, -d.y / den);
      b_ = make_double2(beta, 0.0);
    }
    sc[0] = t_;
    sc[1] = s_;
    if (blockIdx.x == 0) {
      tau[j] = t_;
      betas[j] = b_;
    }
  }
  __syncthreads();
  const double2 s_ = sc[1];
  for (int64_t t = threadIdx.x; t < len; t += NTH) {
    const double2 v = (t == 0) ? make_double2(1.0, 0.0) : cmul(vs[t], s_);
    vs[t] = v;
    if (blockIdx.x == 0) V[j * m + j + t] = v;
  }
  __syncthreads();
  const int64_t c = j + 1 + blockIdx.x;
  if (c >= k) return;
  double2 w = make_double2(0.0, 0.0);
  for (int64_t t = threadIdx.x; t < len; t += NTH) w = cfmac(vs[t], A[rowoff[j + t] + c * cs], w);
  w = block_sum2<NTH>(w, red);
  double2 f = sc[0];
  f.y = -f.y;  // conj(tau): the factorisation applies H^H
  const double2 fw = cmul(f, w);
  for (int64_t t = threadIdx.x; t < len; t += NTH) {
    double2* p = A + rowoff[j + t] + c * cs;
    *p = csub(*p, cmul(vs[t], fw));
  }
}

// R[r][c]: strictly-upper part from A, diagonal from betas (rows < p), zero elsewhere.
__global__ void extract_r_small(const double2* __restrict__ A, const int64_t* __restrict__ rowoff, int64_t cs,
                                int64_t k, int64_t p, const double2* __restrict__ betas, double2* __restrict__ R) {
  for (int64_t e = blockIdx.x * (int64_t)ST + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * ST) {
    const int64_t r = e / k, c = e - r * k;
    double2 v = make_double2(0.0, 0.0);
    if (r < p) {
      if (c == r) v = betas[r];
      else if (c > r) v = A[rowoff[r] + c * cs];
    }
    R[e] = v;
  }
}

// Step j of forming Q (zung2r): CTAs 0..ncols-1 apply H_j to columns j+1..p-1,
// CTA ncols writes column j itself.
template <int NTH>
__global__ void __launch_bounds__(NTH) hh_form_small(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                    int64_t cs, int64_t m, int64_t p, int64_t j,
                                                    const double2* __restrict__ tau, const double2* __restrict__ V) {
  __shared__ double red[NTH / 32 + 1];
  const int64_t ncols = p - (j + 1);
  const double2 t_ = tau[j];
  const double2* v = V + j * m;
  if (blockIdx.x == ncols) {
    for (int64_t i = threadIdx.x; i < m; i += NTH) {
      double2* q = A + rowoff[i] + j * cs;
      if (i < j) *q = make_double2(0.0, 0.0);
      else if (i == j) *q = make_double2(1.0 - t_.x, -t_.y);
      else *q = make_double2(-(t_.x * v[i].x - t_.y * v[i].y), -(t_.x * v[i].y + t_.y * v[i].x));
    }
    return;
  }
  const int64_t c = j + 1 + blockIdx.x;
  double2 w = make_double2(0.0, 0.0);
  for (int64_t i = j + threadIdx.x; i < m; i += NTH) w = cfmac(v[i], A[rowoff[i] + c * cs], w);
  w = block_sum2<NTH>(w, red);
  const double2 fw = cmul(t_, w);
  for (int64_t i = j + threadIdx.x; i < m; i += NTH) {
    double2* q = A + rowoff[i] + c * cs;
    *q = csub(*q, cmul(v[i], fw));
  }
}

inline unsigned grid1(int64_t n) {
  int64_t b = (n + QT - 1) / QT;
  if (b < 1) b = 1;
  if (b > 2048) b = 2048;
  return (unsigned)b;
}

// ---- small m, one cooperative launch ---------------------------------------------------
// The same Householder steps as hh_fact_small / extract_r_small / hh_form_small,
// with the same arithmetic per column (thread-to-row map, reduction tree,
// scalar formulas), so the results are the same bits; but all of them run in
// one launch. CTA b owns a few columns (snake order, so the Q formation work
// -- column c needs c + 1 reflectors -- is balanced) and keeps them in shared
// memory. Reflector j is computed once, by the owner of column j, as soon as
// column j has received reflectors 0 .. j-1, and published through V, tau and
// a flag; every CTA waits for the flag (bounded), then applies the reflector
// to its own columns. The owner of column j + 1 updates that column first and
// publishes reflector j + 1 right away, so the chain of dependent steps costs
// one flag hand-over each instead of one kernel launch.
constexpr long long HP_WAIT_CYCLES = 4000000000LL;   // ~2 s at 2 GHz

struct HPArgs {
  double2* A;
  const int64_t* rowoff;
  int64_t cs, m, k, p;
  double2* tau;
  double2* betas;
  double2* V;
  double2* R;
  int* ready;     // [p], zero on entry; ready[j] = 1 once reflector j is published
  int* status;    // nonzero: a wait ran out (every CTA stops)
  int G;          // CTAs
  int cpc;        // columns per CTA (upper bound)
};

// i-th column of CTA b (increasing in i)
__device__ __forceinline__ int64_t hp_col(int b, int i, int G) {
  return (int64_t)i * G + ((i & 1) ? (G - 1 - b) : b);
}
__device__ __forceinline__ int hp_owner(int64_t c, int G) {
  const int64_t i = c / G, r = c - i * G;
  return (int)((i & 1) ? (G - 1 - r) : r);
}

__global__ void __launch_bounds__(ST) hh_persistent_kernel(HPArgs a) {
  extern __shared__ double2 hsm[];           // [cpc][m] own columns, then [m] reflector
  __shared__ double red[ST / 32 + 1];
  __shared__ double2 red2[ST / 32 + 1];
  __shared__ double2 sc[2];
  __shared__ int abort_s;
  const int b = blockIdx.x, tid = threadIdx.x, G = a.G;
  const int64_t m = a.m, k = a.k, p = a.p, cs = a.cs;
  double2* vs = hsm + (int64_t)a.cpc * m;
  int nown = 0;
  while (nown < a.cpc && hp_col(b, nown, G) < k) ++nown;
  for (int i = 0; i < nown; ++i) {
    const int64_t c = hp_col(b, i, G);
    for (int64_t t = tid; t < m; t += ST) hsm[i * m + t] = a.A[a.rowoff[t] + c * cs];
  }
  if (tid == 0) abort_s = 0;
  __syncthreads();

  // zlarfg on column j (own slot col) and publication of v_j, tau_j, beta_j
  auto publish = [&](int64_t j, const double2* col) {
    const int64_t len = m - j;
    double acc = 0.0;
    for (int64_t t = tid; t < len; t += ST)
      if (t > 0) acc += cabs2(col[j + t]);
    const double xn2 = block_sum<ST>(acc, red);
    if (tid == 0) {
      const double2 alpha = col[j];
      const double xnorm = sqrt(xn2);
      double2 t_, s_, b_;
      if (xnorm == 0.0 && alpha.y == 0.0) {
        t_ = make_double2(0.0, 0.0);
        s_ = make_double2(0.0, 0.0);
        b_ = alpha;
      } else {
        const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
        const double beta = (alpha.x >= 0.0) ? -nrm : nrm;
        t_ = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
        const double2 d = make_double2(alpha.x - beta, alpha.y);
        const double den = d.x * d.x + d.y * d.y;
        s_ = make_double2(d.x / den, -d.y / den);
        b_ = make_double2(beta, 0.0);
      }
      sc[1] = s_;
      a.tau[j] = t_;
      a.betas[j] = b_;
    }
    __syncthreads();
    const double2 s_ = sc[1];
    for (int64_t t = tid; t < len; t += ST)
      a.V[j * m + j + t] = (t == 0) ? make_double2(1.0, 0.0) : cmul(col[j + t], s_);
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicExch(a.ready + j, 1);
  };

  if (p > 0 && hp_owner(0, G) == b) publish(0, hsm);      // column 0 is this CTA's slot 0
  for (int64_t j = 0; j < p; ++j) {
    if (tid == 0) {
      const volatile int* flag = a.ready + j;
      const volatile int* st = a.status;
      const long long t0 = clock64();
      for (unsigned it = 0;; ++it) {
        if (*flag != 0) break;
        if ((it & 255u) == 0u && *st != 0) { abort_s = 1; break; }
        if (clock64() - t0 > HP_WAIT_CYCLES) {
          atomicExch(a.status, PTN_ERR_TIMEOUT);
          abort_s = 1;
          break;
        }
      }
      __threadfence();
    }
    __syncthreads();
    if (abort_s) break;
    const int64_t len = m - j;
    // v_j and tau_j in one round trip to L2
    if (tid == 0) sc[0] = __ldcg(a.tau + j);
    for (int64_t t = tid; t < len; t += ST) vs[t] = __ldcg(a.V + j * m + j + t);
    __syncthreads();
    double2 f = sc[0];
    f.y = -f.y;  // conj(tau): the factorisation applies H^H
    for (int i = 0; i < nown; ++i) {
      const int64_t c = hp_col(b, i, G);
      if (c <= j) continue;
      double2* col = hsm + i * m;
      double2 w = make_double2(0.0, 0.0);
      for (int64_t t = tid; t < len; t += ST) w = cfmac(vs[t], col[j + t], w);
      w = block_sum2_fused<ST>(w, red2);
      const double2 fw = cmul(f, w);
      for (int64_t t = tid; t < len; t += ST) col[j + t] = csub(col[j + t], cmul(vs[t], fw));
      __syncthreads();
      if (c == j + 1 && j + 1 < p) publish(j + 1, col);
    }
    __syncthreads();
  }
  if (abort_s) {
    if (b == 0 && tid == 0) a.R[0] = make_double2(NAN, NAN);   // the result is not usable
    return;
  }
  // R (rows < p: beta on the diagonal, the stored upper part above it), then Q
  // (zung2r: column c = H_0 ... H_c e_c), KEEP padding past p
  for (int i = 0; i < nown; ++i) {
    const int64_t c = hp_col(b, i, G);
    double2* col = hsm + i * m;
    for (int64_t r = tid; r < k; r += ST) {
      double2 v = make_double2(0.0, 0.0);
      if (r < p) {
        if (c == r) v = a.betas[r];
        else if (c > r) v = col[r];
      }
      a.R[r * k + c] = v;
    }
    __syncthreads();
    if (c >= p) {
      for (int64_t t = tid; t < m; t += ST) a.A[a.rowoff[t] + c * cs] = make_double2(0.0, 0.0);
      continue;
    }
    // reflectors come from other CTAs: read them through L2
    const double2 tc = __ldcg(a.tau + c);
    const double2* vc = a.V + c * m;
    for (int64_t t = tid; t < m; t += ST) {
      if (t < c) {
        col[t] = make_double2(0.0, 0.0);
      } else if (t == c) {
        col[t] = make_double2(1.0 - tc.x, -tc.y);
      } else {
        const double2 vt = __ldcg(vc + t);
        col[t] = make_double2(-(tc.x * vt.x - tc.y * vt.y), -(tc.x * vt.y + tc.y * vt.x));
      }
    }
    __syncthreads();
    // H_{c-1}, ..., H_0 in turn; each step stages its reflector in shared
    // memory, and the next one is fetched while this one is applied
    constexpr int PF = QR_SMALL_M / ST;                // rows per thread
    double2 pre[PF];
    double2 tpre = make_double2(0.0, 0.0);
    if (c > 0) {
      const double2* v = a.V + (c - 1) * m;
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int64_t t = (c - 1) + tid + (int64_t)q * ST;
        pre[q] = t < m ? __ldcg(v + t) : make_double2(0.0, 0.0);
      }
      tpre = __ldcg(a.tau + (c - 1));
    }
    for (int64_t j = c - 1; j >= 0; --j) {
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int64_t t = j + tid + (int64_t)q * ST;
        if (t < m) vs[t] = pre[q];
      }
      const double2 t_ = tpre;
      if (j > 0) {
        const double2* vn = a.V + (j - 1) * m;
#pragma unroll
        for (int q = 0; q < PF; ++q) {
          const int64_t t = (j - 1) + tid + (int64_t)q * ST;
          pre[q] = t < m ? __ldcg(vn + t) : make_double2(0.0, 0.0);
        }
        tpre = __ldcg(a.tau + (j - 1));
      }
      double2 w = make_double2(0.0, 0.0);
      for (int64_t t = j + tid; t < m; t += ST) w = cfmac(vs[t], col[t], w);
      w = block_sum2_fused<ST>(w, red2);
      const double2 fw = cmul(t_, w);
      for (int64_t t = j + tid; t < m; t += ST) col[t] = csub(col[t], cmul(vs[t], fw));
      __syncthreads();
    }
    for (int64_t t = tid; t < m; t += ST) a.A[a.rowoff[t] + c * cs] = col[t];
  }
}

}  // namespace

extern "C" int64_t ptn_zqr_work_bytes(int64_t m, int64_t k) {
  if (m <= QR_SMALL_M) {
    const int64_t p = m < k ? m : k;
    return 16 * (2 * k + m * p) + 4 * (p + 1) + 512;   // tau, betas, V, flags, status
  }
  return 16 * (3 * k + (nrb_for(m) + 1) / 2 + 1 + nrb_for(m) * k) + 256;
}

// Launch shape of the one-launch path for an m x k problem (m <= QR_SMALL_M):
// CTAs, columns per CTA and dynamic shared memory; false when it does not fit
// (columns too many for shared memory, or more CTAs than can be co-resident).
static bool hp_shape(int64_t m, int64_t k, int& G, int& cpc, size_t& smem) {
  // device properties and the kernel's shared-memory limit: once per process
  // (thread-safe static initialisation; the engine drives one device)
  struct Dev {
    int n_sm = 0;
    size_t dyn_max = 0;
  };
  static const Dev dv = []() {
    Dev d;
    int dev = 0;
    cudaDeviceProp pr;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&pr, dev) != cudaSuccess ||
        !pr.cooperativeLaunch)
      return d;
    const size_t dyn = pr.sharedMemPerBlockOptin - 1024;    // room for the static shared memory
    if (cudaFuncSetAttribute(hh_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) !=
        cudaSuccess)
      return d;
    d.n_sm = pr.multiProcessorCount;
    d.dyn_max = dyn;
    return d;
  }();
  if (dv.n_sm <= 0 || m < 1 || k < 1 || m > QR_SMALL_M) return false;
  int64_t g = (k + 1) / 2;                           // two columns per CTA
  if (g > dv.n_sm) g = dv.n_sm;
  const int64_t c = (k + g - 1) / g;
  const size_t bytes = (size_t)(c + 1) * (size_t)m * sizeof(double2);
  if (bytes > dv.dyn_max) return false;
  int max_per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_per_sm, hh_persistent_kernel, ST, bytes) != cudaSuccess ||
      (int64_t)max_per_sm * dv.n_sm < g)
    return false;
  G = (int)g;
  cpc = (int)c;
  smem = bytes;
  return true;
}

extern "C" int ptn_zqr_path(int64_t m, int64_t k) {
  int G, cpc;
  size_t smem;
  if (m <= QR_SMALL_M && hp_shape(m, k, G, cpc, smem)) return 1;
  return 0;
}

static int zqr_keep_persistent(double2* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, double2* R,
                               void* work, cudaStream_t s) {
  int G, cpc;
  size_t smem;
  if (!hp_shape(m, k, G, cpc, smem)) return PTN_ERR_UNSUPPORTED;
  const int64_t p = m < k ? m : k;
  HPArgs a;
  a.A = A;
  a.rowoff = rowoff;
  a.cs = cs;
  a.m = m;
  a.k = k;
  a.p = p;
  a.tau = static_cast<double2*>(work);
  a.betas = a.tau + k;
  a.V = a.betas + k;
  a.ready = reinterpret_cast<int*>(a.V + m * p);
  a.status = a.ready + p;
  a.R = R;
  a.G = G;
  a.cpc = cpc;
  if (cudaMemsetAsync(a.ready, 0, sizeof(int) * (size_t)(p + 1), s) != cudaSuccess) return PTN_ERR_LAUNCH;
  void* args[] = {&a};
  PTN_COUNT(1);
  if (cudaLaunchCooperativeKernel((const void*)hh_persistent_kernel, dim3((unsigned)G), dim3(ST), args, smem, s) !=
      cudaSuccess)
    return PTN_ERR_LAUNCH;
  return ptn_launch_status();
}

static int zqr_keep_small(double2* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, double2* R,
                          void* work, cudaStream_t s) {
  double2* tau = static_cast<double2*>(work);
  double2* betas = tau + k;
  double2* V = betas + k;
  const int64_t p = m < k ? m : k;
  // (one warp per column measured slower than 256 threads at 512 x 256: 6.8 vs 4.2 ms)
  for (int64_t j = 0; j < p; ++j) {
    const int64_t ncols = k - (j + 1);
    PTN_COUNT(1);
    hh_fact_small<ST><<<(unsigned)(ncols > 0 ? ncols : 1), ST, 0, s>>>(A, rowoff, cs, m, k, j, tau, betas, V);
  }
  PTN_COUNT(1);
  extract_r_small<<<grid1(k * k), ST, 0, s>>>(A, rowoff, cs, k, p, betas, R);
  for (int64_t j = p - 1; j >= 0; --j) {
    PTN_COUNT(1);
    hh_form_small<ST><<<(unsigned)(p - j), ST, 0, s>>>(A, rowoff, cs, m, p, j, tau, V);
  }
  if (p < k) { PTN_COUNT(1); zero_cols_kernel<<<grid1(m * (k - p)), QT, 0, s>>>(A, rowoff, cs, m, k, p); }
  return ptn_launch_status();
}

// Q[j, j] = 1 for j in [lo, hi): the columns that Householder steps with an
// exactly-zero remaining column (tau = 0) leave as unit vectors.
__global__ void unit_diag_kernel(double2* __restrict__ A, const int64_t* __restrict__ rowoff, int64_t cs,
                                 int64_t lo, int64_t hi) {
  const int64_t j = lo + blockIdx.x * (int64_t)QT + threadIdx.x;
  if (j < hi) A[rowoff[j] + j * cs] = make_double2(1.0, -0.0);
}

static int zqr_keep_impl(double2* A, const int64_t* rowoff, int64_t m_path, int64_t m, int64_t k, int64_t cs,
                         double2* R, void* work, cudaStream_t s);

extern "C" int ptn_zqr_keep(void* Av, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, void* Rv,
                            void* work, void* stream) {
  if (!Av || !rowoff || !Rv || !work || m < 1 || k < 1 || cs < 1) return PTN_ERR_ARG;
  return zqr_keep_impl(static_cast<double2*>(Av), rowoff, m, m, k, cs, static_cast<double2*>(Rv), work,
                       ptn_stream(stream));
}

extern "C" int ptn_zqr_keep_steps(void* Av, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, void* Rv,
                                  void* work, void* stream) {
  if (!Av || !rowoff || !Rv || !work || m < 1 || k < 1 || cs < 1) return PTN_ERR_ARG;
  if (m > QR_SMALL_M)
    return zqr_keep_impl(static_cast<double2*>(Av), rowoff, m, m, k, cs, static_cast<double2*>(Rv), work,
                         ptn_stream(stream));
  return zqr_keep_small(static_cast<double2*>(Av), rowoff, m, k, cs, static_cast<double2*>(Rv), work,
                        ptn_stream(stream));
}

extern "C" int ptn_zqr_keep_rows(void* Av, const int64_t* rowoff, int64_t m, int64_t m_used, int64_t k, int64_t cs,
                                 void* Rv, void* work, void* stream) {
  if (!Av || !rowoff || !Rv || !work || m < 1 || k < 1 || cs < 1 || m_used < 1 || m_used > m) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  double2* A = static_cast<double2*>(Av);
  int st = zqr_keep_impl(A, rowoff, m, m_used, k, cs, static_cast<double2*>(Rv), work, s);
  if (st != PTN_OK) return st;
  // Rows m_used.. are zero, so every step j >= m_used of the full factorisation
  // meets a zero column (tau = 0, beta = 0): R keeps zero rows there and Q the
  // unit vector e_j in column j (up to min(m, k)); columns past min(m, k) stay
  // zero (KEEP padding), as the call on m_used rows already left them.
  const int64_t hi = m < k ? m : k;
  if (m_used < hi) {
    PTN_COUNT(1);
    unit_diag_kernel<<<(unsigned)((hi - m_used + QT - 1) / QT), QT, 0, s>>>(A, rowoff, cs, m_used, hi);
  }
  return ptn_launch_status();
}

// Householder QR of the first m rows, with the kernel sequence (and so the
// rounding) of an m_path-row problem.
static int zqr_keep_impl(double2* A, const int64_t* rowoff, int64_t m_path, int64_t m, int64_t k, int64_t cs,
                         double2* R, void* work, cudaStream_t s) {
  if (m_path <= QR_SMALL_M) {
    const int st = zqr_keep_persistent(A, rowoff, m, k, cs, R, work, s);
    if (st != PTN_ERR_UNSUPPORTED) return st;
    return zqr_keep_small(A, rowoff, m, k, cs, R, work, s);
  }
  QRWork q = carve(work, m, k);
  const int64_t p = m < k ? m : k;
  // factorisation
  for (int64_t j = 0; j < p; ++j) {
    const int64_t below = m - (j + 1);
    const int nb_norm = below > 0 ? (int)((below + RB - 1) / RB) : 0;
    if (nb_norm > 0) { PTN_COUNT(1); colnorm_kernel<<<nb_norm, QT, 0, s>>>(A, rowoff, cs, m, j, q.npart); }
    PTN_COUNT(1);
    reflector_kernel<<<1, 32, 0, s>>>(A, rowoff, cs, j, q.npart, nb_norm, q.tau, q.scal);
    const int64_t ncols = k - (j + 1);
    if (ncols > 0) {
      const int nrb = (int)((m - j + RB - 1) / RB);
      dim3 g(nrb, (unsigned)((ncols + CB - 1) / CB));
      PTN_COUNT(1);
      dots_kernel<<<g, QT, 0, s>>>(A, rowoff, cs, m, k, j, j + 1, q.scal, 0, q.dpart);
      PTN_COUNT(1);
      dots_finish_kernel<<<(unsigned)ncols, 32, 0, s>>>(q.dpart, nrb, k, j + 1, q.w);
      PTN_COUNT(1);
      update_kernel<<<g, QT, 0, s>>>(A, rowoff, cs, m, k, j, j + 1, q.tau, q.scal, q.w, 0, 1);
    }
    if (below > 0) { PTN_COUNT(1); store_v_kernel<<<grid1(below), QT, 0, s>>>(A, rowoff, cs, m, j, q.scal); }
  }
  PTN_COUNT(1);
  extract_r_kernel<<<grid1(k * k), QT, 0, s>>>(A, rowoff, cs, k, p, R);
  // Q formation (zung2r): columns p-1 .. 0
  for (int64_t j = p - 1; j >= 0; --j) {
    const int64_t ncols = p - (j + 1);
    if (ncols > 0) {
      const int nrb = (int)((m - j + RB - 1) / RB);
      dim3 g(nrb, (unsigned)((ncols + CB - 1) / CB));
      PTN_COUNT(1);
      dots_kernel<<<g, QT, 0, s>>>(A, rowoff, cs, m, p, j, j + 1, q.scal, 1, q.dpart);
      PTN_COUNT(1);
      dots_finish_kernel<<<(unsigned)ncols, 32, 0, s>>>(q.dpart, nrb, p, j + 1, q.w);
      PTN_COUNT(1);
      update_kernel<<<g, QT, 0, s>>>(A, rowoff, cs, m, p, j, j + 1, q.tau, q.scal, q.w, 1, 0);
    }
    PTN_COUNT(1);
    qcol_kernel<<<grid1(m), QT, 0, s>>>(A, rowoff, cs, m, j, q.tau);
  }
  if (p < k) { PTN_COUNT(1); zero_cols_kernel<<<grid1(m * (k - p)), QT, 0, s>>>(A, rowoff, cs, m, k, p); }
  return ptn_launch_status();
}

// ---- QR with a library-owned scratch area --------------------------------------------
// Some callers cannot allocate device memory at the moment they need a QR: a
// host framework that binds this library through a plain C FFI and owns no
// CUDA allocator, or code that must not allocate while a stream is being
// captured into a graph. ptn_zqr_keep_noalloc runs the same Householder
// kernels as ptn_zqr_keep but takes its scratch from a fixed array compiled
// into the library (every GPU that loads the library keeps these 4 MiB until
// the process exits).
#include <mutex>

#define PTN_QR_STATIC_SCRATCH_BYTES (4ll << 20)
static __device__ __align__(256) unsigned char g_qr_static_scratch[PTN_QR_STATIC_SCRATCH_BYTES];

namespace {
std::mutex g_qr_static_mu;
void* g_qr_static_ptr[256] = {};  // device address of the array, per device ordinal
}  // namespace

extern "C" int64_t ptn_zqr_noalloc_max_bytes(void) { return PTN_QR_STATIC_SCRATCH_BYTES; }

extern "C" int ptn_zqr_keep_noalloc(void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                                    void* R, void* stream) {
  if (!A || !rowoff || !R || m < 1 || k < 1 || colstride < 1) return PTN_ERR_ARG;
  if (ptn_zqr_work_bytes(m, k) > PTN_QR_STATIC_SCRATCH_BYTES) return PTN_ERR_UNSUPPORTED;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return PTN_ERR_LAUNCH;
  void* work = nullptr;
  {
    std::lock_guard<std::mutex> guard(g_qr_static_mu);
    if (!g_qr_static_ptr[dev]) {
      // Host code cannot pass the array's name to a kernel: it is a host-side
      // stand-in. Resolve its device address once, with this device current.
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_qr_static_scratch) != cudaSuccess || !p) return PTN_ERR_LAUNCH;
      g_qr_static_ptr[dev] = p;
    }
    work = g_qr_static_ptr[dev];
  }
  // Every scratch entry the kernels read is written earlier in the same call
  // (column-norm partials, reflector scalars, dot partials), so nothing needs
  // clearing between calls.
  return ptn_zqr_keep(A, rowoff, m, k, colstride, R, work, stream);
}
