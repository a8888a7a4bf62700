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

// ---- small-m path (m <= QR_SMALL_M) ---------------------------------------------------
// The reflectors go to a separate V buffer and the diagonal of R to `betas`,
// so no CTA writes what another reads in the same launch.
constexpr int64_t QR_SMALL_M = 2048;
constexpr int ST = 256;
constexpr int QR_MULTI_MAX = 8;                   // reflectors per launch
constexpr int64_t QR_MULTI_SMEM = 200 * 1024;     // dynamic shared memory budget

__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < ST / 32; ++i) s += red[i];
    red[ST / 32] = s;
  }
  __syncthreads();
  s = red[ST / 32];
  __syncthreads();
  return s;
}

__device__ __forceinline__ double2 block_sum2(double2 v, double* red) {
  double re = block_sum(v.x, red);
  double im = block_sum(v.y, red);
  return make_double2(re, im);
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

// ---- several reflectors per launch (m <= QR_SMALL_M) ------------------------------------
// Factorisation: every CTA factorises the ns-column panel j0..j0+ns-1
// redundantly in shared memory (identical arithmetic, so identical reflectors
// everywhere; the trailing panel columns are updated a warp per column), then
// applies the ns reflectors to its own trailing column. CTA 0 writes the panel
// back and stores the reflectors. ns launches' worth of dependent steps cost
// one launch; GB300's per-SM FP64 rate keeps ns small (the panel work is
// repeated on every SM).
__global__ void __launch_bounds__(ST) hh_fact_multi(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                    int64_t cs, int64_t m, int64_t k, int64_t j0, int ns,
                                                    double2* __restrict__ tau, double2* __restrict__ betas,
                                                    double2* __restrict__ V) {
  extern __shared__ double2 P[];  // [ns][len] panel, then [len] own column
  __shared__ double red[ST / 32 + 1];
  __shared__ double2 sc[2];
  __shared__ double2 taus[QR_MULTI_MAX];
  const int64_t len = m - j0;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  double2* col = P + (int64_t)ns * len;
  const int64_t c = j0 + ns + blockIdx.x;
  const bool own = c < k;
  for (int64_t e = threadIdx.x; e < ns * len; e += ST) {
    const int64_t cc = e / len, r = e - cc * len;
    P[e] = A[rowoff[j0 + r] + (j0 + cc) * cs];
  }
  if (own)
    for (int64_t t = threadIdx.x; t < len; t += ST) col[t] = A[rowoff[j0 + t] + c * cs];
  __syncthreads();
  for (int i = 0; i < ns; ++i) {
    double2* x = P + (int64_t)i * len;
    double acc = 0.0;
    for (int64_t t = i + 1 + threadIdx.x; t < len; t += ST) acc += cabs2(x[t]);
    const double xn2 = block_sum(acc, red);
    if (threadIdx.x == 0) {
      const double2 alpha = x[i];
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
      taus[i] = t_;
      if (blockIdx.x == 0) {
        tau[j0 + i] = t_;
        betas[j0 + i] = b_;
      }
    }
    __syncthreads();
    const double2 s_ = sc[1];
    const int64_t j = j0 + i;
    for (int64_t t = i + threadIdx.x; t < len; t += ST) {
      const double2 v = (t == i) ? make_double2(1.0, 0.0) : cmul(x[t], s_);
      x[t] = v;
      if (blockIdx.x == 0) V[j * m + j0 + t] = v;
    }
    __syncthreads();
    double2 f = sc[0];
    f.y = -f.y;  // conj(tau): the factorisation applies H^H
    for (int cc = i + 1 + wp; cc < ns; cc += ST / 32) {
      double2* y = P + (int64_t)cc * len;
      double2 w = make_double2(0.0, 0.0);
      for (int64_t t = i + lane; t < len; t += 32) w = cfmac(x[t], y[t], w);
      w = warp_sum2(w);
      const double2 fw = cmul(f, w);
      for (int64_t t = i + lane; t < len; t += 32) y[t] = csub(y[t], cmul(x[t], fw));
    }
    __syncthreads();
  }
  if (own) {
    for (int i = 0; i < ns; ++i) {
      const double2* v = P + (int64_t)i * len;
      double2 w = make_double2(0.0, 0.0);
      for (int64_t t = i + threadIdx.x; t < len; t += ST) w = cfmac(v[t], col[t], w);
      w = block_sum2(w, red);
      double2 f = taus[i];
      f.y = -f.y;
      const double2 fw = cmul(f, w);
      for (int64_t t = i + threadIdx.x; t < len; t += ST) col[t] = csub(col[t], cmul(v[t], fw));
      __syncthreads();
    }
    for (int64_t t = threadIdx.x; t < len; t += ST) A[rowoff[j0 + t] + c * cs] = col[t];
  }
  if (blockIdx.x == 0)
    for (int64_t e = threadIdx.x; e < ns * len; e += ST) {
      const int64_t cc = e / len, r = e - cc * len;
      A[rowoff[j0 + r] + (j0 + cc) * cs] = P[e];
    }
}

// Q formation for reflectors jlo..jhi-1 (zung2r order, descending) in one
// launch: CTA b owns column c = jlo + b (< p). A column c >= jhi receives
// H_{jhi-1} ... H_{jlo}; a panel column c < jhi is first formed from its own
// reflector (rows above c zero) and then receives H_{c-1} ... H_{jlo}.
__global__ void __launch_bounds__(ST) hh_form_multi(double2* __restrict__ A, const int64_t* __restrict__ rowoff,
                                                    int64_t cs, int64_t m, int64_t jlo, int64_t jhi,
                                                    const double2* __restrict__ tau,
                                                    const double2* __restrict__ V) {
  extern __shared__ double2 col[];  // rows jlo..m-1
  __shared__ double red[ST / 32 + 1];
  const int64_t c = jlo + blockIdx.x;
  const int64_t len = m - jlo;
  int64_t top;
  if (c >= jhi) {
    for (int64_t t = threadIdx.x; t < len; t += ST) col[t] = A[rowoff[jlo + t] + c * cs];
    top = jhi - 1;
  } else {
    const double2 tc = tau[c];
    const double2* vc = V + c * m;
    for (int64_t t = threadIdx.x; t < len; t += ST) {
      const int64_t row = jlo + t;
      double2 val;
      if (row < c) val = make_double2(0.0, 0.0);
      else if (row == c) val = make_double2(1.0 - tc.x, -tc.y);
      else {
        const double2 vi = vc[row];
        val = make_double2(-(tc.x * vi.x - tc.y * vi.y), -(tc.x * vi.y + tc.y * vi.x));
      }
      col[t] = val;
    }
    top = c - 1;
  }
  __syncthreads();
  for (int64_t j = top; j >= jlo; --j) {
    const double2 t_ = tau[j];
    const double2* v = V + j * m;
    double2 w = make_double2(0.0, 0.0);
    for (int64_t row = j + threadIdx.x; row < m; row += ST) w = cfmac(v[row], col[row - jlo], w);
    w = block_sum2(w, red);
    const double2 fw = cmul(t_, w);
    for (int64_t row = j + threadIdx.x; row < m; row += ST) col[row - jlo] = csub(col[row - jlo], cmul(v[row], fw));
    __syncthreads();
  }
  for (int64_t t = threadIdx.x; t < len; t += ST) A[rowoff[jlo + t] + c * cs] = col[t];
  if (c < jhi)
    for (int64_t r = threadIdx.x; r < jlo; r += ST) A[rowoff[r] + c * cs] = make_double2(0.0, 0.0);
}

inline unsigned grid1(int64_t n) {
  int64_t b = (n + QT - 1) / QT;
  if (b < 1) b = 1;
  if (b > 2048) b = 2048;
  return (unsigned)b;
}

}  // namespace

extern "C" int64_t ptn_zqr_work_bytes(int64_t m, int64_t k) {
  if (m <= QR_SMALL_M) {
    const int64_t p = m < k ? m : k;
    return 16 * (2 * k + m * p) + 256;   // tau, betas, V
  }
  return 16 * (3 * k + (nrb_for(m) + 1) / 2 + 1 + nrb_for(m) * k) + 256;
}

static int zqr_keep_small(double2* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, double2* R,
                          void* work, cudaStream_t s) {
  double2* tau = static_cast<double2*>(work);
  double2* betas = tau + k;
  double2* V = betas + k;
  const int64_t p = m < k ? m : k;
  // reflectors per launch: the panel and one column must fit the smem budget
  int64_t ns = QR_MULTI_SMEM / (16 * m) - 1;
  if (ns > QR_MULTI_MAX) ns = QR_MULTI_MAX;
  if (ns < 1) ns = 1;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(hh_fact_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QR_MULTI_SMEM) !=
        cudaSuccess)
      return PTN_ERR_LAUNCH;
    attr_set = true;
  }
  for (int64_t j0 = 0; j0 < p; j0 += ns) {
    const int64_t n_ = p - j0 < ns ? p - j0 : ns;
    const int64_t ncols = k - j0 - n_;
    PTN_COUNT(1);
    hh_fact_multi<<<(unsigned)(ncols > 0 ? ncols : 1), ST, (size_t)(n_ + 1) * (m - j0) * 16, s>>>(
        A, rowoff, cs, m, k, j0, (int)n_, tau, betas, V);
  }
  PTN_COUNT(1);
  extract_r_small<<<grid1(k * k), ST, 0, s>>>(A, rowoff, cs, k, p, betas, R);
  for (int64_t jhi = p; jhi > 0; jhi -= ns) {
    const int64_t jlo = jhi - ns > 0 ? jhi - ns : 0;
    PTN_COUNT(1);
    hh_form_multi<<<(unsigned)(p - jlo), ST, (size_t)(m - jlo) * 16, s>>>(A, rowoff, cs, m, jlo, jhi, tau, V);
  }
  if (p < k) { PTN_COUNT(1); zero_cols_kernel<<<grid1(m * (k - p)), QT, 0, s>>>(A, rowoff, cs, m, k, p); }
  return ptn_launch_status();
}

extern "C" int ptn_zqr_keep(void* Av, const int64_t* rowoff, int64_t m, int64_t k, int64_t cs, void* Rv,
                            void* work, void* stream) {
  if (!Av || !rowoff || !Rv || !work || m < 1 || k < 1 || cs < 1) return PTN_ERR_ARG;
  cudaStream_t s = ptn_stream(stream);
  double2* A = static_cast<double2*>(Av);
  double2* R = static_cast<double2*>(Rv);
  if (m <= QR_SMALL_M) return zqr_keep_small(A, rowoff, m, k, cs, R, work, s);
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
