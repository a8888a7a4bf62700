// Singular value decomposition (complex128, FP64) by one-sided Jacobi
// (Hestenes), and a strided permute/conjugate/scale copy.
//
// ptn_zsvd_jacobi factors an m x n matrix (m >= n) as A = U diag(S) V^H with S
// sorted in descending order. One-sided Jacobi orthogonalises the columns of a
// working copy of A by plane rotations applied from the right; V accumulates
// the rotations. A sweep visits every column pair once in the round-robin
// (circle) order: n_even - 1 rounds of n_even / 2 disjoint pairs, one warp per
// pair. Rounds are separated by a grid-wide barrier; the kernel is launched
// cooperatively so all CTAs are resident. A pair (a, b) is rotated when
// |a^H b| > tol * |a| |b| (tol = 8 sqrt(m) * 2^-53); the
// iteration stops after the first sweep without a rotation. Every barrier wait
// is bounded: on timeout the kernel records PTN_ERR_TIMEOUT in *status and all
// CTAs leave. A sweep limit that is reached records PTN_ERR_NOCONVERGE (the
// outputs are still written).
//
// The reference computes this step with np.linalg.svd (LAPACK gesdd) inside
// tensor_svd / truncated_tensor_svd (util/tensor_splitting.py:122-177, 488-527).
#include <mutex>

#include "ptn_common.cuh"
#include "coop.cuh"

namespace {

constexpr int SVD_WARPS = 4;
constexpr int SVD_THREADS = SVD_WARPS * 32;
constexpr int SVD_MAX_SWEEPS = 56;
constexpr long long SVD_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
constexpr int CTRL_WORDS = 64;                       // barrier words + per-sweep rotation counts
constexpr int64_t CTRL_BYTES = 256;

struct SvdArgs {
  const double2* src;
  int64_t rs, cs;
  int64_t m, n;
  double2* Aw;   // m x n column-major working copy
  double2* Vw;   // n x n column-major accumulated rotations
  double* sig;   // n column norms
  unsigned* ctrl;
  double2* U;
  int64_t ldu;
  double* S;
  double2* V;
  int64_t ldv;
  double tol;
  int32_t* status;
};

__device__ __forceinline__ double2 ldcg2(const double2* p) { return __ldcg(p); }
__device__ __forceinline__ void stcg2(double2* p, double2 v) { __stcg(p, v); }

// Grid-wide barrier (coop.cuh); a timeout is also recorded in *status.
__device__ bool grid_barrier(unsigned* ctrl, int32_t* status) {
  const bool ok = ptn_grid_barrier(ctrl, SVD_WAIT_CYCLES);
  if (!ok && threadIdx.x == 0 && *((volatile unsigned*)(ctrl + 2)) != 0u) atomicCAS(status, 0, PTN_ERR_TIMEOUT);
  return ok;
}

// Rotate columns i and j of Aw (and of Vw) so that they become orthogonal.
// Columns whose squared norm is at most `zero2` (numerically zero: norm below
// tol times the largest input column norm) are left alone; their directions
// are rounding noise, and rotating such pairs can cycle without converging.
// Returns true when a rotation was applied.
__device__ bool rotate_pair(const SvdArgs& a, int64_t i, int64_t j, int lane, double zero2) {
  double2* ci = a.Aw + i * a.m;
  double2* cj = a.Aw + j * a.m;
  double al = 0.0, be = 0.0;
  double2 ga = make_double2(0.0, 0.0);
  for (int64_t k = lane; k < a.m; k += 32) {
    const double2 x = ldcg2(ci + k), y = ldcg2(cj + k);
    al += cabs2(x);
    be += cabs2(y);
    ga = cfmac(x, y, ga);  // conj(x) * y
  }
  al = warp_sum(al);
  be = warp_sum(be);
  ga = warp_sum2(ga);
  if (al <= zero2 || be <= zero2) return false;
  const double g = hypot(ga.x, ga.y);
  if (!(g > a.tol * sqrt(al) * sqrt(be))) return false;
  // Real rotation on (a, e^{-i phi} b), e^{i phi} = ga / |ga|, angle from
  // cot(2 theta) = (|b|^2 - |a|^2) / (2 |a^H b|), smaller root for t = tan(theta).
  const double zeta = (be - al) / (2.0 * g);
  double t;
  if (fabs(zeta) > 1e150) {
    t = 0.5 / zeta;
  } else {
    t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  }
  const double c = 1.0 / sqrt(1.0 + t * t);
  const double s = c * t;
  const double2 e = make_double2(ga.x / g, ga.y / g);
  const double2 s_em = make_double2(s * e.x, -s * e.y);  // s e^{-i phi}
  const double2 s_ep = make_double2(s * e.x, s * e.y);   // s e^{+i phi}
  for (int64_t k = lane; k < a.m; k += 32) {
    const double2 x = ldcg2(ci + k), y = ldcg2(cj + k);
    stcg2(ci + k, csub(cscale(x, c), cmul(s_em, y)));
    stcg2(cj + k, cadd(cmul(s_ep, x), cscale(y, c)));
  }
  double2* vi = a.Vw + i * a.n;
  double2* vj = a.Vw + j * a.n;
  for (int64_t k = lane; k < a.n; k += 32) {
    const double2 x = ldcg2(vi + k), y = ldcg2(vj + k);
    stcg2(vi + k, csub(cscale(x, c), cmul(s_em, y)));
    stcg2(vj + k, cadd(cmul(s_ep, x), cscale(y, c)));
  }
  return true;
}

__global__ void __launch_bounds__(SVD_THREADS) zsvd_jacobi_kernel(SvdArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * SVD_WARPS + (threadIdx.x >> 5);
  const int64_t nw = (int64_t)gridDim.x * SVD_WARPS;
  const int64_t gt = (int64_t)blockIdx.x * SVD_THREADS + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * SVD_THREADS;
  const int64_t m = a.m, n = a.n;
  for (int64_t e = gt; e < m * n; e += nt) {
    const int64_t i = e % m, j = e / m;
    stcg2(a.Aw + e, a.src[i * a.rs + j * a.cs]);
  }
  for (int64_t e = gt; e < n * n; e += nt) {
    const int64_t i = e % n, j = e / n;
    stcg2(a.Vw + e, make_double2(i == j ? 1.0 : 0.0, 0.0));
  }
  if (!grid_barrier(a.ctrl, a.status)) return;
  // largest squared column norm (non-negative doubles order like their bit patterns)
  unsigned long long* amax_bits = reinterpret_cast<unsigned long long*>(a.ctrl + 4);
  for (int64_t j = gw; j < n; j += nw) {
    double s2 = 0.0;
    for (int64_t k = lane; k < m; k += 32) s2 += cabs2(ldcg2(a.Aw + j * m + k));
    s2 = warp_sum(s2);
    if (lane == 0) atomicMax(amax_bits, (unsigned long long)__double_as_longlong(s2));
  }
  if (!grid_barrier(a.ctrl, a.status)) return;
  const double amax2 = __longlong_as_double((long long)*((volatile unsigned long long*)amax_bits));
  const double zero2 = a.tol * a.tol * amax2;

  const int64_t np = (n + 1) & ~int64_t(1);
  int sweep = 0;
  bool converged = (n < 2);
  for (; sweep < SVD_MAX_SWEEPS && !converged; ++sweep) {
    for (int64_t r = 0; r + 1 < np; ++r) {
      for (int64_t p = gw; p < np / 2; p += nw) {
        const int64_t x = p, y = np - 1 - p;
        const int64_t i = (x == 0) ? 0 : 1 + (x - 1 + r) % (np - 1);
        const int64_t j = 1 + (y - 1 + r) % (np - 1);
        if (i >= n || j >= n) continue;
        const bool rot = rotate_pair(a, i < j ? i : j, i < j ? j : i, lane, zero2);
        if (rot && lane == 0) atomicAdd(a.ctrl + 8 + (sweep % (CTRL_WORDS - 8)), 1u);
      }
      if (!grid_barrier(a.ctrl, a.status)) return;
    }
    const unsigned cnt = *((volatile unsigned*)(a.ctrl + 8 + (sweep % (CTRL_WORDS - 8))));
    converged = (cnt == 0u);
  }
  if (!converged && blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(a.status, 0, PTN_ERR_NOCONVERGE);

  for (int64_t j = gw; j < n; j += nw) {
    double s2 = 0.0;
    for (int64_t k = lane; k < m; k += 32) s2 += cabs2(ldcg2(a.Aw + j * m + k));
    s2 = warp_sum(s2);
    if (lane == 0) __stcg(a.sig + j, sqrt(s2));
  }
  if (!grid_barrier(a.ctrl, a.status)) return;

  // Sort by rank: position of column j = #{i : sig_i > sig_j or (sig_i == sig_j and i < j)}.
  for (int64_t j = gw; j < n; j += nw) {
    const double sj = __ldcg(a.sig + j);
    int64_t cnt = 0;
    for (int64_t i = lane; i < n; i += 32) {
      const double si = __ldcg(a.sig + i);
      cnt += (si > sj || (si == sj && i < j)) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
    for (int64_t k = lane; k < m; k += 32) a.U[cnt * a.ldu + k] = cscale(ldcg2(a.Aw + j * m + k), inv);
    for (int64_t k = lane; k < n; k += 32) a.V[cnt * a.ldv + k] = ldcg2(a.Vw + j * n + k);
    if (lane == 0) a.S[cnt] = sj;
  }
}

// ---- small matrices: one CTA, everything in shared memory --------------------------------
// For n <= SVD_SMALL_N columns whose working copy and rotations fit in shared
// memory (SVD_SMALL_BYTES) the same sweeps run in one CTA with CTA barriers
// between rounds (no cooperative launch, no global traffic). Same pair
// schedule, rotation formula, thresholds and ordering as the kernel above, one
// warp per pair (the pairs of a round are disjoint, so how they are spread over
// the warps does not matter), so the results are the same bit for bit.
constexpr int64_t SVD_SMALL_N = 64;
constexpr int64_t SVD_SMALL_BYTES = 200 * 1024;
constexpr int SVD_SMALL_THREADS = 1024;

__device__ bool rotate_pair_smem(double2* A, double2* V, int64_t m, int64_t n, int64_t i, int64_t j, double tol,
                                 double zero2, int lane) {
  double2* ci = A + i * m;
  double2* cj = A + j * m;
  double al = 0.0, be = 0.0;
  double2 ga = make_double2(0.0, 0.0);
  for (int64_t k = lane; k < m; k += 32) {
    const double2 x = ci[k], y = cj[k];
    al += cabs2(x);
    be += cabs2(y);
    ga = cfmac(x, y, ga);
  }
  al = warp_sum(al);
  be = warp_sum(be);
  ga = warp_sum2(ga);
  if (al <= zero2 || be <= zero2) return false;
  const double g = hypot(ga.x, ga.y);
  if (!(g > tol * sqrt(al) * sqrt(be))) return false;
  const double zeta = (be - al) / (2.0 * g);
  double t;
  if (fabs(zeta) > 1e150) {
    t = 0.5 / zeta;
  } else {
    t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  }
  const double c = 1.0 / sqrt(1.0 + t * t);
  const double s = c * t;
  const double2 e = make_double2(ga.x / g, ga.y / g);
  const double2 s_em = make_double2(s * e.x, -s * e.y);
  const double2 s_ep = make_double2(s * e.x, s * e.y);
  for (int64_t k = lane; k < m; k += 32) {
    const double2 x = ci[k], y = cj[k];
    ci[k] = csub(cscale(x, c), cmul(s_em, y));
    cj[k] = cadd(cmul(s_ep, x), cscale(y, c));
  }
  double2* vi = V + i * n;
  double2* vj = V + j * n;
  for (int64_t k = lane; k < n; k += 32) {
    const double2 x = vi[k], y = vj[k];
    vi[k] = csub(cscale(x, c), cmul(s_em, y));
    vj[k] = cadd(cmul(s_ep, x), cscale(y, c));
  }
  return true;
}

__global__ void __launch_bounds__(SVD_SMALL_THREADS) zsvd_jacobi_small_kernel(SvdArgs a) {
  extern __shared__ double2 sm[];
  __shared__ double sig[SVD_SMALL_N];
  __shared__ unsigned rot;
  __shared__ double amax2s;
  const int64_t m = a.m, n = a.n;
  double2* A = sm;
  double2* V = sm + m * n;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  constexpr int NW = SVD_SMALL_THREADS / 32;
  for (int64_t e = threadIdx.x; e < m * n; e += SVD_SMALL_THREADS) {
    const int64_t i = e % m, j = e / m;
    A[e] = a.src[i * a.rs + j * a.cs];
  }
  for (int64_t e = threadIdx.x; e < n * n; e += SVD_SMALL_THREADS) {
    const int64_t i = e % n, j = e / n;
    V[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int64_t j = wp; j < n; j += NW) {
    double s2 = 0.0;
    for (int64_t k = lane; k < m; k += 32) s2 += cabs2(A[j * m + k]);
    s2 = warp_sum(s2);
    if (lane == 0) sig[j] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int64_t j = 0; j < n; ++j) mx = sig[j] > mx ? sig[j] : mx;
    amax2s = mx;
  }
  __syncthreads();
  const double zero2 = a.tol * a.tol * amax2s;
  const int64_t np = (n + 1) & ~int64_t(1);
  bool converged = (n < 2);
  int sweep = 0;
  for (; sweep < SVD_MAX_SWEEPS && !converged; ++sweep) {
    if (threadIdx.x == 0) rot = 0u;
    __syncthreads();
    for (int64_t r = 0; r + 1 < np; ++r) {
      for (int64_t p = wp; p < np / 2; p += NW) {
        const int64_t x = p, y = np - 1 - p;
        const int64_t i = (x == 0) ? 0 : 1 + (x - 1 + r) % (np - 1);
        const int64_t j = 1 + (y - 1 + r) % (np - 1);
        if (i >= n || j >= n) continue;
        const bool did = rotate_pair_smem(A, V, m, n, i < j ? i : j, i < j ? j : i, a.tol, zero2, lane);
        if (did && lane == 0) atomicAdd(&rot, 1u);
      }
      __syncthreads();
    }
    converged = (rot == 0u);
    __syncthreads();
  }
  if (!converged && threadIdx.x == 0) atomicCAS(a.status, 0, PTN_ERR_NOCONVERGE);
  for (int64_t j = wp; j < n; j += NW) {
    double s2 = 0.0;
    for (int64_t k = lane; k < m; k += 32) s2 += cabs2(A[j * m + k]);
    s2 = warp_sum(s2);
    if (lane == 0) sig[j] = sqrt(s2);
  }
  __syncthreads();
  for (int64_t j = wp; j < n; j += NW) {
    const double sj = sig[j];
    int64_t cnt = 0;
    for (int64_t i = lane; i < n; i += 32) {
      const double si = sig[i];
      cnt += (si > sj || (si == sj && i < j)) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
    for (int64_t k = lane; k < m; k += 32) a.U[cnt * a.ldu + k] = cscale(A[j * m + k], inv);
    for (int64_t k = lane; k < n; k += 32) a.V[cnt * a.ldv + k] = V[j * n + k];
    if (lane == 0) a.S[cnt] = sj;
  }
}

int g_svd_max_blocks[64] = {0};
std::mutex g_svd_mutex;

int svd_max_blocks() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  std::lock_guard<std::mutex> lock(g_svd_mutex);
  if (g_svd_max_blocks[dev] == 0) {
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zsvd_jacobi_kernel, SVD_THREADS, 0) != cudaSuccess)
      return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    g_svd_max_blocks[dev] = per_sm * sms;
  }
  return g_svd_max_blocks[dev];
}

inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// ---- strided permute / conjugate / scale ---------------------------------------
__global__ void zpermute_kernel(ptn_permute_desc d, int64_t total) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = e, so = 0, dof = 0, sidx = 0;
    for (int i = d.n - 1; i >= 0; --i) {
      const int64_t q = rem / d.dim[i];
      const int64_t x = rem - q * d.dim[i];
      rem = q;
      so += x * d.stride_src[i];
      dof += x * d.stride_dst[i];
      if (i == d.scale_mode) sidx = x;
    }
    double2 v = static_cast<const double2*>(d.src)[so];
    if (d.conj) v.y = -v.y;
    if (d.scale) v = cscale(v, d.scale[sidx]);
    static_cast<double2*>(d.dst)[dof] = v;
  }
}

}  // namespace

extern "C" int64_t ptn_zsvd_work_bytes(int64_t m, int64_t n) {
  if (m < 1 || n < 1) return 0;
  return CTRL_BYTES + align256(16 * m * n) + align256(16 * n * n) + align256(8 * n);
}

extern "C" int ptn_zsvd_jacobi(const ptn_svd_desc* d, void* stream) {
  if (!d || !d->A || !d->U || !d->S || !d->V || !d->work || !d->status) return PTN_ERR_ARG;
  if (d->n < 1 || d->m < d->n || d->ldu < d->m || d->ldv < d->n) return PTN_ERR_ARG;
  SvdArgs a;
  a.src = static_cast<const double2*>(d->A);
  a.rs = d->row_stride;
  a.cs = d->col_stride;
  a.m = d->m;
  a.n = d->n;
  uint8_t* w = static_cast<uint8_t*>(d->work);
  a.ctrl = reinterpret_cast<unsigned*>(w);
  a.Aw = reinterpret_cast<double2*>(w + CTRL_BYTES);
  a.Vw = reinterpret_cast<double2*>(w + CTRL_BYTES + align256(16 * d->m * d->n));
  a.sig = reinterpret_cast<double*>(w + CTRL_BYTES + align256(16 * d->m * d->n) + align256(16 * d->n * d->n));
  a.U = static_cast<double2*>(d->U);
  a.ldu = d->ldu;
  a.S = d->S;
  a.V = static_cast<double2*>(d->V);
  a.ldv = d->ldv;
  // sqrt(m) * 2^-53 (LAPACK's zgesvj) sits at the rounding floor of one
  // rotation for small m, and a pair can then cycle without ever passing the
  // test; 8 sqrt(m) * 2^-53 keeps U and V orthonormal to ~1e-14.
  a.tol = 8.0 * sqrt((double)d->m) * 1.1102230246251565e-16;
  a.status = d->status;
  cudaStream_t s = ptn_stream(stream);
  const size_t smem = (size_t)(d->m * d->n + d->n * d->n) * sizeof(double2);
  if (d->n <= SVD_SMALL_N && smem <= (size_t)SVD_SMALL_BYTES) {
    static const cudaError_t attr = cudaFuncSetAttribute(
        zsvd_jacobi_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SVD_SMALL_BYTES);
    if (attr != cudaSuccess) return PTN_ERR_LAUNCH;
    PTN_COUNT(1);
    zsvd_jacobi_small_kernel<<<1, SVD_SMALL_THREADS, smem, s>>>(a);
    return ptn_launch_status();
  }
  const int maxb = svd_max_blocks();
  if (maxb <= 0) return PTN_ERR_LAUNCH;
  if (cudaMemsetAsync(a.ctrl, 0, CTRL_BYTES, s) != cudaSuccess) return PTN_ERR_LAUNCH;
  const int64_t pairs = (((d->n + 1) & ~int64_t(1)) / 2);
  int64_t blocks = (pairs + SVD_WARPS - 1) / SVD_WARPS;
  if (blocks < 1) blocks = 1;
  if (blocks > maxb) blocks = maxb;
  void* args[] = {&a};
  PTN_COUNT(1);
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)zsvd_jacobi_kernel, dim3((unsigned)blocks),
                                                    dim3(SVD_THREADS), args, 0, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PTN_ERR_LAUNCH;
  }
  return PTN_OK;
}

extern "C" int ptn_zpermute(const ptn_permute_desc* d, void* stream) {
  if (!d || !d->src || !d->dst || d->n < 0 || d->n > PTN_MAX_MODES) return PTN_ERR_ARG;
  if (d->scale && (d->scale_mode < 0 || d->scale_mode >= d->n)) return PTN_ERR_ARG;
  int64_t total = 1;
  for (int i = 0; i < d->n; ++i) {
    if (d->dim[i] < 0) return PTN_ERR_ARG;
    total *= d->dim[i];
  }
  if (total == 0) return PTN_OK;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  PTN_COUNT(1);
  zpermute_kernel<<<(unsigned)blocks, 256, 0, ptn_stream(stream)>>>(*d, total);
  return ptn_launch_status();
}
