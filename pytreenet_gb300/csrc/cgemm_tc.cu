// Mixed-precision complex contraction on the 5th-generation tensor cores.
//
// C[m, n] = sum_k A[m, k] * B[n, k] (complex), with A and B split into L BF16
// levels (x = x0 + x1 [+ x2], each bf16, 8 more mantissa bits per level) and
// the products of levels i + j < L accumulated in FP32 in TMEM:
//   L = 2 ("BF16x3"): A0B0 + A0B1 + A1B0, relative error ~2^-16;
//   L = 3 ("BF16x6"): + A0B2 + A1B1 + A2B0, relative error ~2^-24 (FP32 level).
// The complex product is written as one real product with doubled width:
//   [Cr | Ci] = Ar * [Br | Bi] + Ai * [-Bi | Br]
// so each (i, j) term issues two tcgen05.mma (M=128, N=2*NT, K=16). The
// expanded B keeps the three blocks [-Bi; Br; Bi] of a level adjacent in shared
// memory, so the Ar operand is the window [Br; Bi] and the Ai operand the
// window [-Bi; Br].
//
// Operands (both K-major, K contiguous):
//   A: 2L bf16 planes (Ar_0, Ai_0, Ar_1, Ai_1, ...), each [M][lda]
//   Bx: bf16 [level][block(-Bi, Br, Bi)][N][ldb]
// Tiles are staged by TMA (32-byte swizzle, K=16 per stage, up to 8 stages)
// through an mbarrier ring; two stages make one 32-wide accumulation round;
// one warp issues TMA, one warp issues MMA and owns the TMEM allocation, four
// warps run the epilogue (TMEM -> registers -> global, strided by output mode
// tables so the result lands directly in the layout the next step reads).
// Every mbarrier wait is bounded; a timeout sets *status and the CTA exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "ptn_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int MT = 128;         // rows of C per CTA
constexpr int NT = 64;          // complex columns of C per CTA (MMA N = 2*NT)
constexpr int KT = 32;          // K per accumulation round (the unit of the K split)
constexpr int KS = 16;          // K per shared-memory stage (one 32-byte swizzle row, one MMA K)
constexpr int A_PLANE_BYTES = MT * 2 * KS;         // 4 KB
constexpr int B_BLOCK_BYTES = NT * 2 * KS;         // 2 KB
constexpr int SMEM_LIMIT = 227 * 1024;
constexpr int THREADS = 192;

// Stages of KS: as many as fit (at most 8). Two stages make one accumulation
// round, so the TMEM partial sums still cover 32 K values; the deeper ring
// hides the TMA latency that two 84 KB stages of 32 K values left exposed
// (ncu at the chi=128 root: tensor pipe 39 % active, long-scoreboard stalls).
template <int L>
struct Cfg {
  static constexpr int A_STAGE = 2 * L * A_PLANE_BYTES;
  static constexpr int B_STAGE = 3 * L * B_BLOCK_BYTES;
  static constexpr int STAGE = A_STAGE + B_STAGE;
  static constexpr int STAGES = (SMEM_LIMIT - 2048) / STAGE > 8 ? 8 : (SMEM_LIMIT - 2048) / STAGE;
  static constexpr int SMEM = STAGES * STAGE + 1024;
};
constexpr long long WAIT_CYCLES = 4000000000LL;    // ~2 s at 2 GHz

struct OutModes {
  int n;
  int64_t dim[PTN_MAX_MODES];
  int64_t stride[PTN_MAX_MODES];
};

struct GemmArgs {
  int64_t M, N, K;
  int out_kind;              // 0: complex128, 1: bf16 planes
  void* C;
  int64_t c_plane;           // plane stride (elements) for out_kind 1
  OutModes mo, no;
  int32_t* status;
  int64_t tiles_n;
  int64_t tiles;             // output tiles (tiles_m * tiles_n)
  int32_t splits;            // K ranges per tile (1: no split)
  int32_t ksplit;            // K tiles per range
  float2* partial;           // [splits][M][N] FP32 partial sums when splits > 1
};

// Split-K: outputs with fewer tiles than this many CTAs get their K range
// split so the launch fills the GPU (one CTA per SM, 152 SMs, two waves);
// each range keeps at least SPLIT_MIN_KT K tiles.
constexpr int64_t SPLIT_TARGET_CTAS = 304;
constexpr int64_t SPLIT_MIN_KT = 4;
// Products with fewer K tiles than this are not split: measured on GB300, the
// partial-sum pass costs more than the parallelism gains below K = 1024
// (512 x 1280 x 256: 70 us split, 47 us not; 256 x 256 x 1280: 54 vs 84 us).
constexpr int64_t SPLIT_MIN_KT_TOTAL = 32;

__device__ __forceinline__ int64_t decode_off(const OutModes& md, int64_t idx) {
  int64_t o = 0;
  for (int d = md.n - 1; d >= 0; --d) {
    int64_t q = idx / md.dim[d];
    o += (idx - q * md.dim[d]) * md.stride[d];
    idx = q;
  }
  return o;
}

template <int L>
__global__ void __launch_bounds__(THREADS, 1)
    cgemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const GemmArgs g) {
  using C_ = Cfg<L>;
  constexpr int STAGES = C_::STAGES;
  constexpr int STAGE_BYTES = C_::STAGE;
  constexpr int A_STAGE_BYTES = C_::A_STAGE;
  constexpr uint32_t ACC_COLS = 2 * NT;          // one accumulator: [Re | Im]
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES], tfull_bar[2], tempty_bar[2], drain_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int64_t noff[NT];
  __shared__ int s_abort;
  const volatile int32_t* vstatus = g.status;
  if (threadIdx.x == 0) s_abort = *vstatus;
  __syncthreads();
  if (s_abort != 0) return;  // an earlier CTA failed: skip the work

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = blockIdx.x % g.tiles;
  const int split = (int)(blockIdx.x / g.tiles);
  const int64_t tm = tile / g.tiles_n, tn = tile - tm * g.tiles_n;
  const int64_t m0 = tm * MT, n0 = tn * NT;
  // stages of KS K values; the split ranges are whole accumulation rounds (KT)
  const int kt_all = (int)((g.K + KS - 1) / KS);
  const int kt0 = split * g.ksplit * (KT / KS);
  const int ktiles = min(kt_all, kt0 + g.ksplit * (KT / KS)) - kt0;   // stages of this CTA's range
  const int nacc = (ktiles + 1) / 2;                                   // accumulation rounds

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full_bar[s], 1);
      tc::mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&tfull_bar[b], 1);
      tc::mbar_init(&tempty_bar[b], 4);   // one arrival per epilogue warp
    }
    tc::mbar_init(&drain_bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(&tmem_base, 2 * ACC_COLS);
    tc::tmem_relinquish();
  }
  if (threadIdx.x >= 64 && threadIdx.x < 64 + NT) {
    const int j = threadIdx.x - 64;
    const int64_t n = n0 + j;
    noff[j] = (n < g.N) ? decode_off(g.no, n) : -1;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      tc::prefetch_tmap(&tmA);
      tc::prefetch_tmap(&tmB);
      int issued = 0;
      bool aborted = false;
      for (int kt = 0; kt < ktiles; ++kt) {
        const int s = kt % STAGES;
        const int use = kt / STAGES;
        if (use > 0 && !tc::mbar_wait_abortable(&empty_bar[s], (use - 1) & 1, WAIT_CYCLES, vstatus)) {
          atomicExch(g.status, PTN_ERR_TIMEOUT);
          aborted = true;
          break;
        }
        uint8_t* st = smem + s * STAGE_BYTES;
        tc::mbar_arrive_expect_tx(&full_bar[s], STAGE_BYTES);
        const int kx = (kt0 + kt) * KS;
        for (int p = 0; p < 2 * L; ++p)
          tc::tma_load_3d(st + p * A_PLANE_BYTES, &tmA, &full_bar[s], kx, (int)m0, p);
        for (int b = 0; b < 3 * L; ++b)
          tc::tma_load_3d(st + A_STAGE_BYTES + b * B_BLOCK_BYTES, &tmB, &full_bar[s], kx, (int)n0, b);
        ++issued;
      }
      if (aborted) {
        // Drain before the CTA gives up its shared memory: wait (bounded) for
        // the last load issued into each stage. A stage's phase for its last
        // use is the only one still to complete, so a completed one returns
        // at once.
        for (int s = 0; s < STAGES && s < issued; ++s) {
          const int kt_last = s + ((issued - 1 - s) / STAGES) * STAGES;
          tc::mbar_wait(&full_bar[s], (uint32_t)((kt_last / STAGES) & 1), WAIT_CYCLES);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    // Each K tile accumulates into a fresh TMEM buffer (two, alternating); the
    // epilogue warps add the tile's partial sum into FP32 registers. The
    // tensor-core accumulator loses precision in proportion to the number of
    // accumulations it absorbs, so this bounds that loss to one tile.
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16(MT, 2 * NT);
      bool aborted = false, any_mma = false;
      for (int kt = 0; kt < ktiles; ++kt) {
        const int s = kt % STAGES;
        const int a = kt >> 1;                  // accumulation round: stages 2a, 2a + 1
        const int b = a & 1, ub = a >> 1;
        const bool round_start = (kt & 1) == 0;
        if (round_start && ub > 0 &&
            !tc::mbar_wait_abortable(&tempty_bar[b], (ub - 1) & 1, WAIT_CYCLES, vstatus)) {
          atomicExch(g.status, PTN_ERR_TIMEOUT);
          aborted = true;
          break;
        }
        if (!tc::mbar_wait_abortable(&full_bar[s], (kt / STAGES) & 1, WAIT_CYCLES, vstatus)) {
          atomicExch(g.status, PTN_ERR_TIMEOUT);
          aborted = true;
          break;
        }
        any_mma = true;
        tc::fence_after();
        const uint32_t sa = tc::smem_u32(smem + s * STAGE_BYTES);
        const uint32_t sb = sa + A_STAGE_BYTES;
        const uint32_t acc = tmem + (uint32_t)b * ACC_COLS;
        bool first = round_start;
        // smallest split products first, the leading (0, 0) product last
#pragma unroll
        for (int lvl = L - 1; lvl >= 0; --lvl) {
#pragma unroll
          for (int i = 0; i <= lvl; ++i) {
            const int j = lvl - i;
            // A planes: 2i = Re level i, 2i+1 = Im level i.
            // B level j at sb + 3j*B_BLOCK: window [Br; Bi] at +1 block, [-Bi; Br] at +0.
            const uint64_t ar = tc::sdesc_sw32(sa + (2 * i) * A_PLANE_BYTES);
            const uint64_t ai = tc::sdesc_sw32(sa + (2 * i + 1) * A_PLANE_BYTES);
            const uint64_t bt = tc::sdesc_sw32(sb + (3 * j + 1) * B_BLOCK_BYTES);
            const uint64_t bb = tc::sdesc_sw32(sb + (3 * j) * B_BLOCK_BYTES);
            tc::mma_bf16(acc, ar, bt, idesc, first ? 0u : 1u);
            tc::mma_bf16(acc, ai, bb, idesc, 1u);
            first = false;
          }
        }
        tc::mma_commit(&empty_bar[s]);
        if (!round_start || kt == ktiles - 1) tc::mma_commit(&tfull_bar[b]);
      }
      if (aborted && any_mma) {
        // every MMA this thread issued completes before TMEM is freed
        tc::mma_commit(&drain_bar);
        tc::mbar_wait(&drain_bar, 0, WAIT_CYCLES);
      }
    }
  } else {
    // ---------------- epilogue (warps 2..5) ----------------
    const int q = warp & 3;                 // TMEM lane quarter of this warp
    const int row = q * 32 + lane;
    const int64_t m = m0 + row;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    float acc_re[NT], acc_im[NT];
#pragma unroll
    for (int i = 0; i < NT; ++i) {
      acc_re[i] = 0.f;
      acc_im[i] = 0.f;
    }
    bool ok = true;
    for (int a = 0; a < nacc && ok; ++a) {
      const int b = a & 1;
      ok = tc::mbar_wait_abortable(&tfull_bar[b], (a >> 1) & 1, WAIT_CYCLES, vstatus);
      if (!ok) break;
      tc::fence_after();
      const uint32_t tb = tmem + lane_off + (uint32_t)b * ACC_COLS;
      // two loads in flight per wait (re and im of 16 columns)
#pragma unroll
      for (int j0 = 0; j0 < NT; j0 += 16) {
        uint32_t vr[16], vi[16];
        tc::tmem_ld16_nowait(tb + (uint32_t)j0, vr);
        tc::tmem_ld16_nowait(tb + (uint32_t)(NT + j0), vi);
        tc::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          acc_re[j0 + i] += __uint_as_float(vr[i]);
          acc_im[j0 + i] += __uint_as_float(vi[i]);
        }
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tempty_bar[b]);
    }
    if (!ok) {
      if (lane == 0) atomicExch(g.status, PTN_ERR_TIMEOUT);
    } else if (m < g.M && g.splits > 1) {
      // this K range's FP32 partial sums; splitk_reduce_kernel adds the ranges
      float2* P = g.partial + ((int64_t)split * g.M + m) * g.N + n0;
#pragma unroll
      for (int i = 0; i < NT; ++i)
        if (n0 + i < g.N) P[i] = make_float2(acc_re[i], acc_im[i]);
    } else if (m < g.M) {
      const int64_t moff = decode_off(g.mo, m);
      if (g.out_kind == 0) {
        double2* C = static_cast<double2*>(g.C);
#pragma unroll
        for (int i = 0; i < NT; ++i) {
          const int64_t no = noff[i];
          if (no >= 0) C[moff + no] = make_double2((double)acc_re[i], (double)acc_im[i]);
        }
      } else {
        __nv_bfloat16* C = static_cast<__nv_bfloat16*>(g.C);
        const int64_t ps = g.c_plane;
#pragma unroll
        for (int i = 0; i < NT; ++i) {
          const int64_t no = noff[i];
          if (no < 0) continue;
          const int64_t o = moff + no;
          float r = acc_re[i], v = acc_im[i];
#pragma unroll
          for (int lv = 0; lv < L; ++lv) {
            const __nv_bfloat16 rb = __float2bfloat16_rn(r);
            const __nv_bfloat16 ib = __float2bfloat16_rn(v);
            C[(2 * lv) * ps + o] = rb;
            C[(2 * lv + 1) * ps + o] = ib;
            r -= __bfloat162float(rb);
            v -= __bfloat162float(ib);
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, 2 * ACC_COLS);
}

// ---- tensor maps ---------------------------------------------------------------------
// cuTensorMapEncodeTiled is fetched through the runtime's driver entry point so
// the library does not link libcuda (it still loads on a machine without a driver).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // initialised once, thread-safe (C++11 static initialisation)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return nullptr;
  }();
  return fn;
}

int make_map_3d(CUtensorMap* map, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1_bytes,
                uint64_t s2_bytes, uint32_t b0, uint32_t b1) {
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {s1_bytes, s2_bytes};
  cuuint32_t box[3] = {b0, b1, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return PTN_ERR_LAUNCH;
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims,
                                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? PTN_OK : PTN_ERR_ARG;
}

// ---- conversions ---------------------------------------------------------------------
// planes[p][m * lda + k] <- split(src[off_m(m) + off_k(k)]) for the complex128 source.
// x ~ out[0] + ... + out[L-1] in BF16 pieces. Only the first remainder needs
// double precision: x - bf16(x) is exact in FP64 (Sterbenz) and is rounded
// once to FP32 (error <= 2^-32 |x|, below the 2^-25 |x| the three pieces
// leave); the later pieces are split in FP32. GB300 issues FP64 at 1/64 of the
// FP32 rate, and a split done wholly in FP64 made the conversion of the χ=256
// root vector FP64-bound (0.93 ms for 33.5 M entries).
__device__ __forceinline__ void split_levels(double x, int L, __nv_bfloat16* out) {
  const __nv_bfloat16 b0 = __double2bfloat16(x);
  out[0] = b0;
  float r = (float)(x - (double)__bfloat162float(b0));
  for (int lv = 1; lv < L; ++lv) {
    const __nv_bfloat16 b = __float2bfloat16_rn(r);
    out[lv] = b;
    r -= __bfloat162float(b);
  }
}

__global__ void to_planes_kernel(const double2* __restrict__ src, OutModes mm, OutModes km, int64_t M, int64_t K,
                                 int64_t lda, int64_t plane, int conj, int L, __nv_bfloat16* __restrict__ dst) {
  const int64_t total = M * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / K, k = e - (e / K) * K;
    double2 v = src[decode_off(mm, m) + decode_off(km, k)];
    if (conj) v.y = -v.y;
    __nv_bfloat16 re[3], im[3];
    split_levels(v.x, L, re);
    split_levels(v.y, L, im);
    const int64_t o = m * lda + k;
    for (int lv = 0; lv < L; ++lv) {
      dst[(2 * lv) * plane + o] = re[lv];
      dst[(2 * lv + 1) * plane + o] = im[lv];
    }
  }
}

// The same conversion through a 32 x 32 shared-memory tile, for operands
// whose rows are contiguous in the source while the K index is not (the first
// step of a matvec contracting the parent leg reads x with a stride of the
// whole rest of the tensor): the tile is read with the row index across the
// threads and written with the K index across them, so both sides coalesce.
// Each element is converted exactly as in to_planes_kernel.
__global__ void __launch_bounds__(256) to_planes_tiled_kernel(const double2* __restrict__ src, OutModes mm,
                                                              OutModes km, int64_t M, int64_t K, int64_t lda,
                                                              int64_t plane, int conj, int L,
                                                              __nv_bfloat16* __restrict__ dst) {
  __shared__ double2 tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t tiles_k = (K + 31) / 32;
  const int64_t tiles = ((M + 31) / 32) * tiles_k;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t m0 = (t / tiles_k) * 32, k0 = (t - (t / tiles_k) * tiles_k) * 32;
    for (int r = ty; r < 32; r += 8) {
      const int64_t m = m0 + tx, k = k0 + r;
      double2 v = make_double2(0.0, 0.0);
      if (m < M && k < K) v = src[decode_off(mm, m) + decode_off(km, k)];
      tile[r][tx] = v;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int64_t m = m0 + r, k = k0 + tx;
      if (m < M && k < K) {
        double2 v = tile[tx][r];
        if (conj) v.y = -v.y;
        __nv_bfloat16 re[3], im[3];
        split_levels(v.x, L, re);
        split_levels(v.y, L, im);
        const int64_t o = m * lda + k;
        for (int lv = 0; lv < L; ++lv) {
          dst[(2 * lv) * plane + o] = re[lv];
          dst[(2 * lv + 1) * plane + o] = im[lv];
        }
      }
    }
    __syncthreads();
  }
}

// Bx[level][block][n][k]: block 0 = -Bi, 1 = Br, 2 = Bi.
__global__ void expand_b_kernel(const double2* __restrict__ src, OutModes nm, OutModes km, int64_t N, int64_t K,
                                int64_t ldb, int conj, int L, __nv_bfloat16* __restrict__ dst) {
  const int64_t total = N * K;
  const int64_t blk = N * ldb;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = e / K, k = e - (e / K) * K;
    double2 v = src[decode_off(nm, n) + decode_off(km, k)];
    if (conj) v.y = -v.y;
    __nv_bfloat16 re[3], im[3];
    split_levels(v.x, L, re);
    split_levels(v.y, L, im);
    const int64_t o = n * ldb + k;
    for (int lv = 0; lv < L; ++lv) {
      dst[(3 * lv + 0) * blk + o] = __hneg(im[lv]);
      dst[(3 * lv + 1) * blk + o] = re[lv];
      dst[(3 * lv + 2) * blk + o] = im[lv];
    }
  }
}

// ---- skinny products on the CUDA cores ----------------------------------------------
// A product with K <= SMALLK_MAX_K (one 32-wide K tile) and N <= SMALLK_MAX_N
// (the contraction with a TTNO tensor over its bond and physical legs, K =
// w d = 10) does too little arithmetic per output for a tensor-core tile
// pipeline: its set-up per CTA dominates (65536 x 10 x 10 measured 60 us).
// Here one thread owns one row: it rebuilds A's row from the BF16 level planes,
// B (same operand layout, staged in shared memory) likewise, accumulates in
// FP32 as the tensor cores do, and writes through the same output modes; the
// cost is the operand traffic.
constexpr int64_t SMALLK_MAX_K = 32;
constexpr int64_t SMALLK_MAX_N = 128;
constexpr int SMALLK_T = 128;

// KK: the K of the instance (EXACT) or an upper bound with K read at run time;
// an exact K leaves no predicated-off steps in the unrolled K loops.
template <int KK, bool EXACT>
__global__ void __launch_bounds__(SMALLK_T)
    cgemm_smallk_kernel(const __nv_bfloat16* __restrict__ A, int64_t lda, int64_t a_plane,
                        const __nv_bfloat16* __restrict__ Bx, int64_t ldb, GemmArgs g, int L) {
  __shared__ float2 sB[SMALLK_MAX_N * KK];
  __shared__ int64_t noff[SMALLK_MAX_N];
  if (*(volatile int32_t*)g.status != 0) return;
  const int N = (int)g.N, K = EXACT ? KK : (int)g.K;
  const int64_t blk = (int64_t)N * ldb;
  for (int e = threadIdx.x; e < N * K; e += SMALLK_T) {
    const int n = e / K, kk = e - n * K;
    float re = 0.f, im = 0.f;
    for (int lv = 0; lv < L; ++lv) {
      re += __bfloat162float(Bx[(3 * lv + 1) * blk + (int64_t)n * ldb + kk]);
      im += __bfloat162float(Bx[(3 * lv + 2) * blk + (int64_t)n * ldb + kk]);
    }
    sB[n * KK + kk] = make_float2(re, im);
  }
  for (int n = threadIdx.x; n < N; n += SMALLK_T) noff[n] = decode_off(g.no, n);
  __syncthreads();
  for (int64_t m = blockIdx.x * (int64_t)SMALLK_T + threadIdx.x; m < g.M; m += (int64_t)gridDim.x * SMALLK_T) {
    float2 a[KK];
#pragma unroll
    for (int kk = 0; kk < KK; ++kk) {
      float re = 0.f, im = 0.f;
      if (EXACT || kk < K) {
        for (int lv = 0; lv < L; ++lv) {
          re += __bfloat162float(A[(2 * lv) * a_plane + m * lda + kk]);
          im += __bfloat162float(A[(2 * lv + 1) * a_plane + m * lda + kk]);
        }
      }
      a[kk] = make_float2(re, im);
    }
    const int64_t moff = decode_off(g.mo, m);
    for (int n = 0; n < N; ++n) {
      float cr = 0.f, ci = 0.f;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk) {
        if (EXACT || kk < K) {
          const float2 b = sB[n * KK + kk];
          cr = fmaf(a[kk].x, b.x, cr);
          cr = fmaf(-a[kk].y, b.y, cr);
          ci = fmaf(a[kk].x, b.y, ci);
          ci = fmaf(a[kk].y, b.x, ci);
        }
      }
      const int64_t o = moff + noff[n];
      if (g.out_kind == 0) {
        static_cast<double2*>(g.C)[o] = make_double2((double)cr, (double)ci);
      } else {
        __nv_bfloat16* C = static_cast<__nv_bfloat16*>(g.C);
        for (int lv = 0; lv < L; ++lv) {
          const __nv_bfloat16 rb = __float2bfloat16_rn(cr);
          const __nv_bfloat16 ib = __float2bfloat16_rn(ci);
          C[(2 * lv) * g.c_plane + o] = rb;
          C[(2 * lv + 1) * g.c_plane + o] = ib;
          cr -= __bfloat162float(rb);
          ci -= __bfloat162float(ib);
        }
      }
    }
  }
}

// The same product for BF16-plane outputs whose rows come in adjacent pairs:
// thread t computes rows 2t and 2t + 1 and stores each plane entry of the pair
// as one 4-byte bf16x2 (the host checks that the innermost row mode has
// output stride 1 and an even extent and that every other stride is even, so
// the pair is adjacent and 4-byte aligned). Half the store instructions, and a
// warp writes 128 contiguous bytes per plane. Same arithmetic per output.
template <int KK>
__global__ void __launch_bounds__(SMALLK_T)
    cgemm_smallk_pair_kernel(const __nv_bfloat16* __restrict__ A, int64_t lda, int64_t a_plane,
                             const __nv_bfloat16* __restrict__ Bx, int64_t ldb, GemmArgs g, int L) {
  __shared__ float2 sB[SMALLK_MAX_N * KK];
  __shared__ int64_t noff[SMALLK_MAX_N];
  if (*(volatile int32_t*)g.status != 0) return;
  const int N = (int)g.N;
  const int64_t blk = (int64_t)N * ldb;
  for (int e = threadIdx.x; e < N * KK; e += SMALLK_T) {
    const int n = e / KK, kk = e - n * KK;
    float re = 0.f, im = 0.f;
    for (int lv = 0; lv < L; ++lv) {
      re += __bfloat162float(Bx[(3 * lv + 1) * blk + (int64_t)n * ldb + kk]);
      im += __bfloat162float(Bx[(3 * lv + 2) * blk + (int64_t)n * ldb + kk]);
    }
    sB[n * KK + kk] = make_float2(re, im);
  }
  for (int n = threadIdx.x; n < N; n += SMALLK_T) noff[n] = decode_off(g.no, n);
  __syncthreads();
  const int64_t pairs = g.M / 2;
  for (int64_t pr = blockIdx.x * (int64_t)SMALLK_T + threadIdx.x; pr < pairs;
       pr += (int64_t)gridDim.x * SMALLK_T) {
    const int64_t m = 2 * pr;
    float2 a0[KK], a1[KK];
#pragma unroll
    for (int kk = 0; kk < KK; ++kk) {
      float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f;
      for (int lv = 0; lv < L; ++lv) {
        r0 += __bfloat162float(A[(2 * lv) * a_plane + m * lda + kk]);
        i0 += __bfloat162float(A[(2 * lv + 1) * a_plane + m * lda + kk]);
        r1 += __bfloat162float(A[(2 * lv) * a_plane + (m + 1) * lda + kk]);
        i1 += __bfloat162float(A[(2 * lv + 1) * a_plane + (m + 1) * lda + kk]);
      }
      a0[kk] = make_float2(r0, i0);
      a1[kk] = make_float2(r1, i1);
    }
    const int64_t moff = decode_off(g.mo, m);
    __nv_bfloat16* C = static_cast<__nv_bfloat16*>(g.C);
    for (int n = 0; n < N; ++n) {
      float cr0 = 0.f, ci0 = 0.f, cr1 = 0.f, ci1 = 0.f;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk) {
        const float2 b = sB[n * KK + kk];
        cr0 = fmaf(a0[kk].x, b.x, cr0);
        cr0 = fmaf(-a0[kk].y, b.y, cr0);
        ci0 = fmaf(a0[kk].x, b.y, ci0);
        ci0 = fmaf(a0[kk].y, b.x, ci0);
        cr1 = fmaf(a1[kk].x, b.x, cr1);
        cr1 = fmaf(-a1[kk].y, b.y, cr1);
        ci1 = fmaf(a1[kk].x, b.y, ci1);
        ci1 = fmaf(a1[kk].y, b.x, ci1);
      }
      const int64_t o = moff + noff[n];
      for (int lv = 0; lv < L; ++lv) {
        const __nv_bfloat16 rb0 = __float2bfloat16_rn(cr0), ib0 = __float2bfloat16_rn(ci0);
        const __nv_bfloat16 rb1 = __float2bfloat16_rn(cr1), ib1 = __float2bfloat16_rn(ci1);
        *reinterpret_cast<__nv_bfloat162*>(C + (2 * lv) * g.c_plane + o) = __halves2bfloat162(rb0, rb1);
        *reinterpret_cast<__nv_bfloat162*>(C + (2 * lv + 1) * g.c_plane + o) = __halves2bfloat162(ib0, ib1);
        cr0 -= __bfloat162float(rb0);
        ci0 -= __bfloat162float(ib0);
        cr1 -= __bfloat162float(rb1);
        ci1 -= __bfloat162float(ib1);
      }
    }
  }
}

// Whether the rows of a BF16-plane output come in adjacent, 4-byte aligned
// pairs (cgemm_smallk_pair_kernel).
static bool smallk_pairs_ok(const GemmArgs& g, int64_t M) {
  if (g.out_kind != 1 || M < 2 || M % 2 || g.mo.n < 1 || (g.c_plane & 1)) return false;
  if (g.mo.stride[g.mo.n - 1] != 1 || g.mo.dim[g.mo.n - 1] % 2) return false;
  for (int i = 0; i + 1 < g.mo.n; ++i)
    if (g.mo.stride[i] & 1) return false;
  for (int i = 0; i < g.no.n; ++i)
    if (g.no.stride[i] & 1) return false;
  return true;
}

// Sum of the split-K partial sums (compensated FP32, ranges in order: deterministic),
// written like the GEMM epilogue: complex128 through the output modes, or as
// BF16 level planes.
__global__ void splitk_reduce_kernel(const float2* __restrict__ partial, int splits, int64_t M, int64_t N,
                                     OutModes mo, OutModes no, int out_kind, void* C, int64_t c_plane, int L,
                                     const int32_t* __restrict__ status) {
  if (*status != 0) return;
  const int64_t total = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / N, n = e - (e / N) * N;
    // compensated (Kahan) sums in FP32, ranges in order: the FP32 pipe runs at
    // 64x the FP64 rate on GB300, and the compensation keeps the error at the
    // level of the partials' own rounding
    float sr = 0.f, si = 0.f, cr = 0.f, ci = 0.f;
    for (int s = 0; s < splits; ++s) {
      const float2 p = partial[((int64_t)s * M + m) * N + n];
      const float yr = p.x - cr, yi = p.y - ci;
      const float tr = sr + yr, ti = si + yi;
      cr = (tr - sr) - yr;
      ci = (ti - si) - yi;
      sr = tr;
      si = ti;
    }
    const double re = (double)sr - (double)cr, im = (double)si - (double)ci;
    const int64_t o = decode_off(mo, m) + decode_off(no, n);
    if (out_kind == 0) {
      static_cast<double2*>(C)[o] = make_double2(re, im);
    } else {
      __nv_bfloat16* Cb = static_cast<__nv_bfloat16*>(C);
      __nv_bfloat16 rb[3], ib[3];
      split_levels(re, L, rb);
      split_levels(im, L, ib);
      for (int lv = 0; lv < L; ++lv) {
        Cb[(2 * lv) * c_plane + o] = rb[lv];
        Cb[(2 * lv + 1) * c_plane + o] = ib[lv];
      }
    }
  }
}

// Split of the K range for an M x N x K product: (splits, K tiles per split).
void split_plan(int64_t M, int64_t N, int64_t K, int64_t& splits, int64_t& ksplit) {
  const int64_t tiles = ((M + MT - 1) / MT) * ((N + NT - 1) / NT);
  const int64_t kt_all = (K + KT - 1) / KT;
  splits = 1;
  ksplit = kt_all;
  if (tiles >= SPLIT_TARGET_CTAS / 2 || kt_all < SPLIT_MIN_KT_TOTAL) return;
  int64_t s = (SPLIT_TARGET_CTAS + tiles - 1) / tiles;
  const int64_t smax = kt_all / SPLIT_MIN_KT;
  if (s > smax) s = smax;
  if (s < 2) return;
  ksplit = (kt_all + s - 1) / s;
  splits = (kt_all + ksplit - 1) / ksplit;
  if (splits < 2) {
    splits = 1;
    ksplit = kt_all;
  }
}

int fill_out(const ptn_modes& src, OutModes& dst) {
  if (src.n < 0 || src.n > PTN_MAX_MODES) return PTN_ERR_ARG;
  dst.n = src.n;
  for (int i = 0; i < src.n; ++i) {
    if (src.dim[i] <= 0) return PTN_ERR_ARG;
    dst.dim[i] = src.dim[i];
    dst.stride[i] = src.stride_c[i];
  }
  return PTN_OK;
}

int fill_src(const ptn_modes& src, OutModes& dst, int64_t& total) {
  if (src.n < 0 || src.n > PTN_MAX_MODES) return PTN_ERR_ARG;
  dst.n = src.n;
  total = 1;
  for (int i = 0; i < src.n; ++i) {
    if (src.dim[i] <= 0) return PTN_ERR_ARG;
    dst.dim[i] = src.dim[i];
    dst.stride[i] = src.stride_a[i];
    total *= src.dim[i];
  }
  return PTN_OK;
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 4096) b = 4096;
  return (unsigned)b;
}

}  // namespace

extern "C" int ptn_cgemm_smem_bytes(int32_t levels) { return levels == 3 ? Cfg<3>::SMEM : Cfg<2>::SMEM; }

extern "C" int64_t ptn_cgemm_partial_bytes(int64_t M, int64_t N, int64_t K) {
  if (M < 1 || N < 1 || K < 1) return 0;
  int64_t splits, ksplit;
  split_plan(M, N, K, splits, ksplit);
  return splits > 1 ? splits * M * N * (int64_t)sizeof(float2) : 0;
}

template <int L>
int launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g, unsigned grid, cudaStream_t st) {
  // once per process, thread-safe; a failure is returned on every call
  static const cudaError_t attr =
      cudaFuncSetAttribute(cgemm_bf16_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<L>::SMEM);
  if (attr != cudaSuccess) return PTN_ERR_LAUNCH;
  PTN_COUNT(1);
  cgemm_bf16_kernel<L><<<grid, THREADS, Cfg<L>::SMEM, st>>>(ta, tb, g);
  if (g.splits > 1) {
    PTN_COUNT(1);
    splitk_reduce_kernel<<<grid_for(g.M * g.N), 256, 0, st>>>(g.partial, g.splits, g.M, g.N, g.mo, g.no,
                                                              g.out_kind, g.C, g.c_plane, L, g.status);
  }
  return ptn_launch_status();
}

extern "C" int ptn_cgemm_bf16x3(const ptn_cgemm_desc* d, void* stream) {
  if (!d || !d->A || !d->Bx || !d->C || !d->status) return PTN_ERR_ARG;
  if (d->M < 1 || d->N < 1 || d->K < 1) return PTN_ERR_ARG;
  if (d->levels != 2 && d->levels != 3) return PTN_ERR_ARG;
  // the CUDA-core path (K <= 32, N <= 128) reads A without TMA: any lda >= K
  const bool smallk = d->K <= SMALLK_MAX_K && d->N <= SMALLK_MAX_N;
  if ((!smallk && d->lda % 8) || d->ldb % 8 || d->lda < d->K || d->ldb < d->K) return PTN_ERR_ARG;
  if (d->a_plane % 8 || (reinterpret_cast<uintptr_t>(d->A) & 15) || (reinterpret_cast<uintptr_t>(d->Bx) & 15))
    return PTN_ERR_ARG;
  if (d->M > 0x7fffffffLL || d->N > 0x7fffffffLL) return PTN_ERR_UNSUPPORTED;
  GemmArgs g;
  g.M = d->M;
  g.N = d->N;
  g.K = d->K;
  g.out_kind = d->out_kind;
  g.C = d->C;
  g.c_plane = d->c_plane;
  g.status = d->status;
  if (fill_out(d->m_out, g.mo) || fill_out(d->n_out, g.no)) return PTN_ERR_ARG;
  if (smallk) {
    int64_t blocks = (d->M + SMALLK_T - 1) / SMALLK_T;
    if (blocks > 152 * 16) blocks = 152 * 16;
    PTN_COUNT(1);
    const __nv_bfloat16* A = static_cast<const __nv_bfloat16*>(d->A);
    const __nv_bfloat16* B = static_cast<const __nv_bfloat16*>(d->Bx);
    cudaStream_t st = ptn_stream(stream);
    if (smallk_pairs_ok(g, d->M)) {
      int64_t pb = (d->M / 2 + SMALLK_T - 1) / SMALLK_T;
      if (pb > 152 * 16) pb = 152 * 16;
      switch (d->K) {
#define PTN_SMALLK_PAIR(k)                                                                                     \
  case k:                                                                                                       \
    cgemm_smallk_pair_kernel<k><<<(unsigned)pb, SMALLK_T, 0, st>>>(A, d->lda, d->a_plane, B, d->ldb, g, d->levels); \
    return ptn_launch_status();
        PTN_SMALLK_PAIR(2)
        PTN_SMALLK_PAIR(4)
        PTN_SMALLK_PAIR(6)
        PTN_SMALLK_PAIR(10)
#undef PTN_SMALLK_PAIR
        default:
          break;
      }
    }
    switch (d->K) {
#define PTN_SMALLK_CASE(k)                                                                              \
  case k:                                                                                               \
    cgemm_smallk_kernel<k, true><<<(unsigned)blocks, SMALLK_T, 0, st>>>(A, d->lda, d->a_plane, B, d->ldb, g, \
                                                                        d->levels);                     \
    break;
      PTN_SMALLK_CASE(2)
      PTN_SMALLK_CASE(3)
      PTN_SMALLK_CASE(4)
      PTN_SMALLK_CASE(5)
      PTN_SMALLK_CASE(6)
      PTN_SMALLK_CASE(8)
      PTN_SMALLK_CASE(10)
      PTN_SMALLK_CASE(12)
      PTN_SMALLK_CASE(16)
      PTN_SMALLK_CASE(20)
#undef PTN_SMALLK_CASE
      default:
        cgemm_smallk_kernel<(int)SMALLK_MAX_K, false><<<(unsigned)blocks, SMALLK_T, 0, st>>>(
            A, d->lda, d->a_plane, B, d->ldb, g, d->levels);
    }
    return ptn_launch_status();
  }
  CUtensorMap ta, tb;
  const int L = d->levels;
  if (make_map_3d(&ta, d->A, (uint64_t)d->K, (uint64_t)d->M, 2 * L, (uint64_t)d->lda * 2,
                  (uint64_t)d->a_plane * 2, KS, MT))
    return PTN_ERR_ARG;
  if (make_map_3d(&tb, d->Bx, (uint64_t)d->K, (uint64_t)d->N, 3 * L, (uint64_t)d->ldb * 2,
                  (uint64_t)d->N * (uint64_t)d->ldb * 2, KS, NT))
    return PTN_ERR_ARG;
  const int64_t tm = (d->M + MT - 1) / MT, tn = (d->N + NT - 1) / NT;
  g.tiles_n = tn;
  g.tiles = tm * tn;
  int64_t splits = 1, ksplit = (d->K + KT - 1) / KT;
  if (d->partial) {
    int64_t s_, k_;
    split_plan(d->M, d->N, d->K, s_, k_);
    if (s_ > 1 && s_ * d->M * d->N * (int64_t)sizeof(float2) <= d->partial_bytes &&
        !(reinterpret_cast<uintptr_t>(d->partial) & 7)) {
      splits = s_;
      ksplit = k_;
    }
  }
  g.splits = (int32_t)splits;
  g.ksplit = (int32_t)ksplit;
  g.partial = static_cast<float2*>(d->partial);
  if (tm * tn * splits > 0x7fffffffLL) return PTN_ERR_UNSUPPORTED;
  const unsigned grid = (unsigned)(tm * tn * splits);
  return L == 3 ? launch_gemm<3>(ta, tb, g, grid, ptn_stream(stream)) : launch_gemm<2>(ta, tb, g, grid, ptn_stream(stream));
}

extern "C" int ptn_to_planes(const ptn_convert_desc* d, void* stream) {
  if (!d || !d->src || !d->dst || (d->levels != 2 && d->levels != 3)) return PTN_ERR_ARG;
  OutModes mm, km;
  int64_t M, K;
  if (fill_src(d->rows, mm, M) || fill_src(d->cols, km, K)) return PTN_ERR_ARG;
  if (d->ld < K) return PTN_ERR_ARG;
  PTN_COUNT(1);
  // innermost (fastest) source strides of the row and K indices
  const int64_t sm = mm.n > 0 ? mm.stride[mm.n - 1] : 0, sk = km.n > 0 ? km.stride[km.n - 1] : 0;
  const int64_t asm_ = sm < 0 ? -sm : sm, ask = sk < 0 ? -sk : sk;
  if (M >= 32 && K >= 32 && asm_ <= 2 && ask > 2) {
    const int64_t tiles = ((M + 31) / 32) * ((K + 31) / 32);
    to_planes_tiled_kernel<<<(unsigned)(tiles < 152 * 16 ? tiles : 152 * 16), 256, 0, ptn_stream(stream)>>>(
        static_cast<const double2*>(d->src), mm, km, M, K, d->ld, d->plane, d->conj, d->levels,
        static_cast<__nv_bfloat16*>(d->dst));
    return ptn_launch_status();
  }
  to_planes_kernel<<<grid_for(M * K), 256, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(d->src), mm, km, M, K, d->ld, d->plane, d->conj, d->levels,
      static_cast<__nv_bfloat16*>(d->dst));
  return ptn_launch_status();
}

extern "C" int ptn_expand_b(const ptn_convert_desc* d, void* stream) {
  if (!d || !d->src || !d->dst || (d->levels != 2 && d->levels != 3)) return PTN_ERR_ARG;
  OutModes nm, km;
  int64_t N, K;
  if (fill_src(d->rows, nm, N) || fill_src(d->cols, km, K)) return PTN_ERR_ARG;
  if (d->ld < K) return PTN_ERR_ARG;
  PTN_COUNT(1);
  expand_b_kernel<<<grid_for(N * K), 256, 0, ptn_stream(stream)>>>(
      static_cast<const double2*>(d->src), nm, km, N, K, d->ld, d->conj, d->levels,
      static_cast<__nv_bfloat16*>(d->dst));
  return ptn_launch_status();
}
