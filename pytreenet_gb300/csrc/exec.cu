// Native executor for contraction chains and Krylov steps.
//
// A plan (a chain of strided contractions, or of tensor-core GEMMs with their
// operand conversions) is a fixed list of descriptors whose operand pointers
// are only known when the plan runs (the Krylov vector in and out, workspace
// slots that may have moved). ptn_exec_ops patches those pointers from a small
// table and issues every launch from C++, so a host language pays one foreign
// call per matvec instead of one per kernel. ptn_krylov_gs_step does the same
// for the vector work of one Lanczos/Arnoldi step.
#include "ptn_common.cuh"

extern "C" int ptn_exec_ops(const ptn_exec_op* ops, int32_t nops, void* const* ptrs, int32_t nptrs,
                            void* stream) {
  if (!ops || nops < 0 || (nops > 0 && (!ptrs || nptrs < 1))) return PTN_ERR_ARG;
  for (int32_t i = 0; i < nops; ++i) {
    const ptn_exec_op& op = ops[i];
    if (!op.desc || op.a < 0 || op.a >= nptrs || op.b < -1 || op.b >= nptrs || op.c < 0 || op.c >= nptrs ||
        op.d < -1 || op.d >= nptrs)
      return PTN_ERR_ARG;
    int st;
    switch (op.kind) {
      case PTN_OP_ZCONTRACT: {
        ptn_contract_desc d = *static_cast<const ptn_contract_desc*>(op.desc);
        d.A = ptrs[op.a];
        d.B = op.b >= 0 ? ptrs[op.b] : nullptr;
        d.C = ptrs[op.c];
        st = ptn_zcontract(&d, stream);
        break;
      }
      case PTN_OP_CGEMM: {
        ptn_cgemm_desc d = *static_cast<const ptn_cgemm_desc*>(op.desc);
        d.A = ptrs[op.a];
        d.Bx = op.b >= 0 ? ptrs[op.b] : nullptr;
        d.C = ptrs[op.c];
        if (op.d >= 0) d.partial = ptrs[op.d];
        st = ptn_cgemm_bf16x3(&d, stream);
        break;
      }
      case PTN_OP_TO_PLANES:
      case PTN_OP_EXPAND_B: {
        ptn_convert_desc d = *static_cast<const ptn_convert_desc*>(op.desc);
        d.src = ptrs[op.a];
        d.dst = ptrs[op.c];
        st = op.kind == PTN_OP_TO_PLANES ? ptn_to_planes(&d, stream) : ptn_expand_b(&d, stream);
        break;
      }
      default:
        return PTN_ERR_ARG;
    }
    if (st != PTN_OK) return st;
  }
  return PTN_OK;
}

int ptn_gs_step_passes(const void* Q, int64_t ldq, int32_t nq, void* w, int64_t n, void* h, void* partial,
                       double* norms, void* qnext, void* stream);

extern "C" int ptn_krylov_gs_step(const void* Q, int64_t ldq, int32_t nq, void* w, int64_t n, void* h,
                                  void* partial, double* norms, void* qnext, void* stream) {
  if (!Q || !w || !h || !partial || !norms || nq < 1 || n < 1 || ldq < n) return PTN_ERR_ARG;
  int st = ptn_gs_step_passes(Q, ldq, nq, w, n, h, partial, norms, qnext, stream);
  if (st != PTN_ERR_UNSUPPORTED) return st;
  st = ptn_dznrm2(w, n, norms, partial, stream);
  if (st != PTN_OK) return st;
  double2* h1 = static_cast<double2*>(h);
  double2* h2 = h1 + nq;
  for (double2* hp : {h1, h2}) {
    st = ptn_zdot_multi(Q, ldq, nq, w, n, hp, 0, partial, stream);
    if (st != PTN_OK) return st;
    st = ptn_zaxpy_multi(Q, ldq, nq, hp, w, n, stream);
    if (st != PTN_OK) return st;
  }
  st = ptn_dznrm2(w, n, norms + 1, partial, stream);
  if (st != PTN_OK) return st;
  if (qnext) st = ptn_zscal_inv(w, norms + 1, qnext, n, stream);
  return st;
}
