// drot_solve_ldu.cu -- the single-barrier (LDU) instances of the solve kernel
// (drot_kernels.cuh), compiled apart from drot_api.cu so that the two
// translation units build in parallel.
#include "drot_kernels.cuh"

namespace drot {

typedef void (*SolveFn)(const SolveParams);

template <int MODE, typename CT>
static SolveFn ldu_kv(int kv) {
  if (kv == 1) return drot_solve_kernel<MODE, 4, 1, false, CT, true>;
  if (kv == 2) return drot_solve_kernel<MODE, 4, 2, false, CT, true>;
  if (kv == 4) return drot_solve_kernel<MODE, 4, 4, false, CT, true>;
  if constexpr (MODE == MODE_GL) {
    if (kv == 8) return drot_solve_kernel<MODE, 4, 8, false, CT, true>;
  }
  return nullptr;
}

// LDU instance for (mode, vectors per lane, cost type): register path,
// 4-wide vectors.  nullptr when there is none.
SolveFn solve_kernel_ldu(int mode, int kv, bool bf16) {
  if (mode == MODE_QR) return bf16 ? ldu_kv<MODE_QR, __nv_bfloat16>(kv) : ldu_kv<MODE_QR, float>(kv);
  if (mode == MODE_GL) return bf16 ? ldu_kv<MODE_GL, __nv_bfloat16>(kv) : ldu_kv<MODE_GL, float>(kv);
  return nullptr;
}

}  // namespace drot
