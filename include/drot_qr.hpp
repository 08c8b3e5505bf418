// drot_qr.hpp -- drop-in replacement of the reference's core/drot_qr.hpp.
//
// Same template names and signatures as WangZesen/Regularized-DROT
// core/drot_qr.hpp, forwarding to the C ABI of libdrot_gb300.so
// (drot_gb300.h).  Link with -ldrot_gb300.  Only T = float exists (the
// reference's only instantiation).
//
//   quadratic_regularizer_drot<T>         core/drot_qr.hpp:159-234
//   _q_get_work_size_update_x             core/drot_qr.hpp:236-239
//   quadratic_regularizer_drot_wrapper<T> core/drot_qr.hpp:241-393
//
// Differences a caller can observe: errors are reported (the reference
// ignores them) -- the device loop returns silently with *n_iter == -1 on
// failure and the wrapper returns NULL; drot_last_status() gives the code.
#ifndef DROT_GB300_QR_HPP_
#define DROT_GB300_QR_HPP_

#include <cuda_runtime.h>

#include <type_traits>

#include "drot_gb300.h"

// Columns-per-block heuristic (core/drot_qr.hpp:236-239); callers size the
// reference's partial-sum buffers with it.
inline int _q_get_work_size_update_x(int n_rows, int n_cols) {
  return drot_q_get_work_size_update_x(n_rows, n_cols);
}

namespace drot_compat {

// Scratch for the solve: the caller's row_sum_1 buffer (n_rows *
// ceil(n_cols / work_size) elements in the reference's sizing) when it is
// large enough, otherwise a temporary device allocation.
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  bool owned = false;
  Scratch(void* candidate, size_t candidate_bytes, size_t need) {
    if (candidate && candidate_bytes >= need && (((size_t)candidate) & 255u) == 0) {
      ptr = candidate;
      bytes = candidate_bytes;
    } else if (need > 0 && cudaMalloc(&ptr, need) == cudaSuccess) {
      bytes = need;
      owned = true;
    }
  }
  ~Scratch() {
    if (owned) cudaFree(ptr);
  }
};

}  // namespace drot_compat

// Device-pointer solve loop.  x, a, b, phi1, phi2 and aux[4] (alpha) hold the
// initial state (warm or cold start, prepared by the caller as in the
// reference) and receive the final state; *n_iter and *objective are set as
// the reference sets them.  row_sum, row_sum_2, col_sum, col_sum_1,
// col_sum_2 and aux[0..3] are not used; row_sum_1 serves as scratch when it
// is large enough.  Runs on the legacy default stream and returns when the
// solve has finished.
template <typename T>
void quadratic_regularizer_drot(const T* c, const T* p, const T* q, const int n_rows,
                                const int n_cols, const T step_size, const T scale,
                                const T r_weight, const int max_iters, const T eps,
                                const int work_size_update_x, T* x, T* a, T* row_sum,
                                T* row_sum_1, T* row_sum_2, T* b, T* col_sum, T* col_sum_1,
                                T* col_sum_2, T* phi1, T* phi2, T* aux, int* _n_iter,
                                T* _objective) {
  static_assert(std::is_same<T, float>::value, "the GB300 solver is FP32");
  (void)r_weight; (void)row_sum; (void)row_sum_2; (void)col_sum; (void)col_sum_1;
  (void)col_sum_2;
  const int ws = work_size_update_x > 0 ? work_size_update_x : 1;
  const size_t have = sizeof(T) * (size_t)n_rows * (size_t)((n_cols + ws - 1) / ws);
  drot_compat::Scratch scratch(row_sum_1, have, drot_qr_workspace_bytes(n_rows, n_cols));
  drot_result res;
  const int rc = scratch.ptr
      ? drot_qr_solve(c, p, q, n_rows, n_cols, step_size, scale, max_iters, eps, x, a, b, phi1,
                      phi2, aux + 4, scratch.ptr, scratch.bytes, &res, nullptr)
      : DROT_ERR_CUDA;
  if (rc != DROT_OK) {
    *_n_iter = -1;
    return;
  }
  *_n_iter = res.n_iter;
  if (res.objective_valid) *_objective = res.objective;
}

// Host-buffer wrapper: allocation, copies, warm or cold start, solve, copy
// back (core/drot_qr.hpp:241-393).  Returns a malloc'd column-major X when
// return_x, else NULL.
template <typename T>
T* quadratic_regularizer_drot_wrapper(const T* _c, const T* _p, const T* _q, const int n_rows,
                                      const int n_cols, const T step_size, const T r_weight,
                                      const int max_iters, const T eps, float* dur_in_ms,
                                      float* prep_dur_in_ms, int* _n_iter, T* _objective,
                                      bool use_warmup_init, bool return_x) {
  static_assert(std::is_same<T, float>::value, "the GB300 solver is FP32");
  return drot_qr_wrapper(_c, _p, _q, n_rows, n_cols, step_size, r_weight, max_iters, eps,
                         dur_in_ms, prep_dur_in_ms, _n_iter, _objective,
                         use_warmup_init ? 1 : 0, return_x ? 1 : 0);
}

#endif  // DROT_GB300_QR_HPP_
