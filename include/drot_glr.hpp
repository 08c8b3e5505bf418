// drot_glr.hpp -- drop-in replacement of the reference's core/drot_glr.hpp.
//
// Same template names and signatures as WangZesen/Regularized-DROT
// core/drot_glr.hpp, forwarding to the C ABI of libdrot_gb300.so
// (drot_gb300.h).  Only T = float exists.
//
//   group_lasso_regularizer_drot<T>         core/drot_glr.hpp:242-355
//   _gl_get_work_size_update_x              core/drot_glr.hpp:357-360
//   group_lasso_regularizer_drot_wrapper<T> core/drot_glr.hpp:362-527
//
// Groups are the NGROUPS contiguous row blocks the reference kernels use
// (drot_gl_group_bounds).  On failure the device loop sets *n_iter = -1 and
// the wrapper returns NULL; drot_last_status() gives the code.
#ifndef DROT_GB300_GLR_HPP_
#define DROT_GB300_GLR_HPP_

#include <cuda_runtime.h>

#include <type_traits>

#include "drot_gb300.h"
#include "drot_qr.hpp"  // drot_compat::Scratch

inline int _gl_get_work_size_update_x(int n_rows, int n_cols) {
  return drot_gl_get_work_size_update_x(n_rows, n_cols);
}

// Device-pointer solve loop (core/drot_glr.hpp:242-355).  lambda is the
// shrink threshold itself (the reference's wrapper derives it from r_weight).
// x, a, b, phi1, phi2 and aux[4] (alpha) carry the state in and out; the
// other buffers are not used except row_sum_1, which serves as scratch when
// it is large enough.
template <typename T>
void group_lasso_regularizer_drot(const T* c, const T* p, const T* q, const int n_rows,
                                  const int n_cols, const int NGROUPS, const T step_size,
                                  const T lambda, const int max_iters, const T eps,
                                  const int work_size_update_x, T* x, T* a, T* row_sum,
                                  T* row_sum_1, T* row_sum_2, T* b, T* col_sum, T* col_sum_1,
                                  T* col_sum_2, T* col_obj_sum, T* col_norm_sum, T* group_sum,
                                  T* group_obj_sum, T* group_norm_sum, T* phi1, T* phi2, T* aux,
                                  int* _n_iter, T* _objective) {
  static_assert(std::is_same<T, float>::value, "the GB300 solver is FP32");
  (void)row_sum; (void)row_sum_2; (void)col_sum; (void)col_sum_1; (void)col_sum_2;
  (void)col_obj_sum; (void)col_norm_sum; (void)group_sum; (void)group_obj_sum;
  (void)group_norm_sum;
  const int ws = work_size_update_x > 0 ? work_size_update_x : 1;
  const size_t have = sizeof(T) * (size_t)n_rows * (size_t)((n_cols + ws - 1) / ws);
  drot_compat::Scratch scratch(row_sum_1, have, drot_gl_workspace_bytes(n_rows, n_cols, NGROUPS));
  drot_result res;
  const int rc = scratch.ptr
      ? drot_gl_solve(c, p, q, n_rows, n_cols, NGROUPS, step_size, lambda, max_iters, eps, x, a,
                      b, phi1, phi2, aux + 4, scratch.ptr, scratch.bytes, &res, nullptr)
      : DROT_ERR_CUDA;
  if (rc != DROT_OK) {
    *_n_iter = -1;
    return;
  }
  *_n_iter = res.n_iter;
  if (res.objective_valid) *_objective = res.objective;
}

// Host-buffer wrapper (core/drot_glr.hpp:362-527); lambda = r_weight /
// sqrt(n_rows / NGROUPS) as in the reference wrapper.
template <typename T>
T* group_lasso_regularizer_drot_wrapper(const T* _c, const T* _p, const T* _q, const int n_rows,
                                        const int n_cols, const int NGROUPS, const T step_size,
                                        const T r_weight, const int max_iters, const T eps,
                                        float* dur_in_ms, float* prep_dur_in_ms, int* _n_iter,
                                        T* _objective, bool use_warmup_init, bool return_x) {
  static_assert(std::is_same<T, float>::value, "the GB300 solver is FP32");
  return drot_gl_wrapper(_c, _p, _q, n_rows, n_cols, NGROUPS, step_size, r_weight, max_iters,
                         eps, dur_in_ms, prep_dur_in_ms, _n_iter, _objective,
                         use_warmup_init ? 1 : 0, return_x ? 1 : 0);
}

#endif  // DROT_GB300_GLR_HPP_
