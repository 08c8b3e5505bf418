/*
 * drot_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle), never shipped.
 *
 * A plain-C CPU restatement of the reference DROT hot path
 * (WangZesen/Regularized-DROT, core/drot_qr.hpp, core/drot_glr.hpp,
 * core/kernel_qr.hpp, core/kernel_glr.hpp, pytorch/src/qr_drot_cuda_kernel.cu,
 * pytorch/src/glr_drot_cuda_kernel.cu).
 * It is the checker for the CUDA solver: tests, the smoke check and the CPU
 * baseline leg of the benchmark call it; the solver library never does.
 *
 * Pinned against the reference's own numpy implementation
 * (numpy/npdrot/solver.py, numpy/npdrot/proximal/proximal.py) through the
 * fixtures in tests/golden/, which tests/golden/gen_golden.py produced by
 * importing that code: with the reference's cold start (X = p q^T, which is
 * numpy's init) or, for uniform marginals, its warm start (numpy init = s*1),
 * both implementations run the same iterates.
 *
 * Build: oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off).
 * Host arithmetic is compiled without FP contraction so that the parameter
 * mapping below rounds the way the reference's x86-64 host code does.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------
 * Host-side parameter arithmetic of the reference, restated.
 * ------------------------------------------------------------------------- */

/* step_size = rho / (float(n_rows) + float(n_cols))
 * (pytorch/src/qr_drot_cuda_kernel.cu:100, glr_drot_cuda_kernel.cu:255). */
float oracle_step_size(float rho, int nr, int nc) {
  return rho / ((float)nr + (float)nc);
}

/* QR divisor of the PyTorch operator:
 * 1 + step_size * r_weight * float(n_rows + n_cols) (qr_drot_cuda_kernel.cu:102). */
float oracle_qr_scale_torch(float s, float r, int nr, int nc) {
  float t = s * r;
  t = t * (float)(nr + nc);
  return 1.0f + t;
}

/* QR divisor of the C++ wrapper:
 * 1 + step_size * T(n_rows + n_cols) * r_weight (drot_qr.hpp:262). */
float oracle_qr_scale_wrapper(float s, float r, int nr, int nc) {
  float t = s * (float)(nr + nc);
  t = t * r;
  return 1.0f + t;
}

/* GL threshold of the PyTorch operator:
 * r_weight * sqrt(n_rows / NGROUPS), integer division inside the sqrt
 * (glr_drot_cuda_kernel.cu:257). */
float oracle_gl_lambda_torch(float r, int nr, int G) {
  return (float)((double)r * sqrt((double)(nr / G)));
}

/* GL threshold of the C++ wrapper:
 * r_weight / sqrt(n_rows / NGROUPS) (drot_glr.hpp:385). */
float oracle_gl_lambda_wrapper(float r, int nr, int G) {
  return (float)((double)r / sqrt((double)(nr / G)));
}

/* Group row boundaries.  The reference picks the single-pass kernel when
 * ceil(n_rows / G) <= 256 (drot_glr.hpp:280, param_glr.hpp:31-32) and that
 * kernel rounds with +0.49 (kernel_glr.hpp:79-80); the multi-pass kernels
 * round with +0.49999 (kernel_glr.hpp:185-186, 344-345).  Both compute
 * float(n_rows) / G * float(k) in float and add the double constant. */
void oracle_group_bounds(int nr, int G, int *bounds) {
  const int small = ((nr + G - 1) / G) <= 256;
  const double off = small ? 0.49 : 0.49999;
  const float per = (float)nr / (float)G;
  for (int k = 0; k <= G; ++k) {
    const float f = per * (float)k;
    bounds[k] = (int)((double)f + off);
  }
}

/* Warm start (drot_qr.hpp:321-346, qr_drot_cuda_kernel.cu:107-133, and the
 * same lines in the GL files).  Writes the five constants
 * {phi1, phi2, a, b, alpha}; X starts at zero. */
void oracle_warm_start(float s, int nr, int nc, float *out5) {
  const float n = (float)nr;
  const float m = (float)nc;
  float k = 1.0f * s;
  k = k * n;
  k = k * m;
  k = k - 2.0f;
  float t = (k + 2.0f) / n;
  out5[0] = t / (m + n);
  t = (k + 2.0f) / m;
  out5[1] = t / (m + n);
  out5[2] = (k + 1.0f) / n;
  out5[3] = (k + 1.0f) / m;
  out5[4] = k + 1.0f;
}

/* ---------------------------------------------------------------------------
 * Solve loops in FP32 (reference arithmetic) and FP64.
 * ------------------------------------------------------------------------- */

#define REAL float
#define RFMA fmaf
#define RSQRT sqrtf
#define SFX _f32
#include "drot_oracle_impl.h"
#undef REAL
#undef RFMA
#undef RSQRT
#undef SFX

#define REAL double
#define RFMA fma
#define RSQRT sqrt
#define SFX _f64
#include "drot_oracle_impl.h"
#undef REAL
#undef RFMA
#undef RSQRT
#undef SFX

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
