/*
 * drot_oracle_impl.h -- TEST INFRASTRUCTURE ONLY (the oracle), never shipped.
 *
 * Body of the CPU restatement of the reference DROT solve loops.  It is
 * included twice by drot_oracle.c: once with REAL=float (the reference's own
 * arithmetic: FP32 element operations with the same fused multiply-adds the
 * reference kernels compile to, and the FP64 promotions that its double
 * literals cause), once with REAL=double (the FP64 oracle).
 *
 * Sums (row sums, column sums, the total mass, the objective, the residual)
 * are accumulated in FP64 and rounded to REAL where the reference keeps them
 * in a REAL-typed buffer.  The reference accumulates them with float atomics
 * in an unspecified order, so no CPU order can reproduce its bits; FP64
 * accumulation keeps the oracle within an ulp of the exact sum.
 *
 * Expected macros: REAL, RFMA, RSQRT, SFX (name suffix).
 */

#define OR_CAT2(a, b) a##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR_NAME(base) OR_CAT(base, SFX)

/* Dual/aux update shared by both regularisers.
 *   kernel_qr.hpp:405-461 (quadratic_regularizer_update_aux),
 *   kernel_qr.hpp:463-467 (update_alpha),
 *   kernel_glr.hpp:461-526 (group_lasso_regularizer_update_aux, update_alpha).
 * Returns the squared absolute marginal residual ||X1-p||^2 + ||X^T1-q||^2. */
static double OR_NAME(aux_update)(int nr, int nc, const double *rowsum,
                                  const double *colsum, double total,
                                  const REAL *p, const REAL *q, REAL *a,
                                  REAL *b, REAL *phi1, REAL *phi2,
                                  REAL *alpha) {
  /* x_sum lives in a REAL buffer (aux[1]) in the reference. */
  const REAL sigma = (REAL)total;
  /* gamma = (2*(x_sum - 1.) - alpha) / (n_rows + n_cols): the double literal
   * promotes the whole expression, the result is stored in a REAL. */
  const REAL gamma =
      (REAL)((2.0 * ((double)sigma - 1.0) - (double)(*alpha)) / (double)(nr + nc));
  double res = 0.0;
  for (int i = 0; i < nr; ++i) {
    const REAL rs = (REAL)rowsum[i] - p[i];
    const REAL ab = a[i] - rs;
    phi1[i] = ((ab - rs) + gamma) / (REAL)nc;
    a[i] = ab;
    res += (double)rs * (double)rs;
  }
  for (int j = 0; j < nc; ++j) {
    const REAL cs = (REAL)colsum[j] - q[j];
    const REAL ab = b[j] - cs;
    phi2[j] = ((ab - cs) + gamma) / (REAL)nr;
    b[j] = ab;
    res += (double)cs * (double)cs;
  }
  /* alpha = (alpha + 1.) - x_sum, promoted to double, stored as REAL. */
  *alpha = (REAL)(((double)(*alpha) + 1.0) - (double)sigma);
  return res;
}

/* Quadratic-regularised DROT solve loop.
 *   Loop, stop test and iteration count: drot_qr.hpp:159-234.
 *   Even step (reads C, stores X^ - sC): kernel_qr.hpp:171-278 / 50-113.
 *   Odd step (C already folded in):       kernel_qr.hpp:280-376 / 115-169.
 *   Final unfold on convergence:          kernel_qr.hpp:469-482 (fix_x).
 * X is column-major with leading dimension nr.  x, a, b, phi1, phi2 and
 * alpha hold the initial state on entry and the final state on exit.
 * *objective is written on every even iteration (as the reference does) and
 * left untouched when no even iteration runs. */
int OR_NAME(oracle_qr_solve)(const REAL *c, const REAL *p, const REAL *q,
                             int nr, int nc, REAL s, REAL kappa,
                             int max_iters, REAL eps, REAL *x, REAL *a,
                             REAL *b, REAL *phi1, REAL *phi2, REAL *alpha,
                             int *n_iter, REAL *objective, double *residual,
                             int nthreads) {
  double *rowsum = (double *)calloc((size_t)nr, sizeof(double));
  double *colsum = (double *)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  int nt = nthreads > 0 ? nthreads : 1;
  double *rowpart = (double *)calloc((size_t)nr * (size_t)nt, sizeof(double));
  double *objpart = (double *)calloc((size_t)nt, sizeof(double));
  if (!rowsum || !colsum || !rowpart || !objpart) {
    free(rowsum); free(colsum); free(rowpart); free(objpart);
    return -1;
  }
  int it = 0;
  double last_res = -1.0;
  while (it < max_iters) {
    const int even = (it % 2) == 0;
    memset(rowpart, 0, sizeof(double) * (size_t)nr * (size_t)nt);
    memset(objpart, 0, sizeof(double) * (size_t)nt);
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 0; j < nc; ++j) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      double *rp = rowpart + (size_t)tid * (size_t)nr;
      const REAL f2 = phi2[j];
      REAL *xc = x + (size_t)j * (size_t)nr;
      const REAL *cc = c + (size_t)j * (size_t)nr;
      double cs = 0.0, ob = 0.0;
      for (int i = 0; i < nr; ++i) {
        REAL v = (xc[i] + phi1[i]) + f2;
        REAL cv = 0;
        if (even) {
          cv = cc[i];
          v = RFMA(-s, cv, v);
        }
        /* max(v, 0.) / scale: exact in double, correctly rounded to REAL. */
        const REAL y = (v > (REAL)0 ? v : (REAL)0) / kappa;
        xc[i] = even ? RFMA(-s, cv, y) : y;
        rp[i] += (double)y;
        cs += (double)y;
        if (even) ob += (double)y * (double)cv;
      }
      colsum[j] = cs;
      objpart[tid] += ob;
    }
    double total = 0.0, obj = 0.0;
    for (int i = 0; i < nr; ++i) {
      double acc = 0.0;
      for (int t = 0; t < nt; ++t) acc += rowpart[(size_t)t * (size_t)nr + i];
      rowsum[i] = acc;
    }
    for (int j = 0; j < nc; ++j) total += colsum[j];
    for (int t = 0; t < nt; ++t) obj += objpart[t];
    const double res2 = OR_NAME(aux_update)(nr, nc, rowsum, colsum, total, p, q,
                                            a, b, phi1, phi2, alpha);
    if (even) {
      last_res = sqrt(res2);
      *objective = (REAL)obj;
      if (last_res < (double)eps) {
        /* fix_x: X <- max(X + sC, 0.) */
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int j = 0; j < nc; ++j) {
          REAL *xc = x + (size_t)j * (size_t)nr;
          const REAL *cc = c + (size_t)j * (size_t)nr;
          for (int i = 0; i < nr; ++i) {
            const REAL v = RFMA(s, cc[i], xc[i]);
            xc[i] = v > (REAL)0 ? v : (REAL)0;
          }
        }
        break;
      }
    }
    ++it;
  }
  /* drot_qr.hpp:233 reports n_iter + 1 (so max_iters + 1 without convergence). */
  *n_iter = it + 1;
  if (residual) *residual = last_res;
  free(rowsum); free(colsum); free(rowpart); free(objpart);
  return 0;
}

/* Group-lasso-regularised DROT solve loop.
 *   Loop, stop test (<= eps, every iteration): drot_glr.hpp:242-355.
 *   Prox + group shrink: kernel_glr.hpp:59-161 (groups <= 256 rows) and
 *   kernel_glr.hpp:163-399 (update_x, update_norm, apply_norm).
 * bounds[0..G] are the group row boundaries (see oracle_group_bounds).
 * norm_eps is the constant added to the group norm in the shrink factor
 * (1e-9 in the reference kernels; 0 reproduces the numpy prox). */
int OR_NAME(oracle_gl_solve)(const REAL *c, const REAL *p, const REAL *q,
                             int nr, int nc, int G, const int *bounds, REAL s,
                             REAL lambda, double norm_eps, int max_iters,
                             REAL eps, REAL *x, REAL *a, REAL *b, REAL *phi1,
                             REAL *phi2, REAL *alpha, int *n_iter,
                             REAL *objective, double *residual, int nthreads) {
  double *rowsum = (double *)calloc((size_t)nr, sizeof(double));
  double *colsum = (double *)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  int nt = nthreads > 0 ? nthreads : 1;
  double *rowpart = (double *)calloc((size_t)nr * (size_t)nt, sizeof(double));
  double *objpart = (double *)calloc((size_t)nt, sizeof(double));
  if (!rowsum || !colsum || !rowpart || !objpart) {
    free(rowsum); free(colsum); free(rowpart); free(objpart);
    return -1;
  }
  int it = 0;
  double last_res = -1.0;
  while (it < max_iters) {
    memset(rowpart, 0, sizeof(double) * (size_t)nr * (size_t)nt);
    memset(objpart, 0, sizeof(double) * (size_t)nt);
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 0; j < nc; ++j) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      double *rp = rowpart + (size_t)tid * (size_t)nr;
      const REAL f2 = phi2[j];
      REAL *xc = x + (size_t)j * (size_t)nr;
      const REAL *cc = c + (size_t)j * (size_t)nr;
      double cs = 0.0, ob = 0.0;
      for (int g = 0; g < G; ++g) {
        const int i0 = bounds[g], i1 = bounds[g + 1];
        double ns = 0.0;
        for (int i = i0; i < i1; ++i) {
          const REAL v = RFMA(-s, cc[i], (xc[i] + phi1[i]) + f2);
          const REAL y = v > (REAL)0 ? v : (REAL)0;
          xc[i] = y;
          ns += (double)y * (double)y;
        }
        /* scale = max(1. - lambda / (sqrt(norm) + 1e-9), 0.): the norm is a
         * REAL sum, its square root a REAL sqrt, the rest in double. */
        const REAL nsr = (REAL)ns;
        const double sh = 1.0 - (double)lambda / ((double)RSQRT(nsr) + norm_eps);
        const REAL scale = (REAL)(sh > 0.0 ? sh : 0.0);
        for (int i = i0; i < i1; ++i) {
          const REAL xn = xc[i] * scale;
          xc[i] = xn;
          rp[i] += (double)xn;
          cs += (double)xn;
          ob += (double)xn * (double)cc[i];
        }
      }
      colsum[j] = cs;
      objpart[tid] += ob;
    }
    double total = 0.0, obj = 0.0;
    for (int i = 0; i < nr; ++i) {
      double acc = 0.0;
      for (int t = 0; t < nt; ++t) acc += rowpart[(size_t)t * (size_t)nr + i];
      rowsum[i] = acc;
    }
    for (int j = 0; j < nc; ++j) total += colsum[j];
    for (int t = 0; t < nt; ++t) obj += objpart[t];
    const double res2 = OR_NAME(aux_update)(nr, nc, rowsum, colsum, total, p, q,
                                            a, b, phi1, phi2, alpha);
    last_res = sqrt(res2);
    *objective = (REAL)obj;
    ++it;
    if (last_res <= (double)eps) break;
  }
  *n_iter = it;
  if (residual) *residual = last_res;
  free(rowsum); free(colsum); free(rowpart); free(objpart);
  return 0;
}

#undef OR_NAME
#undef OR_CAT
#undef OR_CAT2
