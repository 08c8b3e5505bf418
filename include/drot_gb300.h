/*
 * drot_gb300.h -- C ABI of the GB300 DROT solver (libdrot_gb300.so).
 *
 * Douglas-Rachford optimal transport with quadratic (QR) or group-lasso (GL)
 * regularisation, as solved by WangZesen/Regularized-DROT.  Every entry point
 * below replaces one interface of that reference (cited per declaration).
 *
 * Layout: C, X are column-major n_rows x n_cols float32 matrices (element
 * (i, j) at j*n_rows + i), i.e. the reference's PyTorch [n_cols, n_rows]
 * contiguous tensor.  p has n_rows entries, q has n_cols entries.
 *
 * Errors are returned as drot_status codes; nothing is printed.  Device entry
 * points take an explicit cudaStream_t (0 = legacy default stream, as the
 * reference uses) and a caller-owned workspace whose size the matching
 * *_workspace_bytes function returns for the current device.
 */
#ifndef DROT_GB300_H
#define DROT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *drot_stream_t; /* == cudaStream_t */

typedef enum {
  DROT_OK = 0,
  DROT_ERR_INVALID_ARG = 1,     /* bad shape, null pointer, bad parameter */
  DROT_ERR_CUDA = 2,            /* a CUDA runtime call failed */
  DROT_ERR_BARRIER_TIMEOUT = 3, /* a device-side grid barrier hit its time limit */
  DROT_ERR_UNSUPPORTED = 4,     /* shape outside what the solver plans for */
  DROT_ERR_WORKSPACE = 5        /* workspace too small or misaligned */
} drot_status;

/* Result of one solve, copied back to the host by the blocking entry points. */
typedef struct {
  int n_iter;          /* the reference's count: QR = index of the last
                          iteration + 1 (max_iters + 1 without convergence,
                          core/drot_qr.hpp:233); GL = iterations run
                          (core/drot_glr.hpp:354) */
  int iters_run;       /* iterations actually executed */
  int converged;       /* 1 if the stop test passed */
  int status;          /* drot_status of the device run */
  int objective_valid; /* 0 when no objective-bearing iteration ran */
  float objective;     /* <C, X> of the last even QR / last GL iteration */
  double objective_f64;/* same, FP64 accumulation */
  double residual;     /* absolute marginal residual ||X1-p, X^T1-q||_2 at the
                          last stop test (-1 if none ran) */
  double phase_ms[4];  /* device time of the solve split by stage, summed over
                          iterations: fused X-update, first grid barrier,
                          dual update, second grid barrier + stop test */
} drot_result;

/* Storage types of the cost matrix C for the *_ex entry points.  Iterates
 * and sums stay FP32; a BF16-stored C is widened exactly to FP32 in the
 * kernel, so the solver solves the problem whose cost is the BF16-rounded C
 * (10 bytes per element on iterations that read C instead of 12). */
#define DROT_C_F32 0
#define DROT_C_BF16 1

/* Text for a drot_status code. */
const char *drot_status_string(int status);

/* Status of the last host-buffer wrapper call on this thread
 * (drot_qr_wrapper / drot_gl_wrapper return a pointer, not a status). */
int drot_last_status(void);

/* ---------------------------------------------------------------------------
 * Parameter helpers
 * ------------------------------------------------------------------------- */

/* Columns-per-block heuristic of the reference, kept for callers that size
 * their own buffers with it: core/drot_qr.hpp:236-239 (_q_get_work_size_update_x)
 * and core/drot_glr.hpp:357-360 (_gl_get_work_size_update_x). */
int drot_q_get_work_size_update_x(int n_rows, int n_cols);
int drot_gl_get_work_size_update_x(int n_rows, int n_cols);

/* Group row boundaries bounds[0..n_groups] that the reference GL kernels use
 * for NGROUPS contiguous classes (core/kernel_glr.hpp:79-80, 185-186, with
 * the kernel choice of core/drot_glr.hpp:280). */
int drot_gl_group_bounds(int n_rows, int n_groups, int *bounds);

/* Launch shape of the single-instance solver (drot_*_solve and the entry
 * points built on them).  Replaces the reference's columns-per-block
 * heuristic (core/drot_qr.hpp:236-239) where a caller -- normally the
 * autotuner reg_drot.tune, which times the candidates on the caller's data
 * -- pins one; zero fields keep the planner's choice.
 *   vectors_per_lane  QR: cap 1, 2 or 4 (128-bit vectors per lane: 128-,
 *                     256- or 512-row bands); GL: 1, 2, 4 or 8
 *   warps_per_cta     4..16 (default 8 on the register path, 16 on the ring)
 *   data_path         0 register loads, 1 TMA bulk-copy ring (FP32 C with
 *                     16-byte aligned columns; otherwise the register path
 *                     runs with the other fields)
 *   ctas_per_sm       ring only: 1 or 2 CTAs share an SM's shared memory */
typedef struct {
  int vectors_per_lane, warps_per_cta, data_path, ctas_per_sm;
} drot_launch_choice;

/* Pins `choice` for problems of mode (0 QR, 1 GL), shape n_rows x n_cols
 * (n_groups for GL) and cost type c_dtype on the current device; n_rows =
 * n_cols = 0 pins it for every shape of that mode and cost type without an
 * exact entry.  choice == NULL removes the entry.  DROT_ERR_UNSUPPORTED
 * when the shape cannot be planned with it.  Workspace sizes queried after
 * the call include the pinned plan. */
int drot_set_launch_choice(int mode, int n_rows, int n_cols, int n_groups, int c_dtype,
                           const drot_launch_choice *choice);
int drot_clear_launch_choices(void);

/* Initial state.  warm != 0: the reference warm start (X = 0 and constant
 * phi1, phi2, a, b, alpha from step_size; core/drot_qr.hpp:321-346,
 * pytorch/src/qr_drot_cuda_kernel.cu:107-133).  warm == 0: the cold start
 * X = p q^T, a = b = phi = 0, alpha = 0 (core/kernel_qr.hpp:7-40,
 * core/drot_qr.hpp:308-320).  All pointers are device pointers. */
int drot_init_state(int n_rows, int n_cols, float step_size, int warm,
                    const float *p, const float *q, float *x, float *a,
                    float *b, float *phi1, float *phi2, float *alpha,
                    drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * Device-pointer solve loops (state in/out)
 * ------------------------------------------------------------------------- */

/* Scratch bytes for drot_qr_solve / drot_gl_solve on the current device. */
size_t drot_qr_workspace_bytes(int n_rows, int n_cols);
size_t drot_gl_workspace_bytes(int n_rows, int n_cols, int n_groups);

/* QR solve loop.  Replaces quadratic_regularizer_drot<float>
 * (core/drot_qr.hpp:159-234): same parameters (step_size, scale = the QR
 * divisor, max_iters, eps on the absolute residual), same state arrays x, a,
 * b, phi1, phi2 and alpha (aux[4] there) read on entry and written on exit,
 * same stop rule (even iterations, residual < eps, X unfolded on
 * convergence).  The reference's partial-sum buffers are replaced by
 * `workspace`.  With result != NULL the call waits for the stream and fills
 * *result; with result == NULL it returns after enqueueing the work and the
 * result can be read later with drot_read_result(workspace, ...). */
int drot_qr_solve(const float *c, const float *p, const float *q, int n_rows,
                  int n_cols, float step_size, float scale, int max_iters,
                  float eps, float *x, float *a, float *b, float *phi1,
                  float *phi2, float *alpha, void *workspace,
                  size_t workspace_bytes, drot_result *result,
                  drot_stream_t stream);

/* GL solve loop.  Replaces group_lasso_regularizer_drot<float>
 * (core/drot_glr.hpp:242-355): groups are the n_groups contiguous row blocks
 * of drot_gl_group_bounds, lambda is the threshold used by the shrink
 * max(1 - lambda/(||Y_g|| + 1e-9), 0), the stop test runs every iteration
 * with residual <= eps. */
int drot_gl_solve(const float *c, const float *p, const float *q, int n_rows,
                  int n_cols, int n_groups, float step_size, float lambda,
                  int max_iters, float eps, float *x, float *a, float *b,
                  float *phi1, float *phi2, float *alpha, void *workspace,
                  size_t workspace_bytes, drot_result *result,
                  drot_stream_t stream);

/* The loop of the reference's numpy solvers (numpy/npdrot/solver.py:7-189:
 * regdrot with trace_nonnegative_quad_prox or trace_nonnegative_l1l2_prox)
 * on the device.  mode 0: QR with divisor scale_or_lambda (= 1 + step*reg);
 * the stop test runs on every iteration with residual <= eps, and X is
 * returned unfolded whatever the last step.  mode 1: GL with threshold
 * scale_or_lambda (= reg*step) over the caller's contiguous row groups
 * [bounds[g], bounds[g+1]) (bounds[0] = 0, bounds[n_groups] = n_rows,
 * increasing; numpy's `groups` pairs).  State in / state out as in
 * drot_qr_solve; the numpy loop's final extra prox is one more call with
 * max_iters = 1. */
size_t drot_np_workspace_bytes(int mode, int n_rows, int n_cols, int n_groups,
                               const int *bounds);
int drot_np_solve(int mode, const void *c, int c_dtype, const float *p,
                  const float *q, int n_rows, int n_cols, int n_groups,
                  const int *bounds, float step_size, float scale_or_lambda,
                  int max_iters, float eps, float *x, float *a, float *b,
                  float *phi1, float *phi2, float *alpha, void *workspace,
                  size_t workspace_bytes, drot_result *result,
                  drot_stream_t stream);

/* drot_qr_solve / drot_gl_solve with the cost matrix stored as c_dtype
 * (DROT_C_F32 or DROT_C_BF16).  No counterpart in the reference (its C is
 * float only); the FP32 case is exactly drot_qr_solve / drot_gl_solve. */
int drot_qr_solve_ex(const void *c, int c_dtype, const float *p, const float *q,
                     int n_rows, int n_cols, float step_size, float scale,
                     int max_iters, float eps, float *x, float *a, float *b,
                     float *phi1, float *phi2, float *alpha, void *workspace,
                     size_t workspace_bytes, drot_result *result,
                     drot_stream_t stream);
int drot_gl_solve_ex(const void *c, int c_dtype, const float *p, const float *q,
                     int n_rows, int n_cols, int n_groups, float step_size,
                     float lambda, int max_iters, float eps, float *x, float *a,
                     float *b, float *phi1, float *phi2, float *alpha,
                     void *workspace, size_t workspace_bytes, drot_result *result,
                     drot_stream_t stream);

/* Copy the result block of the last solve that used `workspace` to the host
 * (waits for `stream`). */
int drot_read_result(const void *workspace, drot_result *result,
                     drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * PyTorch-operator equivalents (device pointers, state kept in the workspace)
 * ------------------------------------------------------------------------- */

/* reg_drot.quadratic_drot (pytorch/src/drot_cuda.cpp:26-40,
 * pytorch/src/qr_drot_cuda_kernel.cu:12-148): step = rho/(n_rows+n_cols),
 * divisor = 1 + step*r_weight*(n_rows+n_cols), warm start, solve into x. */
size_t drot_quadratic_drot_workspace_bytes(int n_rows, int n_cols);
int drot_quadratic_drot(const float *c, const float *p, const float *q,
                        int n_rows, int n_cols, float rho, float r_weight,
                        int max_iters, float eps, float *x, void *workspace,
                        size_t workspace_bytes, drot_result *result,
                        drot_stream_t stream);

/* reg_drot.group_lasso_drot (pytorch/src/drot_cuda.cpp:42-57,
 * pytorch/src/glr_drot_cuda_kernel.cu:13-171): lambda =
 * r_weight*sqrt(n_rows/n_class) with integer division, warm start. */
size_t drot_group_lasso_drot_workspace_bytes(int n_rows, int n_cols, int n_class);
int drot_group_lasso_drot(const float *c, const float *p, const float *q,
                          int n_rows, int n_cols, int n_class, float rho,
                          float r_weight, int max_iters, float eps, float *x,
                          void *workspace, size_t workspace_bytes,
                          drot_result *result, drot_stream_t stream);

/* The operator entry points with the cost stored as c_dtype (DROT_C_F32 or
 * DROT_C_BF16); no counterpart in the reference. */
int drot_quadratic_drot_ex(const void *c, int c_dtype, const float *p,
                           const float *q, int n_rows, int n_cols, float rho,
                           float r_weight, int max_iters, float eps, float *x,
                           void *workspace, size_t workspace_bytes,
                           drot_result *result, drot_stream_t stream);
int drot_group_lasso_drot_ex(const void *c, int c_dtype, const float *p,
                             const float *q, int n_rows, int n_cols, int n_class,
                             float rho, float r_weight, int max_iters, float eps,
                             float *x, void *workspace, size_t workspace_bytes,
                             drot_result *result, drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * Host-buffer wrappers
 * ------------------------------------------------------------------------- */

/* quadratic_regularizer_drot_wrapper<float> (core/drot_qr.hpp:241-393):
 * host C, p, q in; device buffers allocated, inputs copied, solved, freed.
 * Returns a malloc'd host copy of X (column-major) when return_x != 0, else
 * NULL; free it with free() or drot_free_host().  *dur_in_ms is the solve
 * time, *prep_dur_in_ms the allocation + copy + initialisation time (CUDA
 * events, as the reference measures them).  On failure returns NULL and
 * drot_last_status() tells why. */
float *drot_qr_wrapper(const float *c, const float *p, const float *q,
                       int n_rows, int n_cols, float step_size,
                       float r_weight, int max_iters, float eps,
                       float *dur_in_ms, float *prep_dur_in_ms, int *n_iter,
                       float *objective, int use_warmup_init, int return_x);

/* group_lasso_regularizer_drot_wrapper<float> (core/drot_glr.hpp:362-527):
 * as above; lambda = r_weight / sqrt(n_rows / NGROUPS) with integer division
 * (core/drot_glr.hpp:385). */
float *drot_gl_wrapper(const float *c, const float *p, const float *q,
                       int n_rows, int n_cols, int n_groups, float step_size,
                       float r_weight, int max_iters, float eps,
                       float *dur_in_ms, float *prep_dur_in_ms, int *n_iter,
                       float *objective, int use_warmup_init, int return_x);

/* Frees a matrix returned by the wrappers. */
void drot_free_host(float *ptr);

/* ---------------------------------------------------------------------------
 * Solve without any device allocation
 * ------------------------------------------------------------------------- */

/* Bytes of the fixed workspace array of drot_quadratic_drot_noalloc.  Every
 * GPU that loads the library holds this much device memory until exit. */
#define DROT_NOALLOC_WORKSPACE_BYTES (16u << 20)

/* No counterpart in the reference.  Same solve as drot_quadratic_drot (the
 * reg_drot.quadratic_drot operator), for callers that may not allocate
 * device memory when they call it -- e.g. a latency-critical loop, where
 * cudaMalloc/cudaFree would synchronise the device, or a host whose device
 * memory belongs to another allocator.  It allocates nothing: its workspace
 * is a fixed 16 MiB array in the library's device memory (one per GPU),
 * enough for n_rows x n_cols problems whose drot_quadratic_drot_workspace_bytes
 * is at most DROT_NOALLOC_WORKSPACE_BYTES (square problems up to about
 * 35 000); larger problems get DROT_ERR_WORKSPACE and nothing runs.  The
 * caller passes the inputs c, p, q and the output x (device pointers).
 * Every call looks up that array's device address (cudaGetSymbolAddress)
 * with the calling thread's current device; the first call on a device also
 * loads the library's device code there, so make that first call before any
 * stream capture.  All calls on a device share the one array:
 * calls whose work overlaps on the GPU (other streams, other host threads)
 * race and corrupt each other; serialise them.  Each call re-initialises
 * everything it reads from the array. */
int drot_quadratic_drot_noalloc(const float *c, const float *p, const float *q,
                                int n_rows, int n_cols, float rho, float r_weight,
                                int max_iters, float eps, float *x,
                                drot_result *result, drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * Batched quadratic-regularised solves
 *
 * No counterpart in the reference, whose callers solve many instances one at
 * a time (core/multiexp_qr.cu:47-49 calls the wrapper once per repetition;
 * benchmark/utils/compute_w2_dist.py:86 calls reg_drot.quadratic_drot once
 * per problem).  Here many independent instances of different shapes run in
 * ONE persistent cooperative launch: per instance the same iteration, warm
 * start, stop test and n_iter as drot_quadratic_drot, each instance stopping
 * on its own.
 *
 * Flow: drot_batch_plan_create (host, once per set of shapes) ->
 * drot_batch_upload (copies the plan's descriptors into the workspace, once
 * per workspace) -> drot_qr_batch_launch (device work only: no allocation,
 * no host synchronisation, so it can be captured in a CUDA graph and
 * replayed) -> drot_batch_results.
 * ------------------------------------------------------------------------- */

/* One instance.  Its C and X are n_rows x n_cols column-major blocks with
 * leading dimension ld (ld >= n_rows, a multiple of 4), starting at element
 * c_offset of the batch's C buffer and x_offset of its X buffer (multiples of
 * 4); X must hold ld * n_cols elements (the rows past n_rows are zeroed).
 * p and q start at p_offset / q_offset of the batch's p and q buffers.
 * rho, r_weight, eps as in drot_quadratic_drot. */
typedef struct {
  int n_rows, n_cols, ld, pad;
  long long c_offset, x_offset, p_offset, q_offset;
  float rho, r_weight, eps, pad2;
} drot_batch_instance;

/* Per-instance outcome; fields as in drot_result. */
typedef struct {
  int n_iter, iters_run, converged, objective_valid;
  double objective, residual;
} drot_batch_result;

typedef struct drot_batch_plan_s *drot_batch_plan;

/* Builds the tile list of n_inst instances on the current device: tiles of
 * 512 rows x cols_per_tile columns (<= 0: 128), plus the launch shape. */
int drot_batch_plan_create(int n_inst, const drot_batch_instance *inst,
                           int cols_per_tile, drot_batch_plan *plan);
/* The same with the tile height: band_rows 512 (the default; required by
 * drot_qr_batch_launch_points) or 128. */
int drot_batch_plan_create_ex(int n_inst, const drot_batch_instance *inst,
                              int cols_per_tile, int band_rows,
                              drot_batch_plan *plan);
/* Batched group-lasso solves (no counterpart in the reference, whose GL
 * callers loop: core/multiexp_glr.cu).  Per instance: n_groups contiguous
 * row classes with the reference's boundaries (drot_gl_group_bounds),
 * lambda the shrink threshold (the lambda of drot_gl_solve: r_weight *
 * sqrt(n_rows / n_groups) for the PyTorch operator, r_weight /
 * sqrt(n_rows / n_groups) for the C++ wrapper), and the GL loop of
 * drot_gl_solve per instance (core/drot_glr.hpp:242-355: stop on residual
 * <= eps tested every iteration, n_iter = iterations run, X never folded).
 * Groups of at most 4096 rows.  Launched with drot_qr_batch_launch like a
 * QR plan (cost-matrix launches only). */
typedef struct {
  int n_rows, n_cols, ld, n_groups;
  long long c_offset, x_offset, p_offset, q_offset;
  float rho, lambda, eps, pad;
} drot_gl_batch_instance;
int drot_gl_batch_plan_create(int n_inst, const drot_gl_batch_instance *inst,
                              int cols_per_tile, drot_batch_plan *plan);
/* Tile-level shape of the batch plans created after the call (process-wide,
 * no counterpart in the reference; NULL restores the defaults).  A field
 * below 0 keeps its default:
 *   fine_cols          128   columns of the second tile level's tiles
 *   finest_cols         32   columns of the third level's tiles (0: no third level)
 *   item_lines        1024   rows + columns per dual-update item
 *   finest_item_lines   64   the same on the third level
 *   level_quarters       8   fewer active tiles than level_quarters / 4 x the
 *                            grid move the solve to the next finer level
 *                            (0: stay on the coarse tiles)
 *   prefetch_distance    1   L2 prefetch of the fused update, warp steps
 *                            ahead (0..8; 0: off)
 *   tail_quarters        4   the smallest unconverged instances, last in
 *                            each iteration's tile order, take the finest
 *                            tiles up to tail_quarters / 4 x the grid of
 *                            them and the fine tiles up to twice that, so
 *                            an iteration ends on short tiles (0: off)
 * Tuning changes the schedule, not the arithmetic of an instance: every
 * setting gives the same iterates up to summation order. */
typedef struct {
  int fine_cols, finest_cols, item_lines, finest_item_lines, level_quarters,
      prefetch_distance, tail_quarters;
} drot_batch_tuning;
int drot_batch_set_tuning(const drot_batch_tuning *tuning);
void drot_batch_plan_destroy(drot_batch_plan plan);
/* Workspace bytes of a plan (device memory, 256-byte aligned). */
size_t drot_batch_plan_workspace_bytes(drot_batch_plan plan);
/* Profiling (no counterpart in the reference): later launches of the plan
 * record, for iterations it < cap, CTA 0's device clock (globaltimer, ns) at
 * the start of iteration it, after its fused-update tiles, after the first
 * grid barrier and after its dual-update items in times[4 it + 0..3] (4 cap
 * entries), and the coarse tiles of unconverged instances at the start in
 * active_tiles[it] (cap entries).  cap = 0 switches the record off.  The
 * buffers must stay allocated while the record is on. */
int drot_batch_set_iteration_log(drot_batch_plan plan, unsigned long long *times,
                                 unsigned *active_tiles, int cap);
/* Number of tiles (work units of one iteration). */
int drot_batch_plan_tiles(drot_batch_plan plan);
/* Copies the plan's descriptors into the workspace; synchronises `stream`. */
int drot_batch_upload(drot_batch_plan plan, void *workspace,
                      size_t workspace_bytes, drot_stream_t stream);
/* Warm start + solve of every instance (one init kernel, one cooperative
 * launch).  c: DROT_C_F32 or DROT_C_BF16 elements.  Asynchronous. */
int drot_qr_batch_launch(drot_batch_plan plan, const void *c, int c_dtype,
                         const float *p, const float *q, float *x,
                         int max_iters, void *workspace, size_t workspace_bytes,
                         drot_stream_t stream);
/* Point-cloud launch: the cost is never stored.  Instance k's C_ij =
 * cost_scale * max(|x_i|^2 + |y_j|^2 - 2 <x_i, y_j>, 0) is recomputed
 * inside the fused update on the iterations that read C, from x_i =
 * xpts[(R_k + i) * dim ...] and y_j = ypts[(S_k + j) * dim ...] (R_k, S_k:
 * the earlier instances' total rows / columns, i.e. the points of all
 * instances concatenated in order, row-major, 16-byte aligned); dim 8 or
 * 16.  The values are those of drot_sqeuclidean_cost (the same split-TF32
 * tcgen05 products, accumulated in TMEM, and the same epilogue), computed
 * per tile on the tensor cores.  8 bytes of traffic per element on every
 * iteration instead of 12 on those that read C.  The plan must have
 * 512-row bands; c_offset of the descriptors is unused. */
int drot_qr_batch_launch_points(drot_batch_plan plan, const float *xpts,
                                const float *ypts, int dim, float cost_scale,
                                const float *p, const float *q, float *x,
                                int max_iters, void *workspace,
                                size_t workspace_bytes, drot_stream_t stream);
/* Group-lasso plans only: n_iters more iterations of every instance from
 * the state left in the workspace by an earlier launch (a, b, phi1, phi2,
 * alpha of parity slot 0 -- see drot_batch_state_ex) and the plans in x,
 * with the stop test off; afterwards alpha is again in slot 0.  The
 * recomputation step of the batched unrolled adjoint.  Asynchronous. */
int drot_batch_resume(drot_batch_plan plan, const void *c, int c_dtype,
                      const float *p, const float *q, float *x, int n_iters,
                      void *workspace, size_t workspace_bytes,
                      drot_stream_t stream);
/* Copies the per-instance outcomes to out[n_inst]; synchronises `stream`.
 * Returns DROT_ERR_BARRIER_TIMEOUT when the launch gave up on a barrier. */
int drot_batch_results(drot_batch_plan plan, const void *workspace,
                       drot_batch_result *out, drot_stream_t stream);
/* Device pointers of the final duals phi1 (all instances' rows, in instance
 * order) and phi2 (all columns) inside a launched workspace; instance k's
 * entries start at the sum of the earlier instances' n_rows / n_cols. */
int drot_batch_state(drot_batch_plan plan, void *workspace, float **phi1,
                     float **phi2);
/* The whole final state inside a launched workspace (device pointers): a,
 * phi1 (rows), b, phi2 (columns), packed as in drot_batch_state, and alpha
 * [2][n_inst] by iteration parity -- instance k's final alpha is
 * alpha[(iters_run & 1) * n_inst + k].  With the plans X this is the state a
 * single-instance solve (drot_qr_solve / drot_gl_solve) continues from. */
int drot_batch_state_ex(drot_batch_plan plan, void *workspace, float **a, float **b,
                        float **phi1, float **phi2, float **alpha);

/* ---------------------------------------------------------------------------
 * Implicit adjoint of the quadratic-regularised plan (autograd backward)
 *
 * No counterpart in the reference (its operators have no backward).  At
 * the solution X of min <C,X> + (lambda/2)||X||^2 over the transport
 * polytope, with support S = {X > 0} and mask M, the adjoint system is
 *     [D_r M; M^T D_c] [a; b] = [rowsum(G o M); colsum(G o M)]
 * (D_r, D_c: row / column support counts), and then
 *     dL/dC = (a_i + b_j - G_ij) / lambda on S, 0 elsewhere;
 *     dL/dp = a, dL/dq = b (up to a + t, b - t).
 * The support is read off the duals of the solve: S = {phi1_i + phi2_j -
 * s C_ij > 0} (at the fixed point of X = max(X + phi1 + phi2 - sC, 0)/kappa
 * the plan is positive exactly there; a finite solve still holds tiny
 * positive entries of X off S that decay towards 0).
 *
 * drot_qr_adjoint_prepare builds the bit-packed support masks (and,
 * optionally, a byte mask in the layout of C); drot_qr_adjoint_solve then
 * forms the right-hand side from the upstream gradient and solves
 * the system of every instance with Jacobi-preconditioned conjugate
 * gradients in one persistent launch whose matvecs walk the mask bits.
 * ------------------------------------------------------------------------- */

/* One instance: C is n_rows x n_cols column-major with leading dimension ld
 * at element c_offset of the C buffer (and of the upstream gradient and
 * dL/dC buffers, which share its layout); its phi1 (n_rows) and phi2
 * (n_cols) start at phi1_offset / phi2_offset of the phi buffers (and its
 * dL/dp, dL/dq at the same offsets of grad_p / grad_q); step_size is the s
 * of its solve and lambda = (scale - 1) / s its regularisation weight; its
 * solution [a (n_rows); b (n_cols)] starts at element v_offset of z. */
typedef struct {
  int n_rows, n_cols, ld, pad;
  long long c_offset, v_offset, phi1_offset, phi2_offset;
  float step_size, lambda;
} drot_adjoint_instance;

/* Workspace of the prepare + solve + grad calls (the same for all three). */
size_t drot_qr_adjoint_workspace_bytes(int n_inst, const drot_adjoint_instance *inst);

/* Support masks of every instance into the workspace; mask (may be NULL)
 * receives 1 / 0 bytes at the positions of C.  c: DROT_C_F32 or DROT_C_BF16.
 * Synchronises `stream`. */
int drot_qr_adjoint_prepare(int n_inst, const drot_adjoint_instance *inst,
                            const void *c, int c_dtype, const float *phi1,
                            const float *phi2, unsigned char *mask,
                            void *workspace, size_t workspace_bytes,
                            drot_stream_t stream);

/* After drot_qr_adjoint_prepare on the same workspace and instances: the
 * right-hand side [rowsum(g o M); colsum(g o M)] from the upstream gradient
 * g = dL/dX (float, layout of C), then Jacobi-preconditioned CG in FP64
 * until ||r|| <= tol * ||r_0|| per instance or max_iters; writes z (FP64,
 * the [a; b] of every instance at its v_offset) and, when iters != NULL,
 * the CG iterations of each instance (host array of n_inst).  Lines per
 * instance: n_rows + n_cols <= 25 600.  Synchronises `stream`. */
int drot_qr_adjoint_solve(int n_inst, const drot_adjoint_instance *inst,
                          const float *g, double *z, double tol, int max_iters,
                          void *workspace, size_t workspace_bytes, int *iters,
                          drot_stream_t stream);

/* After drot_qr_adjoint_solve: the gradients of every instance --
 * grad_c = (a_i + b_j - g_ij) / lambda on the support and 0 elsewhere
 * (every element of the n_rows x n_cols block; padding rows untouched),
 * grad_p = a + t, grad_q = b - t with t = (sum b - sum a) / (n_rows +
 * n_cols) (the gauge sum(dL/dp) = sum(dL/dq)); FP64 arithmetic, rounded
 * once.  Asynchronous (one kernel on `stream`). */
int drot_qr_adjoint_grad(int n_inst, const drot_adjoint_instance *inst,
                         const float *g, const double *z, float *grad_c,
                         float *grad_p, float *grad_q, void *workspace,
                         size_t workspace_bytes, drot_stream_t stream);

/* After drot_qr_adjoint_solve on the same workspace and instances: the
 * final relative residual ||r|| / ||r_0|| of each instance's CG (host array
 * rel_residual[n_inst]; 0 for a zero right-hand side).  An instance stops
 * the first time it is at or below tol and stays stopped.  Synchronises
 * `stream`. */
int drot_qr_adjoint_residuals(int n_inst, const drot_adjoint_instance *inst,
                              const void *workspace, size_t workspace_bytes,
                              double *rel_residual, drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * Unrolled adjoint of the group-lasso iteration (autograd backward)
 *
 * No counterpart in the reference.  One GL iteration (core/drot_glr.hpp:
 * 242-355) maps s_k = (X, phi1, phi2, a, b, alpha) to s_{k+1};
 * drot_gl_adjoint_step applies the transposed Jacobian of that map: given
 * X, phi1, phi2 of s_k (recomputed from a checkpoint) and the adjoint of
 * s_{k+1} in xbar (n_rows x n_cols) and vbar ([phi1bar | phi2bar | abar |
 * bbar | alphabar], 2*(n_rows + n_cols) + 1 floats), it overwrites them with
 * the adjoint of s_k and adds the step's terms to cbar, pbar, qbar.
 * step_size / lambda are the solve's s and group threshold (the lambda of
 * drot_gl_solve).  Asynchronous (four kernels on `stream`).
 * ------------------------------------------------------------------------- */

size_t drot_gl_adjoint_workspace_bytes(int n_rows, int n_cols, int n_groups);

int drot_gl_adjoint_step(const void *c, int c_dtype, int n_rows, int n_cols,
                         int n_groups, float step_size, float lambda,
                         const float *x, const float *phi1, const float *phi2,
                         float *xbar, float *vbar, float *cbar, float *pbar,
                         float *qbar, void *workspace, size_t workspace_bytes,
                         drot_stream_t stream);

/* One checkpoint segment of the backward in one call: from the state at the
 * segment start (x, a, b, phi1, phi2, alpha; advanced in place) it runs
 * n_steps GL iterations with drot_gl_solve_ex (solve_ws: its workspace),
 * keeping X, phi1, phi2 before each in `states` (n_steps * (n_rows*n_cols +
 * n_rows + n_cols) floats), then applies drot_gl_adjoint_step for those
 * iterations in reverse order.  Asynchronous. */
int drot_gl_adjoint_segment(const void *c, int c_dtype, const float *p,
                            const float *q, int n_rows, int n_cols, int n_groups,
                            float step_size, float lambda, float *x, float *a,
                            float *b, float *phi1, float *phi2, float *alpha,
                            int n_steps, float *states, void *solve_ws,
                            size_t solve_ws_bytes, float *xbar, float *vbar,
                            float *cbar, float *pbar, float *qbar, void *adj_ws,
                            size_t adj_ws_bytes, drot_stream_t stream);

/* Batched GL adjoint steps (the reverse step of drot_gl_adjoint_step for
 * many instances in one set of launches).  Instance k: X (and Xbar, Cbar)
 * n_rows x n_cols column-major with leading dimension ld at element
 * x_offset of the packed X buffers, C at c_offset of the packed C, its
 * rows at row_offset of the packed row vectors (phi1, dL/dp) and columns
 * at col_offset of the packed column vectors (phi2, dL/dq); its vector
 * adjoint [phi1bar | phi2bar | abar | bbar | alphabar] (2 (n_rows + n_cols)
 * + 1 floats) follows the earlier instances' in vbar.  The C++ ABI of a
 * batch is: plan_create (host), setup (uploads the parameter blocks with
 * the C / adjoint buffers; synchronises `stream`), then one step per
 * reverse iteration with that iteration's packed state (X, phi1, phi2). */
typedef struct {
  int n_rows, n_cols, ld, n_groups;
  long long x_offset, c_offset, row_offset, col_offset;
  float step_size, lambda;
} drot_gl_adjoint_batch_instance;
typedef struct drot_gl_adjoint_batch_plan_s *drot_gl_adjoint_batch_plan;
int drot_gl_adjoint_batch_plan_create(int n_inst, const drot_gl_adjoint_batch_instance *inst,
                                      drot_gl_adjoint_batch_plan *plan);
void drot_gl_adjoint_batch_plan_destroy(drot_gl_adjoint_batch_plan plan);
size_t drot_gl_adjoint_batch_workspace_bytes(drot_gl_adjoint_batch_plan plan);
int drot_gl_adjoint_batch_setup(drot_gl_adjoint_batch_plan plan,
                                const drot_gl_adjoint_batch_instance *inst, const void *c,
                                int c_dtype, float *xbar, float *vbar, float *cbar,
                                float *pbar, float *qbar, void *workspace,
                                size_t workspace_bytes, drot_stream_t stream);
int drot_gl_adjoint_batch_step(drot_gl_adjoint_batch_plan plan, const float *x,
                               const float *phi1, const float *phi2, void *workspace,
                               size_t workspace_bytes, drot_stream_t stream);

/* ---------------------------------------------------------------------------
 * Cost matrices of point clouds (tensor cores)
 *
 * No counterpart in the reference, whose callers build C on the host
 * (benchmark/utils/compute_w2_dist.py:68-94).  For each instance, points
 * x (m x dim) and y (n x dim), row-major float32:
 *     C[c_offset + j*ld + i] = scale * max(|x_i|^2 + |y_j|^2 - 2 <x_i, y_j>, 0)
 * (no max when clamp == 0): the column-major m x n cost the solvers read.
 * The Gram term runs on the tcgen05 tensor cores in split TF32 ("3xTF32",
 * FP32-level accuracy); norms are FP32.  dim: 8, 16, 24 or 32.
 * ------------------------------------------------------------------------- */

/* x_offset / y_offset: index of the instance's first point in x / y;
 * c_offset: element offset of its C block (leading dimension ld >= m). */
typedef struct {
  int m, n, ld, pad;
  long long x_offset, y_offset, c_offset;
} drot_cost_instance;

/* Up to 256 instances per call (x, y 16-byte aligned).  Synchronises
 * `stream` (it reads back the kernel's error flag). */
int drot_sqeuclidean_cost(int n_inst, const drot_cost_instance *inst,
                          const float *x, const float *y, int dim, float scale,
                          int clamp, float *c, drot_stream_t stream);

/* Backward of drot_sqeuclidean_cost (no counterpart in the reference): for
 * grad_c = dL/dC of every instance (layout of C), the chain rule
 *     grad_x_i = 2 scale (x_i sum_j G_ij - sum_j G_ij y_j)
 *     grad_y_j = 2 scale (y_j sum_i G_ij - sum_i G_ij x_i)
 * with G = grad_c, zeroed where c <= 0 when c != NULL (the clamp of the
 * forward); grad_x / grad_y in the layout of x / y.  FP32 sums in a fixed
 * order (deterministic), one pass over grad_c (and c).  workspace: the
 * per-band partials of grad_y, drot_sqeuclidean_cost_grad_workspace_bytes.
 * grad_c, c 16-byte aligned.  Asynchronous (two kernels on `stream`). */
size_t drot_sqeuclidean_cost_grad_workspace_bytes(int n_inst,
                                                  const drot_cost_instance *inst,
                                                  int dim);
int drot_sqeuclidean_cost_grad(int n_inst, const drot_cost_instance *inst,
                               const float *x, const float *y, int dim,
                               float scale, const float *c, const float *grad_c,
                               float *grad_x, float *grad_y, void *workspace,
                               size_t workspace_bytes, drot_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* DROT_GB300_H */
