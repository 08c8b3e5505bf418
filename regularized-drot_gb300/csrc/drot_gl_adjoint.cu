// drot_gl_adjoint.cu -- reverse-mode step of the group-lasso DROT iteration
// (checkpointed unrolled adjoint for autograd).
//
// No counterpart in the reference (its operators have no backward,
// pytorch/src/drot_cuda.cpp:26-62).  One forward GL iteration
// (core/drot_glr.hpp:242-355; kernel_glr.hpp:59-161 and 461-526) maps the
// state s_k = (X, phi1, phi2, a, b, alpha) to s_{k+1}:
//     t = X + phi1_i + phi2_j - s C,  y = max(t, 0),
//     n_gj = ||y_{g,j}||,  sig_gj = max(1 - lambda / (n_gj + 1e-9), 0),
//     X' = sig_gj y,  r = X' 1,  c = X'^T 1,  sigma = sum X',
//     gamma = (2 (sigma - 1) - alpha) / (m + n),
//     rs = r - p,  a' = a - rs,  phi1' = (a' - rs + gamma) / n_cols,
//     cs = c - q,  b' = b - cs,  phi2' = (b' - cs + gamma) / n_rows,
//     alpha' = alpha + 1 - sigma.
// drot_gl_adjoint_step maps the adjoint of s_{k+1} (Xbar and the vector
// adjoints) to the adjoint of s_k, given X, phi1, phi2 of s_k, and adds the
// step's contributions to Cbar, pbar, qbar:
//     vector part:  rbar = -abar' - 2 phi1bar'/n_cols,  cbar = -bbar' - 2 phi2bar'/n_rows,
//                   gbar = sum phi1bar'/n_cols + sum phi2bar'/n_rows,
//                   sigbar = -alphabar' + 2 gbar/(m+n),
//                   abar = abar' + phi1bar'/n_cols, bbar = bbar' + phi2bar'/n_rows,
//                   alphabar = alphabar' - gbar/(m+n), pbar -= rbar, qbar -= cbar;
//     matrix part:  Xt = Xbar' + rbar_i + cbar_j + sigbar,
//                   ybar = sig_gj Xt + [sig_gj > 0] lambda y / (n (n+eps)^2) <Xt, y>_{g,j},
//                   tbar = [t > 0] ybar,  Xbar = tbar,  Cbar -= s tbar,
//                   phi1bar = tbar 1,  phi2bar = tbar^T 1.
// Kernels: gl_adj_vec (one CTA), gl_adj_groups (one warp per group column:
// norms, shrink factors and <Xt, y>), gl_adj_elems (one CTA per 16 columns x
// 1024 rows: tbar, Xbar, Cbar, row partials in shared memory, column
// partials per row block), gl_adj_rows (partials -> phi1bar, phi2bar).  All
// sums are in a fixed order (deterministic).  drot_gl_adjoint_segment runs a
// whole checkpoint segment (recompute + reverse steps) in one call.
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

constexpr int kGlaChunk = 16;     // columns per CTA in gl_adj_elems
constexpr int kGlaRows = 1024;    // rows per CTA in gl_adj_elems
constexpr int kGlaThreads = 256;
constexpr double kGlaNormEps = 1e-9;

// One instance's step.  X, Xbar, Cbar and C are column-major with leading
// dimension ld (X at element e = j ld + i).  Single-instance steps pass it
// in the kernel parameters with x / phi1 / phi2 pointing at the state;
// batched steps read it from an array in device memory and add xo / ro /
// co to the step's packed state buffers.
struct GlaParams {
  const void* c;
  int c_bf16;
  int nr, nc, G, ld;
  int chunks, rblocks;  // gl_adj_elems grid of this instance
  float s, lambda;
  const float *x, *phi1, *phi2;
  long long xo;   // batched: X's element offset in the packed state
  int ro, co;     // batched: phi1 / phi2 offsets in the packed state
  float *xbar, *vbar, *cbar, *pbar, *qbar;
  // workspace
  float *rbar, *cbarv, *sbar, *sig, *coef, *rowpart, *colpart;
  int bounds[kMaxGroups + 1];  // group row boundaries
};

// The state pointers of one step.
struct GlaState {
  const float *x, *phi1, *phi2;
};

__device__ __forceinline__ float load_cost(const GlaParams& A, long long e) {
  return A.c_bf16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(A.c)[e])
                  : __ldg(reinterpret_cast<const float*>(A.c) + e);
}

// vbar layout: [phi1bar (nr) | phi2bar (nc) | abar (nr) | bbar (nc) | alphabar (1)]
// Grid over the n_rows + n_cols lines; every CTA first forms gbar from all
// of phi1bar', phi2bar' (8 loads in flight per thread, FP64 across the
// block), then updates its own lines; CTA 0 writes sigbar and alphabar.
__device__ __forceinline__ void gl_adj_vec_body(const GlaParams& A) {
  __shared__ double red[kGlaThreads / 32 + 1];
  const int nr = A.nr, nc = A.nc;
  // CTAs past this instance's lines (batched grids are sized for the
  // largest instance) have nothing to do; CTA 0 always runs.
  if (blockIdx.x > 0 && (long long)blockIdx.x * blockDim.x >= nr + nc) return;
  float* f1 = A.vbar;
  float* f2 = f1 + nr;
  float* ab = f2 + nc;
  float* bb = ab + nr;
  float* alb = bb + nc;
  float s1 = 0.0f, s2 = 0.0f;
  for (int i0 = threadIdx.x; i0 < nr + nc; i0 += 8 * blockDim.x) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int l = i0 + u * blockDim.x;
      v[u] = l < nr + nc ? f1[l] : 0.0f;  // f2 follows f1
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int l = i0 + u * blockDim.x;
      if (l < nr) s1 += v[u];
      else s2 += v[u];
    }
  }
  const double g = block_sum_d((double)s1, red) / (double)nc +
                   block_sum_d((double)s2, red) / (double)nr;
  const double mn = (double)nr + (double)nc;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < nr) {
    const float F = f1[l] / (float)nc;
    const float A1 = ab[l];
    const float rs = -A1 - 2.0f * F;
    A.rbar[l] = rs;
    ab[l] = A1 + F;
    A.pbar[l] -= rs;
  } else if (l < nr + nc) {
    const int j = l - nr;
    const float F = f2[j] / (float)nr;
    const float B1 = bb[j];
    const float cs = -B1 - 2.0f * F;
    A.cbarv[j] = cs;
    bb[j] = B1 + F;
    A.qbar[j] -= cs;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const float al = *alb;
    A.sbar[0] = (float)(-(double)al + 2.0 * g / mn);
    *alb = (float)((double)al - g / mn);
  }
}

__global__ void gl_adj_vec(const GlaParams A) { gl_adj_vec_body(A); }
__global__ void gl_adj_vec_batch(const GlaParams* __restrict__ PA) {
  gl_adj_vec_body(PA[blockIdx.y]);
}

// Group of row i: the last g with bounds[g] <= i (binary search; bounds
// travel in the kernel parameters).
__device__ __forceinline__ int group_of(const GlaParams& A, int i) {
  int lo = 0, hi = A.G - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (A.bounds[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One warp per (group g, column j): n_gj, sig_gj and coef_gj.
__device__ __forceinline__ void gl_adj_groups_body(const GlaParams& A, const GlaState S) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const float sb = A.sbar[0];
  for (long long task = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       task < (long long)A.G * A.nc; task += warps) {
    const int g = (int)(task % A.G), j = (int)(task / A.G);
    const int i0 = A.bounds[g], i1 = A.bounds[g + 1];
    const float f2 = S.phi2[j], cb = A.cbarv[j];
    // Lane sums as float pairs (TwoSum), combined in FP64 across the warp
    // (FP64 arithmetic is slow on this part; a per-element FP64 FMA cost
    // more than the loads).
    float n2h = 0.0f, n2l = 0.0f, dth = 0.0f, dtl = 0.0f;
    for (int ib = i0 + lane; ib < i1; ib += 128) {
      float xv[4], cv[4], f1[4], xb[4], rb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {  // all loads of four rows first
        const int i = ib + 32 * u;
        const long long e = (long long)j * A.ld + (i < i1 ? i : i0);
        xv[u] = S.x[e];
        cv[u] = load_cost(A, e);
        f1[u] = S.phi1[i < i1 ? i : i0];
        xb[u] = A.xbar[e];
        rb[u] = A.rbar[i < i1 ? i : i0];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (ib + 32 * u >= i1) break;
        const float t = fmaf(-A.s, cv[u], (xv[u] + f1[u]) + f2);
        const float y = fmaxf(t, 0.0f);
        const float xt = ((xb[u] + rb[u]) + cb) + sb;
        float e1;
        two_sum(n2h, y * y, n2h, e1);
        n2l += e1;
        two_sum(dth, xt * y, dth, e1);
        dtl += e1;
      }
    }
    double n2 = warp_sum_d((double)n2h + (double)n2l);
    double dot = warp_sum_d((double)dth + (double)dtl);
    if (lane == 0) {
      const double n = sqrt(n2);
      const double sh = 1.0 - (double)A.lambda / (n + kGlaNormEps);
      const double den = n * (n + kGlaNormEps) * (n + kGlaNormEps);
      A.sig[task] = (float)(sh > 0.0 ? sh : 0.0);
      A.coef[task] = (sh > 0.0 && n > 0.0) ? (float)((double)A.lambda * dot / den) : 0.0f;
    }
  }
}

__global__ void gl_adj_groups(const GlaParams A) {
  gl_adj_groups_body(A, GlaState{A.x, A.phi1, A.phi2});
}
__global__ void gl_adj_groups_batch(const GlaParams* __restrict__ PA, const float* x,
                                    const float* phi1, const float* phi2) {
  const GlaParams& A = PA[blockIdx.y];
  gl_adj_groups_body(A, GlaState{x + A.xo, phi1 + A.ro, phi2 + A.co});
}

// One CTA per (chunk of kGlaChunk columns, block of kGlaRows rows); thread
// t owns rows r0 + t + 256 u (u < 4) of the CTA's row partial (registers)
// and loads its four rows of a column before using any.  Column sums: one
// FP32 partial per warp and column in shared memory, combined in warp order
// at the end into the row block's column partial.
__device__ __forceinline__ void gl_adj_elems_body(const GlaParams& A, const GlaState S,
                                                  int chunk, int rb) {
  __shared__ float wcol[kGlaThreads / 32][kGlaChunk];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j0 = chunk * kGlaChunk, j1 = min(j0 + kGlaChunk, A.nc);
  const int r0 = rb * kGlaRows, r1 = min(r0 + kGlaRows, A.nr);
  constexpr int U = kGlaRows / kGlaThreads;
  const float sb = A.sbar[0];
  int gi[U];
  float f1[U], rbv[U], racc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int i = r0 + threadIdx.x + u * kGlaThreads;
    const int ic = i < r1 ? i : r0;
    gi[u] = group_of(A, ic);
    f1[u] = S.phi1[ic];
    rbv[u] = A.rbar[ic];
    racc[u] = 0.0f;
  }
  for (int j = j0; j < j1; ++j) {
    const float f2 = S.phi2[j], cb = A.cbarv[j];
    float xv[U], cv[U], xb[U], sg[U], cf[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = r0 + threadIdx.x + u * kGlaThreads;
      const long long e = (long long)j * A.ld + (i < r1 ? i : r0);
      const long long gj = (long long)j * A.G + gi[u];
      xv[u] = S.x[e];
      cv[u] = load_cost(A, e);
      xb[u] = A.xbar[e];
      sg[u] = A.sig[gj];
      cf[u] = A.coef[gj];
    }
    float colp = 0.0f;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = r0 + threadIdx.x + u * kGlaThreads;
      if (i >= r1) continue;
      const long long e = (long long)j * A.ld + i;
      const float t = fmaf(-A.s, cv[u], (xv[u] + f1[u]) + f2);
      const float xt = ((xb[u] + rbv[u]) + cb) + sb;
      const float ybar = fmaf(cf[u], fmaxf(t, 0.0f), sg[u] * xt);
      const float tb = t > 0.0f ? ybar : 0.0f;
      A.xbar[e] = tb;
      A.cbar[e] = fmaf(-A.s, tb, A.cbar[e]);
      racc[u] += tb;
      colp += tb;
    }
    colp = warp_sum(colp);
    if (lane == 0) wcol[warp][j - j0] = colp;
  }
  __syncthreads();
  if (threadIdx.x < j1 - j0) {
    float cs = 0.0f;
    for (int w = 0; w < kGlaThreads / 32; ++w) cs += wcol[w][threadIdx.x];
    A.colpart[(long long)rb * A.nc + j0 + threadIdx.x] = cs;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int i = r0 + threadIdx.x + u * kGlaThreads;
    if (i < r1) A.rowpart[(long long)chunk * A.nr + i] = racc[u];
  }
}

__global__ void __launch_bounds__(kGlaThreads) gl_adj_elems(const GlaParams A) {
  gl_adj_elems_body(A, GlaState{A.x, A.phi1, A.phi2}, blockIdx.x, blockIdx.y);
}
// Batched: blockIdx.z is the instance; CTAs past its chunks / row blocks
// return at once (the grid is sized for the largest instance).
__global__ void __launch_bounds__(kGlaThreads) gl_adj_elems_batch(
    const GlaParams* __restrict__ PA, const float* x, const float* phi1, const float* phi2) {
  const GlaParams& A = PA[blockIdx.z];
  if ((int)blockIdx.x >= A.chunks || (int)blockIdx.y >= A.rblocks) return;
  gl_adj_elems_body(A, GlaState{x + A.xo, phi1 + A.ro, phi2 + A.co}, blockIdx.x, blockIdx.y);
}

// phi1bar = sum over column chunks of the row partials, phi2bar = sum over
// row blocks of the column partials (fixed order).
// One warp per line: lanes take partials lane, lane + 32, ... (fixed order),
// then a shuffle tree.
__device__ __forceinline__ void gl_adj_rows_body(const GlaParams& A, int chunks, int rblocks) {
  const int n = A.nr + A.nc;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); l < n; l += warps) {
    const bool row = l < A.nr;
    const float* base = row ? A.rowpart + l : A.colpart + (l - A.nr);
    const long long stride = row ? A.nr : A.nc;
    const int cnt = row ? chunks : rblocks;
    double s = 0.0;
    for (int c = lane; c < cnt; c += 32) s += (double)base[c * stride];
    s = warp_sum_d(s);
    if (lane == 0) A.vbar[l] = (float)s;  // [phi1bar | phi2bar] of s_k
  }
}

__global__ void gl_adj_rows(const GlaParams A, int chunks, int rblocks) {
  gl_adj_rows_body(A, chunks, rblocks);
}
__global__ void gl_adj_rows_batch(const GlaParams* __restrict__ PA) {
  const GlaParams& A = PA[blockIdx.y];
  gl_adj_rows_body(A, A.chunks, A.rblocks);
}

struct GlaLayout {
  size_t off_rbar, off_cbar, off_sbar, off_sig, off_coef, off_rowpart, off_colpart, total;
  int chunks, rblocks;
};

static GlaLayout gla_layout(int nr, int nc, int G) {
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  GlaLayout L;
  L.chunks = (nc + kGlaChunk - 1) / kGlaChunk;
  L.rblocks = (nr + kGlaRows - 1) / kGlaRows;
  size_t off = 0;
  L.off_rbar = off;    off = al(off + sizeof(float) * nr);
  L.off_cbar = off;    off = al(off + sizeof(float) * nc);
  L.off_sbar = off;    off = al(off + sizeof(float) * 4);
  L.off_sig = off;     off = al(off + sizeof(float) * (size_t)G * nc);
  L.off_coef = off;    off = al(off + sizeof(float) * (size_t)G * nc);
  L.off_rowpart = off; off = al(off + sizeof(float) * (size_t)L.chunks * nr);
  L.off_colpart = off; off = al(off + sizeof(float) * (size_t)L.rblocks * nc);
  L.total = off;
  return L;
}

}  // namespace drot

using namespace drot;

// Batched adjoint: the instances' parameter blocks live in the workspace
// (uploaded once by drot_gl_adjoint_batch_setup), followed by every
// instance's scratch (the single-instance layout, 256-byte aligned).
struct drot_gl_adjoint_batch_plan_s {
  int n_inst = 0;
  std::vector<GlaParams> prm;  // host copies; pointers filled by setup
  std::vector<size_t> ws_off;  // per instance: scratch offset in the workspace
  std::vector<long long> v_off;  // per instance: offset of its vector adjoint in vbar
  size_t off_params = 0, total = 0;
  int max_lines = 0, max_chunks = 0, max_rblocks = 0;
  long long max_tasks = 0;
};

extern "C" {

size_t drot_gl_adjoint_workspace_bytes(int n_rows, int n_cols, int n_groups) {
  if (n_rows <= 0 || n_cols <= 0 || n_groups <= 0 || n_groups > kMaxGroups) return 0;
  return gla_layout(n_rows, n_cols, n_groups).total;
}

int drot_gl_adjoint_step(const void* c, int c_dtype, int n_rows, int n_cols, int n_groups,
                         float step_size, float lambda, const float* x, const float* phi1,
                         const float* phi2, float* xbar, float* vbar, float* cbar, float* pbar,
                         float* qbar, void* workspace, size_t workspace_bytes,
                         drot_stream_t stream) {
  if (!c || !x || !phi1 || !phi2 || !xbar || !vbar || !cbar || !pbar || !qbar || !workspace)
    return DROT_ERR_INVALID_ARG;
  if (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  const size_t need = drot_gl_adjoint_workspace_bytes(n_rows, n_cols, n_groups);
  if (need == 0) return DROT_ERR_UNSUPPORTED;
  if (workspace_bytes < need || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  const GlaLayout L = gla_layout(n_rows, n_cols, n_groups);
  char* ws = (char*)workspace;
  cudaStream_t st = (cudaStream_t)stream;
  GlaParams A;
  memset(&A, 0, sizeof(A));
  if (drot_gl_group_bounds(n_rows, n_groups, A.bounds) != DROT_OK) return DROT_ERR_INVALID_ARG;
  A.c = c;
  A.c_bf16 = c_dtype == DROT_C_BF16;
  A.nr = n_rows;
  A.nc = n_cols;
  A.G = n_groups;
  A.ld = n_rows;
  A.chunks = L.chunks;
  A.rblocks = L.rblocks;
  A.s = step_size;
  A.lambda = lambda;
  A.x = x;
  A.phi1 = phi1;
  A.phi2 = phi2;
  A.xbar = xbar;
  A.vbar = vbar;
  A.cbar = cbar;
  A.pbar = pbar;
  A.qbar = qbar;
  A.rbar = (float*)(ws + L.off_rbar);
  A.cbarv = (float*)(ws + L.off_cbar);
  A.sbar = (float*)(ws + L.off_sbar);
  A.sig = (float*)(ws + L.off_sig);
  A.coef = (float*)(ws + L.off_coef);
  A.rowpart = (float*)(ws + L.off_rowpart);
  A.colpart = (float*)(ws + L.off_colpart);
  gl_adj_vec<<<(n_rows + n_cols + kGlaThreads - 1) / kGlaThreads, kGlaThreads, 0, st>>>(A);
  const long long tasks = (long long)n_groups * n_cols;
  const int gblocks = (int)std::min<long long>((tasks + 7) / 8, 4096);
  gl_adj_groups<<<gblocks, 256, 0, st>>>(A);
  gl_adj_elems<<<dim3(L.chunks, L.rblocks), kGlaThreads, 0, st>>>(A);
  gl_adj_rows<<<(n_rows + n_cols + 7) / 8, 256, 0, st>>>(A, L.chunks, L.rblocks);
  return cudaGetLastError() == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

int drot_gl_adjoint_batch_plan_create(int n_inst, const drot_gl_adjoint_batch_instance* desc,
                                      drot_gl_adjoint_batch_plan* out) {
  if (!out || !desc || n_inst <= 0 || n_inst > 65535) return DROT_ERR_INVALID_ARG;
  *out = nullptr;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  drot_gl_adjoint_batch_plan_s* P = new (std::nothrow) drot_gl_adjoint_batch_plan_s;
  if (!P) return DROT_ERR_UNSUPPORTED;
  P->n_inst = n_inst;
  P->prm.resize(n_inst);
  P->ws_off.resize(n_inst);
  P->v_off.resize(n_inst);
  size_t off = al(sizeof(GlaParams) * (size_t)n_inst);
  long long vo = 0;
  for (int k = 0; k < n_inst; ++k) {
    const drot_gl_adjoint_batch_instance& d = desc[k];
    if (d.n_rows <= 0 || d.n_cols <= 0 || d.ld < d.n_rows || d.n_groups <= 0 ||
        d.n_groups > kMaxGroups || d.n_groups > d.n_rows || d.x_offset < 0 || d.c_offset < 0 ||
        d.row_offset < 0 || d.col_offset < 0 || d.row_offset > INT32_MAX - d.n_rows ||
        d.col_offset > INT32_MAX - d.n_cols || !(d.step_size > 0.0f) || !(d.lambda >= 0.0f)) {
      delete P;
      return DROT_ERR_INVALID_ARG;
    }
    GlaParams& A = P->prm[k];
    memset(&A, 0, sizeof(A));
    if (drot_gl_group_bounds(d.n_rows, d.n_groups, A.bounds) != DROT_OK) {
      delete P;
      return DROT_ERR_INVALID_ARG;
    }
    const GlaLayout L = gla_layout(d.n_rows, d.n_cols, d.n_groups);
    A.nr = d.n_rows;
    A.nc = d.n_cols;
    A.G = d.n_groups;
    A.ld = d.ld;
    A.chunks = L.chunks;
    A.rblocks = L.rblocks;
    A.s = d.step_size;
    A.lambda = d.lambda;
    A.xo = d.x_offset;
    A.ro = (int)d.row_offset;
    A.co = (int)d.col_offset;
    P->v_off[k] = vo;  // the buffers' pointers are filled by setup
    vo += 2LL * (d.n_rows + d.n_cols) + 1;
    P->ws_off[k] = off;
    off = al(off + L.total);
    P->max_lines = std::max(P->max_lines, d.n_rows + d.n_cols);
    P->max_chunks = std::max(P->max_chunks, L.chunks);
    P->max_rblocks = std::max(P->max_rblocks, L.rblocks);
    P->max_tasks = std::max(P->max_tasks, (long long)d.n_groups * d.n_cols);
  }
  P->off_params = 0;
  P->total = off;
  *out = P;
  return DROT_OK;
}

void drot_gl_adjoint_batch_plan_destroy(drot_gl_adjoint_batch_plan plan) { delete plan; }

size_t drot_gl_adjoint_batch_workspace_bytes(drot_gl_adjoint_batch_plan plan) {
  return plan ? plan->total : 0;
}

int drot_gl_adjoint_batch_setup(drot_gl_adjoint_batch_plan plan,
                                const drot_gl_adjoint_batch_instance* desc, const void* c,
                                int c_dtype, float* xbar, float* vbar, float* cbar, float* pbar,
                                float* qbar, void* workspace, size_t workspace_bytes,
                                drot_stream_t stream) {
  if (!plan || !desc || !c || !xbar || !vbar || !cbar || !pbar || !qbar || !workspace)
    return DROT_ERR_INVALID_ARG;
  if (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  if (workspace_bytes < plan->total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  const size_t esz = c_dtype == DROT_C_F32 ? sizeof(float) : 2;
  std::vector<GlaParams> dev(plan->prm);
  for (int k = 0; k < plan->n_inst; ++k) {
    GlaParams& A = dev[k];
    const drot_gl_adjoint_batch_instance& d = desc[k];
    const GlaLayout L = gla_layout(A.nr, A.nc, A.G);
    char* w = ws + plan->ws_off[k];
    A.c = (const char*)c + (size_t)d.c_offset * esz;
    A.c_bf16 = c_dtype == DROT_C_BF16;
    A.xbar = xbar + d.x_offset;
    A.cbar = cbar + d.c_offset;
    A.vbar = vbar + plan->v_off[k];
    A.pbar = pbar + d.row_offset;
    A.qbar = qbar + d.col_offset;
    A.rbar = (float*)(w + L.off_rbar);
    A.cbarv = (float*)(w + L.off_cbar);
    A.sbar = (float*)(w + L.off_sbar);
    A.sig = (float*)(w + L.off_sig);
    A.coef = (float*)(w + L.off_coef);
    A.rowpart = (float*)(w + L.off_rowpart);
    A.colpart = (float*)(w + L.off_colpart);
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(ws + plan->off_params, dev.data(), sizeof(GlaParams) * dev.size(),
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return DROT_ERR_CUDA;
  return DROT_OK;
}

int drot_gl_adjoint_batch_step(drot_gl_adjoint_batch_plan plan, const float* x, const float* phi1,
                               const float* phi2, void* workspace, size_t workspace_bytes,
                               drot_stream_t stream) {
  if (!plan || !x || !phi1 || !phi2 || !workspace) return DROT_ERR_INVALID_ARG;
  if (workspace_bytes < plan->total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  const GlaParams* PA = (const GlaParams*)((char*)workspace + plan->off_params);
  cudaStream_t st = (cudaStream_t)stream;
  const int n = plan->n_inst;
  gl_adj_vec_batch<<<dim3((plan->max_lines + kGlaThreads - 1) / kGlaThreads, n), kGlaThreads, 0,
                     st>>>(PA);
  const int gblocks = (int)std::min<long long>((plan->max_tasks + 7) / 8, 4096);
  gl_adj_groups_batch<<<dim3(gblocks, n), 256, 0, st>>>(PA, x, phi1, phi2);
  gl_adj_elems_batch<<<dim3(plan->max_chunks, plan->max_rblocks, n), kGlaThreads, 0, st>>>(
      PA, x, phi1, phi2);
  gl_adj_rows_batch<<<dim3((plan->max_lines + 7) / 8, n), 256, 0, st>>>(PA);
  return cudaGetLastError() == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

int drot_gl_adjoint_segment(const void* c, int c_dtype, const float* p, const float* q,
                            int n_rows, int n_cols, int n_groups, float step_size, float lambda,
                            float* x, float* a, float* b, float* phi1, float* phi2, float* alpha,
                            int n_steps, float* states, void* solve_ws, size_t solve_ws_bytes,
                            float* xbar, float* vbar, float* cbar, float* pbar, float* qbar,
                            void* adj_ws, size_t adj_ws_bytes, drot_stream_t stream) {
  if (n_steps < 0 || !states || !x || !phi1 || !phi2) return DROT_ERR_INVALID_ARG;
  const size_t mn = (size_t)n_rows * n_cols;
  const size_t per = mn + n_rows + n_cols;
  cudaStream_t st = (cudaStream_t)stream;
  // Recompute: keep X, phi1, phi2 before every iteration of the segment.
  for (int k = 0; k < n_steps; ++k) {
    float* s_k = states + per * k;
    if (cudaMemcpyAsync(s_k, x, sizeof(float) * mn, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(s_k + mn, phi1, sizeof(float) * n_rows, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(s_k + mn + n_rows, phi2, sizeof(float) * n_cols, cudaMemcpyDeviceToDevice,
                        st) != cudaSuccess)
      return DROT_ERR_CUDA;
    // One GL iteration; eps = -1 never stops it early.
    const int rc = drot_gl_solve_ex(c, c_dtype, p, q, n_rows, n_cols, n_groups, step_size, lambda,
                                    1, -1.0f, x, a, b, phi1, phi2, alpha, solve_ws,
                                    solve_ws_bytes, nullptr, stream);
    if (rc != DROT_OK) return rc;
  }
  // Reverse steps.
  for (int k = n_steps - 1; k >= 0; --k) {
    const float* s_k = states + per * k;
    const int rc = drot_gl_adjoint_step(c, c_dtype, n_rows, n_cols, n_groups, step_size, lambda,
                                        s_k, s_k + mn, s_k + mn + n_rows, xbar, vbar, cbar, pbar,
                                        qbar, adj_ws, adj_ws_bytes, stream);
    if (rc != DROT_OK) return rc;
  }
  return DROT_OK;
}

}  // extern "C"
