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
// norms, shrink factors and <Xt, y>), gl_adj_elems (one CTA per 32-column
// chunk: tbar, Xbar, Cbar, column sums, per-chunk row partials in shared
// memory), gl_adj_rows (row partials -> phi1bar).  All sums are in a fixed
// order (deterministic).
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

constexpr int kGlaChunk = 32;     // columns per CTA in gl_adj_elems
constexpr int kGlaThreads = 256;
constexpr double kGlaNormEps = 1e-9;

struct GlaParams {
  const void* c;
  int c_bf16;
  int nr, nc, G;
  float s, lambda;
  const float *x, *phi1, *phi2;
  float *xbar, *vbar, *cbar, *pbar, *qbar;
  // workspace
  float *rbar, *cbarv, *sbar, *sig, *coef, *rowpart;
  int* gid;
  int bounds[kMaxGroups + 1];  // group row boundaries (travel in the parameters)
};

__device__ __forceinline__ float load_cost(const GlaParams& A, long long e) {
  return A.c_bf16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(A.c)[e])
                  : __ldg(reinterpret_cast<const float*>(A.c) + e);
}

// vbar layout: [phi1bar (nr) | phi2bar (nc) | abar (nr) | bbar (nc) | alphabar (1)]
__global__ void gl_adj_vec(const GlaParams A) {
  __shared__ double red[kGlaThreads / 32 + 1];
  const int nr = A.nr, nc = A.nc;
  float* f1 = A.vbar;
  float* f2 = f1 + nr;
  float* ab = f2 + nc;
  float* bb = ab + nr;
  float* alb = bb + nc;
  double g = 0.0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) g += (double)f1[i] / (double)nc;
  for (int j = threadIdx.x; j < nc; j += blockDim.x) g += (double)f2[j] / (double)nr;
  g = block_sum_d(g, red);
  const double mn = (double)nr + (double)nc;
  const float al = *alb;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const float F = f1[i] / (float)nc;
    const float A1 = ab[i];
    const float rs = -A1 - 2.0f * F;
    A.rbar[i] = rs;
    ab[i] = A1 + F;
    A.pbar[i] -= rs;
  }
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    const float F = f2[j] / (float)nr;
    const float B1 = bb[j];
    const float cs = -B1 - 2.0f * F;
    A.cbarv[j] = cs;
    bb[j] = B1 + F;
    A.qbar[j] -= cs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    A.sbar[0] = (float)(-(double)al + 2.0 * g / mn);
    *alb = (float)((double)al - g / mn);
  }
  for (int g2 = threadIdx.x; g2 < A.G; g2 += blockDim.x)
    for (int i = A.bounds[g2]; i < A.bounds[g2 + 1]; ++i) A.gid[i] = g2;
}

// One warp per (group g, column j): n_gj, sig_gj and coef_gj.
__global__ void gl_adj_groups(const GlaParams A) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const float sb = A.sbar[0];
  for (long long task = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       task < (long long)A.G * A.nc; task += warps) {
    const int g = (int)(task % A.G), j = (int)(task / A.G);
    const int i0 = A.bounds[g], i1 = A.bounds[g + 1];
    const float f2 = A.phi2[j], cb = A.cbarv[j];
    double n2 = 0.0, dot = 0.0;
    for (int i = i0 + lane; i < i1; i += 32) {
      const long long e = (long long)j * A.nr + i;
      const float t = fmaf(-A.s, load_cost(A, e), (A.x[e] + A.phi1[i]) + f2);
      const float y = fmaxf(t, 0.0f);
      const float xt = ((A.xbar[e] + A.rbar[i]) + cb) + sb;
      n2 += (double)y * (double)y;
      dot += (double)xt * (double)y;
    }
    n2 = warp_sum_d(n2);
    dot = warp_sum_d(dot);
    if (lane == 0) {
      const double n = sqrt(n2);
      const double sh = 1.0 - (double)A.lambda / (n + kGlaNormEps);
      const double den = n * (n + kGlaNormEps) * (n + kGlaNormEps);
      A.sig[task] = (float)(sh > 0.0 ? sh : 0.0);
      A.coef[task] = (sh > 0.0 && n > 0.0) ? (float)((double)A.lambda * dot / den) : 0.0f;
    }
  }
}

// One CTA per chunk of kGlaChunk columns; each thread owns rows
// tid, tid + 256, ... of the chunk's row partial (shared memory).
__global__ void __launch_bounds__(kGlaThreads) gl_adj_elems(const GlaParams A) {
  extern __shared__ float rowacc[];  // [nr]
  __shared__ double red[kGlaThreads / 32 + 1];
  const int chunk = blockIdx.x;
  const int j0 = chunk * kGlaChunk, j1 = min(j0 + kGlaChunk, A.nc);
  for (int i = threadIdx.x; i < A.nr; i += blockDim.x) rowacc[i] = 0.0f;
  const float sb = A.sbar[0];
  for (int j = j0; j < j1; ++j) {
    const float f2 = A.phi2[j], cb = A.cbarv[j];
    float colp = 0.0f;
    for (int i = threadIdx.x; i < A.nr; i += blockDim.x) {
      const long long e = (long long)j * A.nr + i;
      const float cv = load_cost(A, e);
      const float t = fmaf(-A.s, cv, (A.x[e] + A.phi1[i]) + f2);
      const int g = A.gid[i];
      const long long gj = (long long)j * A.G + g;
      const float xt = ((A.xbar[e] + A.rbar[i]) + cb) + sb;
      const float ybar = fmaf(A.coef[gj], fmaxf(t, 0.0f), A.sig[gj] * xt);
      const float tb = t > 0.0f ? ybar : 0.0f;
      A.xbar[e] = tb;
      A.cbar[e] = fmaf(-A.s, tb, A.cbar[e]);
      rowacc[i] += tb;
      colp += tb;
    }
    const double cs = block_sum_d((double)colp, red);
    if (threadIdx.x == 0) A.vbar[A.nr + j] = (float)cs;  // phi2bar of s_k
  }
  __syncthreads();
  for (int i = threadIdx.x; i < A.nr; i += blockDim.x)
    A.rowpart[(long long)chunk * A.nr + i] = rowacc[i];
}

__global__ void gl_adj_rows(const GlaParams A, int chunks) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.nr; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += (double)A.rowpart[(long long)c * A.nr + i];
    A.vbar[i] = (float)s;  // phi1bar of s_k
  }
}

struct GlaLayout {
  size_t off_rbar, off_cbar, off_sbar, off_sig, off_coef, off_rowpart, off_gid, total;
  int chunks;
};

static GlaLayout gla_layout(int nr, int nc, int G) {
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  GlaLayout L;
  L.chunks = (nc + kGlaChunk - 1) / kGlaChunk;
  size_t off = 0;
  L.off_rbar = off;    off = al(off + sizeof(float) * nr);
  L.off_cbar = off;    off = al(off + sizeof(float) * nc);
  L.off_sbar = off;    off = al(off + sizeof(float) * 4);
  L.off_sig = off;     off = al(off + sizeof(float) * (size_t)G * nc);
  L.off_coef = off;    off = al(off + sizeof(float) * (size_t)G * nc);
  L.off_rowpart = off; off = al(off + sizeof(float) * (size_t)L.chunks * nr);
  L.off_gid = off;     off = al(off + sizeof(int) * nr);
  L.total = off;
  return L;
}

}  // namespace drot

using namespace drot;

extern "C" {

size_t drot_gl_adjoint_workspace_bytes(int n_rows, int n_cols, int n_groups) {
  if (n_rows <= 0 || n_cols <= 0 || n_groups <= 0 || n_groups > kMaxGroups ||
      n_rows > 48 * 1024)
    return 0;
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
  A.gid = (int*)(ws + L.off_gid);
  gl_adj_vec<<<1, kGlaThreads, 0, st>>>(A);
  const long long tasks = (long long)n_groups * n_cols;
  const int gblocks = (int)std::min<long long>((tasks + 7) / 8, 4096);
  gl_adj_groups<<<gblocks, 256, 0, st>>>(A);
  const size_t smem = sizeof(float) * (size_t)n_rows;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)gl_adj_elems, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return DROT_ERR_CUDA;
  gl_adj_elems<<<L.chunks, kGlaThreads, smem, st>>>(A);
  gl_adj_rows<<<(n_rows + 255) / 256, 256, 0, st>>>(A, L.chunks);
  return cudaGetLastError() == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

}  // extern "C"
