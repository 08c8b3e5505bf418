// drot_adjoint.cu -- implicit adjoint of the quadratic-regularised DROT plan.
//
// No counterpart in the reference (its operators return plans without
// autograd, pytorch/src/drot_cuda.cpp:26-44).  At the solution of
//     min <C, X> + (lambda / 2) ||X||_F^2  s.t.  X 1 = p, X^T 1 = q, X >= 0
// (the fixed point of the QR iteration, lambda = (kappa - 1) / s), the plan on
// its support S is X_ij = (u_i + v_j - C_ij) / lambda.  Differentiating the
// marginal constraints on a fixed support gives, for an upstream gradient
// G = dL/dX, the adjoint system
//     [ D_r  M  ] [a]   [ rowsum(G o M) ]
//     [ M^T  D_c] [b] = [ colsum(G o M) ]
// with M the 0/1 support mask and D_r, D_c its row / column counts; then
// dL/dC = (a_i + b_j - G_ij) / lambda on S (0 elsewhere), dL/dp = a,
// dL/dq = b.  The matrix is a graph Laplacian (of the bipartite support
// graph, after b -> -b): singular but the right-hand side is consistent, so
// conjugate gradients converge; a and b are determined up to a + t, b - t.
//
// The support is read off the duals, not off X: at the fixed point of
// X = max(X + phi1 + phi2 - sC, 0) / kappa the plan is positive exactly where
// D_ij = phi1_i + phi2_j - s C_ij > 0, while a finite solve still carries
// entries of X that decay geometrically towards 0 off the support (tiny but
// positive); counting those would add wrong equations to the system.
//
// Kernels here:
//   adj_mask_kernel  -- the support bitmasks of D > 0 in both layouts
//                       (column words: 32 rows of a column; row words: 32
//                       columns of a row) and a byte mask in the layout of C,
//                       one warp per 32 x 32 block.
//   adj_pcg_kernel   -- Jacobi-preconditioned CG for a batch of instances in
//                       one persistent cooperative launch.  Every matvec
//                       line (a row or a column of an instance) is one warp
//                       walking the set bits of its mask words and summing
//                       the search direction staged in shared memory.
//                       Two grid barriers per iteration; each instance
//                       stops on its own relative residual.
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

struct AdjInst {
  long long c_off;   // element offset of C (column-major, leading dimension ld)
  long long f1_off, f2_off;  // offsets of the instance's phi1 / phi2
  long long mc_off;  // word offset of the column-word mask [nc][nwr]
  long long mr_off;  // word offset of the row-word mask [nr][nwc]
  int nr, nc, ld, nwr, nwc;
  int v_off;         // offset of [a; b] in the packed vectors (nr + nc entries)
  int seg0, nseg;    // its segments (contiguous)
  int owner;         // CTA that counts its convergence
  float s;           // step size of the solve
  float lam;         // regularisation weight lambda = (kappa - 1) / s
};

struct AdjSeg {
  int inst, l0, l1, cta;  // lines [l0, l1) of instance inst, processed by CTA cta
};

struct AdjParams {
  const void* c;
  int c_bf16;
  const float *phi1, *phi2;
  unsigned char* mask;  // byte mask, layout of C (may be null)
  const float* g;       // upstream gradient dL/dX, layout of C
  double* z;            // solution [a; b]
  double *r, *d0, *d1, *q, *invdiag, *deg;
  unsigned *mcol, *mrow;
  const AdjInst* inst;
  const AdjSeg* seg;
  const int* cta_seg0;  // [grid + 1]: the segments of CTA c are cta_seg0[c] .. cta_seg0[c+1]
  double* slot_dq;      // per segment: d.q
  double* slot_ry;      // [2][n_seg]: r.y (y = M^-1 r), by iteration parity
  double* slot_rr;      // [2][n_seg]: r.r, by iteration parity
  double* slot_rr0;     // per segment: initial r.r
  int* iters;           // per instance: CG iterations run
  int* conv;            // per instance: converged flag (owner CTA only)
  double* relres;       // per instance: final relative residual ||r|| / ||r0||
  unsigned* conv_count;
  unsigned* bar;
  int* abort_flag;
  long long timeout_ns;
  int n_inst, n_seg, max_iters;
  double tol;
};

// ---------------------------------------------------------------------------
// support masks
// ---------------------------------------------------------------------------

// grid: (blocks, n_inst); a warp per 32 x 32 block (row word w, column word v).
__global__ void adj_mask_kernel(const AdjParams A) {
  const int k = blockIdx.y;
  const AdjInst I = A.inst[k];
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const long long nblk = (long long)I.nwr * I.nwc;
  for (long long blk = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); blk < nblk;
       blk += (long long)gridDim.x * wpb) {
    const int w = (int)(blk % I.nwr);  // row word
    const int v = (int)(blk / I.nwr);  // column word
    const int i = w * 32 + lane;
    const float f1 = i < I.nr ? __ldg(A.phi1 + I.f1_off + i) : 0.0f;
    unsigned mine = 0u, rowword = 0u;
    for (int c = 0; c < 32; ++c) {
      const int j = v * 32 + c;
      bool on = false;
      if (i < I.nr && j < I.nc) {
        const long long e = I.c_off + (long long)j * I.ld + i;
        const float cv = A.c_bf16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(A.c)[e])
                                  : __ldg(reinterpret_cast<const float*>(A.c) + e);
        const float f2 = __ldg(A.phi2 + I.f2_off + j);
        on = fmaf(-I.s, cv, f1 + f2) > 0.0f;
        if (A.mask) A.mask[e] = on ? 1 : 0;
      }
      const unsigned word = __ballot_sync(0xffffffffu, on);
      if (lane == c) mine = word;
      rowword |= ((word >> lane) & 1u) << c;
    }
    const int j = v * 32 + lane;
    if (j < I.nc) A.mcol[I.mc_off + (long long)j * I.nwr + w] = mine;
    if (i < I.nr) A.mrow[I.mr_off + (long long)i * I.nwc + v] = rowword;
  }
}

// ---------------------------------------------------------------------------
// batched PCG (FP64 vectors)
// ---------------------------------------------------------------------------

// Lines per warp step and 32-word blocks per line held in registers: a
// warp loads the mask words of 4 lines (up to 128 words = 4096 bits each per
// pass) before it walks any bit, so 16 loads per lane are in flight.
constexpr int kAdjLines = 4;
constexpr int kAdjWords = 4;

// Sum over the set bits of line l's mask words of the staged vector entries
// (rows sum the column half, columns the row half); lanes split the words,
// bits are walked in order, then a shuffle tree.  Deterministic.
__device__ __forceinline__ void lines_dot(const AdjParams& A, const AdjInst& I, int l0, int l1,
                                          const double* sv, int lane, double (&out)[kAdjLines]) {
  double s[kAdjLines];
#pragma unroll
  for (int u = 0; u < kAdjLines; ++u) s[u] = 0.0;
  const int nwmax = max(I.nwr, I.nwc);
  for (int w0 = 0; w0 < nwmax; w0 += 32 * kAdjWords) {
    unsigned wd[kAdjLines][kAdjWords];
#pragma unroll
    for (int u = 0; u < kAdjLines; ++u) {
      const int l = l0 + u;
      const bool row = l < I.nr;
      const int nw = row ? I.nwc : I.nwr;
      const unsigned* words = row ? A.mrow + I.mr_off + (long long)l * I.nwc
                                  : A.mcol + I.mc_off + (long long)(l - I.nr) * I.nwr;
#pragma unroll
      for (int kk = 0; kk < kAdjWords; ++kk) {
        const int w = w0 + kk * 32 + lane;
        wd[u][kk] = (l < l1 && w < nw) ? __ldcg(words + w) : 0u;
      }
    }
#pragma unroll
    for (int u = 0; u < kAdjLines; ++u) {
      const double* base = (l0 + u < I.nr) ? sv + I.nr : sv;
#pragma unroll
      for (int kk = 0; kk < kAdjWords; ++kk) {
        unsigned m = wd[u][kk];
        const double* b0 = base + (w0 + kk * 32 + lane) * 32;
        while (m) {
          const int b = __ffs(m) - 1;
          s[u] += b0[b];
          m &= m - 1u;
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < kAdjLines; ++u) out[u] = warp_sum_d(s[u]);
}

// Degree of line l and the right-hand side entry of the adjoint system: the
// sum of the upstream gradient g over the line's support (rowsum(g o M) for
// a row, colsum(g o M) for a column), in FP64.  Lanes split the mask words;
// fixed shuffle trees, so the result is deterministic.
__device__ __forceinline__ void line_degree_rhs(const AdjParams& A, const AdjInst& I, int l,
                                                int lane, int& deg, double& rhs) {
  int c = 0;
  double s = 0.0;
  const float* g = A.g + I.c_off;
  if (l < I.nr) {  // row i = l: set bits are columns j, g at j * ld + i (strided gather)
    const unsigned* words = A.mrow + I.mr_off + (long long)l * I.nwc;
    for (int w = lane; w < I.nwc; w += 32) {
      unsigned m = __ldcg(words + w);
      c += __popc(m);
      while (m) {
        const int j = 32 * w + __ffs(m) - 1;
        s += (double)__ldg(g + (long long)j * I.ld + l);
        m &= m - 1u;
      }
    }
  } else {  // column j = l - nr: set bits are rows i, g contiguous down the column
    const int j = l - I.nr;
    const unsigned* words = A.mcol + I.mc_off + (long long)j * I.nwr;
    const float* gc = g + (long long)j * I.ld;
    for (int w = lane; w < I.nwr; w += 32) {
      unsigned m = __ldcg(words + w);
      c += __popc(m);
      while (m) {
        const int i = 32 * w + __ffs(m) - 1;
        s += (double)__ldg(gc + i);
        m &= m - 1u;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  deg = c;
  rhs = warp_sum_d(s);
}

// Sum over the segments of an instance of slot[] (fixed order).
__device__ __forceinline__ double inst_sum(const double* slot, const AdjInst& I) {
  double s = 0.0;
  for (int t = 0; t < I.nseg; ++t) s += __ldcg(slot + I.seg0 + t);
  return s;
}

// Vectors (r, d, q, z) and the staged direction are FP64: the adjoint system
// is a graph Laplacian whose support graph is often close to a forest (as
// many edges as vertices), so it is badly conditioned, and an FP32 CG stops
// at a solution error far above its residual.  The FP64 work is one add per
// set mask bit and O(lines) vector updates -- small beside the mask traffic.
__global__ void __launch_bounds__(256, 2) adj_pcg_kernel(const AdjParams A) {
  extern __shared__ __align__(16) double sv[];  // the staged direction of one instance
  __shared__ int s_flag;
  __shared__ double s_red[32 + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
  const int sg0 = A.cta_seg0[blockIdx.x], sg1 = A.cta_seg0[blockIdx.x + 1];
  const double tol2 = A.tol * A.tol;
  unsigned epoch = 0;

  // Prologue: degrees, the right-hand side from g, r = rhs, z = 0; parity-0
  // slots r.y and r.r.
  for (int sg = sg0; sg < sg1; ++sg) {
    const AdjSeg S = A.seg[sg];
    const AdjInst I = A.inst[S.inst];
    double ry = 0.0, rr = 0.0;
    for (int l = S.l0 + warp; l < S.l1; l += W) {
      int dg;
      double rhs;
      line_degree_rhs(A, I, l, lane, dg, rhs);
      if (lane == 0) {
        const int gi = I.v_off + l;
        const double inv = dg > 0 ? 1.0 / (double)dg : 0.0;
        const double r0 = dg > 0 ? rhs : 0.0;
        A.invdiag[gi] = inv;
        A.deg[gi] = (double)dg;
        A.r[gi] = r0;
        A.z[gi] = 0.0;
        ry += r0 * (inv * r0);
        rr += r0 * r0;
      }
    }
    ry = block_sum_d(ry, s_red);
    rr = block_sum_d(rr, s_red);
    if (threadIdx.x == 0) {
      A.slot_ry[sg] = ry;
      A.slot_rr[sg] = rr;
      A.slot_rr0[sg] = rr;
    }
  }
  if (!grid_barrier(A.bar, A.abort_flag, A.timeout_ns, epoch, &s_flag)) return;

  int it = 0;
  for (; it < A.max_iters; ++it) {
    const int par = it & 1;
    double* dcur = par ? A.d1 : A.d0;
    const double* dold = par ? A.d0 : A.d1;
    const double* ry_cur = A.slot_ry + (size_t)par * A.n_seg;
    const double* ry_prev = A.slot_ry + (size_t)(par ^ 1) * A.n_seg;
    const double* rr_cur = A.slot_rr + (size_t)par * A.n_seg;

    // ---- phase A: d = y + beta d_old (staged), q = A d on this CTA's lines
    for (int sg = sg0; sg < sg1; ++sg) {
      const AdjSeg S = A.seg[sg];
      const int k = S.inst;
      const AdjInst I = A.inst[k];
      const bool done = !(inst_sum(rr_cur, I) > tol2 * inst_sum(A.slot_rr0, I));
      if (done) {
        if (sg == I.seg0 && threadIdx.x == 0 && !A.conv[k]) {
          A.conv[k] = 1;
          atomicAdd(A.conv_count, 1u);
        }
        continue;
      }
      const double beta = it == 0 ? 0.0 : inst_sum(ry_cur, I) / inst_sum(ry_prev, I);
      const int nv = I.nr + I.nc;
      __syncthreads();
      // Stage d = M^-1 r + beta d_old for the whole instance: a thread takes
      // 4 entries and issues their 12 loads before using any.
      for (int t0 = threadIdx.x; t0 < nv; t0 += 4 * blockDim.x) {
        double iv[4], rv[4], dv0[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          const int gi = I.v_off + (t < nv ? t : 0);
          iv[u] = __ldcg(A.invdiag + gi);
          rv[u] = __ldcg(A.r + gi);
          dv0[u] = it == 0 ? 0.0 : __ldcg(dold + gi);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          if (t >= nv) break;
          const double y = iv[u] * rv[u];
          const double dv = it == 0 ? y : fma(beta, dv0[u], y);
          sv[t] = dv;
          if (t >= S.l0 && t < S.l1) dcur[I.v_off + t] = dv;
        }
      }
      __syncthreads();
      double dq = 0.0;
      for (int l0 = S.l0 + warp * kAdjLines; l0 < S.l1; l0 += W * kAdjLines) {
        double s[kAdjLines];
        lines_dot(A, I, l0, S.l1, sv, lane, s);
        if (lane == 0) {
#pragma unroll
          for (int u = 0; u < kAdjLines; ++u) {
            const int l = l0 + u;
            if (l < S.l1) {
              const int gi = I.v_off + l;
              const double dl = sv[l];
              const double qv = fma(__ldcg(A.deg + gi), dl, s[u]);
              A.q[gi] = qv;
              dq += dl * qv;
            }
          }
        }
      }
      dq = block_sum_d(dq, s_red);
      if (threadIdx.x == 0) A.slot_dq[sg] = dq;
    }
    if (!grid_barrier(A.bar, A.abort_flag, A.timeout_ns, epoch, &s_flag)) return;
    if (__ldcg(A.conv_count) >= (unsigned)A.n_inst) break;

    // ---- phase B: z += alpha d, r -= alpha q; next-parity slots r.y, r.r
    double* ry_next = A.slot_ry + (size_t)(par ^ 1) * A.n_seg;
    double* rr_next = A.slot_rr + (size_t)(par ^ 1) * A.n_seg;
    for (int sg = sg0; sg < sg1; ++sg) {
      const AdjSeg S = A.seg[sg];
      const AdjInst I = A.inst[S.inst];
      if (!(inst_sum(rr_cur, I) > tol2 * inst_sum(A.slot_rr0, I))) {
        // Converged: carry this segment's r.y and r.r into the next parity's
        // slots, so the instance reads the same (converged) sums on every
        // later iteration and stays stopped.  Without the copy the next
        // iteration would read the slots of two iterations back, find the
        // instance unconverged and step it again with stale CG scalars.
        if (threadIdx.x == 0) {
          ry_next[sg] = __ldcg(ry_cur + sg);
          rr_next[sg] = __ldcg(rr_cur + sg);
        }
        continue;
      }
      const double dq = inst_sum(A.slot_dq, I);
      const double alpha = dq > 0.0 ? inst_sum(ry_cur, I) / dq : 0.0;
      double ry = 0.0, rr = 0.0;
      for (int l = S.l0 + threadIdx.x; l < S.l1; l += blockDim.x) {
        const int gi = I.v_off + l;
        const double zl = fma(alpha, __ldcg(dcur + gi), A.z[gi]);
        const double rl = fma(-alpha, __ldcg(A.q + gi), A.r[gi]);
        A.z[gi] = zl;
        A.r[gi] = rl;
        const double yl = __ldcg(A.invdiag + gi) * rl;
        ry += rl * yl;
        rr += rl * rl;
      }
      ry = block_sum_d(ry, s_red);
      rr = block_sum_d(rr, s_red);
      if (threadIdx.x == 0) {
        ry_next[sg] = ry;
        rr_next[sg] = rr;
        if (sg == I.seg0) A.iters[S.inst] = it + 1;
      }
    }
    if (!grid_barrier(A.bar, A.abort_flag, A.timeout_ns, epoch, &s_flag)) return;
  }
  // Final relative residual of each instance, from the slots of the parity
  // the last phase A read (written, and made visible by a grid barrier,
  // before the loop ended); the CTA of the instance's first segment writes it.
  const double* rr_fin = A.slot_rr + (size_t)(it & 1) * A.n_seg;
  for (int sg = sg0; sg < sg1; ++sg) {
    const AdjSeg S = A.seg[sg];
    const AdjInst I = A.inst[S.inst];
    if (sg == I.seg0 && threadIdx.x == 0) {
      const double r0 = inst_sum(A.slot_rr0, I);
      A.relres[S.inst] = r0 > 0.0 ? sqrt(inst_sum(rr_fin, I) / r0) : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// gradient assembly
// ---------------------------------------------------------------------------

// dL/dC = (a_i + b_j - g_ij) / lambda on the support, 0 elsewhere (FP64
// arithmetic on the support entries, rounded once), for every element of an
// instance's n_rows x n_cols block; grid (column blocks, instances), a warp
// per column, a lane per 4 rows (one 128-row chunk per step).  Off-support
// groups of 4 rows are written as zeros without reading g.  Block 0 of each
// instance also writes dL/dp = a + t, dL/dq = b - t with the gauge t =
// (sum b - sum a) / (n_rows + n_cols) (FP64 sums in a fixed order).
__global__ void __launch_bounds__(256) adj_grad_kernel(const AdjParams A, float* __restrict__ gc,
                                                       float* __restrict__ gp,
                                                       float* __restrict__ gq) {
  __shared__ double s_red[32 + 1];
  const int k = blockIdx.y;
  const AdjInst I = A.inst[k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
  const double* za = A.z + I.v_off;
  const double* zb = za + I.nr;
  const double inv_lam = 1.0 / (double)I.lam;
  for (int j = blockIdx.x * W + warp; j < I.nc; j += gridDim.x * W) {
    const unsigned* words = A.mcol + I.mc_off + (long long)j * I.nwr;
    const float* gcol = A.g + I.c_off + (long long)j * I.ld;
    float* ocol = gc + I.c_off + (long long)j * I.ld;
    const double bj = __ldcg(zb + j);
    for (int i0 = 0; i0 < I.nr; i0 += 128) {
      const int i = i0 + 4 * lane;
      if (i >= I.nr) continue;
      const unsigned wd = __ldcg(words + (i >> 5));
      const unsigned m4 = (wd >> (i & 31)) & 0xfu;
      float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      if (m4) {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (((m4 >> e) & 1u) && i + e < I.nr)
            o[e] = (float)(((__ldcg(za + i + e) + bj) - (double)__ldg(gcol + i + e)) * inv_lam);
      }
      if (i + 4 <= I.nr && (((I.c_off + (long long)j * I.ld + i) & 3) == 0)) {
        *reinterpret_cast<float4*>(ocol + i) = make_float4(o[0], o[1], o[2], o[3]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (i + e < I.nr) ocol[i + e] = o[e];
      }
    }
  }
  if (blockIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int i = threadIdx.x; i < I.nr; i += blockDim.x) sa += __ldcg(za + i);
    for (int j = threadIdx.x; j < I.nc; j += blockDim.x) sb += __ldcg(zb + j);
    sa = block_sum_d(sa, s_red);
    sb = block_sum_d(sb, s_red);
    const double t = (sb - sa) / (double)(I.nr + I.nc);
    for (int i = threadIdx.x; i < I.nr; i += blockDim.x) gp[I.f1_off + i] = (float)(za[i] + t);
    for (int j = threadIdx.x; j < I.nc; j += blockDim.x) gq[I.f2_off + j] = (float)(zb[j] - t);
  }
}

}  // namespace drot

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

using namespace drot;

namespace {

struct AdjLayout {
  int grid = 0, threads = 256, n_seg = 0, V = 0;
  size_t smem = 0;
  std::vector<AdjInst> inst;
  std::vector<AdjSeg> seg;
  std::vector<int> cta_seg0;
  long long mcol_words = 0, mrow_words = 0;
  size_t off_ctrl = 0, off_inst = 0, off_seg = 0, off_cta = 0, off_mcol = 0, off_mrow = 0,
         off_vec = 0, off_slots = 0, off_iters = 0, off_conv = 0, off_relres = 0, total = 0;
};

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

int adj_layout(int n_inst, const drot_adjoint_instance* d, AdjLayout& L) {
  if (n_inst <= 0 || n_inst > 65535 || !d) return DROT_ERR_INVALID_ARG;
  L.inst.resize(n_inst);
  long long V = 0, mc = 0, mr = 0, lines = 0;
  int maxv = 0;
  for (int k = 0; k < n_inst; ++k) {
    const drot_adjoint_instance& a = d[k];
    if (a.n_rows <= 0 || a.n_cols <= 0 || a.ld < a.n_rows || a.c_offset < 0 ||
        a.v_offset < 0 || a.phi1_offset < 0 || a.phi2_offset < 0 || !(a.step_size > 0.0f) ||
        !(a.lambda > 0.0f) ||
        (long long)a.n_rows + a.n_cols > (1 << 24))
      return DROT_ERR_INVALID_ARG;
    AdjInst& I = L.inst[k];
    memset(&I, 0, sizeof(I));
    I.nr = a.n_rows;
    I.nc = a.n_cols;
    I.ld = a.ld;
    I.nwr = (a.n_rows + 31) / 32;
    I.nwc = (a.n_cols + 31) / 32;
    I.c_off = a.c_offset;
    I.f1_off = a.phi1_offset;
    I.f2_off = a.phi2_offset;
    I.s = a.step_size;
    I.lam = a.lambda;
    I.v_off = (int)a.v_offset;
    I.mc_off = mc;
    I.mr_off = mr;
    mc += (long long)a.n_cols * I.nwr;
    mr += (long long)a.n_rows * I.nwc;
    V = std::max(V, a.v_offset + a.n_rows + a.n_cols);
    lines += a.n_rows + a.n_cols;
    maxv = std::max(maxv, a.n_rows + a.n_cols);
  }
  if (V > INT32_MAX / 2) return DROT_ERR_UNSUPPORTED;
  L.V = (int)V;
  L.mcol_words = mc;
  L.mrow_words = mr;
  L.smem = sizeof(double) * (size_t)maxv;
  if (L.smem > 200 * 1024) return DROT_ERR_UNSUPPORTED;

  int dev = 0, sms = 0, coop = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return DROT_ERR_CUDA;
  if (L.smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)adj_pcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)L.smem) != cudaSuccess)
    return DROT_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)adj_pcg_kernel, L.threads,
                                                    L.smem) != cudaSuccess || occ <= 0)
    return DROT_ERR_CUDA;
  // At least ~64 lines per CTA: tiny batches do not spread over every SM.
  const long long want = std::max(1LL, lines / 64);
  L.grid = (int)std::min<long long>((long long)occ * sms, want);

  // Lines [c*lines/G, (c+1)*lines/G) go to CTA c, cut at instance boundaries.
  L.cta_seg0.assign(L.grid + 1, 0);
  long long base = 0;
  int k = 0;
  for (int c = 0; c < L.grid; ++c) {
    L.cta_seg0[c] = (int)L.seg.size();
    const long long g0 = lines * c / L.grid, g1 = lines * (c + 1) / L.grid;
    long long g = g0;
    while (g < g1) {
      while (g >= base + L.inst[k].nr + L.inst[k].nc) {
        base += L.inst[k].nr + L.inst[k].nc;
        ++k;
      }
      const long long end = std::min(g1, base + L.inst[k].nr + L.inst[k].nc);
      AdjSeg S;
      S.inst = k;
      S.l0 = (int)(g - base);
      S.l1 = (int)(end - base);
      S.cta = c;
      L.seg.push_back(S);
      g = end;
    }
  }
  L.cta_seg0[L.grid] = (int)L.seg.size();
  L.n_seg = (int)L.seg.size();
  for (int t = 0; t < L.n_seg; ++t) {
    AdjInst& I = L.inst[L.seg[t].inst];
    if (I.nseg == 0) {
      I.seg0 = t;
      I.owner = L.seg[t].cta;
    }
    ++I.nseg;
  }

  size_t off = 0;
  L.off_ctrl = off;  off = al256(off + 512);
  L.off_inst = off;  off = al256(off + sizeof(AdjInst) * n_inst);
  L.off_seg = off;   off = al256(off + sizeof(AdjSeg) * L.n_seg);
  L.off_cta = off;   off = al256(off + sizeof(int) * (L.grid + 1));
  L.off_mcol = off;  off = al256(off + sizeof(unsigned) * (size_t)mc);
  L.off_mrow = off;  off = al256(off + sizeof(unsigned) * (size_t)mr);
  L.off_vec = off;   off = al256(off + sizeof(double) * (size_t)V * 6);
  L.off_slots = off; off = al256(off + sizeof(double) * (size_t)L.n_seg * 6);
  L.off_iters = off; off = al256(off + sizeof(int) * n_inst);
  L.off_conv = off;  off = al256(off + sizeof(int) * n_inst);
  L.off_relres = off; off = al256(off + sizeof(double) * n_inst);
  L.total = off;
  return DROT_OK;
}

}  // namespace

// Device pointers of a workspace laid out by L.
static void adj_params(const AdjLayout& L, char* ws, AdjParams& A) {
  memset(&A, 0, sizeof(A));
  double* vec = (double*)(ws + L.off_vec);
  A.r = vec;
  A.d0 = vec + (size_t)L.V;
  A.d1 = vec + 2 * (size_t)L.V;
  A.q = vec + 3 * (size_t)L.V;
  A.invdiag = vec + 4 * (size_t)L.V;
  A.deg = vec + 5 * (size_t)L.V;
  A.mcol = (unsigned*)(ws + L.off_mcol);
  A.mrow = (unsigned*)(ws + L.off_mrow);
  A.inst = (const AdjInst*)(ws + L.off_inst);
  A.seg = (const AdjSeg*)(ws + L.off_seg);
  A.cta_seg0 = (const int*)(ws + L.off_cta);
  double* slots = (double*)(ws + L.off_slots);
  A.slot_dq = slots;
  A.slot_ry = slots + L.n_seg;
  A.slot_rr = slots + 3 * (size_t)L.n_seg;
  A.slot_rr0 = slots + 5 * (size_t)L.n_seg;
  A.iters = (int*)(ws + L.off_iters);
  A.conv = (int*)(ws + L.off_conv);
  A.relres = (double*)(ws + L.off_relres);
  A.bar = (unsigned*)(ws + L.off_ctrl);
  A.abort_flag = (int*)(ws + L.off_ctrl + 64);
  A.conv_count = (unsigned*)(ws + L.off_ctrl + 128);
  const char* e = getenv("DROT_BARRIER_TIMEOUT_MS");
  const long long ms = (e && atoll(e) > 0) ? atoll(e) : 10000LL;
  A.timeout_ns = ms * 1000000LL;
  A.n_seg = L.n_seg;
}

extern "C" {

size_t drot_qr_adjoint_workspace_bytes(int n_inst, const drot_adjoint_instance* inst) {
  AdjLayout L;
  return adj_layout(n_inst, inst, L) == DROT_OK ? L.total : 0;
}

int drot_qr_adjoint_prepare(int n_inst, const drot_adjoint_instance* inst, const void* c,
                            int c_dtype, const float* phi1, const float* phi2,
                            unsigned char* mask, void* workspace, size_t workspace_bytes,
                            drot_stream_t stream) {
  if (!c || !phi1 || !phi2 || !workspace) return DROT_ERR_INVALID_ARG;
  if (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  AdjLayout L;
  int rc = adj_layout(n_inst, inst, L);
  if (rc != DROT_OK) return rc;
  if (workspace_bytes < L.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  cudaStream_t st = (cudaStream_t)stream;
  AdjParams A;
  adj_params(L, ws, A);
  A.c = c;
  A.c_bf16 = c_dtype == DROT_C_BF16;
  A.phi1 = phi1;
  A.phi2 = phi2;
  A.mask = mask;
  A.n_inst = n_inst;
  if (cudaMemcpyAsync(ws + L.off_inst, L.inst.data(), sizeof(AdjInst) * n_inst,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws + L.off_seg, L.seg.data(), sizeof(AdjSeg) * L.n_seg,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws + L.off_cta, L.cta_seg0.data(), sizeof(int) * (L.grid + 1),
                      cudaMemcpyHostToDevice, st) != cudaSuccess)
    return DROT_ERR_CUDA;
  long long maxblk = 0;
  for (const AdjInst& I : L.inst) maxblk = std::max(maxblk, (long long)I.nwr * I.nwc);
  const int mblocks = (int)std::min<long long>((maxblk + 7) / 8, 2048);
  adj_mask_kernel<<<dim3(mblocks, n_inst), 256, 0, st>>>(A);
  if (cudaGetLastError() != cudaSuccess) return DROT_ERR_CUDA;
  // The descriptors above are copied from pageable host memory that dies
  // with this call: wait for the copies (and the mask) to finish.
  return cudaStreamSynchronize(st) == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

int drot_qr_adjoint_solve(int n_inst, const drot_adjoint_instance* inst, const float* g,
                          double* z, double tol, int max_iters, void* workspace,
                          size_t workspace_bytes, int* iters, drot_stream_t stream) {
  if (!g || !z || !workspace || max_iters < 0 || !(tol >= 0.0)) return DROT_ERR_INVALID_ARG;
  AdjLayout L;
  int rc = adj_layout(n_inst, inst, L);
  if (rc != DROT_OK) return rc;
  if (workspace_bytes < L.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  cudaStream_t st = (cudaStream_t)stream;
  AdjParams A;
  adj_params(L, ws, A);
  A.g = g;
  A.z = z;
  A.n_inst = n_inst;
  A.max_iters = max_iters;
  A.tol = tol;
  if (cudaMemsetAsync(ws + L.off_ctrl, 0, 512, st) != cudaSuccess ||
      cudaMemsetAsync(ws + L.off_iters, 0, L.total - L.off_iters, st) != cudaSuccess)
    return DROT_ERR_CUDA;
  void* args[] = {(void*)&A};
  if (cudaLaunchCooperativeKernel((const void*)adj_pcg_kernel, dim3(L.grid), dim3(L.threads), args,
                                  L.smem, st) != cudaSuccess) {
    cudaGetLastError();
    return DROT_ERR_CUDA;
  }
  int abort_flag = 0;
  if ((iters && cudaMemcpyAsync(iters, ws + L.off_iters, sizeof(int) * n_inst,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
      cudaMemcpyAsync(&abort_flag, ws + L.off_ctrl + 64, sizeof(int), cudaMemcpyDeviceToHost,
                      st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return DROT_ERR_CUDA;
  return abort_flag ? DROT_ERR_BARRIER_TIMEOUT : DROT_OK;
}

int drot_qr_adjoint_grad(int n_inst, const drot_adjoint_instance* inst, const float* g,
                         const double* z, float* grad_c, float* grad_p, float* grad_q,
                         void* workspace, size_t workspace_bytes, drot_stream_t stream) {
  if (!g || !z || !grad_c || !grad_p || !grad_q || !workspace) return DROT_ERR_INVALID_ARG;
  AdjLayout L;
  int rc = adj_layout(n_inst, inst, L);
  if (rc != DROT_OK) return rc;
  if (workspace_bytes < L.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  AdjParams A;
  adj_params(L, (char*)workspace, A);
  A.g = g;
  A.z = const_cast<double*>(z);
  A.n_inst = n_inst;
  int maxc = 1;
  for (const AdjInst& I : L.inst) maxc = std::max(maxc, I.nc);
  const int blocks = std::min((maxc + 7) / 8, 1024);
  adj_grad_kernel<<<dim3(blocks, n_inst), 256, 0, (cudaStream_t)stream>>>(A, grad_c, grad_p,
                                                                        grad_q);
  return cudaGetLastError() == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

int drot_qr_adjoint_residuals(int n_inst, const drot_adjoint_instance* inst,
                              const void* workspace, size_t workspace_bytes, double* rel_residual,
                              drot_stream_t stream) {
  if (!workspace || !rel_residual) return DROT_ERR_INVALID_ARG;
  AdjLayout L;
  int rc = adj_layout(n_inst, inst, L);
  if (rc != DROT_OK) return rc;
  if (workspace_bytes < L.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(rel_residual, (const char*)workspace + L.off_relres,
                      sizeof(double) * n_inst, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return DROT_ERR_CUDA;
  return DROT_OK;
}

}  // extern "C"
