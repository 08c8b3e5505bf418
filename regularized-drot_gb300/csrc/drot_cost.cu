// drot_cost.cu -- squared-Euclidean cost matrices of point clouds on the
// 5th-generation tensor cores (tcgen05.mma kind::tf32, accumulator in TMEM).
//
// No counterpart in the reference, whose callers build C on the host
// (benchmark/utils/compute_w2_dist.py:68-94) and hand it to the solver.  For
// point clouds x (m x d) and y (n x d), row-major:
//     C[j*ld + i] = scale * max(||x_i||^2 + ||y_j||^2 - 2 <x_i, y_j>, 0)
// i.e. the column-major m x n cost the solver reads (the reference's PyTorch
// layout [n, m]).  The Gram term is one GEMM with K = d, done in "3xTF32":
// x = x_hi + x_lo with x_hi = RN_tf32(x), x_lo = RN_tf32(x - x_hi) (same
// for y), <x, y> ~ x_hi.y_hi + x_hi.y_lo + x_lo.y_hi accumulated in FP32 --
// the split-precision scheme that gives FP32-level accuracy on TF32 tensor
// cores (the dropped x_lo.y_lo term is below 2^-22 relative).  Norms are
// FP32 FMA sums in k order.
//
// Persistent kernel (at most two CTAs per SM, each walking the tiles of all
// instances with stride grid): per 128 x 128 tile, 256 threads stage the
// hi / lo operand tiles in shared memory (K-major, no swizzle: 8-row x
// 16-byte core matrices), one thread issues 3 * d/8 MMAs into a 128-lane x
// 128-column TMEM accumulator and a tcgen05.commit arrives on an mbarrier;
// then each warp reads its TMEM lane quadrant for half of the columns
// (tcgen05.ld 32x32b) and writes those rows of each column (128 bytes per
// warp store).  Operands and accumulators are double-buffered, so tile n+1's
// loads and MMAs run while tile n's C is stored.  The kernel is bound by the
// C stores (4 bytes per element).
#include <cuda_runtime.h>

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

constexpr int kCostM = 128;        // tile rows (x points) = TMEM lanes
constexpr int kCostN = 128;        // tile columns (y points) = TMEM columns
constexpr int kCostMaxInst = 256;  // instances per launch (descriptors travel in the parameters)
constexpr int kCostThreads = 256;  // 8 warps: x / y rows staged one per thread

struct CostInst {
  long long x_off, y_off, c_off;  // element offsets: x (m x d), y (n x d), C (ld x n)
  int m, n, ld, tiles_m, tiles;
  int tile0;  // tiles of the earlier instances
};

struct CostParams {
  const float* x;
  const float* y;
  float* c;
  int* err;
  long long timeout_ns;
  int dim, n_inst, clamp, total_tiles;
  float scale, pad2;
  CostInst inst[kCostMaxInst];
};

// Instruction descriptor of the tile's MMAs (M = 128 x points, N = 128 y points).
constexpr uint32_t kCostIdesc = tf32_idesc(kCostM, kCostN);

// Stage tile (i0, j0) of instance I into one operand buffer: x rows by
// threads 0..127, y rows by threads 128..255 (one row each): hi / lo TF32
// parts in the K-major layout, FP32 norms in k order.
__device__ __forceinline__ void cost_stage(const CostParams& P, const CostInst& I, int i0, int j0,
                                           unsigned char* buf, uint32_t op_bytes, float* norms) {
  const int d = P.dim, kc = d >> 2, tid = threadIdx.x;
  const bool is_y = tid >= kCostM;
  const int r = is_y ? tid - kCostM : tid;
  const int row = (is_y ? j0 : i0) + r;
  const bool in = row < (is_y ? I.n : I.m);
  const float4* src = reinterpret_cast<const float4*>(
      (is_y ? P.y + I.y_off : P.x + I.x_off) + (long long)(in ? row : 0) * d);
  unsigned char* hi_t = buf + (is_y ? 2 * op_bytes : 0);
  unsigned char* lo_t = hi_t + op_bytes;
  float nrm = 0.0f;
  for (int c4 = 0; c4 < kc; ++c4) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in) v = __ldg(src + c4);
    const float e[4] = {v.x, v.y, v.z, v.w};
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      hi[q] = to_tf32(e[q]);
      lo[q] = to_tf32(e[q] - __uint_as_float(hi[q]));
      nrm = fmaf(e[q], e[q], nrm);
    }
    const uint32_t off = kmaj_off(r, c4 * 4, kc);
    *reinterpret_cast<uint4*>(hi_t + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(lo_t + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
  norms[tid] = nrm;  // x norms [0, 128), y norms [128, 256)
}

// The 3 x d/8 MMAs of one tile into a 128-column TMEM accumulator, then a
// commit arriving on `bar` (one thread).
__device__ __forceinline__ void cost_issue(unsigned char* buf, uint32_t op_bytes, int d,
                                           uint32_t tmem, uint64_t* bar) {
  const uint32_t ah = smem_u32(buf), al = ah + op_bytes;
  const uint32_t bh = al + op_bytes, bl = bh + op_bytes;
  gram_tf32x3(ah, al, bh, bl, d, tmem, kCostIdesc);
  tc_commit(bar);
}

// Instance and tile coordinates of global tile g (k advances monotonically).
__device__ __forceinline__ void cost_locate(const CostParams& P, int g, int& k, int& i0, int& j0) {
  while (g >= P.inst[k].tile0 + P.inst[k].tiles) ++k;
  const int t = g - P.inst[k].tile0;
  i0 = (t % P.inst[k].tiles_m) * kCostM;
  j0 = (t / P.inst[k].tiles_m) * kCostN;
}

// Persistent: CTA b takes tiles b, b + grid, ... of all instances in order.
// Operand buffers and TMEM accumulators are double-buffered, so while the
// eight warps stage tile n+1 and then store tile n's C, the tensor core
// computes tile n+1: the MMA and the operand loads hide behind the stores.
__global__ void __launch_bounds__(kCostThreads, 1) cost_sqeuclid_kernel(const __grid_constant__ CostParams P) {
  const int d = P.dim;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t op_bytes = (uint32_t)kCostM * d * 4;  // one hi or lo tile (x or y: 128 rows)
  const uint32_t buf_bytes = 4 * op_bytes;
  // norms of tile n in slot n % 3: staging writes tile n+1's while slower
  // warps may still read tile n-1's
  float* norms = reinterpret_cast<float*>(smem + 2 * buf_bytes);  // [3][256]
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_tmem;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&s_tmem)), "r"((uint32_t)(2 * kCostN)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  int g = blockIdx.x, kk = 0, i0 = 0, j0 = 0;
  if (g < P.total_tiles) {
    cost_locate(P, g, kk, i0, j0);
    cost_stage(P, P.inst[kk], i0, j0, smem, op_bytes, norms);
  }
  fence_proxy_async_shared();  // generic-proxy smem writes -> visible to the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  if (tid == 0 && g < P.total_tiles) cost_issue(smem, op_bytes, d, tmem, &mbar[0]);

  // Epilogue split: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its lane
  // quadrant) and columns 64 (w / 4) .. + 63 of the accumulator.
  const int quad = warp & 3, half = warp >> 2;
  for (int n = 0; g < P.total_tiles; ++n, g += gridDim.x) {
    const int b = n & 1;
    const int g_next = g + (int)gridDim.x;
    int kn = kk, in0 = 0, jn0 = 0;
    if (g_next < P.total_tiles) {
      cost_locate(P, g_next, kn, in0, jn0);
      cost_stage(P, P.inst[kn], in0, jn0, smem + (b ^ 1) * buf_bytes, op_bytes,
                 norms + ((n + 1) % 3) * 256);
    }
    fence_proxy_async_shared();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0 && g_next < P.total_tiles)
      cost_issue(smem + (b ^ 1) * buf_bytes, op_bytes, d, tmem + (uint32_t)((b ^ 1) * kCostN),
                 &mbar[b ^ 1]);
    // tile n's accumulator: use n >> 1 of buffer b
    bool got = mbar_wait(&mbar[b], (uint32_t)((n >> 1) & 1), P.timeout_ns);
    if (!__syncthreads_and(got ? 1 : 0)) {
      // An MMA that never completed: report it, give the MMAs in flight a
      // second bounded chance to land, and stop without storing.
      if (tid == 0) atomicExch(P.err, 1);
      mbar_wait(&mbar[b], (uint32_t)((n >> 1) & 1), P.timeout_ns);
      if (g_next < P.total_tiles) mbar_wait(&mbar[b ^ 1], (uint32_t)(((n + 1) >> 1) & 1), P.timeout_ns);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    const CostInst& I = P.inst[kk];
    const int i = i0 + quad * 32 + lane;
    const float* nb = norms + (n % 3) * 256;
    const float xi = nb[quad * 32 + lane];
    float* crow = P.c + I.c_off + (long long)(j0 + half * 64) * I.ld + i;
    const bool full = i0 + kCostM <= I.m && j0 + kCostN <= I.n;
    const bool row_in = i < I.m;
#pragma unroll
    for (int cb = 0; cb < 64; cb += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + (uint32_t)(b * kCostN) + ((uint32_t)(quad * 32) << 16) +
                             (uint32_t)(half * 64 + cb);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
            "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
            "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
            "=r"(r[31])
          : "r"(taddr) : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const float* yn = nb + kCostM + half * 64 + cb;
      float* cp = crow + (long long)cb * I.ld;
      if (full) {
#pragma unroll
        for (int e = 0; e < 32; ++e) {
          float v = fmaf(-2.0f, __uint_as_float(r[e]), xi + yn[e]);
          if (P.clamp) v = fmaxf(v, 0.0f);
          cp[(long long)e * I.ld] = v * P.scale;
        }
      } else if (row_in) {
        const int jb = j0 + half * 64 + cb;
#pragma unroll
        for (int e = 0; e < 32; ++e) {
          if (jb + e < I.n) {
            float v = fmaf(-2.0f, __uint_as_float(r[e]), xi + yn[e]);
            if (P.clamp) v = fmaxf(v, 0.0f);
            cp[(long long)e * I.ld] = v * P.scale;
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    kk = kn;
    i0 = in0;
    j0 = jn0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"((uint32_t)(2 * kCostN)) : "memory");
}

static size_t cost_smem_bytes(int dim) {
  // two operand buffers (x hi / lo, y hi / lo: 4 x 128 rows x dim floats) + [3][256] norms
  return (size_t)2 * 4 * kCostM * dim * 4 + sizeof(float) * 3 * 256;
}

// ---------------------------------------------------------------------------
// chain rule of the cost to the points (autograd backward of the cost)
// ---------------------------------------------------------------------------
//
// For G = dL/dC of one instance (column-major m x n, the layout of C),
//     dL/dx_i = 2 scale (x_i sum_j G_ij - sum_j G_ij y_j)
//     dL/dy_j = 2 scale (y_j sum_i G_ij - sum_i G_ij x_i)
// (G zeroed where C = 0 when the cost was clamped).  CTA (band b, instance
// k) owns rows [256 b, 256 b + 256) and walks the columns in tiles of 64:
// the G tile goes to shared memory (row pitch 65: conflict-free both ways),
// thread t accumulates row t's sums over the columns (its dL/dx, written at
// the end), and thread (column c, k-group) the column sums of the tile over
// the band's rows, written as the band's partial of dL/dy; a second kernel
// adds the bands' partials in band order.  No atomics: deterministic.

constexpr int kGradRows = 256;  // rows per CTA (= threads)
constexpr int kGradCols = 64;   // columns per tile
constexpr int kGradPitch = kGradCols + 1;

struct GradInst {
  long long x_off, y_off, c_off;  // element offsets: x (m x d), y (n x d), G / C (ld x n)
  long long part_off;             // float offset of its partials [bands][n][d + 1]
  int m, n, ld, bands, aligned;
  int pad;
};

struct GradParams {
  const float* x;
  const float* y;
  const float* g;
  const float* c;  // null: no clamp mask
  float* gx;
  float* gy;
  float* part;
  int n_inst;
  float scale2;  // 2 * scale
  GradInst inst[kCostMaxInst];
};

template <int DIM>
__global__ void __launch_bounds__(kGradRows, 2) cost_grad_kernel(const GradParams P) {
  extern __shared__ __align__(16) float gsm[];
  float* gt = gsm;                               // [kGradRows][kGradPitch]
  float* xs = gt + kGradRows * kGradPitch;       // [kGradRows][DIM]
  float* ys = xs + kGradRows * DIM;              // [kGradCols][DIM]
  const GradInst I = P.inst[blockIdx.y];
  const int b = blockIdx.x;
  if (b >= I.bands) return;
  const int t = threadIdx.x;
  const int r0 = b * kGradRows;
  constexpr int KG = DIM / 4;  // k values per column thread
  for (int e = t; e < kGradRows * DIM; e += kGradRows) {
    const int r = e / DIM, k = e - r * DIM;
    xs[e] = r0 + r < I.m ? __ldg(P.x + I.x_off + (long long)(r0 + r) * DIM + k) : 0.0f;
  }
  float ax[DIM], rs = 0.0f;
#pragma unroll
  for (int k = 0; k < DIM; ++k) ax[k] = 0.0f;
  const int cc = t % kGradCols, kg = t / kGradCols;
  const float* gbase = P.g + I.c_off;
  const float* cbase = P.c ? P.c + I.c_off : nullptr;
  for (int c0 = 0; c0 < I.n; c0 += kGradCols) {
    __syncthreads();  // the previous tile's readers are done
    for (int e = t; e < kGradCols * DIM; e += kGradRows) {
      const int c = e / DIM, k = e - c * DIM;
      ys[e] = c0 + c < I.n ? __ldg(P.y + I.y_off + (long long)(c0 + c) * DIM + k) : 0.0f;
    }
    // G tile: a column is 256 contiguous rows; 64 threads per column, 4 rows each.
    for (int pass = 0; pass < kGradCols / 4; ++pass) {
      const int c = pass * 4 + t / 64, rr = 4 * (t % 64);
      const int j = c0 + c, i = r0 + rr;
      float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      if (j < I.n && i < I.m) {
        const long long off = (long long)j * I.ld + i;
        if (I.aligned && i + 4 <= I.m) {
          const float4 q = __ldg(reinterpret_cast<const float4*>(gbase + off));
          v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
          if (cbase) {
            const float4 cq = __ldg(reinterpret_cast<const float4*>(cbase + off));
            v[0] = cq.x > 0.0f ? v[0] : 0.0f;
            v[1] = cq.y > 0.0f ? v[1] : 0.0f;
            v[2] = cq.z > 0.0f ? v[2] : 0.0f;
            v[3] = cq.w > 0.0f ? v[3] : 0.0f;
          }
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (i + e < I.m) {
              const float gv = __ldg(gbase + off + e);
              v[e] = (!cbase || __ldg(cbase + off + e) > 0.0f) ? gv : 0.0f;
            }
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) gt[(rr + e) * kGradPitch + c] = v[e];
    }
    __syncthreads();
    // row t: sums over the tile's columns
    {
      const float* grow = gt + t * kGradPitch;
#pragma unroll 4
      for (int c = 0; c < kGradCols; ++c) {
        const float gv = grow[c];
        rs += gv;
#pragma unroll
        for (int k = 0; k < DIM; ++k) ax[k] = fmaf(gv, ys[c * DIM + k], ax[k]);
      }
    }
    // column cc, k-group kg: sums over the band's rows -> the band's partial
    {
      float ay[KG], cs = 0.0f;
#pragma unroll
      for (int k = 0; k < KG; ++k) ay[k] = 0.0f;
#pragma unroll 4
      for (int r = 0; r < kGradRows; ++r) {
        const float gv = gt[r * kGradPitch + cc];
        cs += gv;
#pragma unroll
        for (int k = 0; k < KG; ++k) ay[k] = fmaf(gv, xs[r * DIM + kg * KG + k], ay[k]);
      }
      const int j = c0 + cc;
      if (j < I.n) {
        float* pp = P.part + I.part_off + ((long long)b * I.n + j) * (DIM + 1);
#pragma unroll
        for (int k = 0; k < KG; ++k) pp[kg * KG + k] = ay[k];
        if (kg == 0) pp[DIM] = cs;
      }
    }
  }
  const int i = r0 + t;
  if (i < I.m) {
    float* o = P.gx + I.x_off + (long long)i * DIM;
#pragma unroll
    for (int k = 0; k < DIM; ++k) o[k] = P.scale2 * fmaf(xs[t * DIM + k], rs, -ax[k]);
  }
}

// dL/dy_j from the bands' partials, added in band order.
template <int DIM>
__global__ void cost_grad_reduce_kernel(const GradParams P) {
  const GradInst I = P.inst[blockIdx.y];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < I.n; j += gridDim.x * blockDim.x) {
    float a[DIM + 1];
#pragma unroll
    for (int k = 0; k <= DIM; ++k) a[k] = 0.0f;
    for (int b = 0; b < I.bands; ++b) {
      const float* pp = P.part + I.part_off + ((long long)b * I.n + j) * (DIM + 1);
#pragma unroll
      for (int k = 0; k <= DIM; ++k) a[k] += __ldcg(pp + k);
    }
    const float* yj = P.y + I.y_off + (long long)j * DIM;
    float* o = P.gy + I.y_off + (long long)j * DIM;
#pragma unroll
    for (int k = 0; k < DIM; ++k) o[k] = P.scale2 * fmaf(__ldg(yj + k), a[DIM], -a[k]);
  }
}

static size_t grad_smem_bytes(int dim) {
  return sizeof(float) * ((size_t)kGradRows * kGradPitch + (size_t)kGradRows * dim +
                          (size_t)kGradCols * dim);
}

// Partials layout; returns the floats they need (0: invalid descriptors).
static long long grad_layout(int n_inst, const drot_cost_instance* inst, int dim, GradParams* P) {
  long long part = 0;
  for (int k = 0; k < n_inst; ++k) {
    const drot_cost_instance& a = inst[k];
    if (a.m <= 0 || a.n <= 0 || a.ld < a.m || a.x_offset < 0 || a.y_offset < 0 || a.c_offset < 0)
      return 0;
    const int bands = (a.m + kGradRows - 1) / kGradRows;
    if (P) {
      GradInst& I = P->inst[k];
      I.x_off = a.x_offset * dim;
      I.y_off = a.y_offset * dim;
      I.c_off = a.c_offset;
      I.part_off = part;
      I.m = a.m;
      I.n = a.n;
      I.ld = a.ld;
      I.bands = bands;
      I.aligned = (a.ld % 4 == 0) && (a.c_offset % 4 == 0);
    }
    part += (long long)bands * a.n * (dim + 1);
  }
  return part;
}

}  // namespace drot

using namespace drot;

extern "C" {

size_t drot_sqeuclidean_cost_grad_workspace_bytes(int n_inst, const drot_cost_instance* inst,
                                                  int dim) {
  if (n_inst <= 0 || n_inst > kCostMaxInst || !inst || dim <= 0 || dim > 32 || (dim & 7))
    return 0;
  const long long f = grad_layout(n_inst, inst, dim, nullptr);
  return f > 0 ? (size_t)f * sizeof(float) : 0;
}

int drot_sqeuclidean_cost_grad(int n_inst, const drot_cost_instance* inst, const float* x,
                               const float* y, int dim, float scale, const float* c,
                               const float* grad_c, float* grad_x, float* grad_y,
                               void* workspace, size_t workspace_bytes, drot_stream_t stream) {
  if (n_inst <= 0 || n_inst > kCostMaxInst || !inst || !x || !y || !grad_c || !grad_x ||
      !grad_y || !workspace)
    return DROT_ERR_INVALID_ARG;
  if (dim <= 0 || dim > 32 || (dim & 7) != 0) return DROT_ERR_UNSUPPORTED;
  if (((uintptr_t)grad_c & 15u) || (c && ((uintptr_t)c & 15u))) return DROT_ERR_INVALID_ARG;
  static GradParams P;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  memset(&P, 0, sizeof(P));
  const long long nf = grad_layout(n_inst, inst, dim, &P);
  if (nf <= 0) return DROT_ERR_INVALID_ARG;
  if (workspace_bytes < (size_t)nf * sizeof(float)) return DROT_ERR_WORKSPACE;
  int max_bands = 0, max_n = 0;
  for (int k = 0; k < n_inst; ++k) {
    max_bands = std::max(max_bands, P.inst[k].bands);
    max_n = std::max(max_n, P.inst[k].n);
  }
  P.x = x;
  P.y = y;
  P.g = grad_c;
  P.c = c;
  P.gx = grad_x;
  P.gy = grad_y;
  P.part = (float*)workspace;
  P.n_inst = n_inst;
  P.scale2 = 2.0f * scale;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = grad_smem_bytes(dim);
  const void* k1 = dim == 8 ? (const void*)cost_grad_kernel<8>
                 : dim == 16 ? (const void*)cost_grad_kernel<16>
                 : dim == 24 ? (const void*)cost_grad_kernel<24>
                             : (const void*)cost_grad_kernel<32>;
  const void* k2 = dim == 8 ? (const void*)cost_grad_reduce_kernel<8>
                 : dim == 16 ? (const void*)cost_grad_reduce_kernel<16>
                 : dim == 24 ? (const void*)cost_grad_reduce_kernel<24>
                             : (const void*)cost_grad_reduce_kernel<32>;
  if (cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return DROT_ERR_CUDA;
  void* args[] = {(void*)&P};
  if (cudaLaunchKernel(k1, dim3(max_bands, n_inst), dim3(kGradRows), args, smem, st) !=
          cudaSuccess ||
      cudaLaunchKernel(k2, dim3(std::min((max_n + 255) / 256, 64), n_inst), dim3(256), args, 0,
                       st) != cudaSuccess) {
    cudaGetLastError();
    return DROT_ERR_CUDA;
  }
  return DROT_OK;
}


int drot_sqeuclidean_cost(int n_inst, const drot_cost_instance* inst, const float* x,
                          const float* y, int dim, float scale, int clamp, float* c,
                          drot_stream_t stream) {
  if (n_inst <= 0 || n_inst > kCostMaxInst || !inst || !x || !y || !c) return DROT_ERR_INVALID_ARG;
  if (dim <= 0 || dim > 32 || (dim & 7) != 0) return DROT_ERR_UNSUPPORTED;
  if (((uintptr_t)x & 15u) || ((uintptr_t)y & 15u)) return DROT_ERR_INVALID_ARG;
  // The parameter block (descriptors included) is about 12 KB: kept off the
  // stack, filled and launched under a lock (launch copies it).
  static CostParams P;
  static int* err_flag[64] = {};
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DROT_ERR_CUDA;
  if (!err_flag[dev] && cudaMalloc(&err_flag[dev], sizeof(int)) != cudaSuccess) return DROT_ERR_CUDA;
  int* err = err_flag[dev];
  memset(&P, 0, sizeof(P));
  long long total_tiles = 0;
  for (int k = 0; k < n_inst; ++k) {
    const drot_cost_instance& a = inst[k];
    if (a.m <= 0 || a.n <= 0 || a.ld < a.m || a.x_offset < 0 || a.y_offset < 0 ||
        a.c_offset < 0 || ((a.x_offset * dim) & 3) || ((a.y_offset * dim) & 3))
      return DROT_ERR_INVALID_ARG;
    CostInst& I = P.inst[k];
    I.x_off = a.x_offset * dim;
    I.y_off = a.y_offset * dim;
    I.c_off = a.c_offset;
    I.m = a.m;
    I.n = a.n;
    I.ld = a.ld;
    I.tiles_m = (a.m + kCostM - 1) / kCostM;
    const long long tiles = (long long)I.tiles_m * ((a.n + kCostN - 1) / kCostN);
    if (tiles > 65535LL * 1024) return DROT_ERR_UNSUPPORTED;
    I.tiles = (int)tiles;
    I.tile0 = (int)total_tiles;
    total_tiles += tiles;
    if (total_tiles > (1LL << 30)) return DROT_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  P.x = x;
  P.y = y;
  P.c = c;
  P.err = err;
  P.timeout_ns = 2000000000LL;
  P.dim = dim;
  P.n_inst = n_inst;
  P.clamp = clamp ? 1 : 0;
  P.scale = scale;
  P.total_tiles = (int)total_tiles;
  const size_t smem = cost_smem_bytes(dim);
  if (cudaFuncSetAttribute((const void*)cost_sqeuclid_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute((const void*)cost_sqeuclid_kernel,
                           cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
    return DROT_ERR_CUDA;
  // Persistent grid of two CTAs per SM: each holds 256 of the SM's 512 TMEM
  // columns, and the registers (under 128 per thread, 256 threads) and
  // shared memory (under 100 KB at d <= 24) of two fit an SM.  CTAs that do
  // not fit (d = 32) start when one finishes; the tile stride keeps every
  // tile covered either way.
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return DROT_ERR_CUDA;
  const int grid = (int)std::min<long long>(total_tiles, 2LL * sms);
  if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return DROT_ERR_CUDA;
  cost_sqeuclid_kernel<<<grid, kCostThreads, smem, st>>>(P);
  if (cudaGetLastError() != cudaSuccess) return DROT_ERR_CUDA;
  int h_err = 0;
  if (cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return DROT_ERR_CUDA;
  return h_err ? DROT_ERR_BARRIER_TIMEOUT : DROT_OK;
}

}  // extern "C"
