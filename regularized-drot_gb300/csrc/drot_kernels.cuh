// drot_kernels.cuh -- persistent fused DROT solve kernel for sm_103a.
//
// One cooperative launch runs the whole Douglas-Rachford solve of the
// reference's quadratic-regularised (core/drot_qr.hpp:159-234) or
// group-lasso-regularised (core/drot_glr.hpp:242-355) loop.
//
// Work split.  X and C are column-major (element (i, j) at j*ld + i).  Rows
// are cut into "bands": fixed-height bands for QR, the reference's group row
// ranges for GL.  CTA b owns band b / P and column chunk b % P for the whole
// solve.  Inside a CTA, warps form teams of Wt warps; a team processes one
// column of the band at a time, warp k of the team covering sub-band k
// (S = 32*VEC*KV rows; lane l holds rows base + k*S + v*32*VEC + l*VEC + e,
// v < KV, e < VEC).  One (band, column) segment is register resident, so the
// GL group norm needs no second pass over X.
//
// Data path.  When X and C are 16-byte aligned with a leading dimension that
// is a multiple of 4 (TMA = true), every warp streams its column segments
// through a private ring of shared-memory stages filled by cp.async.bulk
// (TMA bulk copies) and tracked by mbarriers, NS columns ahead of the one it
// computes; the bytes in flight are bounded by shared memory, not registers.
// Otherwise (TMA = false) the warp loads its segment straight into registers.
//
// Per iteration (all on device, no host round trip):
//   phase 1  fused X-update over the CTA's tile: prox (QR divisor or GL group
//            shrink), store, per-lane row partials, per-warp column partials,
//            per-CTA mass and objective partials (float pairs);
//   barrier A
//   phase 2  CTA b reduces rows [b*nr/G, (b+1)*nr/G) and the same share of
//            columns: marginal residuals, duals a/b, phi1/phi2 (the
//            reference's update_aux, kernel_qr.hpp:405-467), and a
//            float-pair partial of the squared residual;
//   barrier B
//   stop test on the squared residual (QR: even iterations only, "< eps";
//            GL: every iteration, "<= eps"), identical in every CTA.
//
// Every wait is bounded by wall time (globaltimer): a grid barrier or an
// mbarrier that waits longer than the limit raises an abort flag, every CTA
// leaves its loop, and the host reads DROT_ERR_BARRIER_TIMEOUT.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "drot_math.cuh"

namespace drot {

enum { MODE_QR = 0, MODE_GL = 1 };

// Largest number of GL groups (classes); the boundaries travel in the
// kernel parameter block.
constexpr int kMaxGroups = 256;

// Device-side result block (lives at offset 0 of the workspace).
struct DeviceStats {
  int n_iter;          // reference convention (see drot_gb300.h)
  int iters_run;       // iterations actually executed
  int converged;
  int status;          // 0 ok, 3 wait time limit hit
  int objective_valid; // QR: 0 until an even iteration ran
  int pad;
  double objective;    // <C, X> of the last objective-bearing iteration
  double residual;     // absolute marginal residual at the last stop test
  double sigma;        // total mass sum(X) of the last iteration
  // Wall time of CTA 0 per stage, summed over iterations (globaltimer ns):
  // phase 1, barrier A, phase 2, barrier B + stop test.
  double phase_ns[4];
};

struct SolveParams {
  const void* c;       // float or __nv_bfloat16 (the kernel's CT)
  const float* p;
  const float* q;
  float* x;
  float* a;
  float* b;
  float* phi1;
  float* phi2;
  float* alpha;        // device scalar
  long long ld;        // leading dimension of X and C (elements)
  int nr, nc;
  float s;             // step size
  float kappa;         // QR divisor
  float kappa_rcp;     // RN(1 / kappa)
  float nc_rcp;        // RN(1 / float(nc))
  float nr_rcp;        // RN(1 / float(nr))
  float lambda;        // GL threshold
  double res2_stop;    // stop when the squared residual (FP64) is below this:
                       // the exact image of the "< eps" / "<= eps" test on
                       // its square root of the absolute tolerance eps
                       // (set by the host)
  int max_iters;
  int stop_every;      // QR: test every iteration (numpy-API loop), not only even ones
  int stop_le;         // QR: stop on residual <= eps (numpy-API loop) instead of < eps
  int nbands;          // QR: row bands; GL: groups
  int P;               // CTAs per band (column chunks)
  int Wt;              // warps per team (sub-bands per band)
  int nsb;             // nbands * Wt sub-bands (column partial rows)
  int band_h;          // QR: rows per band
  int ns;              // TMA ring stages per warp
  int p2_smem;         // phase-2 state (p, q, a, b slices) in shared memory
  int p2_cap_r;        // rows / columns per CTA slice (multiples of 4)
  int p2_cap_c;
  float* rowpart;      // [P][nr]
  float* colpart;      // [nsb][nc]
  float2* cta_sum;     // [grid] float pairs (hi, lo)
  float2* cta_obj;     // [grid]
  float2* cta_res;     // [grid]
  unsigned int* bar;   // barrier arrival counter (zeroed before launch)
  int* abort_flag;     // zeroed before launch
  DeviceStats* stats;
  int timer_cta;       // CTA whose stage times are recorded (phase_ns)
  int stall_cta;       // test hook of the bounded waits (grid_barrier); -1 off
  long long timeout_ns;
  int gbounds[kMaxGroups + 1];  // GL: group row boundaries
};


// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Hint: fetch the 128-byte line holding p into L2 (no register, no wait).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" :: "l"(p));
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  int v;
  asm volatile("ld.volatile.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp sum of float pairs (fixed butterfly order; lane 0's result is the
// one used, so runs are bitwise repeatable).
__device__ __forceinline__ fpair warp_sum_fp(fpair v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const fpair u{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = fp_add(v, u);
  }
  return v;
}

// Sum of the float pairs v[0..n) over one warp: 16 strided loads per lane in
// flight at once (grids up to 512 CTAs take one round trip), a fixed add
// tree, then the shuffle tree.
__device__ __forceinline__ fpair warp_sum_strided_fp(const float2* v, int n, int lane) {
  fpair a[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int i = lane + 32 * u;
    const float2 t = i < n ? __ldcg(v + i) : make_float2(0.0f, 0.0f);
    a[u] = fpair{t.x, t.y};
  }
#pragma unroll
  for (int w = 8; w > 0; w >>= 1)
#pragma unroll
    for (int u = 0; u < w; ++u) a[u] = fp_add(a[u], a[u + w]);
  fpair t = a[0];
  for (int i = lane + 512; i < n; i += 32) {
    const float2 x = __ldcg(v + i);
    t = fp_add(t, fpair{x.x, x.y});
  }
  return warp_sum_fp(t);
}

// Deterministic block-wide FP64 sum; every thread receives the result.
// `scratch` holds blockDim/32 + 1 doubles.  FP64 runs on a narrow pipe here,
// so only warp 0 combines the per-warp sums.
__device__ __forceinline__ double block_sum_d(double v, double* scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < nw ? scratch[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) scratch[nw] = t;
  }
  __syncthreads();
  return scratch[nw];
}

// Deterministic block-wide sum of float pairs; every thread receives the
// result.  `scratch` holds blockDim/32 + 1 pairs.
__device__ __forceinline__ fpair block_sum_fp(fpair v, fpair* scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum_fp(v);
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  if (w == 0) {
    fpair t = lane < nw ? scratch[lane] : fp_make(0.0f);
    t = warp_sum_fp(t);
    if (lane == 0) scratch[nw] = t;
  }
  __syncthreads();
  return scratch[nw];
}

// Grid barrier.  Returns false when the run was aborted (time limit hit here
// or in another CTA).  `epoch` counts barriers passed by this CTA.
// stall_cta >= 0 is the failure-detection test hook: that CTA does not
// arrive at its first barrier, so every CTA's bounded wait runs out and the
// launch ends with the time-limit status (no fault, no unbounded wait).  The
// CTA
// barrier orders every thread's writes before thread 0's release add, and
// thread 0's acquire load before every thread's later reads (the release /
// acquire pattern needs no separate fences: 1.5 us per barrier at 300 CTAs
// against 1.8 us with a fence on each side).
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* abort_flag, long long timeout_ns,
                                             unsigned& epoch, int* s_flag, int stall_cta = -1) {
  __syncthreads();
  if (threadIdx.x == 0) {
    epoch += 1u;
    const unsigned target = epoch * gridDim.x;
    if (!(epoch == 1u && (int)blockIdx.x == stall_cta)) red_release_add_u32(bar, 1u);
    int ok = 1;
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    while ((int)(ld_acquire_u32(bar) - target) < 0) {
      if ((++spins & 31u) == 0u) {
        if (ld_volatile_i32(abort_flag)) { ok = 0; break; }
        if ((long long)(globaltimer_ns() - t0) > timeout_ns) {
          atomicExch(abort_flag, 1);
          ok = 0;
          break;
        }
      }
    }
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

__device__ __forceinline__ bool grid_barrier(const SolveParams& P, unsigned& epoch, int* s_flag) {
  return grid_barrier(P.bar, P.abort_flag, P.timeout_ns, epoch, s_flag, P.stall_cta);
}

// ---- shared-memory addresses, mbarriers and TMA bulk copies -------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait for the phase `parity` of an mbarrier.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  unsigned spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if ((++spins & 63u) == 0u && (long long)(globaltimer_ns() - t0) > limit_ns) return false;
  }
  return true;
}

// 1-D TMA bulk copy global -> shared, completing on `bar` (both addresses
// 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_all() {
  asm volatile("fence.proxy.async;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// ---- tcgen05 split-TF32 Gram products (5th-generation tensor cores) ------
//
// <x_i, y_j> for 128 x points (MMA M) against N y points with K = d:
// x = x_hi + x_lo, x_hi = RN_tf32(x), x_lo = RN_tf32(x - x_hi) (the same for
// y), accumulated in FP32 as x_hi.y_hi, then x_hi.y_lo, then x_lo.y_hi
// (the split-precision scheme that gives FP32-level products on TF32 tensor
// cores; the dropped x_lo.y_lo term is below 2^-22 relative).  Operands are
// K-major tiles in shared memory without swizzle: 8-row x 16-byte core
// matrices, kc = d / 4 of them per 8-row group.

__device__ __forceinline__ uint32_t to_tf32(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return r;
}

// Shared-memory matrix descriptor: start address, leading byte offset
// (between core matrices along K), stride byte offset (between 8-row
// groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tf32_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// Byte offset of element (r, k) of a K-major tile with kc = d / 4 core
// matrices per 8-row group.
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int kc) {
  return (uint32_t)((((r >> 3) * kc + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// Splits 4 consecutive k of one row into its tf32 hi / lo parts in the
// K-major tiles hi_t / lo_t.
__device__ __forceinline__ void stage_split4(unsigned char* hi_t, unsigned char* lo_t, int r,
                                             int k, int kc, float4 v) {
  const float e[4] = {v.x, v.y, v.z, v.w};
  uint32_t hi[4], lo[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    hi[q] = to_tf32(e[q]);
    lo[q] = to_tf32(e[q] - __uint_as_float(hi[q]));
  }
  const uint32_t off = kmaj_off(r, k, kc);
  *reinterpret_cast<uint4*>(hi_t + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
  *reinterpret_cast<uint4*>(lo_t + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
}

// The 3 x d / 8 MMAs of one split-TF32 Gram tile into the accumulator at
// tmem (shared-memory addresses of the four operand tiles; one thread).
__device__ __forceinline__ void gram_tf32x3(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl,
                                            int d, uint32_t tmem, uint32_t idesc) {
  const uint32_t sbo = (uint32_t)(d >> 2) * 128u;
  const int ks_n = d >> 3;  // K = 8 per kind::tf32 MMA = 2 core matrices
  for (int ks = 0; ks < ks_n; ++ks)
    mma_tf32(tmem, smem_desc(ah + ks * 256, 128, sbo), smem_desc(bh + ks * 256, 128, sbo), idesc,
             ks > 0 ? 1u : 0u);
  for (int ks = 0; ks < ks_n; ++ks)
    mma_tf32(tmem, smem_desc(ah + ks * 256, 128, sbo), smem_desc(bl + ks * 256, 128, sbo), idesc,
             1u);
  for (int ks = 0; ks < ks_n; ++ks)
    mma_tf32(tmem, smem_desc(al + ks * 256, 128, sbo), smem_desc(bh + ks * 256, 128, sbo), idesc,
             1u);
}

// Arrive on `bar` once every MMA this thread issued has completed.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(smem_u32(bar)) : "memory");
}

// 16 consecutive TMEM columns of the warp's lane quadrant (thread = lane).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Packed FP32 pairs: the sm_100-family add/mul/fma .f32x2 instructions work
// on two floats in a 64-bit register pair, each lane rounded exactly as the
// scalar instruction (round to nearest, no contraction), at half the issue
// slots.  The fused updates are issue-bound while X and C sit in L2.
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 x2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void x2_unpack(f32x2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 x2_add(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
// div_rn_by_fma on both lanes (nb = (-b, -b), y = (RN(1/b), RN(1/b))).
__device__ __forceinline__ f32x2 x2_div_rn_by_fma(f32x2 a, f32x2 nb, f32x2 y) {
  const f32x2 q0 = x2_mul(a, y);
  const f32x2 r0 = x2_fma(nb, q0, a);
  const f32x2 q1 = x2_fma(r0, y, q0);
  const f32x2 r1 = x2_fma(nb, q1, a);
  return x2_fma(r1, y, q1);
}

template <int VEC>
__device__ __forceinline__ void load_vec(const float* ptr, float (&v)[VEC]) {
  if constexpr (VEC == 4) {
    const float4 t = *reinterpret_cast<const float4*>(ptr);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
    v[0] = *ptr;
  }
}

template <int VEC>
__device__ __forceinline__ void load_vec_nc(const float* ptr, float (&v)[VEC]) {
  if constexpr (VEC == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(ptr));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
    v[0] = __ldg(ptr);
  }
}

// Cost loads: float, or bfloat16 widened exactly to float (a bf16 value is
// the top 16 bits of the float with the same value).
template <int VEC, typename CT>
__device__ __forceinline__ void load_c(const CT* ptr, float (&v)[VEC]) {
  if constexpr (std::is_same<CT, float>::value) {
    load_vec_nc<VEC>(ptr, v);
  } else if constexpr (VEC == 4) {
    const uint2 t = __ldg(reinterpret_cast<const uint2*>(ptr));
    v[0] = __uint_as_float(t.x << 16);
    v[1] = __uint_as_float(t.x & 0xffff0000u);
    v[2] = __uint_as_float(t.y << 16);
    v[3] = __uint_as_float(t.y & 0xffff0000u);
  } else {
    const unsigned short t = __ldg(reinterpret_cast<const unsigned short*>(ptr));
    v[0] = __uint_as_float((unsigned)t << 16);
  }
}

// C in the registers of the fused update: FP32 as loaded; BF16 kept as the
// raw packed pairs (two bf16 per 32-bit word: half the registers of the
// widened values, so the BF16 kernel fits the register budget without
// spilling) and widened exactly where it is used (c_at).
template <int VEC, typename CT>
__device__ __forceinline__ void load_c_raw(const CT* ptr, float (&v)[VEC]) {
  if constexpr (std::is_same<CT, float>::value) {
    load_vec_nc<VEC>(ptr, v);
  } else if constexpr (VEC == 4) {
    const uint2 t = __ldg(reinterpret_cast<const uint2*>(ptr));
    v[0] = __uint_as_float(t.x);
    v[1] = __uint_as_float(t.y);
    v[2] = 0.0f;
    v[3] = 0.0f;
  } else {
    v[0] = __uint_as_float((unsigned)__ldg(reinterpret_cast<const unsigned short*>(ptr)));
  }
}

template <typename CT, int VEC>
__device__ __forceinline__ float c_at(const float (&v)[VEC], int e) {
  if constexpr (std::is_same<CT, float>::value) {
    return v[e];
  } else {
    const unsigned w = __float_as_uint(v[e >> 1]);
    return __uint_as_float((e & 1) ? (w & 0xffff0000u) : (w << 16));
  }
}

template <int VEC>
__device__ __forceinline__ void store_vec(float* ptr, const float (&v)[VEC]) {
  if constexpr (VEC == 4) {
    *reinterpret_cast<float4*>(ptr) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    *ptr = v[0];
  }
}

// Sums the partials of the CTA's rows [r0, r1) (np_r partials, row i's
// partial k at rowpart[k * nr + i]) and columns [k0, k1) (np_c partials at
// colpart[k * nc + j]) in one pass: g threads per item, g a power of two
// <= 32 chosen so the items fill the block, every thread's loads issued
// together; load order, add tree and shuffle tree are fixed, so the sums are
// deterministic.  fin_r(i, sum) / fin_c(j, sum) run on the item's first thread.
template <typename FinR, typename FinC>
__device__ __forceinline__ void reduce_partials(int r0, int r1, int k0, int k1,
                                                const float* rowpart, const float* colpart,
                                                long long nr, long long nc, int np_r, int np_c,
                                                FinR fin_r, FinC fin_c) {
  const int R = r1 - r0;
  const int items = R + (k1 - k0);
  if (items <= 0) return;
  int g = 32;
  while (g > 1 && items * g > (int)blockDim.x) g >>= 1;
  const int per_round = blockDim.x / g;
  const int sub = threadIdx.x & (g - 1);
  for (int base = 0; base < items; base += per_round) {
    const int idx = base + (int)threadIdx.x / g;
    const bool live = idx < items;
    const bool is_row = idx < R;
    const float* pp = is_row ? rowpart + r0 + idx : colpart + k0 + (idx - R);
    const long long stride = is_row ? nr : nc;
    const int np = is_row ? np_r : np_c;
    float t = 0.0f;
    if (live) {
      float a[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int kk = sub + u * g;
        a[u] = kk < np ? __ldcg(pp + (long long)kk * stride) : 0.0f;
      }
      t = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
      for (int kk = sub + 8 * g; kk < np; kk += g) t += __ldcg(pp + (long long)kk * stride);
    }
    for (int o = g >> 1; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (live && sub == 0) {
      if (is_row) fin_r(r0 + idx, t);
      else fin_c(k0 + idx - R, t);
    }
  }
}

// Dynamic shared memory of the solve kernel (must match the device layout).
//   ring    TMA: W * ns * 2 * S floats (stage: X segment, C segment)
//           reg: W * S floats (row-partial staging only)
//   f1s     Wt * S floats (phi1 of the band rows)
//   st2     3 * (cap_r + cap_c) floats when the phase-2 state is in shared
//           memory (p, a, staged phi1 of the CTA's rows; q, b, phi2 of its columns)
//   dscr    W + 1 float pairs (per-warp mass / residual sums)
//   nslot   2 * W float pairs (per-warp objective sums; GL team norms)
//   mbar    W * ns uint64 (TMA only)
__host__ __device__ constexpr size_t solve_smem_bytes(int warps, int wt, int S, int ns, bool tma,
                                                      int p2_floats = 0) {
  return sizeof(float) * (size_t)warps * S * (tma ? 2 * ns : 1) + sizeof(float) * (size_t)wt * S +
         sizeof(float) * (size_t)p2_floats + sizeof(double) * (warps + 1) +
         sizeof(double) * 2 * warps + (tma ? sizeof(uint64_t) * (size_t)warps * ns : 0);
}

// ---------------------------------------------------------------------------
// The solve kernel
// ---------------------------------------------------------------------------

template <int MODE, int VEC, int KV, bool TMA, typename CT = float>
__global__ void __launch_bounds__(512, 1)
drot_solve_kernel(const SolveParams P) {
  static_assert(!TMA || VEC == 4, "the TMA path moves 16-byte vectors");
  static_assert(!TMA || std::is_same<CT, float>::value, "the TMA path streams float costs");
  const CT* const cbase = reinterpret_cast<const CT*>(P.c);
  constexpr int SV = 32 * VEC;        // rows per vector slot of a warp
  constexpr int S = SV * KV;          // rows per sub-band (one warp)
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int W = blockDim.x >> 5;
  const int Wt = P.Wt;
  const int NS = TMA ? P.ns : 1;
  const int capr = P.p2_smem ? P.p2_cap_r : 0;
  const int capc = P.p2_smem ? P.p2_cap_c : 0;
  float* ring = reinterpret_cast<float*>(smem_raw);
  float* red = ring;  // row-partial staging aliases the ring (ring idle then)
  float* f1s = ring + (size_t)W * S * (TMA ? 2 * NS : 1);
  float* s_p = f1s + (size_t)Wt * S;
  float* s_a = s_p + capr;
  float* s_t1 = s_a + capr;
  float* s_q = s_t1 + capr;
  float* s_b = s_q + capc;
  float* s_t2 = s_b + capc;
  fpair* dscr = reinterpret_cast<fpair*>(s_t2 + capc);
  fpair* nslot = dscr + W + 1;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(nslot + 2 * W);
  __shared__ int s_flag;
  __shared__ int s_stop;
  __shared__ float s_misc_f[2];
  __shared__ double s_misc_d[2];

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nteams = W / Wt;
  const int team = warp / Wt;
  const int k = warp - team * Wt;     // sub-band within the band
  const bool active_warp = team < nteams;

  const int band = blockIdx.x / P.P;
  const int chunk = blockIdx.x - band * P.P;
  int lo, hi;
  if constexpr (MODE == MODE_QR) {
    lo = min(band * P.band_h, P.nr);
    hi = min(lo + P.band_h, P.nr);
  } else {
    lo = P.gbounds[band];
    hi = P.gbounds[band + 1];
  }
  const int base = lo - (lo % VEC);
  const int c0 = (int)(((long long)P.nc * chunk) / P.P);
  const int c1 = (int)(((long long)P.nc * (chunk + 1)) / P.P);
  const long long ld = P.ld;
  const int sb = band * Wt + k;

  // Rows owned by this lane; validity is recomputed where needed (masks held
  // in registers would cost more than the two compares).
  const int lrow = base + k * S + lane * VEC;
  auto row0f = [&](int v) { return lrow + v * SV; };
  auto einf = [&](int v, int e) {
    const int r = lrow + v * SV + e;
    return active_warp && r >= lo && r < hi;
  };
  auto vanyf = [&](int v) {
    const int r = lrow + v * SV;
    return active_warp && r + VEC > lo && r < hi;
  };
  auto vallf = [&](int v) {
    const int r = lrow + v * SV;
    return active_warp && r >= lo && r + VEC <= hi;
  };
  bool full = active_warp;
#pragma unroll
  for (int v = 0; v < KV; ++v) full &= vallf(v);
  // Interior sub-bands (every lane's rows inside the band) skip all masking.
  const bool wfull = __all_sync(0xffffffffu, full);

  // TMA segment of this warp: rows [seg_lo, seg_lo + seg_rows), 16-byte granular.
  const int seg_lo = base + k * S;
  const int hi4 = (hi + 3) & ~3;
  const int seg_rows = (TMA && active_warp) ? max(0, min(seg_lo + S, hi4) - seg_lo) : 0;
  const uint32_t seg_bytes = (uint32_t)seg_rows * 4u;
  float* wring = ring + (size_t)warp * NS * 2 * S;
  uint64_t* wbar = mbar + (size_t)warp * NS;
  uint32_t pipe_cnt = 0;  // columns waited on by this warp (monotonic)
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      for (int i = 0; i < W * NS; ++i) mbar_init(mbar + i, 1);
      fence_mbar_init();
      fence_proxy_async_shared();
    }
  }

  // Phase-2 slices; their marginals and duals stay in shared memory.
  const int G = gridDim.x;
  const int r_lo = (int)(((long long)P.nr * blockIdx.x) / G);
  const int r_hi = (int)(((long long)P.nr * (blockIdx.x + 1)) / G);
  const int k_lo = (int)(((long long)P.nc * blockIdx.x) / G);
  const int k_hi = (int)(((long long)P.nc * (blockIdx.x + 1)) / G);
  if (P.p2_smem) {
    for (int i = threadIdx.x; i < r_hi - r_lo; i += blockDim.x) {
      s_p[i] = P.p[r_lo + i];
      s_a[i] = P.a[r_lo + i];
    }
    for (int j = threadIdx.x; j < k_hi - k_lo; j += blockDim.x) {
      s_q[j] = P.q[k_lo + j];
      s_b[j] = P.b[k_lo + j];
    }
  }
  __syncthreads();

  const float s = P.s;
  const float kappa = P.kappa;
  const float kappa_rcp = P.kappa_rcp;
  const float nc_f = (float)P.nc, nr_f = (float)P.nr;
  const float nc_rcp = P.nc_rcp, nr_rcp = P.nr_rcp;
  float alpha = *P.alpha;  // maintained by thread 0
  unsigned epoch = 0;
  int it = 0;
  bool converged = false;
  bool aborted = false;
  double last_obj = 0.0;
  int obj_valid = 0;
  double last_res = -1.0;
  double last_sigma = 0.0;

  // Stage timers of one CTA (thread 0, in shared memory to keep them out of
  // the registers of every thread).
  const bool timer = blockIdx.x == P.timer_cta;
  __shared__ unsigned long long s_tp;
  __shared__ unsigned long long s_tacc[4];
  if (threadIdx.x == 0) {
    s_tp = 0;
    for (int q = 0; q < 4; ++q) s_tacc[q] = 0ull;
  }
  auto stamp = [&](int k2) {  // CTA 0 only (block-uniform)
    if (timer) {
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned long long now = globaltimer_ns();
        if (k2 > 0) s_tacc[k2 - 1] += now - s_tp;
        s_tp = now;
      }
    }
  };

  for (; it < P.max_iters; ++it) {
    const bool even = (it & 1) == 0;
    const bool with_c = (MODE == MODE_GL) || even;
    stamp(0);

    // ------------------------------------------------------------ phase 1
    // phi1 of the band rows -> shared memory.
    for (int idx = threadIdx.x; idx < Wt * S; idx += blockDim.x) {
      const int r = base + idx;
      f1s[idx] = (r >= lo && r < hi) ? __ldcg(P.phi1 + r) : 0.0f;
    }
    __syncthreads();
    float acc[KV][VEC];
#pragma unroll
    for (int v = 0; v < KV; ++v)
#pragma unroll
      for (int e = 0; e < VEC; ++e) acc[v][e] = 0.0f;
    // Per-lane mass and objective sums over the warp's columns, carried as
    // exact float pairs (TwoSum); FP64 only once per iteration.
    float ms_hi = 0.0f, ms_lo = 0.0f, ob_hi = 0.0f, ob_lo = 0.0f;
    bool wfail = false;

    // One column of the band per team step.  EV selects the QR step that
    // reads C and stores the folded value X^ - sC (kernel_qr.hpp:171-278);
    // the odd QR step reads X only (kernel_qr.hpp:280-376).  FULL drops the
    // row masks of interior sub-bands.
    auto run_columns = [&](auto even_tag, auto full_tag) {
      constexpr bool EV = decltype(even_tag)::value;
      constexpr bool FULL = decltype(full_tag)::value;
      constexpr bool WITH_C = (MODE == MODE_GL) || EV;
      const int ncw = (c1 - c0 - team + nteams - 1) / nteams;  // columns of this warp
      const uint32_t tx_bytes = seg_bytes * (WITH_C ? 2u : 1u);
      uint32_t issued = pipe_cnt;
      auto issue = [&](int n) {  // lane 0: fetch column n of this warp into its stage
        const int jn = c0 + team + n * nteams;
        const int st = (int)(issued % (uint32_t)NS);
        float* dx = wring + (size_t)st * 2 * S;
        mbar_arrive_expect_tx(wbar + st, tx_bytes);
        bulk_g2s(dx, P.x + (long long)jn * ld + seg_lo, seg_bytes, wbar + st);
        if constexpr (WITH_C) bulk_g2s(dx + S, cbase + (long long)jn * ld + seg_lo, seg_bytes, wbar + st);
        ++issued;
      };

      // Register path: the warp's segment of column j straight into registers.
      auto load_reg = [&](int j, float (&xv)[KV][VEC], float (&cv)[KV][VEC]) {
        const float* xcol = P.x + (long long)j * ld;
        const CT* ccol = cbase + (long long)j * ld;
#pragma unroll
        for (int v = 0; v < KV; ++v) {
          if (FULL || vanyf(v)) {
            load_vec<VEC>(xcol + row0f(v), xv[v]);
            if constexpr (WITH_C) load_c_raw<VEC, CT>(ccol + row0f(v), cv[v]);
            else {
#pragma unroll
              for (int e = 0; e < VEC; ++e) cv[v][e] = 0.0f;
            }
          } else {
#pragma unroll
            for (int e = 0; e < VEC; ++e) { xv[v][e] = 0.0f; cv[v][e] = 0.0f; }
          }
        }
      };

      // TMA path: wait for the stage of this warp's next column and read it.
      auto load_tma = [&](int n, float (&xv)[KV][VEC], float (&cv)[KV][VEC]) {
        if (seg_rows > 0) {
          const int st = (int)(pipe_cnt % (uint32_t)NS);
          const uint32_t parity = (pipe_cnt / (uint32_t)NS) & 1u;
          if (!wfail && !mbar_wait(wbar + st, parity, P.timeout_ns)) wfail = true;
          ++pipe_cnt;
          const float* sx = wring + (size_t)st * 2 * S;
#pragma unroll
          for (int v = 0; v < KV; ++v) {
            const float4 t = *reinterpret_cast<const float4*>(sx + v * SV + lane * 4);
            xv[v][0] = t.x; xv[v][1] = t.y; xv[v][2] = t.z; xv[v][3] = t.w;
            if constexpr (WITH_C) {
              const float4 u = *reinterpret_cast<const float4*>(sx + S + v * SV + lane * 4);
              cv[v][0] = u.x; cv[v][1] = u.y; cv[v][2] = u.z; cv[v][3] = u.w;
            } else {
              cv[v][0] = cv[v][1] = cv[v][2] = cv[v][3] = 0.0f;
            }
            if (!FULL && !vallf(v)) {
              // Stage bytes outside this warp's rows are stale: zero them so
              // masked lanes add exact zeros to the objective.
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                xv[v][e] = einf(v, e) ? xv[v][e] : 0.0f;
                cv[v][e] = einf(v, e) ? cv[v][e] : 0.0f;
              }
            }
          }
          __syncwarp();
          if (lane == 0 && n + NS < ncw && !wfail) {
            fence_proxy_async_shared();
            issue(n + NS);
          }
        } else {
#pragma unroll
          for (int v = 0; v < KV; ++v)
#pragma unroll
            for (int e = 0; e < VEC; ++e) { xv[v][e] = 0.0f; cv[v][e] = 0.0f; }
        }
      };

      // Prox, store and partial sums of column j (segment in xv / cv).
      auto finish = [&](int j, float (&xv)[KV][VEC], const float (&cv)[KV][VEC], int par) {
        const float f2 = __ldcg(P.phi2 + j);
        float* xcol = P.x + (long long)j * ld;
        float f1[KV][VEC];
#pragma unroll
        for (int v = 0; v < KV; ++v) {
          if constexpr (VEC == 4) {
            const float4 t = *reinterpret_cast<const float4*>(f1s + k * S + v * SV + lane * 4);
            f1[v][0] = t.x; f1[v][1] = t.y; f1[v][2] = t.z; f1[v][3] = t.w;
          } else {
            f1[v][0] = f1s[k * S + v * SV + lane];
          }
        }

        float colp = 0.0f, objp = 0.0f;
        if constexpr (MODE == MODE_QR) {
          // t = X + phi1 + phi2 (- sC); the rare nonzero t below 2^-90 sends
          // the whole column through the IEEE division (one warp vote).
          // 4-wide vectors run the element math on packed pairs (.f32x2).
          const f32x2 ns2 = x2_pack(-s, -s);
          unsigned tmin = 0xffffffffu;
          if constexpr (VEC == 4) {
            const f32x2 f2b = x2_pack(f2, f2);
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int h = 0; h < 4; h += 2) {
                f32x2 t = x2_add(x2_add(x2_pack(xv[v][h], xv[v][h + 1]),
                                        x2_pack(f1[v][h], f1[v][h + 1])), f2b);
                if constexpr (EV)
                  t = x2_fma(ns2, x2_pack(c_at<CT>(cv[v], h), c_at<CT>(cv[v], h + 1)), t);
                x2_unpack(t, xv[v][h], xv[v][h + 1]);
              }
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int e = 0; e < VEC; ++e)
                tmin = min(tmin, (unsigned)__float_as_int(xv[v][e]) - 1u);
          } else {
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int e = 0; e < VEC; ++e) {
                float t = (xv[v][e] + f1[v][e]) + f2;
                if constexpr (EV) t = fmaf(-s, c_at<CT>(cv[v], e), t);
                xv[v][e] = t;
                tmin = min(tmin, (unsigned)__float_as_int(t) - 1u);
              }
          }
          const bool slow = __any_sync(0xffffffffu, tmin < kDivTinyBitsM1);
          auto body = [&](auto slow_tag) {
            constexpr bool SLOW = decltype(slow_tag)::value;
            if constexpr (VEC == 4 && !SLOW) {
              const f32x2 nk = x2_pack(-kappa, -kappa);
              const f32x2 ky = x2_pack(kappa_rcp, kappa_rcp);
              f32x2 col2 = x2_pack(0.0f, 0.0f), obj2 = x2_pack(0.0f, 0.0f);
#pragma unroll
              for (int v = 0; v < KV; ++v)
#pragma unroll
                for (int h = 0; h < 4; h += 2) {
                  f32x2 y = x2_div_rn_by_fma(
                      x2_pack(fmaxf(xv[v][h], 0.0f), fmaxf(xv[v][h + 1], 0.0f)), nk, ky);
                  if constexpr (!FULL) {
                    float y0, y1;
                    x2_unpack(y, y0, y1);
                    y = x2_pack(einf(v, h) ? y0 : 0.0f, einf(v, h + 1) ? y1 : 0.0f);
                  }
                  if constexpr (EV) {
                    const f32x2 c2 = x2_pack(c_at<CT>(cv[v], h), c_at<CT>(cv[v], h + 1));
                    x2_unpack(x2_fma(ns2, c2, y), xv[v][h], xv[v][h + 1]);
                    obj2 = x2_fma(y, c2, obj2);
                  } else {
                    x2_unpack(y, xv[v][h], xv[v][h + 1]);
                  }
                  x2_unpack(x2_add(x2_pack(acc[v][h], acc[v][h + 1]), y), acc[v][h], acc[v][h + 1]);
                  col2 = x2_add(col2, y);
                }
              float u0, u1;
              x2_unpack(col2, u0, u1);
              colp = u0 + u1;
              if constexpr (EV) {
                x2_unpack(obj2, u0, u1);
                objp = u0 + u1;
              }
            } else {
#pragma unroll
              for (int v = 0; v < KV; ++v)
#pragma unroll
                for (int e = 0; e < VEC; ++e) {
                  const float a = fmaxf(xv[v][e], 0.0f);
                  float y = SLOW ? a / kappa : div_rn_by_fma(a, kappa, kappa_rcp);
                  if constexpr (!FULL) y = einf(v, e) ? y : 0.0f;
                  if constexpr (EV) {
                    const float c = c_at<CT>(cv[v], e);
                    xv[v][e] = fmaf(-s, c, y);
                    objp = fmaf(y, c, objp);
                  } else {
                    xv[v][e] = y;
                  }
                  acc[v][e] += y;
                  colp += y;
                }
            }
          };
          if (slow) body(std::true_type());
          else body(std::false_type());
        } else {
          // y = max((X + phi1) + phi2 - sC, 0); 4-wide vectors on packed
          // pairs (each lane rounded as the scalar code), the group norm's
          // lane part then in two partial sums.
          float nsl = 0.0f;
          if constexpr (VEC == 4) {
            const f32x2 ms2 = x2_pack(-s, -s), f2b = x2_pack(f2, f2);
            f32x2 n2 = x2_pack(0.0f, 0.0f);
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int h = 0; h < 4; h += 2) {
                const f32x2 c2 = x2_pack(c_at<CT>(cv[v], h), c_at<CT>(cv[v], h + 1));
                float t0, t1;
                x2_unpack(x2_fma(ms2, c2, x2_add(x2_add(x2_pack(xv[v][h], xv[v][h + 1]),
                                                        x2_pack(f1[v][h], f1[v][h + 1])), f2b)),
                          t0, t1);
                float y0 = fmaxf(t0, 0.0f), y1 = fmaxf(t1, 0.0f);
                if constexpr (!FULL) {
                  y0 = einf(v, h) ? y0 : 0.0f;
                  y1 = einf(v, h + 1) ? y1 : 0.0f;
                }
                xv[v][h] = y0;
                xv[v][h + 1] = y1;
                const f32x2 y2 = x2_pack(y0, y1);
                n2 = x2_fma(y2, y2, n2);
              }
            float u0, u1;
            x2_unpack(n2, u0, u1);
            nsl = u0 + u1;
          } else {
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int e = 0; e < VEC; ++e) {
                const float t = fmaf(-s, c_at<CT>(cv[v], e), (xv[v][e] + f1[v][e]) + f2);
                float y = fmaxf(t, 0.0f);
                if constexpr (!FULL) y = einf(v, e) ? y : 0.0f;
                xv[v][e] = y;
                nsl = fmaf(y, y, nsl);
              }
          }
          // Group norm: a float sum, as the reference's atomics make it.
          nsl = warp_sum(nsl);
          if (Wt > 1) {
            float* slot = reinterpret_cast<float*>(nslot) + par * W + team * Wt;
            if (lane == 0) slot[k] = nsl;
            asm volatile("bar.sync %0, %1;" :: "r"(1 + team), "r"(Wt * 32) : "memory");
            nsl = 0.0f;
            for (int kk = 0; kk < Wt; ++kk) nsl += slot[kk];
          }
          const float scale = gl_shrink(nsl, P.lambda);
          if constexpr (VEC == 4) {
            const f32x2 sc2 = x2_pack(scale, scale);
            f32x2 col2 = x2_pack(0.0f, 0.0f), obj2 = col2;
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int h = 0; h < 4; h += 2) {
                const f32x2 y2 = x2_mul(x2_pack(xv[v][h], xv[v][h + 1]), sc2);
                x2_unpack(y2, xv[v][h], xv[v][h + 1]);
                x2_unpack(x2_add(x2_pack(acc[v][h], acc[v][h + 1]), y2), acc[v][h], acc[v][h + 1]);
                col2 = x2_add(col2, y2);
                obj2 = x2_fma(y2, x2_pack(c_at<CT>(cv[v], h), c_at<CT>(cv[v], h + 1)), obj2);
              }
            float u0, u1;
            x2_unpack(col2, u0, u1);
            colp = u0 + u1;
            x2_unpack(obj2, u0, u1);
            objp = u0 + u1;
          } else {
#pragma unroll
            for (int v = 0; v < KV; ++v)
#pragma unroll
              for (int e = 0; e < VEC; ++e) {
                const float y = xv[v][e] * scale;
                xv[v][e] = y;
                acc[v][e] += y;
                colp += y;
                objp = fmaf(y, c_at<CT>(cv[v], e), objp);
              }
          }
        }

#pragma unroll
        for (int v = 0; v < KV; ++v) {
          if (FULL || vallf(v)) {
            store_vec<VEC>(xcol + row0f(v), xv[v]);
          } else if (vanyf(v)) {
#pragma unroll
            for (int e = 0; e < VEC; ++e)
              if (einf(v, e)) xcol[row0f(v) + e] = xv[v][e];
          }
        }

        float e1;
        two_sum(ms_hi, colp, ms_hi, e1);
        ms_lo += e1;
        if constexpr (WITH_C) {
          two_sum(ob_hi, objp, ob_hi, e1);
          ob_lo += e1;
        }
        colp = warp_sum(colp);
        if (lane == 0) P.colpart[(long long)sb * P.nc + j] = colp;
      };

      if constexpr (TMA) {
        if (seg_rows > 0 && lane == 0) {
          // X was last written by generic stores; order them before the
          // async-proxy reads.
          fence_proxy_async_all();
          const int pre = min(NS, ncw);
          for (int n = 0; n < pre; ++n) issue(n);
        }
        int par = 0;
        for (int n = 0; n < ncw; ++n, par ^= 1) {
          float xv[KV][VEC], cv[KV][VEC];
          load_tma(n, xv, cv);
          finish(c0 + team + n * nteams, xv, cv, par);
        }
      } else if constexpr (!WITH_C) {
        // X-only QR step: two columns in flight per warp (the registers the
        // C segment uses on even steps).
        float cz[KV][VEC];
#pragma unroll
        for (int v = 0; v < KV; ++v)
#pragma unroll
          for (int e = 0; e < VEC; ++e) cz[v][e] = 0.0f;
        for (int n = 0; n < ncw; n += 2) {
          const int ja = c0 + team + n * nteams;
          const bool two = n + 1 < ncw;
          float xa[KV][VEC], xb[KV][VEC], dummy[KV][VEC];
          load_reg(ja, xa, dummy);
          if (two) load_reg(ja + nteams, xb, dummy);
          finish(ja, xa, cz, 0);
          if (two) finish(ja + nteams, xb, cz, 0);
        }
      } else {
        int par = 0;
        for (int n = 0; n < ncw; ++n, par ^= 1) {
          float xv[KV][VEC], cv[KV][VEC];
          load_reg(c0 + team + n * nteams, xv, cv);
          finish(c0 + team + n * nteams, xv, cv, par);
        }
      }
    };
    if (active_warp) {
      if (with_c) {
        if (wfull) run_columns(std::true_type(), std::true_type());
        else run_columns(std::true_type(), std::false_type());
      } else {
        if (wfull) run_columns(std::false_type(), std::true_type());
        else run_columns(std::false_type(), std::false_type());
      }
    }
    if (wfail && lane == 0) atomicExch(P.abort_flag, 1);

    // CTA reduction of the row partials (fixed order over teams) and of the
    // mass / objective (float pairs across lanes and warps).
    const fpair wsum = warp_sum_fp(fpair{ms_hi, ms_lo});
    const fpair wobj = with_c ? warp_sum_fp(fpair{ob_hi, ob_lo}) : fp_make(0.0f);
    __syncthreads();
#pragma unroll
    for (int v = 0; v < KV; ++v)
#pragma unroll
      for (int e = 0; e < VEC; ++e)
        red[(size_t)warp * S + v * SV + lane * VEC + e] = acc[v][e];
    if (lane == 0) {
      dscr[warp] = wsum;
      nslot[warp] = wobj;
    }
    __syncthreads();
    {
      const int cover = Wt * S;
      for (int idx = threadIdx.x; idx < cover; idx += blockDim.x) {
        const int row = base + idx;
        if (row >= lo && row < hi) {
          const int kk = idx / S, r = idx - kk * S;
          float t = 0.0f;
          for (int tm = 0; tm < nteams; ++tm) t += red[(size_t)(tm * Wt + kk) * S + r];
          P.rowpart[(long long)chunk * P.nr + row] = t;
        }
      }
    }
    if (warp == 0) {
      fpair t = lane < W ? dscr[lane] : fp_make(0.0f);
      fpair o = lane < W ? nslot[lane] : fp_make(0.0f);
      t = warp_sum_fp(t);
      if (with_c) o = warp_sum_fp(o);
      if (lane == 0) {
        P.cta_sum[blockIdx.x] = make_float2(t.hi, t.lo);
        if (with_c) P.cta_obj[blockIdx.x] = make_float2(o.hi, o.lo);
      }
    }

    stamp(1);
    if (!grid_barrier(P, epoch, &s_flag)) { aborted = true; break; }
    stamp(2);

    // ------------------------------------------------------------ phase 2
    // (a) warp 0 sums the CTA masses (FP64) into sigma and derives gamma and
    //     the next alpha (thread 0 owns alpha);
    // (b) meanwhile every thread reduces the partials of its rows / columns
    //     (float tree, fixed order) and updates the marginal residuals and
    //     the duals a, b; (dual - residual) is staged until gamma is known;
    // (c) one block sync, then phi = (staged + gamma) / n_cols (or n_rows).
    const bool check = (MODE == MODE_GL) || even || P.stop_every;
    if (warp == 0) {
      const fpair ts = warp_sum_strided_fp(P.cta_sum, G, lane);
      if (lane == 0) {
        // The float total mass: RN(hi + lo) of the normalised pair.
        const float sigma = ts.hi + ts.lo;
        const double t = fp_value(ts);
        s_misc_f[0] = (float)((2.0 * ((double)sigma - 1.0) - (double)alpha) /
                              (double)(P.nr + P.nc));
        alpha = (float)(((double)alpha + 1.0) - (double)sigma);
        s_misc_d[0] = t;
      }
    }
    fpair res = fp_make(0.0f);
    const bool sm2 = P.p2_smem != 0;
    reduce_partials(
        r_lo, r_hi, k_lo, k_hi, P.rowpart, P.colpart, P.nr, P.nc, P.P, P.nsb,
        [&](int i, float t) {
          const int li = i - r_lo;
          const float rs = t - (sm2 ? s_p[li] : __ldg(P.p + i));
          const float ab = (sm2 ? s_a[li] : P.a[i]) - rs;
          if (sm2) {
            s_a[li] = ab;
            s_t1[li] = ab - rs;
          } else {
            P.a[i] = ab;
            P.phi1[i] = ab - rs;
          }
          res = fp_add(res, fp_sqr(rs));
        },
        [&](int j, float t) {
          const int lj = j - k_lo;
          const float cs = t - (sm2 ? s_q[lj] : __ldg(P.q + j));
          const float ab = (sm2 ? s_b[lj] : P.b[j]) - cs;
          if (sm2) {
            s_b[lj] = ab;
            s_t2[lj] = ab - cs;
          } else {
            P.b[j] = ab;
            P.phi2[j] = ab - cs;
          }
          res = fp_add(res, fp_sqr(cs));
        });
    if (check) {
      res = warp_sum_fp(res);
      if (lane == 0) dscr[warp] = res;
    }
    __syncthreads();
    {
      const float gamma = s_misc_f[0];
      for (int i = threadIdx.x; i < r_hi - r_lo; i += blockDim.x) {
        const float t = sm2 ? s_t1[i] : __ldcg(P.phi1 + r_lo + i);
        P.phi1[r_lo + i] = div_rn_by(t + gamma, nc_f, nc_rcp);
      }
      for (int j = threadIdx.x; j < k_hi - k_lo; j += blockDim.x) {
        const float t = sm2 ? s_t2[j] : __ldcg(P.phi2 + k_lo + j);
        P.phi2[k_lo + j] = div_rn_by(t + gamma, nr_f, nr_rcp);
      }
    }
    if (check && warp == 0) {
      fpair t = lane < W ? dscr[lane] : fp_make(0.0f);
      t = warp_sum_fp(t);
      if (lane == 0) P.cta_res[blockIdx.x] = make_float2(t.hi, t.lo);
    }
    last_sigma = s_misc_d[0];
    if (with_c) obj_valid = 1;

    stamp(3);
    if (!grid_barrier(P, epoch, &s_flag)) { aborted = true; break; }

    if (check) {
      // One thread turns the squared residual into the decision; the square
      // root is taken once, after the loop.
      if (warp == 0) {
        const fpair t = warp_sum_strided_fp(P.cta_res, G, lane);
        if (lane == 0) {
          const double r2 = fp_value(t);
          s_misc_d[1] = r2;
          s_stop = r2 < P.res2_stop ? 1 : 0;
        }
      }
      __syncthreads();
      last_res = s_misc_d[1];  // squared until the epilogue
      if (s_stop) {
        converged = true;
        stamp(4);
        break;
      }
    }
    stamp(4);
  }

  // ------------------------------------------------------------ epilogue
  // fix_x (kernel_qr.hpp:469-482): undo the fold of the last step when it
  // was even and the solve converged -- or, in the numpy-API loop
  // (stop_every), whenever it ends on an even step (that loop always hands
  // back an unfolded X).  An odd last step stores X as is.
  const int last_it = converged ? it : it - 1;
  if (MODE == MODE_QR && (converged || P.stop_every) && last_it >= 0 && (last_it & 1) == 0 &&
      !aborted && active_warp) {
    for (int j = c0 + team; j < c1; j += nteams) {
      float* xcol = P.x + (long long)j * ld;
      const CT* ccol = cbase + (long long)j * ld;
#pragma unroll
      for (int v = 0; v < KV; ++v) {
        if (!vanyf(v)) continue;
        float xv[VEC], cv[VEC];
        load_vec<VEC>(xcol + row0f(v), xv);
        load_c<VEC, CT>(ccol + row0f(v), cv);
#pragma unroll
        for (int e = 0; e < VEC; ++e) xv[e] = fmaxf(fmaf(s, cv[e], xv[e]), 0.0f);
        if (vallf(v)) store_vec<VEC>(xcol + row0f(v), xv);
        else {
#pragma unroll
          for (int e = 0; e < VEC; ++e)
            if (einf(v, e)) xcol[row0f(v) + e] = xv[e];
        }
      }
    }
  }
  // Duals of this CTA's slice back to global memory (the state outputs).
  if (P.p2_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < r_hi - r_lo; i += blockDim.x) P.a[r_lo + i] = s_a[i];
    for (int j = threadIdx.x; j < k_hi - k_lo; j += blockDim.x) P.b[k_lo + j] = s_b[j];
  }
  // <C, X> of the last objective-bearing iteration: the CTA partials of that
  // iteration are the last ones written (visible since its barriers).
  if (blockIdx.x == 0 && warp == 0 && obj_valid && !aborted)
    last_obj = fp_value(warp_sum_strided_fp(P.cta_obj, G, lane));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    DeviceStats* st = P.stats;
    st->iters_run = converged ? it + 1 : it;
    // QR reports the index of the last iteration + 1, and max_iters + 1 when
    // it never converged (drot_qr.hpp:233); GL the iterations run (drot_glr.hpp:354).
    st->n_iter = (MODE == MODE_QR) ? it + 1 : st->iters_run;
    st->converged = converged ? 1 : 0;
    st->status = (aborted || ld_volatile_i32(P.abort_flag)) ? 3 : 0;
    st->objective_valid = obj_valid;
    st->objective = last_obj;
    st->residual = last_res >= 0.0 ? sqrt(last_res) : last_res;
    st->sigma = last_sigma;
    *P.alpha = alpha;
  }
  if (timer && threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) P.stats->phase_ns[q] = (double)s_tacc[q];
}

}  // namespace drot
