// drot_batch.cu -- batched quadratic-regularised DROT: many independent
// instances of uneven shape solved in one persistent cooperative launch.
//
// Work units are tiles (instance, row band, column chunk).  In the fused
// update every CTA takes tiles from a per-iteration atomic counter until the
// list is exhausted (instances of very different sizes balance out), and
// every tile writes its own partial-sum slots, so the sums do not depend on
// which CTA ran which tile (results are deterministic).  The dual update is
// split into items of at most 1024 lines (rows or columns) of one instance,
// spread over the CTAs; the stop test and the bookkeeping of an instance
// belong to the CTA of its first item and run after a third grid barrier on
// the iterations that test (even ones).  Converged instances drop out of
// the tile list; once fewer coarse tiles stay active than half the CTAs the
// solve moves to a list of 128-column tiles, so the last large instances
// still spread over more of the GPU.  The launch ends when every instance has
// converged or max_iters is reached.  Per instance the iteration map, fold, stop rule and counts are
// those of the single-instance solver (core/drot_qr.hpp:159-234).
#include <cuda_runtime.h>

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

struct BatchInst {
  long long c_off, x_off, p_off, q_off;  // element offsets into the caller's buffers
  long long ld;                          // leading dimension of its C and X
  long long rp_off;                      // row partials [P][nr] (floats)
  long long cp_off;                      // column partials [nbands][nc] (floats)
  int nr, nc;
  int nbands, band_h;
  int tile0, ntiles, P;                  // coarse tiles (global indices), column chunks
  int tile0f, ntilesf, Pf;               // fine tiles (global indices), column chunks
  int tile0x, ntilesx, Px;               // finest tiles (global indices), column chunks
  int item0, nitems;                     // dual-update items (contiguous)
  int item0x, nitemsx;                   // short items of the finest level (contiguous)
  int row_off, col_off;                  // its rows / columns in the packed state arrays
  float s, kappa, kappa_rcp, eps, nc_rcp, nr_rcp;
  float w_phi1, w_phi2, w_a, w_b, w_alpha;  // warm-start constants
  float lambda;      // GL plans: the group threshold of the shrink
  double res2_stop;  // converged when the squared residual is below this (res2_threshold)
};

struct BatchTile {
  int inst, band, chunk, lo, hi, c0, c1;
  int kvr;  // 128-row blocks per warp step: 1, 2 or 4 (band height <= 128 * kvr)
};

struct BatchItem {
  int inst, l0, l1, pad;  // lines [l0, l1) of instance inst: row l < nr, column l - nr
};

struct BatchStat {
  int n_iter, iters_run, converged, objective_valid;
  double objective, residual;  // residual: squared on the device, rooted by the host
};

struct BatchParams {
  const void* c;
  const float* p;
  const float* q;
  float* x;
  const BatchInst* inst;
  const BatchTile* tiles;
  const BatchItem* items;
  int n_inst, n_tiles, max_iters, n_items;
  int n_tiles_f;       // fine tiles, stored after the n_tiles coarse ones
  int n_tiles_x;       // finest tiles, stored after the fine ones
  int n_items_x;       // short items of the finest level, stored after the n_items others
  const int* order;    // instances by decreasing size (the order of the active lists)
  int* act;            // active lists: tile indices (at most n_tiles + n_tiles_f + n_tiles_x
                       // entries), then dual-update item indices
  int* ilvl;           // per instance: its tile level in the current lists
  int fine_threshold;  // next (finer) base level once fewer active tiles of the current one remain
  int tail_tiles;      // smallest instances at finer levels (build_active_lists); 0 off
  float *a, *b, *phi1, *phi2;  // packed state
  float* alpha;                // [2][n_inst], by iteration parity
  float2* res_slot;            // per item: squared residual (float pair)
  double* obj_slot;            // per instance: objective
  float *rowpart, *colpart;
  float2 *tile_sum, *tile_obj; // per tile: mass and objective (float pairs)
  int* conv;
  BatchStat* stats;
  // On-the-fly cost (point-cloud launches): C_ij = cscale * max(|x_i|^2 +
  // |y_j|^2 - 2 <x_i, y_j>, 0) with x_i = xpts[row_off + i], y_j =
  // ypts[col_off + j] (dim floats each), norms precomputed.
  const float *xpts, *ypts, *xnorm, *ynorm;
  float cscale;
  int dim;
  unsigned* counters;  // [0], [1]: tile counters of even / odd iterations; [2]: converged
                       // instances; [3]: coarse tiles of unconverged instances;
                       // [8..10]: their tiles per level; [13]: base level;
                       // [14], [15]: lengths of the tile and item lists
  unsigned* bar;
  int* abort_flag;
  long long timeout_ns;
  int stall_cta;       // test hook of the bounded waits (grid_barrier); -1 off
  int band_cover;      // GL plans: rows of shared staging per band (>= every group's cover)
  int pf_dist;         // L2 prefetch distance of the fused update, in warp steps (0 off)
  int resume;          // start from the state in the workspace and X (no warm start)
  int no_stop;         // run max_iters iterations on every instance (stop test off)
  // Optional profile of CTA 0 for iterations it < iter_log_cap: globaltimer
  // at the start of the iteration, after its fused-update tiles, after the
  // first barrier and after its dual-update items (iter_log[4 it + 0..3]),
  // and the active coarse tiles at the start.
  unsigned long long* iter_log;
  unsigned* iter_tiles;
  int iter_log_cap;
};

constexpr int kBatchKV = 4;
constexpr int kBatchS = 32 * 4 * kBatchKV;  // rows per band (one warp covers a band)

// Warm start of every instance (core/drot_qr.hpp:321-346): X = 0 over its
// ld x nc block, constant phi1, phi2, a, b, alpha.
__global__ void batch_init_kernel(const BatchParams P) {
  const int k = blockIdx.y;
  if (k >= P.n_inst) return;
  const BatchInst I = P.inst[k];
  const long long nx = I.ld * I.nc;
  if (!P.resume)
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx;
         t += (long long)gridDim.x * blockDim.x)
      P.x[I.x_off + t] = 0.0f;
  if (blockIdx.x == 0 && P.resume) {
    if (threadIdx.x == 0) {
      if (k == 0) P.counters[3] = (unsigned)P.n_tiles;
      P.conv[k] = 0;
      BatchStat st = {0, 0, 0, 0, 0.0, -1.0};
      P.stats[k] = st;
    }
  } else if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < I.nr; i += blockDim.x) {
      P.a[I.row_off + i] = I.w_a;
      P.phi1[I.row_off + i] = I.w_phi1;
    }
    for (int j = threadIdx.x; j < I.nc; j += blockDim.x) {
      P.b[I.col_off + j] = I.w_b;
      P.phi2[I.col_off + j] = I.w_phi2;
    }
    if (threadIdx.x == 0) {
      if (k == 0) P.counters[3] = (unsigned)P.n_tiles;
      P.alpha[k] = I.w_alpha;
      P.conv[k] = 0;
      BatchStat st = {0, 0, 0, 0, 0.0, -1.0};
      P.stats[k] = st;
    }
  }
}

// The column loop of one tile.  A warp step covers 512 elements per lane
// group: KVR row blocks of 128 rows (32 lanes x float4) times 4 / KVR columns,
// so short bands (the last band of an instance, or instances under 512 rows)
// still put 16 loads per lane in flight.  EV: even iteration (reads C, stores
// the folded X - sC), else odd (reads X only).  FULL: the band is exactly
// 128 * KVR rows (no row masks).  Element arithmetic as in the
// single-instance kernel: t = (X + phi1) + phi2 (- sC), y = max(t, 0) / kappa.
template <int KVR, bool EV, bool FULL, typename CT>
__device__ __forceinline__ void batch_tile_columns(const BatchParams& P, const BatchInst& I,
                                                   const BatchTile& T, const float* f1s,
                                                   float (&acc)[4][4], float& ms_hi,
                                                   float& ms_lo, float& ob_hi, float& ob_lo,
                                                   int lane, int warp, int W) {
  constexpr int VEC = 4, SV = 128, NCOL = 4 / KVR;
  const CT* const cbase = reinterpret_cast<const CT*>(P.c);
  const int lo = T.lo, hi = T.hi, c1 = T.c1;
  const float s = I.s, kappa = I.kappa, krcp = I.kappa_rcp;
  for (int j0 = T.c0 + warp * NCOL; j0 < c1; j0 += W * NCOL) {
    // L2 prefetch of this warp's step pf_dist steps ahead (its X segment,
    // and C on even iterations): one 128-byte line per lane, no registers
    // held, so more of the tile's bytes are in flight from DRAM than the
    // register-resident loads of the 16 warps of an SM alone keep.
    if (P.pf_dist > 0) {
      const int jn = j0 + P.pf_dist * W * NCOL;
      if (jn < c1) {
        constexpr int RPC = 128 * KVR;  // rows per column of a warp step
        if (lane < 16) {
          const int cc = lane / (4 * KVR), r = lo + (lane % (4 * KVR)) * 32;
          if (jn + cc < c1 && r < hi) prefetch_l2(P.x + I.x_off + (long long)(jn + cc) * I.ld + r);
        } else if constexpr (EV) {
          constexpr int EPL = 128 / (int)sizeof(CT);  // elements per line
          constexpr int LPC = (RPC + EPL - 1) / EPL;  // lines per column
          const int li = lane - 16, cc = li / LPC, r = lo + (li % LPC) * EPL;
          if (cc < NCOL && jn + cc < c1 && r < hi)
            prefetch_l2(cbase + I.c_off + (long long)(jn + cc) * I.ld + r);
        }
      }
    }
    float xv[4][VEC], cv[4][VEC], f2[NCOL];
    // All loads of the step first (nothing consumes them before the last
    // one is issued).
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int jc = j0 + v / KVR;
      const int r = lo + (v % KVR) * SV + lane * VEC;
      if ((NCOL == 1 || jc < c1) && (FULL || r < hi)) {
        load_vec<VEC>(P.x + I.x_off + (long long)jc * I.ld + r, xv[v]);
        if constexpr (EV)
          load_c_raw<VEC, CT>(cbase + I.c_off + (long long)jc * I.ld + r, cv[v]);
        else {
#pragma unroll
          for (int e = 0; e < VEC; ++e) cv[v][e] = 0.0f;
        }
      } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) { xv[v][e] = 0.0f; cv[v][e] = 0.0f; }
      }
    }
#pragma unroll
    for (int cc = 0; cc < NCOL; ++cc)
      f2[cc] = (NCOL == 1 || j0 + cc < c1) ? __ldcg(P.phi2 + I.col_off + j0 + cc) : 0.0f;
    auto valid = [&](int v, int e) -> bool {
      if constexpr (FULL && NCOL == 1) return true;
      const bool colok = (NCOL == 1) || (j0 + v / KVR < c1);
      return colok && (FULL || lo + (v % KVR) * SV + lane * VEC + e < hi);
    };
    unsigned tmin = 0xffffffffu;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const float4 f1 = *reinterpret_cast<const float4*>(f1s + (v % KVR) * SV + lane * VEC);
      const float f1a[VEC] = {f1.x, f1.y, f1.z, f1.w};
      // Element math on packed pairs (.f32x2; each lane rounds as the scalar
      // instruction).
      const f32x2 f2b = x2_pack(f2[v / KVR], f2[v / KVR]);
#pragma unroll
      for (int h = 0; h < VEC; h += 2) {
        f32x2 tt = x2_add(x2_add(x2_pack(xv[v][h], xv[v][h + 1]), x2_pack(f1a[h], f1a[h + 1])), f2b);
        if constexpr (EV)
          tt = x2_fma(x2_pack(-s, -s), x2_pack(c_at<CT>(cv[v], h), c_at<CT>(cv[v], h + 1)), tt);
        x2_unpack(tt, xv[v][h], xv[v][h + 1]);
      }
#pragma unroll
      for (int e = 0; e < VEC; ++e) {
        const unsigned key = (unsigned)__float_as_int(xv[v][e]) - 1u;
        tmin = min(tmin, valid(v, e) ? key : 0xffffffffu);
      }
    }
    // A nonzero t below 2^-90 anywhere in the step sends the whole step
    // through the IEEE division (one warp vote).
    const bool slow = __any_sync(0xffffffffu, tmin < kDivTinyBitsM1);
    float colp[NCOL], objp = 0.0f;
#pragma unroll
    for (int cc = 0; cc < NCOL; ++cc) colp[cc] = 0.0f;
    auto body = [&](auto slow_tag) {
      constexpr bool SLOW = decltype(slow_tag)::value;
      if constexpr (!SLOW) {
        const f32x2 nk = x2_pack(-kappa, -kappa), ky = x2_pack(krcp, krcp);
        const f32x2 ns2 = x2_pack(-s, -s);
        f32x2 col2[NCOL], obj2 = x2_pack(0.0f, 0.0f);
#pragma unroll
        for (int cc = 0; cc < NCOL; ++cc) col2[cc] = x2_pack(0.0f, 0.0f);
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int h = 0; h < VEC; h += 2) {
            const bool ok0 = valid(v, h), ok1 = valid(v, h + 1);
            f32x2 y = x2_div_rn_by_fma(
                x2_pack(fmaxf(xv[v][h], 0.0f), fmaxf(xv[v][h + 1], 0.0f)), nk, ky);
            if constexpr (!(FULL && NCOL == 1)) {
              float y0, y1;
              x2_unpack(y, y0, y1);
              y = x2_pack(ok0 ? y0 : 0.0f, ok1 ? y1 : 0.0f);
            }
            if constexpr (EV) {
              // the caller's padding may hold anything
              const f32x2 c2 = x2_pack(ok0 ? c_at<CT>(cv[v], h) : 0.0f,
                                       ok1 ? c_at<CT>(cv[v], h + 1) : 0.0f);
              x2_unpack(x2_fma(ns2, c2, y), xv[v][h], xv[v][h + 1]);
              obj2 = x2_fma(y, c2, obj2);
            } else {
              x2_unpack(y, xv[v][h], xv[v][h + 1]);
            }
            float* ac = acc[v % KVR];
            x2_unpack(x2_add(x2_pack(ac[h], ac[h + 1]), y), ac[h], ac[h + 1]);
            col2[v / KVR] = x2_add(col2[v / KVR], y);
          }
        float u0, u1;
#pragma unroll
        for (int cc = 0; cc < NCOL; ++cc) {
          x2_unpack(col2[cc], u0, u1);
          colp[cc] = u0 + u1;
        }
        if constexpr (EV) {
          x2_unpack(obj2, u0, u1);
          objp = u0 + u1;
        }
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int e = 0; e < VEC; ++e) {
            const bool ok = valid(v, e);
            const float a0 = fmaxf(xv[v][e], 0.0f);
            float y = a0 / kappa;
            y = ok ? y : 0.0f;
            if constexpr (EV) {
              const float c = ok ? c_at<CT>(cv[v], e) : 0.0f;  // the caller's padding may hold anything
              xv[v][e] = fmaf(-s, c, y);
              objp = fmaf(y, c, objp);
            } else {
              xv[v][e] = y;
            }
            acc[v % KVR][e] += y;
            colp[v / KVR] += y;
          }
      }
    };
    if (slow) body(std::true_type());
    else body(std::false_type());
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int jc = j0 + v / KVR;
      const int r = lo + (v % KVR) * SV + lane * VEC;
      if ((NCOL == 1 || jc < c1) && (FULL || r < hi)) {
        float* xp = P.x + I.x_off + (long long)jc * I.ld + r;
        if (FULL || r + VEC <= hi) {
          store_vec<VEC>(xp, xv[v]);
        } else {
#pragma unroll
          for (int e = 0; e < VEC; ++e)
            if (r + e < hi) xp[e] = xv[v][e];
        }
      }
    }
    float e1;
#pragma unroll
    for (int cc = 0; cc < NCOL; ++cc) {
      two_sum(ms_hi, colp[cc], ms_hi, e1);
      ms_lo += e1;
    }
    if constexpr (EV) {
      two_sum(ob_hi, objp, ob_hi, e1);
      ob_lo += e1;
    }
#pragma unroll
    for (int cc = 0; cc < NCOL; ++cc) {
      const float cs = warp_sum(colp[cc]);
      if (lane == 0 && (NCOL == 1 || j0 + cc < c1))
        P.colpart[I.cp_off + (long long)T.band * I.nc + j0 + cc] = cs;
    }
  }
}

// GL tile: the band is one group [lo, hi) of the instance (the rows of one
// class, any height up to the plan's band cover), columns [c0, c1).  A warp
// takes one column at a time.  Pass A walks the group in 512-row steps (four
// 128-bit vectors per lane, all loads issued first): y = max((X + phi1) +
// phi2 - sC, 0) (kernel_glr.hpp:163-305), stored back, and the float sum of
// y^2 -- the group norm, a float sum as the reference's atomics make it.
// phi1 is staged as -inf on the rows of the 16-byte vectors that lie
// outside [lo, hi), so y = 0 there with no per-element masks (only the C
// of the caller's padding rows is zeroed, for <C, y>).  The shrink factor
// max(1 - lambda / (||y|| + 1e-9), 0) follows (kernel_glr.hpp:307-326).
// Pass B re-reads the column's y -- just touched, so from L2 -- stores X = y
// * scale and adds the column, row (per-warp shared row partials
// wred[row - base]) and mass sums; the column's objective term <C, X> =
// scale <C, y> comes from pass A.  The element math runs on packed pairs.
// DRAM traffic stays 12 bytes per element, as in the single-pass update.
// Stores the vector of rows r..r+3 that lie inside [lo, hi); a vector that
// straddles a group boundary is stored element by element (the rows of the
// neighbouring group belong to another tile, possibly in flight).
__device__ __forceinline__ void gl_store(float* xcol, int r, int lo, int hi, const float (&v)[4]) {
  if (r >= lo && r + 4 <= hi) {
    store_vec<4>(xcol + r, v);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (r + e >= lo && r + e < hi) xcol[r + e] = v[e];
  }
}

template <typename CT>
__device__ __forceinline__ void batch_gl_tile_columns(const BatchParams& P, const BatchInst& I,
                                                      const BatchTile& T, const float* f1s,
                                                      float* wred, float& ms_hi, float& ms_lo,
                                                      float& ob_hi, float& ob_lo, int lane,
                                                      int warp, int W) {
  constexpr int VEC = 4;
  const CT* const cbase = reinterpret_cast<const CT*>(P.c);
  const int lo = T.lo, hi = T.hi, base = lo & ~3;
  const int nsub = (hi - base + 511) / 512;
  const int pad = (hi == I.nr && (hi & 3)) ? hi : INT_MAX;  // first padding row, if any
  const f32x2 ms2 = x2_pack(-I.s, -I.s);
  for (int j = T.c0 + warp; j < T.c1; j += W) {
    const float f2 = __ldcg(P.phi2 + I.col_off + j);
    const f32x2 f2b = x2_pack(f2, f2);
    float* xcol = P.x + I.x_off + (long long)j * I.ld;
    const CT* ccol = cbase + I.c_off + (long long)j * I.ld;
    // the column's |y|^2 and <C, y> (lane parts, two per lane)
    f32x2 ns2 = x2_pack(0.0f, 0.0f), cy2 = ns2;
    for (int sb = 0; sb < nsub; ++sb) {
      float xv[4][VEC], cv[4][VEC];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = base + sb * 512 + v * 128 + lane * VEC;
        if (r < hi) {
          load_vec<VEC>(xcol + r, xv[v]);
          load_c<VEC, CT>(ccol + r, cv[v]);
        } else {
#pragma unroll
          for (int e = 0; e < VEC; ++e) { xv[v][e] = 0.0f; cv[v][e] = 0.0f; }
        }
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = base + sb * 512 + v * 128 + lane * VEC;
        // The caller's padding rows below ld (the last class's vector that
        // holds row n_rows - 1) may hold any value: their C is zeroed, as y
        // = 0 there and <C, y> must not see a NaN (a neighbouring class's
        // rows hold finite costs).
        if (r + 4 > pad) {
#pragma unroll
          for (int e = 0; e < VEC; ++e)
            if (r + e >= hi) cv[v][e] = 0.0f;
        }
        const float4 f1 = *reinterpret_cast<const float4*>(f1s + (r - base));
        const f32x2 f1p[2] = {x2_pack(f1.x, f1.y), x2_pack(f1.z, f1.w)};
#pragma unroll
        for (int h = 0; h < VEC; h += 2) {
          const f32x2 c2 = x2_pack(cv[v][h], cv[v][h + 1]);
          float t0, t1;
          x2_unpack(x2_fma(ms2, c2, x2_add(x2_add(x2_pack(xv[v][h], xv[v][h + 1]), f1p[h / 2]),
                                           f2b)), t0, t1);
          xv[v][h] = fmaxf(t0, 0.0f);
          xv[v][h + 1] = fmaxf(t1, 0.0f);
          const f32x2 y2 = x2_pack(xv[v][h], xv[v][h + 1]);
          ns2 = x2_fma(y2, y2, ns2);
          cy2 = x2_fma(y2, c2, cy2);
        }
        if (r < hi) gl_store(xcol, r, lo, hi, xv[v]);
      }
    }
    float a0, a1;
    x2_unpack(ns2, a0, a1);
    const float scale = gl_shrink(warp_sum(a0 + a1), I.lambda);
    const f32x2 sc2 = x2_pack(scale, scale);
    x2_unpack(cy2, a0, a1);
    // Pass B re-reads only y: the objective's <C, X> of the column is
    // scale <C, y>, summed in pass A.
    const float objp = scale * (a0 + a1);
    f32x2 col2 = x2_pack(0.0f, 0.0f);
    for (int sb = 0; sb < nsub; ++sb) {
      float xv[4][VEC];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = base + sb * 512 + v * 128 + lane * VEC;
        if (r < hi) load_vec<VEC>(xcol + r, xv[v]);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = base + sb * 512 + v * 128 + lane * VEC;
        if (r >= hi) continue;
        // rows of the vector outside [lo, hi) hold another group's X
        if (r < lo || r + 4 > hi) {
#pragma unroll
          for (int e = 0; e < VEC; ++e)
            if (r + e < lo || r + e >= hi) xv[v][e] = 0.0f;
        }
        float4 acc = *reinterpret_cast<float4*>(wred + (r - base));
        const f32x2 x01 = x2_mul(x2_pack(xv[v][0], xv[v][1]), sc2);
        const f32x2 x23 = x2_mul(x2_pack(xv[v][2], xv[v][3]), sc2);
        x2_unpack(x2_add(x2_pack(acc.x, acc.y), x01), acc.x, acc.y);
        x2_unpack(x2_add(x2_pack(acc.z, acc.w), x23), acc.z, acc.w);
        col2 = x2_add(col2, x2_add(x01, x23));
        *reinterpret_cast<float4*>(wred + (r - base)) = acc;
        x2_unpack(x01, xv[v][0], xv[v][1]);
        x2_unpack(x23, xv[v][2], xv[v][3]);
        gl_store(xcol, r, lo, hi, xv[v]);
      }
    }
    x2_unpack(col2, a0, a1);
    const float colp = a0 + a1;
    float e1;
    two_sum(ms_hi, colp, ms_hi, e1);
    ms_lo += e1;
    two_sum(ob_hi, objp, ob_hi, e1);
    ob_lo += e1;
    const float cs = warp_sum(colp);
    if (lane == 0) P.colpart[I.cp_off + (long long)T.band * I.nc + j] = cs;
  }
}

// Line sums of `n` partial vectors (partial c of line l at base[c * stride
// + l]) for lines lo + threadIdx.x + k * blockDim.x below hi.  A thread takes
// 4 lines and issues the loads of 8 partials of each before adding any (one
// L2 round trip per 32 loads instead of one per line); per line the
// partials are added in index order.  use(l, sum) consumes each line.
// Short ranges (fewer lines than threads / 2) take g = 2..32 threads per
// line instead: thread `sub` of a line adds partials sub, sub + g, ... in
// index order and a shuffle tree of fixed shape combines the g sums.
template <typename F>
__device__ __forceinline__ void reduce_lines(const float* base, int stride, int lo, int hi, int n,
                                             F&& use) {
  const int nt = blockDim.x;
  if (hi <= lo) return;
  int g = 1;
  while (g < 32 && (hi - lo) * g * 2 <= nt) g <<= 1;
  if (g > 1) {
    const int sub = threadIdx.x & (g - 1);
    const int l = lo + (int)threadIdx.x / g;
    float t = 0.0f;
    if (l < hi) {
      for (int c0 = sub; c0 < n; c0 += 8 * g) {
        float v[8];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const int c = c0 + cc * g;
          v[cc] = c < n ? __ldcg(base + (long long)c * stride + l) : 0.0f;
        }
#pragma unroll
        for (int cc = 0; cc < 8; ++cc)
          if (c0 + cc * g < n) t += v[cc];
      }
    }
    for (int o = g >> 1; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (sub == 0 && l < hi) use(l, t);
    return;
  }
  for (int l0 = lo + threadIdx.x; l0 < hi; l0 += 4 * nt) {
    float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int c0 = 0; c0 < n; c0 += 8) {
      float v[4][8];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const int l = l0 + u * nt, c = c0 + cc;
          v[u][cc] = (l < hi && c < n) ? __ldcg(base + (long long)c * stride + l) : 0.0f;
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int cc = 0; cc < 8; ++cc)
          if (c0 + cc < n) s[u] += v[u][cc];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (l0 + u * nt < hi) use(l0 + u * nt, s[u]);
  }
}

// ---------------------------------------------------------------------------
// Point-cloud launches: the cost recomputed on the tensor cores
// ---------------------------------------------------------------------------
//
// On the iterations that read C (even QR iterations and the final unfold) a
// point launch recomputes the tile's C_ij = cscale * max(|x_i|^2 + |y_j|^2 -
// 2 <x_i, y_j>, 0) with the split-TF32 tcgen05 Gram product of the cost
// kernel -- the same MMAs in the same order and the same epilogue, so the
// values equal the stored cost's -- straight into TMEM, and the fused update
// reads them from there: 8 bytes of DRAM traffic per element instead of 12.
//
// The tile is a 512-row band in four 128-row sub-bands; its columns go in
// rounds of kPtCols = 64.  Per round, lane 0 of warp 4 v issues sub-band v's
// 3 x DIM/8 MMAs (M = 128 rows, N = 64 columns) into its quarter of a
// 256-column TMEM buffer and commits; the round's mbarrier completes on the
// four commits.  The buffers alternate, so round n+1's MMAs run while round
// n is updated.  Warp w (of 16) reads TMEM lane quadrant q = w % 4 -- rows
// 128 v + 32 q + lane -- for the round's columns 16 (w / 4) .. + 15: each
// lane updates one row of each sub-band (its row partials stay in
// registers) and the column sums are warp reductions, combined over the
// quadrants in shared memory in a fixed order.
constexpr int kPtCols = 64;    // columns per round (MMA N)
constexpr int kPtTmemCols = 2 * 4 * kPtCols;  // two buffers x four sub-bands

// Shared memory of the point path (after the common part of the kernel's).
struct PointSmem {
  unsigned char* xa;  // x band: 4 sub-bands x [hi | lo] x 128 rows x DIM (K-major)
  unsigned char* yb;  // y of a round: 2 buffers x [hi | lo] x 16 rows x DIM
  float* ycol;        // per round n % 3: |y_j|^2 [16], phi2_j [16] (a round's are
                      // staged two rounds ahead, while the round before is read)
  float* cpart;       // per buffer: column partials [4 quadrants][16]
  float* xn;          // |x_i|^2 of the band's 512 rows
};

__host__ __device__ constexpr size_t point_smem_bytes(int dim) {
  return 1024 /* alignment */ + (size_t)4 * 2 * 128 * dim * 4 + (size_t)2 * 2 * kPtCols * dim * 4 +
         sizeof(float) * (3 * 2 * kPtCols + 2 * 4 * kPtCols + 512);
}

__device__ __forceinline__ PointSmem point_smem(void* base, int dim) {
  unsigned char* p = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(base) + 1023) & ~static_cast<uintptr_t>(1023));
  PointSmem S;
  S.xa = p;
  p += (size_t)4 * 2 * 128 * dim * 4;
  S.yb = p;
  p += (size_t)2 * 2 * kPtCols * dim * 4;
  S.ycol = reinterpret_cast<float*>(p);
  S.cpart = S.ycol + 3 * 2 * kPtCols;
  S.xn = S.cpart + 2 * 4 * kPtCols;
  return S;
}

// One tile of a point launch on an iteration that reads C.  UNFOLD: the
// final unfold X = max(X + sC, 0) of a converged instance; otherwise the
// even QR update (t = (X + phi1) + phi2 - sC, y = max(t, 0) / kappa, X =
// y - sC stored folded), with the row partials left in red[w][row] (warps w
// and w + 4 share a quadrant: rows of quadrant q in red[q] and red[q + 4]),
// the column partials written to colpart and the mass / objective lane sums
// in the float pairs.  mw: per buffer, the mbarrier phases waited so far.
// False when an MMA did not complete within the time limit (every thread
// returns the same).
template <int DIM, bool UNFOLD>
__device__ bool point_tile(const BatchParams& P, const BatchInst& I, const BatchTile& T,
                           const float* f1s, const PointSmem& S, uint32_t tmem, uint64_t* mbar,
                           unsigned (&mw)[2], float* red, float& ms_hi, float& ms_lo,
                           float& ob_hi, float& ob_lo) {
  constexpr int kc = DIM / 4;
  constexpr uint32_t sub = 128u * DIM * 4;      // one hi or lo tile of a sub-band
  constexpr uint32_t ysub = kPtCols * DIM * 4;  // one hi or lo tile of a round's y
  constexpr uint32_t idesc = tf32_idesc(128, kPtCols);
  constexpr int YT = 64;                        // threads staging a round's y (the last two warps)
  constexpr int YV = (kPtCols * kc + YT - 1) / YT;  // float4 of y per staging thread
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int lo = T.lo, hi = T.hi, c0 = T.c0, c1 = T.c1;
  // x of the band's rows, split, K-major per sub-band; their norms
  for (int idx = tid; idx < 512 * kc; idx += nt) {
    const int r = idx / kc, c4 = idx - r * kc;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lo + r < hi)
      v = __ldg(reinterpret_cast<const float4*>(P.xpts + (long long)(I.row_off + lo + r) * DIM) + c4);
    unsigned char* h = S.xa + (r >> 7) * 2 * sub;
    stage_split4(h, h + sub, r & 127, 4 * c4, kc, v);
  }
  for (int r = tid; r < 512; r += nt) S.xn[r] = lo + r < hi ? __ldg(P.xnorm + I.row_off + lo + r) : 0.0f;
  const int rounds = (c1 - c0 + kPtCols - 1) / kPtCols;
  // Round n's y: loaded into registers (y_load) by the staging threads,
  // split into buffer n & 1 with norms and phi2 into slot n % 3 (y_store).
  const int yt = tid - (nt - YT);  // staging thread index, < 0 for the others
  float4 yreg[YV];
  float ynr = 0.0f, yph = 0.0f;
  auto y_load = [&](int n) {
    if (yt < 0) return;
#pragma unroll
    for (int u = 0; u < YV; ++u) {
      const int idx = yt + u * YT, jl = idx / kc, c4 = idx - jl * kc, j = c0 + n * kPtCols + jl;
      yreg[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (idx < kPtCols * kc && j < c1)
        yreg[u] = __ldg(reinterpret_cast<const float4*>(P.ypts + (long long)(I.col_off + j) * DIM) + c4);
    }
    if (yt < kPtCols) {
      const int j = c0 + n * kPtCols + yt;
      ynr = j < c1 ? __ldg(P.ynorm + I.col_off + j) : 0.0f;
      yph = (!UNFOLD && j < c1) ? __ldcg(P.phi2 + I.col_off + j) : 0.0f;
    }
  };
  auto y_store = [&](int n) {
    if (yt < 0) return;
    unsigned char* h = S.yb + (n & 1) * 2 * ysub;
#pragma unroll
    for (int u = 0; u < YV; ++u) {
      const int idx = yt + u * YT, jl = idx / kc, c4 = idx - jl * kc;
      if (idx < kPtCols * kc) stage_split4(h, h + ysub, jl, 4 * c4, kc, yreg[u]);
    }
    if (yt < kPtCols) {
      float* yc = S.ycol + (n % 3) * 2 * kPtCols;
      yc[yt] = ynr;
      yc[kPtCols + yt] = yph;
    }
    fence_proxy_async_shared();
  };
  // Round n's MMAs: sub-band v's chain issued by lane 0 of warp 4 v (four
  // issuing threads share the work), each followed by its commit (the
  // round's mbarrier completes on the four arrivals).
  const bool issuer = lane == 0 && (warp & 3) == 0 && warp < 16;
  auto issue = [&](int n) {
    const int v = warp >> 2;
    const uint32_t yh = smem_u32(S.yb + (n & 1) * 2 * ysub);
    const uint32_t xh = smem_u32(S.xa + v * 2 * sub);
    gram_tf32x3(xh, xh + sub, yh, yh + ysub, DIM,
                tmem + (uint32_t)((n & 1) * 4 * kPtCols + v * kPtCols), idesc);
    tc_commit(&mbar[n & 1]);
  };
  // lane quadrant and column group (16 of the round's 64 columns; 16 warps)
  const int q = warp & 3, hcol = warp >> 2;
  constexpr int WC = kPtCols / 4;  // columns of a warp per round
  float f1[4], xnr[4], racc[4];
  bool rowok[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int r = 128 * v + 32 * q + lane;
    rowok[v] = lo + r < hi;
    f1[v] = UNFOLD ? 0.0f : f1s[r];
    racc[v] = 0.0f;
  }
  float* const xbase = P.x + I.x_off + lo + 32 * q + lane;
  // L2 prefetch of the X lines of the warp's columns of round n (WC columns
  // x 4 sub-bands of its quadrant: WC / 8 128-byte lines per lane)
  auto prefetch_round = [&](int n) {
#pragma unroll
    for (int u = 0; u < WC / 8; ++u) {
      const int line = lane + 32 * u, jn = c0 + n * kPtCols + WC * hcol + (line >> 2), vv = line & 3;
      if (n < rounds && jn < c1 && rowok[vv]) prefetch_l2(xbase + (long long)jn * I.ld + 128 * vv);
    }
  };
  y_load(0);
  y_store(0);
  if (rounds > 1) {
    y_load(1);
    y_store(1);
  }
  if (P.pf_dist > 0) {
    prefetch_round(0);
    prefetch_round(1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (issuer && rounds > 0) issue(0);
#pragma unroll
  for (int v = 0; v < 4; ++v) xnr[v] = S.xn[128 * v + 32 * q + lane];
  const float s = I.s, kappa = I.kappa, krcp = I.kappa_rcp, cscale = P.cscale;
  bool ok = true;
  for (int n = 0; n < rounds; ++n) {
    const int b = n & 1;
    if (n + 2 < rounds) y_load(n + 2);  // in flight during the round
    if (P.pf_dist > 0) prefetch_round(n + 2);
    const bool got = mbar_wait(&mbar[b], mw[b] & 1u, P.timeout_ns);
    ++mw[b];
    // Round n-1's TMEM reads are done before this barrier, after which
    // round n+1's MMAs may overwrite that buffer.
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if (!__syncthreads_and(got ? 1 : 0)) {
      // an MMA that did not complete: give it a second bounded chance to
      // land (its TMEM and shared memory stay allocated until the end)
      mbar_wait(&mbar[b], (mw[b] - 1u) & 1u, P.timeout_ns);
      ok = false;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (issuer && n + 1 < rounds) issue(n + 1);
    if (!UNFOLD && n > 0 && tid >= 32 && tid < 32 + kPtCols) {  // round n-1's column sums (warps 1, 2)
      const int jl = tid - 32, j = c0 + (n - 1) * kPtCols + jl;
      const float* cp = S.cpart + ((n - 1) & 1) * 4 * kPtCols;
      if (j < c1)
        P.colpart[I.cp_off + (long long)T.band * I.nc + j] =
            ((cp[jl] + cp[kPtCols + jl]) + cp[2 * kPtCols + jl]) + cp[3 * kPtCols + jl];
    }
    // the warp's WC columns of the round, 4 at a time
#pragma unroll 1
    for (int hh = 0; hh < WC / 4; ++hh) {
      const int jb = c0 + n * kPtCols + WC * hcol + 4 * hh;
      const float* yc = S.ycol + (n % 3) * 2 * kPtCols + WC * hcol + 4 * hh;
      float xv[4][4], cv[4][4];
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const bool colok = jb + cc < c1;
#pragma unroll
        for (int v = 0; v < 4; ++v)
          xv[v][cc] = (colok && rowok[v]) ? xbase[(long long)(jb + cc) * I.ld + 128 * v] : 0.0f;
      }
      {
        uint32_t d[4][4];
#pragma unroll
        for (int v = 0; v < 4; ++v)
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                       : "=r"(d[v][0]), "=r"(d[v][1]), "=r"(d[v][2]), "=r"(d[v][3])
                       : "r"(tmem + ((uint32_t)(32 * q) << 16) +
                             (uint32_t)(b * 4 * kPtCols + v * kPtCols + WC * hcol + 4 * hh))
                       : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const float yn = yc[cc];
#pragma unroll
          for (int v = 0; v < 4; ++v)
            cv[v][cc] = cscale * fmaxf(fmaf(-2.0f, __uint_as_float(d[v][cc]), xnr[v] + yn), 0.0f);
        }
      }
      if constexpr (UNFOLD) {
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          if (jb + cc >= c1) continue;
#pragma unroll
          for (int v = 0; v < 4; ++v)
            if (rowok[v])
              xbase[(long long)(jb + cc) * I.ld + 128 * v] =
                  fmaxf(fmaf(s, cv[v][cc], xv[v][cc]), 0.0f);
        }
        continue;
      }
      // t = (X + phi1) + phi2 - sC on packed column pairs
      unsigned tmin = 0xffffffffu;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const f32x2 f1b = x2_pack(f1[v], f1[v]);
#pragma unroll
        for (int cc = 0; cc < 4; cc += 2) {
          f32x2 tt = x2_add(x2_add(x2_pack(xv[v][cc], xv[v][cc + 1]), f1b),
                            x2_pack(yc[kPtCols + cc], yc[kPtCols + cc + 1]));
          tt = x2_fma(x2_pack(-s, -s), x2_pack(cv[v][cc], cv[v][cc + 1]), tt);
          x2_unpack(tt, xv[v][cc], xv[v][cc + 1]);
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const unsigned key = (unsigned)__float_as_int(xv[v][cc]) - 1u;
          tmin = min(tmin, (rowok[v] && jb + cc < c1) ? key : 0xffffffffu);
        }
      }
      const bool slow = __any_sync(0xffffffffu, tmin < kDivTinyBitsM1);
      float colp[4] = {0.0f, 0.0f, 0.0f, 0.0f}, objp = 0.0f;
      if (!slow) {
        const f32x2 nk = x2_pack(-kappa, -kappa), ky = x2_pack(krcp, krcp), ns2 = x2_pack(-s, -s);
        f32x2 obj2 = x2_pack(0.0f, 0.0f);
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int cc = 0; cc < 4; cc += 2) {
            const bool ok0 = rowok[v] && jb + cc < c1, ok1 = rowok[v] && jb + cc + 1 < c1;
            f32x2 y = x2_div_rn_by_fma(
                x2_pack(fmaxf(xv[v][cc], 0.0f), fmaxf(xv[v][cc + 1], 0.0f)), nk, ky);
            float y0, y1;
            x2_unpack(y, y0, y1);
            y0 = ok0 ? y0 : 0.0f;
            y1 = ok1 ? y1 : 0.0f;
            y = x2_pack(y0, y1);
            const f32x2 c2 = x2_pack(ok0 ? cv[v][cc] : 0.0f, ok1 ? cv[v][cc + 1] : 0.0f);
            x2_unpack(x2_fma(ns2, c2, y), xv[v][cc], xv[v][cc + 1]);
            obj2 = x2_fma(y, c2, obj2);
            racc[v] = (racc[v] + y0) + y1;
            colp[cc] += y0;
            colp[cc + 1] += y1;
          }
        float u0, u1;
        x2_unpack(obj2, u0, u1);
        objp = u0 + u1;
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const bool okk = rowok[v] && jb + cc < c1;
            float y = fmaxf(xv[v][cc], 0.0f) / kappa;
            y = okk ? y : 0.0f;
            const float c = okk ? cv[v][cc] : 0.0f;
            xv[v][cc] = fmaf(-s, c, y);
            objp = fmaf(y, c, objp);
            racc[v] += y;
            colp[cc] += y;
          }
      }
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        if (jb + cc >= c1) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v)
          if (rowok[v]) xbase[(long long)(jb + cc) * I.ld + 128 * v] = xv[v][cc];
      }
      float e1;
      const float msum = ((colp[0] + colp[1]) + colp[2]) + colp[3];
      two_sum(ms_hi, msum, ms_hi, e1);
      ms_lo += e1;
      two_sum(ob_hi, objp, ob_hi, e1);
      ob_lo += e1;
      float* cp = S.cpart + b * 4 * kPtCols + q * kPtCols + WC * hcol + 4 * hh;
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const float cs = warp_sum(colp[cc]);
        if (lane == 0) cp[cc] = cs;
      }
    }
    if (n + 2 < rounds) y_store(n + 2);  // read by round n+2's MMAs, issued after the next barrier
  }
  // every warp past its last round (or the failed one): the last round's
  // column sums, then the row partials
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (!UNFOLD && ok && rounds > 0 && tid < kPtCols) {
    const int n = rounds - 1;
    const int j = c0 + n * kPtCols + tid;
    const float* cp = S.cpart + (n & 1) * 4 * kPtCols;
    if (j < c1)
      P.colpart[I.cp_off + (long long)T.band * I.nc + j] =
          ((cp[tid] + cp[kPtCols + tid]) + cp[2 * kPtCols + tid]) + cp[3 * kPtCols + tid];
  }
  if (!UNFOLD) {  // the warp's rows of red hold its partials, the other rows zeros
#pragma unroll
    for (int r0 = 0; r0 < 512; r0 += 32)
      red[(size_t)warp * 512 + r0 + lane] = ((r0 >> 5) & 3) == q ? racc[r0 >> 7] : 0.0f;
  }
  return ok;
}

// Norms |x_i|^2 (k ascending, FMA) of n points of dimension dim.
__global__ void point_norms_kernel(const float* pts, int n, int dim, float* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < dim; ++k) {
      const float v = pts[(long long)i * dim + k];
      s = fmaf(v, v, s);
    }
    out[i] = s;
  }
}

// Inclusive block-wide scan of Q ints per thread over `scan` (Q * blockDim
// ints of shared memory); every thread gets its inclusive prefix.
template <int Q>
__device__ __forceinline__ void block_scan_incl(int (&v)[Q], int* scan) {
  const int tid = threadIdx.x, nt = blockDim.x;
#pragma unroll
  for (int l = 0; l < Q; ++l) scan[l * nt + tid] = v[l];
  __syncthreads();
  for (int o = 1; o < nt; o <<= 1) {  // Hillis-Steele
    int u[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) u[l] = tid >= o ? scan[l * nt + tid - o] : 0;
    __syncthreads();
#pragma unroll
    for (int l = 0; l < Q; ++l) scan[l * nt + tid] += u[l];
    __syncthreads();
  }
#pragma unroll
  for (int l = 0; l < Q; ++l) v[l] = scan[l * nt + tid];
  __syncthreads();
}

// Active lists (CTA 0, all threads), rebuilt at the start and whenever an
// instance converged (at most once per instance; a grid barrier publishes
// them).  Every unconverged instance gets a tile level: the run's base level
// -- coarse tiles, then the fine ones once fewer than fine_threshold coarse
// tiles remain, then the finest ones likewise -- or a finer one for the
// smallest instances, those at the end of the order: the instances whose
// finest tiles, counted from the end, number at most tail_tiles take the
// finest level, those whose fine tiles number at most 2 tail_tiles the fine
// one.  The tile list holds each instance's tiles at its level, the item
// list its dual-update items (the finest level's short ones at level 2),
// largest instances first (P.order): the fused update and the dual update
// never step over converged instances, and the last tiles taken in an
// iteration are short ones (the wait at the following barrier is about the
// length of the last tile).  Published: ilvl[k], counters[8..10] the tiles
// of each level over unconverged instances, [13] the base level, [14] / [15]
// the lengths of the tile / item lists.  scan: 2 * blockDim ints.
__device__ void build_active_lists(const BatchParams& P, int* scan) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int T = P.n_tiles + P.n_tiles_f + P.n_tiles_x;  // item list offset in P.act
  const bool has_f = P.n_tiles_f > 0, has_x = P.n_tiles_x > 0;
  __shared__ int s_tot[3], s_carry[4];
  if (tid < 3) s_tot[tid] = 0;
  if (tid < 4) s_carry[tid] = 0;
  __syncthreads();
  // Tiles of every level over the unconverged instances.
  {
    int c[3] = {0, 0, 0};
    for (int k = tid; k < P.n_inst; k += nt) {
      if (__ldcg(P.conv + k)) continue;
      c[0] += P.inst[k].ntiles;
      c[1] += has_f ? P.inst[k].ntilesf : 0;
      c[2] += has_x ? P.inst[k].ntilesx : 0;
    }
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      for (int o = 16; o > 0; o >>= 1) c[l] += __shfl_xor_sync(0xffffffffu, c[l], o);
      if ((tid & 31) == 0) atomicAdd(&s_tot[l], c[l]);
    }
  }
  __syncthreads();
  int L = (int)__ldcg(P.counters + 13);
  if (L == 0 && has_f && s_tot[0] < P.fine_threshold) L = 1;
  if (L == 1 && has_x && s_tot[1] < P.fine_threshold) L = 2;
  for (int k0 = 0; k0 < P.n_inst; k0 += nt) {
    const int k = k0 + tid < P.n_inst ? P.order[k0 + tid] : -1;
    const bool live = k >= 0 && !__ldcg(P.conv + k);
    BatchInst I;
    if (live) I = P.inst[k];
    // finest / fine tiles from the start of the order through this instance
    int pre[2] = {live && has_x ? I.ntilesx : 0, live && has_f ? I.ntilesf : 0};
    const int own[2] = {pre[0], pre[1]};
    block_scan_incl<2>(pre, scan);
    int lvl = L;
    if (live) {
      const int suf_x = s_tot[2] - (s_carry[0] + pre[0] - own[0]);  // this one and later ones
      const int suf_f = s_tot[1] - (s_carry[1] + pre[1] - own[1]);
      if (has_x && suf_x <= P.tail_tiles) lvl = 2;
      else if (has_f && L < 1 && suf_f <= 2 * P.tail_tiles) lvl = 1;
    }
    int cnt[2] = {0, 0};
    if (live) {
      cnt[0] = lvl == 0 ? I.ntiles : (lvl == 1 ? I.ntilesf : I.ntilesx);
      cnt[1] = lvl == 2 ? I.nitemsx : I.nitems;
    }
    int off[2] = {cnt[0], cnt[1]};
    block_scan_incl<2>(off, scan);
    if (live) {
      P.ilvl[k] = lvl;
      const int t0 = lvl == 0 ? I.tile0 : (lvl == 1 ? I.tile0f : I.tile0x);
      const int q0 = lvl == 2 ? I.item0x : I.item0;
      int* dt = P.act + s_carry[2] + off[0] - cnt[0];
      int* dq = P.act + T + s_carry[3] + off[1] - cnt[1];
      for (int u = 0; u < cnt[0]; ++u) dt[u] = t0 + u;
      for (int u = 0; u < cnt[1]; ++u) dq[u] = q0 + u;
    }
    __syncthreads();
    if (tid == nt - 1) {
      s_carry[0] += pre[0];
      s_carry[1] += pre[1];
      s_carry[2] += off[0];
      s_carry[3] += off[1];
    }
    __syncthreads();
  }
  if (tid < 3) P.counters[8 + tid] = (unsigned)s_tot[tid];
  if (tid == 0) {
    P.counters[13] = (unsigned)L;
    P.counters[14] = (unsigned)s_carry[2];
    P.counters[15] = (unsigned)s_carry[3];
  }
}

// GL = true: the group-lasso iteration (core/drot_glr.hpp:242-355) on plans
// made by drot_gl_batch_plan_create -- bands are the instances' groups, the
// stop test runs on every iteration with "<=", no fold, and n_iter counts
// the iterations run.
// Point launches (DIM > 0) run one 512-thread CTA per SM: a kernel that
// allocates TMEM is given one resident CTA per SM by the runtime's occupancy
// rule, so a cooperative launch of two per SM is refused.
template <typename CT, int DIM, bool GL = false>
__global__ void __launch_bounds__(DIM > 0 ? 512 : 256, DIM > 0 ? 1 : 2)
    batch_solve_kernel(const BatchParams P) {
  constexpr int VEC = 4, KV = kBatchKV;
  const int S = GL ? P.band_cover : kBatchS;  // rows of the band staging
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int W = blockDim.x >> 5;
  float* red = reinterpret_cast<float*>(smem_raw);  // [W][S]
  float* f1s = red + (size_t)W * S;                 // [S]
  fpair* dscr = reinterpret_cast<fpair*>(f1s + S);  // [W + 1]
  fpair* oscr = dscr + W + 1;                       // [W]
  __shared__ int s_flag, s_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Point launches: operand staging after the pair scratch, two mbarriers
  // and kPtTmemCols TMEM columns (the round buffers of point_tile), held
  // for the whole launch.
  PointSmem ps{};
  uint32_t tmem = 0;
  unsigned mw[2] = {0u, 0u};
  __shared__ __align__(8) uint64_t s_mbar[2];
  __shared__ uint32_t s_tmem;
  if constexpr (DIM > 0) {
    ps = point_smem(oscr + W, DIM);
    if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                   :: "r"(smem_u32(&s_tmem)), "r"((uint32_t)kPtTmemCols) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
      mbar_init(&s_mbar[0], 4);  // one commit per sub-band (point_tile)
      mbar_init(&s_mbar[1], 4);
      fence_mbar_init();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem = s_tmem;
  }
  const int G = gridDim.x;
  const CT* const cbase = reinterpret_cast<const CT*>(P.c);
  unsigned epoch = 0;
  bool aborted = false;
  int it = 0;
  // Tile and item lists of the iteration (each unconverged instance at its
  // own tile level, build_active_lists), read after the barrier that
  // publishes them, so every CTA uses the same lists.
  const int items0 = P.n_tiles + P.n_tiles_f + P.n_tiles_x;  // item part of P.act
  int n_list = 0, nq = 0;  // active tiles / dual-update items
  unsigned conv_seen;      // converged instances when the lists were last built
  // Builds the lists (CTA 0) and publishes them.  False when the run was
  // aborted.
  auto rebuild = [&]() -> bool {
    if (blockIdx.x == 0) build_active_lists(P, reinterpret_cast<int*>(smem_raw));
    if (!grid_barrier(P.bar, P.abort_flag, P.timeout_ns, epoch, &s_flag, P.stall_cta)) return false;
    n_list = (int)__ldcg(P.counters + 14);
    nq = (int)__ldcg(P.counters + 15);
    conv_seen = __ldcg(P.counters + 2);
    return true;
  };
  if (!rebuild()) aborted = true;

  for (; it < P.max_iters && !aborted; ++it) {
    const bool even = (it & 1) == 0;
    unsigned* counter = P.counters + (it & 1);
    const bool logit = P.iter_log && it < P.iter_log_cap && blockIdx.x == 0 && threadIdx.x == 0;
    if (logit) {
      P.iter_log[4 * it] = globaltimer_ns();
      P.iter_tiles[it] = __ldcg(P.counters + 3);
    }
    const int qa = items0;  // active dual-update items: P.act[qa + 0 .. nq)

    // ---------------------------------------------------------- fused update
    // A CTA takes its next list slot only when it is free: taking it earlier
    // (as a tile starts, to hide the atomic) reserves tiles that idle CTAs
    // could run at the end of the iteration (measured: barrier wait 8 -> 13
    // us, solve +1.5 %).  The lists hold unconverged instances only (rebuilt
    // after every stop test that converged one).
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
      __syncthreads();
      if (s_tile >= n_list) break;
      const int t = __ldcg(P.act + s_tile);
      const BatchTile T = P.tiles[t];
      const BatchInst I = P.inst[T.inst];
      const int lo = T.lo, hi = T.hi;
      if constexpr (GL) {
        // phi1 of the group's rows from the 16-byte boundary below lo (-inf
        // on the rows outside [lo, hi), through the last 512-row step) and
        // zeroed per-warp row partials, then the two-pass column walk.
        const int base = lo & ~3, cover = hi - base, span = (cover + 511) / 512 * 512;
        for (int idx = threadIdx.x; idx < span; idx += blockDim.x) {
          const int r = base + idx;
          f1s[idx] = (r >= lo && r < hi) ? __ldcg(P.phi1 + I.row_off + r) : -INFINITY;
        }
        for (int idx = threadIdx.x; idx < W * S; idx += blockDim.x) red[idx] = 0.0f;
        __syncthreads();
        float ms_hi = 0.0f, ms_lo = 0.0f, ob_hi = 0.0f, ob_lo = 0.0f;
        batch_gl_tile_columns<CT>(P, I, T, f1s, red + (size_t)warp * S, ms_hi, ms_lo, ob_hi,
                                  ob_lo, lane, warp, W);
        const fpair wsum = warp_sum_fp(fpair{ms_hi, ms_lo});
        const fpair wobj = warp_sum_fp(fpair{ob_hi, ob_lo});
        if (lane == 0) {
          dscr[warp] = wsum;
          oscr[warp] = wobj;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < cover; idx += blockDim.x) {
          const int r = base + idx;
          if (r >= lo) {
            float tsum = 0.0f;
            for (int w = 0; w < W; ++w) tsum += red[(size_t)w * S + idx];
            P.rowpart[I.rp_off + (long long)T.chunk * I.nr + r] = tsum;
          }
        }
        if (warp == 0) {
          fpair a1 = lane < W ? dscr[lane] : fp_make(0.0f);
          fpair a2 = lane < W ? oscr[lane] : fp_make(0.0f);
          a1 = warp_sum_fp(a1);
          a2 = warp_sum_fp(a2);
          if (lane == 0) {
            P.tile_sum[t] = make_float2(a1.hi, a1.lo);
            P.tile_obj[t] = make_float2(a2.hi, a2.lo);
          }
        }
      } else {
        for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
          const int r = lo + idx;
          f1s[idx] = r < hi ? __ldcg(P.phi1 + I.row_off + r) : 0.0f;
        }
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int e = 0; e < 4; ++e) acc[v][e] = 0.0f;
        float ms_hi = 0.0f, ms_lo = 0.0f, ob_hi = 0.0f, ob_lo = 0.0f;
        auto run = [&](auto kvr_tag, auto ev_tag) {
          constexpr int KVR = decltype(kvr_tag)::value;
          constexpr bool EV = decltype(ev_tag)::value;
          if (hi - lo == 128 * KVR)
            batch_tile_columns<KVR, EV, true, CT>(P, I, T, f1s, acc, ms_hi, ms_lo, ob_hi, ob_lo,
                                                  lane, warp, W);
          else
            batch_tile_columns<KVR, EV, false, CT>(P, I, T, f1s, acc, ms_hi, ms_lo, ob_hi, ob_lo,
                                                   lane, warp, W);
        };
        using K1 = std::integral_constant<int, 1>;
        using K2 = std::integral_constant<int, 2>;
        using K4 = std::integral_constant<int, 4>;
        bool point_even = false;
        if constexpr (DIM > 0) point_even = even;
        if (point_even) {
          // the cost from the points on the tensor cores (512-row bands)
          if constexpr (DIM > 0) {
            if (!point_tile<DIM, false>(P, I, T, f1s, ps, tmem, s_mbar, mw, red, ms_hi, ms_lo,
                                        ob_hi, ob_lo)) {
              aborted = true;
              atomicExch(P.abort_flag, 1);
              break;
            }
          }
        } else if (even) {
          if (T.kvr == 1) run(K1(), std::true_type());
          else if (T.kvr == 2) run(K2(), std::true_type());
          else run(K4(), std::true_type());
        } else {
          if (T.kvr == 1) run(K1(), std::false_type());
          else if (T.kvr == 2) run(K2(), std::false_type());
          else run(K4(), std::false_type());
        }
        // Tile partials: rows (fixed warp order), mass and objective (float pairs).
        const fpair wsum = warp_sum_fp(fpair{ms_hi, ms_lo});
        const fpair wobj = even ? warp_sum_fp(fpair{ob_hi, ob_lo}) : fp_make(0.0f);
        if (!point_even) {
#pragma unroll
          for (int v = 0; v < 4; ++v)
            if (v < T.kvr)
              *reinterpret_cast<float4*>(red + (size_t)warp * S + v * 128 + lane * 4) =
                  make_float4(acc[v][0], acc[v][1], acc[v][2], acc[v][3]);
        }
        if (lane == 0) {
          dscr[warp] = wsum;
          oscr[warp] = wobj;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
          const int r = lo + idx;
          if (r < hi) {
            float tsum = 0.0f;
            for (int w = 0; w < W; ++w) tsum += red[(size_t)w * S + idx];
            P.rowpart[I.rp_off + (long long)T.chunk * I.nr + r] = tsum;
          }
        }
        if (warp == 0) {
          fpair a1 = lane < W ? dscr[lane] : fp_make(0.0f);
          fpair a2 = lane < W ? oscr[lane] : fp_make(0.0f);
          a1 = warp_sum_fp(a1);
          if (even) a2 = warp_sum_fp(a2);
          if (lane == 0) {
            P.tile_sum[t] = make_float2(a1.hi, a1.lo);
            if (even) P.tile_obj[t] = make_float2(a2.hi, a2.lo);
          }
        }
      }
    }

    if (logit) P.iter_log[4 * it + 1] = globaltimer_ns();
    if (!grid_barrier(P.bar, P.abort_flag, P.timeout_ns, epoch, &s_flag, P.stall_cta)) {
      aborted = true;
      break;
    }

    if (logit) P.iter_log[4 * it + 2] = globaltimer_ns();
    // ---------------------------------------------------------- dual update
    // Item q: lines [l0, l1) of one instance (kernel_qr.hpp:405-467).  Every
    // item of the instance recomputes sigma from the tile sums; alpha is
    // read from this iteration's parity and written (by the first item) to
    // the other one.
    if (blockIdx.x == 0 && threadIdx.x == 0) P.counters[(it + 1) & 1] = 0u;
    for (int qq = blockIdx.x; qq < nq; qq += G) {
      const int qi = __ldcg(P.act + qa + qq);
      const BatchItem Q = P.items[qi];
      const int k = Q.inst;
      if (__ldcg(P.conv + k)) continue;
      const BatchInst I = P.inst[k];
      const int lvl = __ldcg(P.ilvl + k);
      const bool first = qi == (lvl == 2 ? I.item0x : I.item0);
      const int t0 = lvl == 0 ? I.tile0 : (lvl == 1 ? I.tile0f : I.tile0x);
      const int ntl = lvl == 0 ? I.ntiles : (lvl == 1 ? I.ntilesf : I.ntilesx);
      const int nchunks = lvl == 0 ? I.P : (lvl == 1 ? I.Pf : I.Px);
      fpair sg = fp_make(0.0f), og = fp_make(0.0f);
      for (int i = threadIdx.x; i < ntl; i += blockDim.x) {
        const float2 u = __ldcg(P.tile_sum + t0 + i);
        sg = fp_add(sg, fpair{u.x, u.y});
        if ((even || GL) && first) {
          const float2 o = __ldcg(P.tile_obj + t0 + i);
          og = fp_add(og, fpair{o.x, o.y});
        }
      }
      sg = block_sum_fp(sg, dscr);
      if ((even || GL) && first) og = block_sum_fp(og, dscr);
      const float sigma = sg.hi + sg.lo;  // the float total mass
      const float alpha = __ldcg(P.alpha + (size_t)(it & 1) * P.n_inst + k);
      const float gamma =
          (float)((2.0 * ((double)sigma - 1.0) - (double)alpha) / (double)(I.nr + I.nc));
      if (first && threadIdx.x == 0)
        P.alpha[(size_t)((it + 1) & 1) * P.n_inst + k] =
            (float)(((double)alpha + 1.0) - (double)sigma);
      fpair res = fp_make(0.0f);
      const float ncf = (float)I.nc, nrf = (float)I.nr;
      reduce_lines(P.rowpart + I.rp_off, I.nr, Q.l0, min(Q.l1, I.nr), nchunks, [&](int i, float r) {
        const float rs = r - __ldg(P.p + I.p_off + i);
        const float ab = P.a[I.row_off + i] - rs;
        P.phi1[I.row_off + i] = div_rn_by((ab - rs) + gamma, ncf, I.nc_rcp);
        P.a[I.row_off + i] = ab;
        res = fp_add(res, fp_sqr(rs));
      });
      reduce_lines(P.colpart + I.cp_off, I.nc, max(Q.l0 - I.nr, 0), Q.l1 - I.nr, I.nbands,
                   [&](int j, float cs_) {
        const float cs = cs_ - __ldg(P.q + I.q_off + j);
        const float ab = P.b[I.col_off + j] - cs;
        P.phi2[I.col_off + j] = div_rn_by((ab - cs) + gamma, nrf, I.nr_rcp);
        P.b[I.col_off + j] = ab;
        res = fp_add(res, fp_sqr(cs));
      });
      res = block_sum_fp(res, dscr);
      if (threadIdx.x == 0) {
        P.res_slot[qi] = make_float2(res.hi, res.lo);
        if ((even || GL) && first) P.obj_slot[k] = fp_value(og);
      }
      __syncthreads();
    }

    if (logit) P.iter_log[4 * it + 3] = globaltimer_ns();
    if (!grid_barrier(P.bar, P.abort_flag, P.timeout_ns, epoch, &s_flag, P.stall_cta)) {
      aborted = true;
      break;
    }

    if (even || GL) {
      // Stop test (drot_qr.hpp:219-229: even iterations, residual < eps), by
      // the CTA of each instance's first item, then one more barrier so the
      // next fused update sees every decision.
      // Warp 0 sums an instance's item residuals (lanes in parallel, fixed
      // order), lane 0 decides.
      if (warp == 0) {
        for (int qq = blockIdx.x; qq < nq; qq += G) {
          const int qi = __ldcg(P.act + qa + qq);
          const int k = P.items[qi].inst;
          const BatchInst& I = P.inst[k];
          const int lvl = __ldcg(P.ilvl + k);
          const int i0 = lvl == 2 ? I.item0x : I.item0;
          const int ni = lvl == 2 ? I.nitemsx : I.nitems;
          if (qi != i0 || __ldcg(P.conv + k)) continue;
          fpair r2 = fp_make(0.0f);
          for (int t = lane; t < ni; t += 32) {
            const float2 u = __ldcg(P.res_slot + i0 + t);
            r2 = fp_add(r2, fpair{u.x, u.y});
          }
          r2 = warp_sum_fp(r2);
          if (lane != 0) continue;
          BatchStat st = P.stats[k];
          st.objective = __ldcg(P.obj_slot + k);
          st.objective_valid = 1;
          st.residual = fp_value(r2);
          if (!P.no_stop && st.residual < I.res2_stop) {
            // Converged at iteration it: the instance keeps its folded X
            // until the unfold pass at the end of the launch.
            st.converged = 1;
            st.n_iter = it + 1;
            st.iters_run = it + 1;
            P.conv[k] = 1;
            atomicAdd(P.counters + 2, 1u);
            atomicSub(P.counters + 3, (unsigned)I.ntiles);
          }
          P.stats[k] = st;
        }
      }
      if (!grid_barrier(P.bar, P.abort_flag, P.timeout_ns, epoch, &s_flag, P.stall_cta)) {
        aborted = true;
        break;
      }
      if (__ldcg(P.counters + 2) >= (unsigned)P.n_inst) {
        ++it;
        break;
      }
      if (__ldcg(P.counters + 2) != conv_seen && !rebuild()) {
        aborted = true;
        break;
      }
    }
  }

  // ------------------------------------------------------------ epilogue
  // Unfold the X of converged instances (fix_x, kernel_qr.hpp:469-482);
  // static tile assignment (the last barrier ordered every earlier write).
  // GL stores X unfolded on every iteration.
  if (!GL && !aborted) {
    for (int t = blockIdx.x; t < P.n_tiles; t += G) {
      const BatchTile T = P.tiles[t];
      if (!__ldcg(P.conv + T.inst)) continue;
      const BatchInst I = P.inst[T.inst];
      if constexpr (DIM > 0) {  // the same C as the fold's, from the points
        float u0 = 0.0f, u1 = 0.0f, u2 = 0.0f, u3 = 0.0f;
        __syncthreads();  // the previous tile's staging is no longer read
        if (!point_tile<DIM, true>(P, I, T, nullptr, ps, tmem, s_mbar, mw, red, u0, u1, u2, u3)) {
          aborted = true;
          atomicExch(P.abort_flag, 1);
          break;
        }
      } else {
      for (int j = T.c0 + warp; j < T.c1; j += W) {
        float* xcol = P.x + I.x_off + (long long)j * I.ld;
        const CT* ccol = cbase + I.c_off + (long long)j * I.ld;
#pragma unroll
        for (int v = 0; v < KV; ++v) {
          const int r = T.lo + lane * VEC + v * 128;
          if (r >= T.hi) continue;
          float xv[VEC], cv[VEC];
          load_vec<VEC>(xcol + r, xv);
          load_c<VEC, CT>(ccol + r, cv);
#pragma unroll
          for (int e = 0; e < VEC; ++e) xv[e] = fmaxf(fmaf(I.s, cv[e], xv[e]), 0.0f);
          if (r + VEC <= T.hi) store_vec<VEC>(xcol + r, xv);
          else {
#pragma unroll
            for (int e = 0; e < VEC; ++e)
              if (r + e < T.hi) xcol[r + e] = xv[e];
          }
        }
      }
      }
    }
  }
  for (int k = blockIdx.x; k < P.n_inst; k += G) {
    if (threadIdx.x == 0) {
      BatchStat st = P.stats[k];
      if (!st.converged) {
        // drot_qr.hpp:233 without convergence (QR); GL counts the
        // iterations run (drot_glr.hpp:354)
        st.n_iter = GL ? P.max_iters : P.max_iters + 1;
        st.iters_run = aborted ? it : P.max_iters;
      }
      P.stats[k] = st;
    }
  }
  if (aborted && blockIdx.x == 0 && threadIdx.x == 0) atomicExch(P.abort_flag, 1);
  if constexpr (DIM > 0) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                   :: "r"(tmem), "r"((uint32_t)kPtTmemCols) : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static const size_t kAl = 256;
static inline size_t al(size_t v) { return (v + kAl - 1) / kAl * kAl; }

// Tile-level shape of the plans created after drot_batch_set_tuning (one
// process-wide setting, read once per plan).  Defaults, measured:
//  * fine_cols 128, level_quarters 8: on 256 instances of U{64..2048}^2 with
//    256-column coarse tiles, 128-column fine tiles and the switch at grid / 2
//    gave 3.20 s against 3.45 s without the fine list (32-column fine tiles:
//    3.45-3.85 s).  On the 64-instance differentiable workload the switch at
//    2 / 8 / 16 / 32 quarters of the grid gave 5.70 / 5.66 / 5.72 / 5.76 s per
//    solve (finer tiles balance the tail's CTAs -- barrier wait 14 -> 6 us --
//    until their per-tile cost wins).
//  * finest_cols 32, finest_item_lines 64: the level used once the fine list
//    too leaves CTAs idle (in the 256-instance workload the last few
//    instances, mostly the largest, for the last two thirds of the
//    iterations); a lone 2048-column instance still spreads over ~250 CTAs.
//  * item_lines 1024: rows + columns per dual-update item.
//  * prefetch_distance 1: on the 64-instance workload (377 M elements, all
//    active) one warp step ahead took an iteration from 663 to 601 us (0.85
//    -> 0.94 of the measured HBM copy bandwidth); 2 steps 606 us, 4 steps 647.
//  * tail_quarters 4: the smallest instances (at the end of every
//    iteration's tile order) take the finest tiles up to tail_quarters / 4 x
//    the grid of them, and the fine tiles up to twice that, so the last
//    tiles of an iteration are short (0: every instance at the base level).
struct BatchTuning {
  int fine_cols = 128, finest_cols = 32, item_lines = 1024, finest_item_lines = 64,
      level_quarters = 8, prefetch_distance = 1, tail_quarters = 4;
};
static std::mutex g_tuning_mu;
static BatchTuning g_tuning;
static BatchTuning current_tuning() {
  std::lock_guard<std::mutex> lk(g_tuning_mu);
  return g_tuning;
}

struct BatchPlanImpl {
  int n_inst = 0, n_tiles = 0, n_tiles_f = 0, n_tiles_x = 0, n_items = 0, n_items_x = 0;
  int grid = 0, threads = 256, cols_per_tile = 0;
  int band_rows = 512;
  int gl = 0;                 // group-lasso plan
  int band_cover = kBatchS;   // GL: rows of the band staging (>= every group's cover)
  BatchTuning tune;           // tile-level shape and prefetch (drot_batch_set_tuning)
  size_t smem = 0;     // dynamic shared memory of the cost-matrix launches
  size_t smem_pt = 0;  // and of the point launches
  int grid_pt = 0;     // CTAs of the point launches (one per SM)
  int threads_pt = 512;  // their threads per CTA
  long long rows = 0, cols = 0, rowpart = 0, colpart = 0;
  std::vector<BatchInst> inst;
  std::vector<BatchTile> tiles;  // coarse tiles, then fine tiles, then finest tiles
  // dual-update items (n_items), then the finest level's short ones (n_items_x)
  std::vector<BatchItem> items;
  std::vector<int> order;        // instances by decreasing n_rows * n_cols
  // workspace layout
  size_t off_ctrl = 0, off_inst = 0, off_tiles = 0, off_items = 0, off_a = 0, off_b = 0,
         off_phi1 = 0, off_phi2 = 0, off_alpha = 0, off_rp = 0, off_cp = 0, off_tsum = 0,
         off_tobj = 0, off_res = 0, off_obj = 0, off_conv = 0, off_stats = 0, off_act = 0, off_order = 0,
         off_ilvl = 0, off_xn = 0,
         off_yn = 0, total = 0;
  bool uploaded_any = false;
};

// Tiles of one instance: every 512-row band x `chunks` column chunks.
static void add_tiles(std::vector<BatchTile>& tiles, int k, const BatchInst& I, int chunks) {
  for (int b = 0; b < I.nbands; ++b)
    for (int c = 0; c < chunks; ++c) {
      BatchTile T;
      T.inst = k;
      T.band = b;
      T.chunk = c;
      T.lo = b * I.band_h;
      T.hi = std::min(T.lo + I.band_h, I.nr);
      T.c0 = (int)(((long long)I.nc * c) / chunks);
      T.c1 = (int)(((long long)I.nc * (c + 1)) / chunks);
      const int h = T.hi - T.lo;
      T.kvr = h <= 128 ? 1 : (h <= 256 ? 2 : 4);
      tiles.push_back(T);
    }
}

// GL tiles of one instance: every group (the reference's contiguous class
// row ranges, bounds[0..G]) x `chunks` column chunks.
static void add_gl_tiles(std::vector<BatchTile>& tiles, int k, const BatchInst& I, int chunks,
                         const std::vector<int>& bounds) {
  for (int g = 0; g + 1 < (int)bounds.size(); ++g)
    for (int c = 0; c < chunks; ++c) {
      BatchTile T;
      T.inst = k;
      T.band = g;
      T.chunk = c;
      T.lo = bounds[g];
      T.hi = bounds[g + 1];
      T.c0 = (int)(((long long)I.nc * c) / chunks);
      T.c1 = (int)(((long long)I.nc * (c + 1)) / chunks);
      T.kvr = 4;
      tiles.push_back(T);
    }
}

// Group row boundaries of the reference GL kernels (core/kernel_glr.hpp:79-80
// with +0.49 when ceil(n_rows/G) <= 256, drot_glr.hpp:280; +0.49999
// otherwise, kernel_glr.hpp:185-186), FP32 products as the reference.
static std::vector<int> gl_bounds(int nr, int G) {
  std::vector<int> b(G + 1);
  const double off = ((nr + G - 1) / G) <= 256 ? 0.49 : 0.49999;
  const float per = (float)nr / (float)G;
  for (int k = 0; k <= G; ++k) b[k] = (int)((double)(per * (float)k) + off);
  return b;
}

// Largest group height a GL plan stages (rows of shared memory per warp).
constexpr int kBatchGlMaxCover = 4096;

// Dynamic shared memory: row reduction [warps][S], phi1 stage [S] (S = 512
// rows, or a GL plan's band cover), FP64 scratch, and for point launches the
// band's x (k-major) and norms.
static size_t batch_smem(int warps, int dim, int band_cover = kBatchS) {
  return sizeof(float) * ((size_t)warps * band_cover + band_cover) +
         sizeof(fpair) * (2 * warps + 1) + (dim > 0 ? point_smem_bytes(dim) : 0);
}

}  // namespace drot

using namespace drot;

struct drot_batch_plan_s {
  BatchPlanImpl p;
  unsigned long long* iter_log = nullptr;  // optional profile (drot_batch_set_iteration_log)
  unsigned* iter_tiles = nullptr;
  int iter_log_cap = 0;
};

extern "C" {

int drot_batch_set_tuning(const drot_batch_tuning* t) {
  BatchTuning v;
  if (t) {
    const BatchTuning d;
    if (t->fine_cols > 4096 || t->finest_cols > 4096 || t->item_lines > (1 << 24) ||
        t->finest_item_lines > (1 << 24) || t->level_quarters > 4096 ||
        t->prefetch_distance > 8 || t->tail_quarters > 4096 || t->fine_cols == 0 ||
        t->item_lines == 0 ||
        t->finest_item_lines == 0)
      return DROT_ERR_INVALID_ARG;
    v.fine_cols = t->fine_cols > 0 ? t->fine_cols : d.fine_cols;
    v.finest_cols = t->finest_cols >= 0 ? t->finest_cols : d.finest_cols;
    v.item_lines = t->item_lines > 0 ? t->item_lines : d.item_lines;
    v.finest_item_lines = t->finest_item_lines > 0 ? t->finest_item_lines : d.finest_item_lines;
    v.level_quarters = t->level_quarters >= 0 ? t->level_quarters : d.level_quarters;
    v.prefetch_distance = t->prefetch_distance >= 0 ? t->prefetch_distance : d.prefetch_distance;
    v.tail_quarters = t->tail_quarters >= 0 ? t->tail_quarters : d.tail_quarters;
  }
  std::lock_guard<std::mutex> lk(g_tuning_mu);
  g_tuning = v;
  return DROT_OK;
}

int drot_batch_plan_create(int n_inst, const drot_batch_instance* desc, int cols_per_tile,
                           drot_batch_plan* out) {
  return drot_batch_plan_create_ex(n_inst, desc, cols_per_tile, 512, out);
}

}  // extern "C"

// Plan of a QR batch, or of a GL batch when groups != nullptr (groups[k] the
// class count and lambdas[k] the shrink threshold of instance k; the
// descriptors' r_weight is then unused).
static int batch_plan_create_impl(int n_inst, const drot_batch_instance* desc, int cols_per_tile,
                                  int band_rows, const int* groups, const float* lambdas,
                                  drot_batch_plan* out) {
  if (!out || n_inst <= 0 || n_inst > 65535 || !desc) return DROT_ERR_INVALID_ARG;
  if (band_rows != 128 && band_rows != 512) return DROT_ERR_INVALID_ARG;
  const bool gl = groups != nullptr;
  if (gl && band_rows != 512) return DROT_ERR_INVALID_ARG;
  *out = nullptr;
  if (cols_per_tile <= 0) cols_per_tile = 128;
  BatchPlanImpl P;
  P.tune = current_tuning();
  const int fine_cols = P.tune.fine_cols, finest_cols = P.tune.finest_cols;
  P.n_inst = n_inst;
  P.cols_per_tile = cols_per_tile;
  P.gl = gl ? 1 : 0;
  P.inst.resize(n_inst);
  std::vector<std::vector<int>> bounds(gl ? n_inst : 0);
  if (gl) {
    int cover = 0;
    for (int k = 0; k < n_inst; ++k) {
      if (groups[k] <= 0 || groups[k] > desc[k].n_rows || !(lambdas[k] >= 0.0f))
        return DROT_ERR_INVALID_ARG;
      bounds[k] = gl_bounds(desc[k].n_rows, groups[k]);
      for (int g = 0; g < groups[k]; ++g) {
        if (bounds[k][g + 1] <= bounds[k][g]) return DROT_ERR_INVALID_ARG;
        cover = std::max(cover, bounds[k][g + 1] - (bounds[k][g] & ~3));
      }
    }
    P.band_cover = (cover + kBatchS - 1) / kBatchS * kBatchS;
    if (P.band_cover > kBatchGlMaxCover) return DROT_ERR_UNSUPPORTED;
  }
  long long rows = 0, cols = 0, rp = 0, cpp = 0;
  for (int k = 0; k < n_inst; ++k) {
    const drot_batch_instance& d = desc[k];
    if (d.n_rows <= 0 || d.n_cols <= 0 || d.ld < d.n_rows || (d.ld & 3) != 0 ||
        (long long)d.ld * d.n_cols > (1LL << 40) ||
        (d.c_offset & 3) != 0 || (d.x_offset & 3) != 0 || d.c_offset < 0 || d.x_offset < 0 ||
        d.p_offset < 0 || d.q_offset < 0 || !(d.rho > 0.0f) || !(d.r_weight >= 0.0f))
      return DROT_ERR_INVALID_ARG;
    BatchInst I;
    memset(&I, 0, sizeof(I));
    I.nr = d.n_rows;
    I.nc = d.n_cols;
    I.ld = d.ld;
    I.c_off = d.c_offset;
    I.x_off = d.x_offset;
    I.p_off = d.p_offset;
    I.q_off = d.q_offset;
    // Bands of 512 rows; the last one takes the remainder and the narrowest
    // warp step (128, 256 or 512 rows x 4, 2 or 1 columns) that covers it.
    I.band_h = band_rows;
    I.nbands = gl ? groups[k] : (d.n_rows + band_rows - 1) / band_rows;
    I.P = (d.n_cols + cols_per_tile - 1) / cols_per_tile;
    I.Pf = (d.n_cols + fine_cols - 1) / fine_cols;
    I.Px = finest_cols > 0 ? (d.n_cols + finest_cols - 1) / finest_cols : 0;
    I.tile0 = (int)P.tiles.size();
    if (gl) add_gl_tiles(P.tiles, k, I, I.P, bounds[k]);
    else add_tiles(P.tiles, k, I, I.P);
    I.ntiles = (int)P.tiles.size() - I.tile0;
    I.row_off = (int)rows;
    I.col_off = (int)cols;
    I.rp_off = rp;
    I.cp_off = cpp;
    rows += d.n_rows;
    cols += d.n_cols;
    rp += (long long)std::max(std::max(I.P, I.Pf), I.Px) * d.n_rows;
    I.item0 = (int)P.items.size();
    const int ilines = P.tune.item_lines;
    for (int l = 0; l < d.n_rows + d.n_cols; l += ilines) {
      BatchItem Q;
      Q.inst = k;
      Q.l0 = l;
      Q.l1 = std::min(l + ilines, d.n_rows + d.n_cols);
      Q.pad = 0;
      P.items.push_back(Q);
    }
    I.nitems = (int)P.items.size() - I.item0;
    cpp += (long long)I.nbands * d.n_cols;
    // Operator parameters (pytorch/src/qr_drot_cuda_kernel.cu:100-102) and
    // the warm start (core/drot_qr.hpp:321-331), in float as the reference.
    const float s = d.rho / ((float)d.n_rows + (float)d.n_cols);
    float t = s * d.r_weight;
    t = t * (float)(d.n_rows + d.n_cols);
    I.s = s;
    I.kappa = 1.0f + t;
    I.kappa_rcp = (float)(1.0 / (double)I.kappa);
    I.eps = d.eps;
    // QR stops on residual < eps, GL on residual <= eps (drot_glr.hpp:348)
    I.res2_stop = res2_threshold(d.eps, !gl);
    I.lambda = gl ? lambdas[k] : 0.0f;
    I.nc_rcp = (float)(1.0 / (double)(float)d.n_cols);
    I.nr_rcp = (float)(1.0 / (double)(float)d.n_rows);
    const float n = (float)d.n_rows, m = (float)d.n_cols;
    float kk = 1.0f * s;
    kk = kk * n;
    kk = kk * m;
    kk = kk - 2.0f;
    float tt = (kk + 2.0f) / n;
    I.w_phi1 = tt / (m + n);
    tt = (kk + 2.0f) / m;
    I.w_phi2 = tt / (m + n);
    I.w_a = (kk + 1.0f) / n;
    I.w_b = (kk + 1.0f) / m;
    I.w_alpha = kk + 1.0f;
    P.inst[k] = I;
  }
  P.n_tiles = (int)P.tiles.size();
  // The fine list (fine_cols-column chunks) after the coarse one; unused when the
  // coarse tiles are no wider.
  for (int k = 0; k < n_inst; ++k) {
    BatchInst& I = P.inst[k];
    I.tile0f = (int)P.tiles.size();
    if (gl) add_gl_tiles(P.tiles, k, I, I.Pf, bounds[k]);
    else add_tiles(P.tiles, k, I, I.Pf);
    I.ntilesf = (int)P.tiles.size() - I.tile0f;
  }
  P.n_tiles_f = fine_cols < cols_per_tile ? (int)P.tiles.size() - P.n_tiles : 0;
  // The finest list after the fine one (only when the fine list is used).
  const bool use_x = P.n_tiles_f > 0 && finest_cols > 0 && finest_cols < fine_cols;
  const int x0 = (int)P.tiles.size();
  P.n_items = (int)P.items.size();
  for (int k = 0; k < n_inst; ++k) {
    BatchInst& I = P.inst[k];
    I.tile0x = (int)P.tiles.size();
    if (use_x) {
      if (gl) add_gl_tiles(P.tiles, k, I, I.Px, bounds[k]);
      else add_tiles(P.tiles, k, I, I.Px);
    }
    I.ntilesx = (int)P.tiles.size() - I.tile0x;
    I.item0x = (int)P.items.size();
    if (use_x) {
      const int xl = P.tune.finest_item_lines;
      for (int l = 0; l < I.nr + I.nc; l += xl) {
        BatchItem Q;
        Q.inst = k;
        Q.l0 = l;
        Q.l1 = std::min(l + xl, I.nr + I.nc);
        Q.pad = 0;
        P.items.push_back(Q);
      }
    }
    I.nitemsx = (int)P.items.size() - I.item0x;
  }
  P.n_tiles_x = (int)P.tiles.size() - x0;
  P.n_items_x = (int)P.items.size() - P.n_items;
  P.order.resize(n_inst);
  for (int k = 0; k < n_inst; ++k) P.order[k] = k;
  std::stable_sort(P.order.begin(), P.order.end(), [&](int a, int b) {
    return (long long)P.inst[a].nr * P.inst[a].nc > (long long)P.inst[b].nr * P.inst[b].nc;
  });
  P.rows = rows;
  P.cols = cols;
  P.rowpart = rp;
  P.colpart = cpp;
  if (rows > INT32_MAX || cols > INT32_MAX) return DROT_ERR_UNSUPPORTED;

  int dev = 0, sms = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return DROT_ERR_CUDA;
  P.threads = 256;
  P.threads_pt = 512;
  P.band_rows = band_rows;
  P.smem = gl ? batch_smem(P.threads / 32, 0, P.band_cover) : batch_smem(P.threads / 32, 0);
  P.smem_pt = gl ? 0 : batch_smem(P.threads_pt / 32, 16);  // point launches (d <= 16)
  struct Variant {
    const void* fn;
    size_t smem;
  };
  const Variant qr_kernels[] = {{(const void*)batch_solve_kernel<float, 0>, P.smem},
                                {(const void*)batch_solve_kernel<__nv_bfloat16, 0>, P.smem},
                                {(const void*)batch_solve_kernel<float, 8>, P.smem_pt},
                                {(const void*)batch_solve_kernel<float, 16>, P.smem_pt}};
  const Variant gl_kernels[] = {{(const void*)batch_solve_kernel<float, 0, true>, P.smem},
                                {(const void*)batch_solve_kernel<__nv_bfloat16, 0, true>, P.smem}};
  auto occupancy = [&](const Variant* v, int n, int threads, int& occ) -> bool {
    occ = 1 << 30;
    for (int i = 0; i < n; ++i) {
      if (v[i].smem > 48 * 1024 &&
          cudaFuncSetAttribute(v[i].fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)v[i].smem) != cudaSuccess)
        return false;
      int o = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, v[i].fn, threads, v[i].smem) !=
          cudaSuccess)
        return false;
      occ = std::min(occ, o);
    }
    return true;
  };
  int occ = 0, occ_pt = 0;
  if (!occupancy(gl ? gl_kernels : qr_kernels, 2, P.threads, occ)) return DROT_ERR_CUDA;
  if (occ <= 0) return DROT_ERR_CUDA;
  P.grid = occ * sms;
  if (!gl) {
    // point launches hold kPtTmemCols TMEM columns per CTA for the whole launch
    if (!occupancy(qr_kernels + 2, 2, P.threads_pt, occ_pt)) return DROT_ERR_CUDA;
    occ_pt = std::min(occ_pt, 512 / kPtTmemCols);
    P.grid_pt = occ_pt * sms;
  }

  size_t off = 0;
  P.off_ctrl = off;  off = al(off + 512);
  P.off_inst = off;  off = al(off + sizeof(BatchInst) * n_inst);
  P.off_tiles = off; off = al(off + sizeof(BatchTile) * P.tiles.size());
  P.off_items = off; off = al(off + sizeof(BatchItem) * P.items.size());
  P.off_a = off;     off = al(off + sizeof(float) * rows);
  P.off_phi1 = off;  off = al(off + sizeof(float) * rows);
  P.off_b = off;     off = al(off + sizeof(float) * cols);
  P.off_phi2 = off;  off = al(off + sizeof(float) * cols);
  P.off_alpha = off; off = al(off + sizeof(float) * 2 * n_inst);
  P.off_rp = off;    off = al(off + sizeof(float) * rp);
  P.off_cp = off;    off = al(off + sizeof(float) * cpp);
  P.off_tsum = off;  off = al(off + sizeof(float2) * P.tiles.size());
  P.off_tobj = off;  off = al(off + sizeof(float2) * P.tiles.size());
  P.off_res = off;   off = al(off + sizeof(float2) * P.items.size());
  P.off_obj = off;   off = al(off + sizeof(double) * n_inst);
  P.off_conv = off;  off = al(off + sizeof(int) * n_inst);
  P.off_stats = off; off = al(off + sizeof(BatchStat) * n_inst);
  P.off_act = off;   off = al(off + sizeof(int) * (P.tiles.size() + P.items.size()));
  P.off_order = off; off = al(off + sizeof(int) * n_inst);
  P.off_ilvl = off;  off = al(off + sizeof(int) * n_inst);
  P.off_xn = off;    off = al(off + sizeof(float) * rows);
  P.off_yn = off;    off = al(off + sizeof(float) * cols);
  P.total = off;

  drot_batch_plan h = new (std::nothrow) drot_batch_plan_s;
  if (!h) return DROT_ERR_CUDA;
  h->p = std::move(P);
  *out = h;
  return DROT_OK;
}

extern "C" {

int drot_batch_plan_create_ex(int n_inst, const drot_batch_instance* desc, int cols_per_tile,
                              int band_rows, drot_batch_plan* out) {
  return batch_plan_create_impl(n_inst, desc, cols_per_tile, band_rows, nullptr, nullptr, out);
}

int drot_gl_batch_plan_create(int n_inst, const drot_gl_batch_instance* desc, int cols_per_tile,
                              drot_batch_plan* out) {
  if (!desc || n_inst <= 0 || n_inst > 65535) return DROT_ERR_INVALID_ARG;
  std::vector<drot_batch_instance> d(n_inst);
  std::vector<int> groups(n_inst);
  std::vector<float> lambdas(n_inst);
  for (int k = 0; k < n_inst; ++k) {
    const drot_gl_batch_instance& g = desc[k];
    memset(&d[k], 0, sizeof(d[k]));
    d[k].n_rows = g.n_rows;
    d[k].n_cols = g.n_cols;
    d[k].ld = g.ld;
    d[k].c_offset = g.c_offset;
    d[k].x_offset = g.x_offset;
    d[k].p_offset = g.p_offset;
    d[k].q_offset = g.q_offset;
    d[k].rho = g.rho;
    d[k].r_weight = 0.0f;
    d[k].eps = g.eps;
    groups[k] = g.n_groups;
    lambdas[k] = g.lambda;
  }
  return batch_plan_create_impl(n_inst, d.data(), cols_per_tile, 512, groups.data(),
                                lambdas.data(), out);
}

void drot_batch_plan_destroy(drot_batch_plan plan) { delete plan; }

size_t drot_batch_plan_workspace_bytes(drot_batch_plan plan) {
  return plan ? plan->p.total : 0;
}

int drot_batch_plan_tiles(drot_batch_plan plan) { return plan ? plan->p.n_tiles : 0; }

int drot_batch_upload(drot_batch_plan plan, void* workspace, size_t workspace_bytes,
                      drot_stream_t stream) {
  if (!plan || !workspace) return DROT_ERR_INVALID_ARG;
  const BatchPlanImpl& P = plan->p;
  if (workspace_bytes < P.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(ws + P.off_inst, P.inst.data(), sizeof(BatchInst) * P.n_inst,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws + P.off_tiles, P.tiles.data(), sizeof(BatchTile) * P.tiles.size(),
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws + P.off_items, P.items.data(), sizeof(BatchItem) * P.items.size(),
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(ws + P.off_order, P.order.data(), sizeof(int) * P.n_inst,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return DROT_ERR_CUDA;
  return DROT_OK;
}

// Shared by the cost-matrix and the point-cloud launches: parameter block,
// control words, warm start, then the cooperative solve kernel `fn`.
static int batch_launch(const BatchPlanImpl& P, const void* fn, BatchParams& B, void* workspace,
                        size_t workspace_bytes, int max_iters, cudaStream_t st,
                        bool points = false) {
  const int grid = points ? P.grid_pt : P.grid;
  const int threads = points ? P.threads_pt : P.threads;
  const size_t smem = points ? P.smem_pt : P.smem;
  if (grid <= 0) return DROT_ERR_INVALID_ARG;
  if (workspace_bytes < P.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  B.inst = (const BatchInst*)(ws + P.off_inst);
  B.tiles = (const BatchTile*)(ws + P.off_tiles);
  B.n_inst = P.n_inst;
  B.n_tiles = P.n_tiles;
  B.n_tiles_f = P.n_tiles_f;
  B.n_tiles_x = P.n_tiles_x;
  B.n_items_x = P.n_items_x;
  // active tiles of a level below which the solve moves to the next finer one
  B.fine_threshold = (int)((long long)grid * P.tune.level_quarters / 4);
  B.tail_tiles = (int)((long long)grid * P.tune.tail_quarters / 4);
  B.items = (const BatchItem*)(ws + P.off_items);
  B.n_items = P.n_items;
  B.res_slot = (float2*)(ws + P.off_res);
  B.obj_slot = (double*)(ws + P.off_obj);
  B.max_iters = max_iters;
  B.a = (float*)(ws + P.off_a);
  B.b = (float*)(ws + P.off_b);
  B.phi1 = (float*)(ws + P.off_phi1);
  B.phi2 = (float*)(ws + P.off_phi2);
  B.alpha = (float*)(ws + P.off_alpha);
  B.rowpart = (float*)(ws + P.off_rp);
  B.colpart = (float*)(ws + P.off_cp);
  B.tile_sum = (float2*)(ws + P.off_tsum);
  B.tile_obj = (float2*)(ws + P.off_tobj);
  B.conv = (int*)(ws + P.off_conv);
  B.stats = (BatchStat*)(ws + P.off_stats);
  B.act = (int*)(ws + P.off_act);
  B.order = (const int*)(ws + P.off_order);
  B.ilvl = (int*)(ws + P.off_ilvl);
  B.counters = (unsigned*)(ws + P.off_ctrl);
  B.bar = (unsigned*)(ws + P.off_ctrl + 64);
  B.abort_flag = (int*)(ws + P.off_ctrl + 128);
  const char* e = getenv("DROT_BARRIER_TIMEOUT_MS");
  const long long ms = (e && atoll(e) > 0) ? atoll(e) : 10000LL;
  B.timeout_ns = ms * 1000000LL;
  // DROT_TEST_STALL_CTA=k: CTA k skips its first grid-barrier arrival (the
  // failure-detection test hook of the bounded waits; off by default).
  const char* sc = getenv("DROT_TEST_STALL_CTA");
  B.stall_cta = (sc && *sc) ? atoi(sc) : -1;
  B.pf_dist = P.tune.prefetch_distance;
  B.band_cover = P.band_cover;
  if (cudaMemsetAsync(ws + P.off_ctrl, 0, 512, st) != cudaSuccess) return DROT_ERR_CUDA;
  batch_init_kernel<<<dim3(64, P.n_inst), 256, 0, st>>>(B);
  if (cudaGetLastError() != cudaSuccess) return DROT_ERR_CUDA;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return DROT_ERR_CUDA;
  void* args[] = {(void*)&B};
  if (cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, st) !=
      cudaSuccess) {
    cudaGetLastError();
    return DROT_ERR_CUDA;
  }
  return DROT_OK;
}

int drot_qr_batch_launch(drot_batch_plan plan, const void* c, int c_dtype, const float* p,
                         const float* q, float* x, int max_iters, void* workspace,
                         size_t workspace_bytes, drot_stream_t stream) {
  if (!plan || !c || !p || !q || !x || !workspace || max_iters < 0) return DROT_ERR_INVALID_ARG;
  if (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  if (((uintptr_t)x & 15u) || ((uintptr_t)c & (c_dtype == DROT_C_F32 ? 15u : 7u)))
    return DROT_ERR_INVALID_ARG;
  BatchParams B;
  memset(&B, 0, sizeof(B));
  B.c = c;
  B.p = p;
  B.q = q;
  B.x = x;
  B.iter_log = plan->iter_log;
  B.iter_tiles = plan->iter_tiles;
  B.iter_log_cap = plan->iter_log_cap;
  const bool gl = plan->p.gl != 0;
  const void* fn = c_dtype == DROT_C_F32
                       ? (gl ? (const void*)batch_solve_kernel<float, 0, true>
                             : (const void*)batch_solve_kernel<float, 0>)
                       : (gl ? (const void*)batch_solve_kernel<__nv_bfloat16, 0, true>
                             : (const void*)batch_solve_kernel<__nv_bfloat16, 0>);
  return batch_launch(plan->p, fn, B, workspace, workspace_bytes, max_iters,
                      (cudaStream_t)stream);
}

int drot_batch_resume(drot_batch_plan plan, const void* c, int c_dtype, const float* p,
                      const float* q, float* x, int n_iters, void* workspace,
                      size_t workspace_bytes, drot_stream_t stream) {
  if (!plan || !c || !p || !q || !x || !workspace || n_iters < 0) return DROT_ERR_INVALID_ARG;
  if (!plan->p.gl) return DROT_ERR_INVALID_ARG;  // QR keeps X folded between iterations
  if (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  if (((uintptr_t)x & 15u) || ((uintptr_t)c & (c_dtype == DROT_C_F32 ? 15u : 7u)))
    return DROT_ERR_INVALID_ARG;
  if (n_iters == 0) return DROT_OK;
  const BatchPlanImpl& P = plan->p;
  BatchParams B;
  memset(&B, 0, sizeof(B));
  B.c = c;
  B.p = p;
  B.q = q;
  B.x = x;
  B.resume = 1;
  B.no_stop = 1;
  const void* fn = c_dtype == DROT_C_F32 ? (const void*)batch_solve_kernel<float, 0, true>
                                         : (const void*)batch_solve_kernel<__nv_bfloat16, 0, true>;
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = batch_launch(P, fn, B, workspace, workspace_bytes, n_iters, st);
  if (rc != DROT_OK) return rc;
  // alpha of the last iteration sits in parity slot n_iters & 1: bring it to
  // slot 0, where the next launch reads it.
  if (n_iters & 1) {
    float* alpha = (float*)((char*)workspace + P.off_alpha);
    if (cudaMemcpyAsync(alpha, alpha + P.n_inst, sizeof(float) * P.n_inst,
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return DROT_ERR_CUDA;
  }
  return DROT_OK;
}

int drot_qr_batch_launch_points(drot_batch_plan plan, const float* xpts, const float* ypts,
                                int dim, float cost_scale, const float* p, const float* q,
                                float* x, int max_iters, void* workspace, size_t workspace_bytes,
                                drot_stream_t stream) {
  if (!plan || !xpts || !ypts || !p || !q || !x || !workspace || max_iters < 0)
    return DROT_ERR_INVALID_ARG;
  if (dim != 8 && dim != 16) return DROT_ERR_UNSUPPORTED;
  if (plan->p.band_rows != 512 || plan->p.gl) return DROT_ERR_INVALID_ARG;  // point tiles: 512-row QR bands
  if (((uintptr_t)x & 15u) || ((uintptr_t)xpts & 15u) || ((uintptr_t)ypts & 15u))
    return DROT_ERR_INVALID_ARG;
  const BatchPlanImpl& P = plan->p;
  if (workspace_bytes < P.total || ((uintptr_t)workspace & 255u)) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  cudaStream_t st = (cudaStream_t)stream;
  BatchParams B;
  memset(&B, 0, sizeof(B));
  B.p = p;
  B.q = q;
  B.x = x;
  B.xpts = xpts;
  B.ypts = ypts;
  B.xnorm = (const float*)(ws + P.off_xn);
  B.ynorm = (const float*)(ws + P.off_yn);
  B.cscale = cost_scale;
  B.dim = dim;
  B.iter_log = plan->iter_log;
  B.iter_tiles = plan->iter_tiles;
  B.iter_log_cap = plan->iter_log_cap;
  point_norms_kernel<<<(int)std::min<long long>((P.rows + 255) / 256, 1024), 256, 0, st>>>(
      xpts, (int)P.rows, dim, (float*)(ws + P.off_xn));
  point_norms_kernel<<<(int)std::min<long long>((P.cols + 255) / 256, 1024), 256, 0, st>>>(
      ypts, (int)P.cols, dim, (float*)(ws + P.off_yn));
  if (cudaGetLastError() != cudaSuccess) return DROT_ERR_CUDA;
  const void* fn = dim == 8 ? (const void*)batch_solve_kernel<float, 8>
                            : (const void*)batch_solve_kernel<float, 16>;
  return batch_launch(P, fn, B, workspace, workspace_bytes, max_iters, st, true);
}

int drot_batch_set_iteration_log(drot_batch_plan plan, unsigned long long* times,
                                 unsigned* active_tiles, int cap) {
  if (!plan || cap < 0 || (cap > 0 && (!times || !active_tiles))) return DROT_ERR_INVALID_ARG;
  plan->iter_log = cap > 0 ? times : nullptr;
  plan->iter_tiles = cap > 0 ? active_tiles : nullptr;
  plan->iter_log_cap = cap;
  return DROT_OK;
}

int drot_batch_state(drot_batch_plan plan, void* workspace, float** phi1, float** phi2) {
  if (!plan || !workspace || !phi1 || !phi2) return DROT_ERR_INVALID_ARG;
  char* ws = (char*)workspace;
  *phi1 = (float*)(ws + plan->p.off_phi1);
  *phi2 = (float*)(ws + plan->p.off_phi2);
  return DROT_OK;
}

int drot_batch_state_ex(drot_batch_plan plan, void* workspace, float** a, float** b,
                        float** phi1, float** phi2, float** alpha) {
  if (!plan || !workspace || !a || !b || !phi1 || !phi2 || !alpha) return DROT_ERR_INVALID_ARG;
  char* ws = (char*)workspace;
  *a = (float*)(ws + plan->p.off_a);
  *b = (float*)(ws + plan->p.off_b);
  *phi1 = (float*)(ws + plan->p.off_phi1);
  *phi2 = (float*)(ws + plan->p.off_phi2);
  *alpha = (float*)(ws + plan->p.off_alpha);
  return DROT_OK;
}

int drot_batch_results(drot_batch_plan plan, const void* workspace, drot_batch_result* out,
                       drot_stream_t stream) {
  if (!plan || !workspace || !out) return DROT_ERR_INVALID_ARG;
  const BatchPlanImpl& P = plan->p;
  const char* ws = (const char*)workspace;
  std::vector<BatchStat> st(P.n_inst);
  int abort_flag = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(st.data(), ws + P.off_stats, sizeof(BatchStat) * P.n_inst,
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&abort_flag, ws + P.off_ctrl + 128, sizeof(int), cudaMemcpyDeviceToHost,
                      s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return DROT_ERR_CUDA;
  for (int k = 0; k < P.n_inst; ++k) {
    out[k].n_iter = st[k].n_iter;
    out[k].iters_run = st[k].iters_run;
    out[k].converged = st[k].converged;
    out[k].objective_valid = st[k].objective_valid;
    out[k].objective = st[k].objective;
    out[k].residual = st[k].residual >= 0.0 ? sqrt(st[k].residual) : st[k].residual;
  }
  return abort_flag ? DROT_ERR_BARRIER_TIMEOUT : DROT_OK;
}

}  // extern "C"
