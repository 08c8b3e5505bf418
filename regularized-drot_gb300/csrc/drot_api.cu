// drot_api.cu -- host side of the GB300 DROT solver: launch planning,
// workspace layout, the cooperative launch, and the extern "C" entry points
// declared in include/drot_gb300.h.
//
// Host arithmetic that mirrors the reference's parameter mapping is compiled
// with -ffp-contract=off (see build.py) so it rounds like the reference's
// x86-64 host code on every host architecture.
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "drot_gb300.h"
#include "drot_kernels.cuh"

namespace drot {

// ---------------------------------------------------------------------------
// kernel table
// ---------------------------------------------------------------------------

typedef void (*SolveFn)(const SolveParams);

template <int MODE, bool TMA, typename CT>
static SolveFn kernel_kv(int vec, int kv) {
  if constexpr (TMA) {
    if (vec != 4) return nullptr;
    if (kv == 1) return drot_solve_kernel<MODE, 4, 1, true, CT>;
    if (kv == 2) return drot_solve_kernel<MODE, 4, 2, true, CT>;
    if (kv == 4) return drot_solve_kernel<MODE, 4, 4, true, CT>;
    if constexpr (MODE == MODE_GL) {
      if (kv == 8) return drot_solve_kernel<MODE, 4, 8, true, CT>;
    }
  } else {
    if (vec == 4) {
      if (kv == 1) return drot_solve_kernel<MODE, 4, 1, false, CT>;
      if (kv == 2) return drot_solve_kernel<MODE, 4, 2, false, CT>;
      if (kv == 4) return drot_solve_kernel<MODE, 4, 4, false, CT>;
      if constexpr (MODE == MODE_GL) {
        if (kv == 8) return drot_solve_kernel<MODE, 4, 8, false, CT>;
      }
    } else {
      if (kv == 1) return drot_solve_kernel<MODE, 1, 1, false, CT>;
      if (kv == 2) return drot_solve_kernel<MODE, 1, 2, false, CT>;
      if (kv == 4) return drot_solve_kernel<MODE, 1, 4, false, CT>;
      if constexpr (MODE == MODE_GL) {
        if (kv == 8) return drot_solve_kernel<MODE, 1, 8, false, CT>;
      }
    }
  }
  return nullptr;
}

// Kernel instance for (mode, vector width, vectors per lane, data path, cost
// type).  The TMA ring exists for float costs only.
static SolveFn kernel_for(int mode, int vec, int kv, bool tma, int ctype = DROT_C_F32) {
  if (ctype == DROT_C_BF16) {
    if (tma) return nullptr;
    return mode == MODE_QR ? kernel_kv<MODE_QR, false, __nv_bfloat16>(vec, kv)
                           : kernel_kv<MODE_GL, false, __nv_bfloat16>(vec, kv);
  }
  if (mode == MODE_QR)
    return tma ? kernel_kv<MODE_QR, true, float>(vec, kv) : kernel_kv<MODE_QR, false, float>(vec, kv);
  return tma ? kernel_kv<MODE_GL, true, float>(vec, kv) : kernel_kv<MODE_GL, false, float>(vec, kv);
}

// ---------------------------------------------------------------------------
// small helper kernels (initial state)
// ---------------------------------------------------------------------------

__global__ void fill_kernel(float* __restrict__ v, long long n, float val) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = val;
}

// Cold start X = p q^T (init_x, core/kernel_qr.hpp:7-40): x = p_i * q_j.
__global__ void outer_kernel(float* __restrict__ x, const float* __restrict__ p,
                             const float* __restrict__ q, int nr, int nc) {
  const long long n = (long long)nr * nc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / nr);
    const int i = (int)(t - (long long)j * nr);
    x[t] = p[i] * q[j];
  }
}

// ---------------------------------------------------------------------------
// planning
// ---------------------------------------------------------------------------

static const size_t kAlign = 256;
static inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }


// Scratch layout (offsets from the workspace base):
//   [0, 256)     DeviceStats
//   [256, 512)   barrier counter + abort flag
//   rowpart      P * nr floats
//   colpart      nsb * nc floats
//   cta_sum/obj/res  grid float pairs (8 bytes) each
struct Plan {
  int mode = 0, vec = 4, kv = 4, wt = 1, threads = 256, nbands = 1, P = 1, grid = 1, nsb = 1;
  int band_h = 0, ns = 1, p2_smem = 0, p2_cap_r = 0, p2_cap_c = 0, ctype = DROT_C_F32;
  bool tma = false;
  size_t smem = 0;
  std::vector<int> bounds;
  size_t off_stats = 0, off_ctrl = 256, off_rowpart = 0, off_colpart = 0, off_sum = 0,
         off_obj = 0, off_res = 0, total = 0;
};

struct DeviceInfo {
  int dev = 0, sms = 0, smem_optin = 0, l2 = 0;
  bool ok = false;
};

static DeviceInfo device_info() {
  DeviceInfo d;
  if (cudaGetDevice(&d.dev) != cudaSuccess) return d;
  if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, d.dev) != cudaSuccess)
    return d;
  cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, d.dev);
  cudaDeviceGetAttribute(&d.l2, cudaDevAttrL2CacheSize, d.dev);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, d.dev);
  d.ok = coop != 0 && d.sms > 0;
  return d;
}

// Reference group boundaries (core/kernel_glr.hpp:79-80 with +0.49 for the
// single-pass kernel chosen when ceil(n_rows/G) <= 256, drot_glr.hpp:280;
// core/kernel_glr.hpp:185-186 with +0.49999 otherwise).
static void group_bounds(int nr, int G, int* out) {
  const int small = ((nr + G - 1) / G) <= 256;
  const double off = small ? 0.49 : 0.49999;
  const float per = (float)nr / (float)G;
  for (int k = 0; k <= G; ++k) {
    const float f = per * (float)k;
    out[k] = (int)((double)f + off);
  }
}

static int occupancy(SolveFn fn, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)fn, threads, smem) !=
      cudaSuccess)
    return 0;
  return nb;
}

// Launch shape pinned for a problem shape (drot_set_launch_choice, set by
// the autotuner); zero fields leave the planner's own choice.
struct LaunchChoice {
  int kv = 0;     // vectors per lane (QR: cap 1, 2, 4; GL: 1, 2, 4, 8)
  int warps = 0;  // warps per CTA, 4..16
  int tma = 0;    // 1: TMA bulk-copy ring (FP32 C, 16-byte aligned columns)
  int ctas = 0;   // TMA ring: CTAs per SM sharing its shared memory (1 or 2)
  bool operator==(const LaunchChoice& o) const {
    return kv == o.kv && warps == o.warps && tma == o.tma && ctas == o.ctas;
  }
};

// Build the launch plan for one data path (tma: shared-memory TMA ring, else
// register loads).  Returns a drot_status.
static int make_plan_uncached(int mode, int nr, int nc, int G, int vec, bool tma, int ctype,
                              Plan& pl, const int* ubounds, const LaunchChoice& ch) {
  if (nr <= 0 || nc <= 0) return DROT_ERR_INVALID_ARG;
  if (tma && vec != 4) return DROT_ERR_UNSUPPORTED;
  const DeviceInfo dev = device_info();
  if (!dev.ok) return DROT_ERR_CUDA;
  pl = Plan();
  pl.mode = mode;
  pl.vec = vec;
  pl.tma = tma;
  const int SV = 32 * vec;
  if (mode == MODE_QR) {
    // Four 128-bit vectors per lane (512-row sub-bands); short panels use
    // fewer so lanes are not left idle.
    pl.kv = nr <= SV ? 1 : (nr <= 2 * SV ? 2 : 4);
    // A pinned choice caps the vectors per lane: shorter bands, fewer
    // registers per thread, more CTAs per SM.
    if (ch.kv == 1 || ch.kv == 2 || ch.kv == 4) pl.kv = std::min(pl.kv, ch.kv);
    pl.wt = 1;
  } else {
    if (G <= 0) return DROT_ERR_INVALID_ARG;
    if (G > kMaxGroups) return DROT_ERR_UNSUPPORTED;
    pl.bounds.resize(G + 1);
    if (ubounds) std::copy(ubounds, ubounds + G + 1, pl.bounds.begin());
    else group_bounds(nr, G, pl.bounds.data());
    int hmax = 0;
    for (int g = 0; g < G; ++g) {
      const int lo = pl.bounds[g];
      const int base = lo - lo % vec;
      hmax = std::max(hmax, pl.bounds[g + 1] - base);
    }
    hmax = std::max(hmax, 1);
    // Vectors per lane: the smallest that covers a group in one warp, up to
    // a cap (a pinned choice, else 8); taller groups use teams of warps.
    const bool kv_pinned = ch.kv == 1 || ch.kv == 2 || ch.kv == 4 || ch.kv == 8;
    int kvcap = kv_pinned ? ch.kv : 8;
    pl.kv = 0;
    for (int kv : {1, 2, 4, 8})
      if (kv <= kvcap && SV * kv >= hmax) { pl.kv = kv; break; }
    if (pl.kv == 0) {
      // Groups taller than one warp covers: teams of 4-vector warps (the
      // 8-vector kernel spills at the register cap; measured at 3000^2 with
      // two 1500-row groups: 26.7 us per iteration against 31.8) -- unless
      // X + C lie beyond L2 and 8-vector teams fill at least 3 more warp
      // slots of the CTA (the kernel holds one CTA per SM, and the update is
      // latency-bound): 6000^2, 3000-row groups, 15 warps against 12: 86.3
      // against 95.4 us per iteration; 10000^2, 5000-row groups, 15 against
      // 10: 213 against 286 us.  With equal warps (5000^2, 8192 x 3000) the
      // 4-vector teams measured as fast or faster.
      if (!kv_pinned) {
        kvcap = 4;
        auto team_warps = [&](int kv) {
          const int wt = (hmax + kv * SV - 1) / (kv * SV);
          const int cap = wt >= 3 ? 16 : 8;
          return wt >= cap ? wt : (cap / wt) * wt;
        };
        const bool beyond_l2 = (double)nr * (double)nc * 8.0 > (double)dev.l2;
        if (!tma && vec == 4 && ctype == DROT_C_F32 && beyond_l2 &&
            team_warps(8) <= 16 && team_warps(8) >= team_warps(4) + 3)
          kvcap = 8;
      }
      pl.kv = kvcap;
      pl.wt = (hmax + kvcap * SV - 1) / (kvcap * SV);
      if (pl.wt > 16) return DROT_ERR_UNSUPPORTED;
    } else {
      pl.wt = 1;
    }
  }
  const int S = SV * pl.kv;
  SolveFn fn = kernel_for(mode, vec, pl.kv, tma, ctype);
  if (!fn) return DROT_ERR_UNSUPPORTED;
  pl.ctype = ctype;
  // TMA ring: 1 (default) or 2 CTAs per SM share the shared memory.
  const int tma_ctas = tma ? std::max(1, std::min(2, ch.ctas > 0 ? ch.ctas : 1)) : 1;
  const size_t budget = (size_t)std::max(dev.smem_optin, 48 * 1024) / tma_ctas - 1024;

  // Warps per CTA: 8 on the register path (two CTAs per SM), up to 16 when
  // a band needs teams of 3 or more warps (fewer CTAs per band keeps the
  // phase-2 partial count down).
  const int wtarget = (ch.warps >= 4 && ch.warps <= 16) ? ch.warps : (tma ? 16 : 8);
  for (int attempt = 0; attempt < 8; ++attempt) {
    const int wcap = (!tma && pl.wt >= 3) ? 16 : wtarget;
    int teams = pl.wt >= wcap ? 1 : std::max(1, wcap / pl.wt);
    int warps = teams * pl.wt;
    if (tma) {
      // Deepest ring that fits; fewer teams when two stages do not fit.
      for (;;) {
        const size_t fixed = solve_smem_bytes(warps, pl.wt, S, 0, true);
        const size_t stage = solve_smem_bytes(warps, pl.wt, S, 1, true) - fixed;
        const size_t fit = budget > fixed ? (budget - fixed) / stage : 0;
        if (fit >= 2) {
          pl.ns = (int)std::min<size_t>(fit, 8);
          break;
        }
        if (teams == 1) return DROT_ERR_UNSUPPORTED;
        teams = teams / 2;
        warps = teams * pl.wt;
      }
    } else {
      pl.ns = 1;
    }
    pl.threads = 32 * warps;
    pl.smem = solve_smem_bytes(warps, pl.wt, S, pl.ns, tma);
    if (pl.smem > budget) return DROT_ERR_UNSUPPORTED;
    if (pl.smem > 48 * 1024 &&
        cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pl.smem) != cudaSuccess)
      return DROT_ERR_CUDA;
    const int occ = occupancy(fn, pl.threads, pl.smem);
    if (occ <= 0) return DROT_ERR_CUDA;
    const int max_grid = occ * dev.sms;
    if (mode == MODE_QR) {
      // Fewest bands of at most wt*S rows, then equal heights (multiples of
      // 4) so every band carries the same work.
      const int cover = pl.wt * S;
      pl.nbands = (nr + cover - 1) / cover;
      if (pl.nbands > max_grid) {
        if (pl.wt >= 16) return DROT_ERR_UNSUPPORTED;
        pl.wt = std::min(16, pl.wt * 2);
        continue;
      }
      pl.band_h = (((nr + pl.nbands - 1) / pl.nbands) + 3) & ~3;
      pl.nbands = (nr + pl.band_h - 1) / pl.band_h;
    } else {
      pl.nbands = G;
      if (G > max_grid) return DROT_ERR_UNSUPPORTED;
    }
    const int per_band = std::max(1, max_grid / pl.nbands);
    const int by_cols = std::max(1, (nc + teams * 2 - 1) / (teams * 2));
    pl.P = std::max(1, std::min(per_band, by_cols));
    pl.grid = pl.nbands * pl.P;
    pl.nsb = pl.nbands * pl.wt;
    break;
  }
  if (pl.grid <= 0 || pl.nbands <= 0) return DROT_ERR_UNSUPPORTED;

  // Phase-2 state of each CTA's row / column slice in shared memory when
  // it is small and the CTAs stay co-resident with it.
  const int capr = ((nr + pl.grid - 1) / pl.grid + 3) & ~3;
  const int capc = ((nc + pl.grid - 1) / pl.grid + 3) & ~3;
  const int p2f = 3 * (capr + capc);
  const int warps = pl.threads / 32;
  const size_t smem2 = solve_smem_bytes(warps, pl.wt, S, pl.ns, tma, p2f);
  pl.p2_smem = 0;
  pl.p2_cap_r = pl.p2_cap_c = 0;
  if ((size_t)p2f * sizeof(float) <= 48 * 1024 && smem2 <= budget) {
    bool ok = true;
    if (smem2 > 48 * 1024)
      ok = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem2) == cudaSuccess;
    if (ok && occupancy(fn, pl.threads, smem2) * dev.sms >= pl.grid) {
      pl.p2_smem = 1;
      pl.p2_cap_r = capr;
      pl.p2_cap_c = capc;
      pl.smem = smem2;
    }
  }

  size_t off = 512;
  pl.off_stats = 0;
  pl.off_ctrl = 256;
  pl.off_rowpart = off;
  off = align_up(off + sizeof(float) * (size_t)pl.P * nr);
  pl.off_colpart = off;
  off = align_up(off + sizeof(float) * (size_t)pl.nsb * nc);
  pl.off_sum = off;
  off = align_up(off + sizeof(float2) * pl.grid);
  pl.off_obj = off;
  off = align_up(off + sizeof(float2) * pl.grid);
  pl.off_res = off;
  off = align_up(off + sizeof(float2) * pl.grid);
  pl.total = off;
  return DROT_OK;
}

// Plans are cached per (device, mode, shape, path): planning queries the
// occupancy calculator, which costs microseconds per call.
struct PlanKey {
  int dev, mode, nr, nc, G, vec, tma, ctype;
  std::vector<int> ubounds;  // caller's GL group boundaries (empty: the reference's)
  LaunchChoice ch;
  bool operator==(const PlanKey& o) const {
    return dev == o.dev && mode == o.mode && nr == o.nr && nc == o.nc && G == o.G &&
           vec == o.vec && tma == o.tma && ctype == o.ctype && ubounds == o.ubounds && ch == o.ch;
  }
};

static std::mutex g_plan_mu;
static std::vector<std::pair<PlanKey, Plan>> g_plans;

static int make_plan(int mode, int nr, int nc, int G, int vec, bool tma, Plan& pl,
                     int ctype = DROT_C_F32, const int* ubounds = nullptr,
                     const LaunchChoice& ch = LaunchChoice()) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DROT_ERR_CUDA;
  PlanKey key = {dev, mode, nr, nc, mode == MODE_GL ? G : 0, vec, tma ? 1 : 0, ctype, {}, ch};
  if (mode == MODE_GL && ubounds) key.ubounds.assign(ubounds, ubounds + G + 1);
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    for (auto& e : g_plans)
      if (e.first == key) { pl = e.second; return DROT_OK; }
  }
  const int rc = make_plan_uncached(mode, nr, nc, G, vec, tma, ctype, pl,
                                    mode == MODE_GL ? ubounds : nullptr, ch);
  if (rc == DROT_OK) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (g_plans.size() >= 64) g_plans.erase(g_plans.begin());
    g_plans.emplace_back(key, pl);
  }
  return rc;
}

// Pinned launch choices per (device, mode, shape, cost type); a key with
// n_rows = n_cols = 0 applies to every shape of its mode and cost type that
// has no exact entry.
struct ChoiceKey {
  int dev, mode, nr, nc, G, ctype;
  bool operator==(const ChoiceKey& o) const {
    return dev == o.dev && mode == o.mode && nr == o.nr && nc == o.nc && G == o.G &&
           ctype == o.ctype;
  }
};

static std::mutex g_choice_mu;
static std::vector<std::pair<ChoiceKey, LaunchChoice>> g_choices;

static LaunchChoice find_choice(int mode, int nr, int nc, int G, int ctype) {
  int dev = 0;
  LaunchChoice ch;
  if (cudaGetDevice(&dev) != cudaSuccess) return ch;
  const ChoiceKey exact = {dev, mode, nr, nc, mode == MODE_GL ? G : 0, ctype};
  const ChoiceKey any = {dev, mode, 0, 0, 0, ctype};
  std::lock_guard<std::mutex> lk(g_choice_mu);
  bool found = false;
  for (auto& e : g_choices) {
    if (e.first == exact) return e.second;
    if (!found && e.first == any) {
      ch = e.second;
      found = true;
    }
  }
  return ch;
}

// Plan for the given alignment.  The register path is the default: on this
// part the fused update is bound by per-warp instruction latency, and two
// 8-warp CTAs per SM with register-resident segments beat one 16-warp CTA
// fed by the shared-memory TMA ring.  A pinned choice can select the ring
// (used when C is FP32 and the columns are 16-byte aligned, else the
// register path runs with the choice's other fields).
static int choose_plan(int mode, int nr, int nc, int G, bool aligned4, Plan& pl,
                       int ctype = DROT_C_F32, const int* ubounds = nullptr) {
  const LaunchChoice ch = find_choice(mode, nr, nc, G, ctype);
  if (ch.tma && aligned4 && ctype == DROT_C_F32 &&
      make_plan(mode, nr, nc, G, 4, true, pl, DROT_C_F32, ubounds, ch) == DROT_OK)
    return DROT_OK;
  return make_plan(mode, nr, nc, G, aligned4 ? 4 : 1, false, pl, ctype, ubounds, ch);
}

static size_t scratch_bytes(int mode, int nr, int nc, int G, const int* ubounds = nullptr) {
  size_t best = 0;
  Plan pl;
  if (make_plan(mode, nr, nc, G, 4, true, pl, DROT_C_F32, ubounds) == DROT_OK)
    best = std::max(best, pl.total);
  if (make_plan(mode, nr, nc, G, 4, false, pl, DROT_C_F32, ubounds) == DROT_OK)
    best = std::max(best, pl.total);
  if (make_plan(mode, nr, nc, G, 1, false, pl, DROT_C_F32, ubounds) == DROT_OK)
    best = std::max(best, pl.total);
  // pinned choices (either cost type) may plan more partials
  for (int ctype : {DROT_C_F32, DROT_C_BF16}) {
    const LaunchChoice ch = find_choice(mode, nr, nc, G, ctype);
    if (ch == LaunchChoice()) continue;
    for (int v : {4, 1})
      if (make_plan(mode, nr, nc, G, v, false, pl, ctype, ubounds, ch) == DROT_OK)
        best = std::max(best, pl.total);
    if (ch.tma && ctype == DROT_C_F32 &&
        make_plan(mode, nr, nc, G, 4, true, pl, ctype, ubounds, ch) == DROT_OK)
      best = std::max(best, pl.total);
  }
  return best;
}

// Column-aligned copies.  Columns of n_rows % 4 != 0 rows are not 16-byte
// aligned, so the 128-bit vector path cannot read them in place; given the
// room, the solve runs on copies of C and X whose leading dimension is
// n_rows rounded up to 4 (the pad rows zero and masked), then copies X back:
// about 24 bytes per element once against 10 per iteration.  Every solve
// that has the room takes it, short ones too, so a solve split into
// segments (checkpointed autograd) keeps the arithmetic of one whole solve.
// The region follows the scratch.
constexpr int kRepackMinIters = 1;
static size_t repack_bytes(int nr, int nc) {
  const size_t ldp = ((size_t)nr + 3) & ~(size_t)3;
  return 2 * align_up(ldp * (size_t)nc * sizeof(float));
}
// Workspace of drot_*_solve: the scratch, then the aligned copies when the
// columns are unaligned.
static size_t solve_ws_bytes(int mode, int nr, int nc, int G, const int* ubounds = nullptr) {
  const size_t sc = scratch_bytes(mode, nr, nc, G, ubounds);
  if (sc == 0) return 0;
  return nr % 4 != 0 ? align_up(sc) + repack_bytes(nr, nc) : sc;
}

static long long barrier_timeout_ns() {
  const char* e = getenv("DROT_BARRIER_TIMEOUT_MS");
  if (e && *e) {
    const long long ms = atoll(e);
    if (ms > 0) return ms * 1000000LL;
  }
  return 10000LL * 1000000LL;  // 10 s
}

// DROT_TEST_STALL_CTA=k: CTA k skips its first grid-barrier arrival, so the
// launch's bounded waits run out and it returns DROT_ERR_BARRIER_TIMEOUT
// (with DROT_BARRIER_TIMEOUT_MS set low, quickly).  Failure-detection test
// hook; off (-1) by default.
static int stall_cta_hook() {
  const char* e = getenv("DROT_TEST_STALL_CTA");
  return (e && *e) ? atoi(e) : -1;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

struct SolveArgs {
  int mode;
  const void* c;
  int ctype;
  const float *p, *q;
  int nr, nc, G;
  float s, kappa, lambda;
  int max_iters;
  float eps;
  float *x, *a, *b, *phi1, *phi2, *alpha;
  void* ws;
  size_t ws_bytes;
  cudaStream_t stream;
  const int* bounds = nullptr;  // GL: caller's group boundaries (null: the reference's)
  int stop_every = 0, stop_le = 0;  // numpy-API stop rule (QR)
};

static int read_stats(const void* ws, drot_result* r, cudaStream_t stream) {
  DeviceStats st;
  if (cudaMemcpyAsync(&st, ws, sizeof(st), cudaMemcpyDeviceToHost, stream) != cudaSuccess)
    return DROT_ERR_CUDA;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return DROT_ERR_CUDA;
  r->n_iter = st.n_iter;
  r->iters_run = st.iters_run;
  r->converged = st.converged;
  r->status = st.status;
  r->objective_valid = st.objective_valid;
  r->objective = (float)st.objective;
  r->objective_f64 = st.objective;
  r->residual = st.residual;
  for (int k = 0; k < 4; ++k) r->phase_ms[k] = st.phase_ns[k] * 1e-6;
  return st.status == 0 ? DROT_OK : st.status;
}

static int run_solve(const SolveArgs& A, drot_result* result) {
  if (!A.c || !A.p || !A.q || !A.x || !A.a || !A.b || !A.phi1 || !A.phi2 || !A.alpha || !A.ws)
    return DROT_ERR_INVALID_ARG;
  if (A.nr <= 0 || A.nc <= 0 || A.max_iters < 0) return DROT_ERR_INVALID_ARG;
  if (((uintptr_t)A.ws & (kAlign - 1)) != 0) return DROT_ERR_WORKSPACE;
  if (A.ctype != DROT_C_F32 && A.ctype != DROT_C_BF16) return DROT_ERR_INVALID_ARG;
  const bool c_aligned = A.ctype == DROT_C_F32 ? aligned16(A.c) : (((uintptr_t)A.c & 7u) == 0);
  const bool aligned4 = A.nr % 4 == 0 && aligned16(A.x) && c_aligned;
  char* ws = (char*)A.ws;
  // Unaligned columns: the aligned copies when the workspace holds them.
  bool repack = false;
  char* cpad = nullptr;
  float* xpad = nullptr;
  const long long ldp = ((long long)A.nr + 3) & ~3LL;
  if (!aligned4 && A.max_iters >= kRepackMinIters) {
    const size_t base = align_up(scratch_bytes(A.mode, A.nr, A.nc, A.G, A.bounds));
    if (base > 0 && A.ws_bytes >= base + repack_bytes(A.nr, A.nc)) {
      repack = true;
      cpad = ws + base;
      xpad = (float*)(cpad + align_up((size_t)ldp * A.nc * sizeof(float)));
    }
  }
  const long long ld = repack ? ldp : A.nr;
  Plan pl;
  int rc = choose_plan(A.mode, A.nr, A.nc, A.G, aligned4 || repack, pl, A.ctype, A.bounds);
  if (rc != DROT_OK) return rc;
  if (A.ws_bytes < pl.total) return DROT_ERR_WORKSPACE;

  SolveParams prm;
  memset(&prm, 0, sizeof(prm));
  prm.c = repack ? (const void*)cpad : A.c; prm.p = A.p; prm.q = A.q;
  prm.x = repack ? xpad : A.x;
  prm.a = A.a; prm.b = A.b; prm.phi1 = A.phi1; prm.phi2 = A.phi2; prm.alpha = A.alpha;
  prm.ld = ld; prm.nr = A.nr; prm.nc = A.nc;
  prm.s = A.s; prm.kappa = A.kappa; prm.lambda = A.lambda;
  // RN(1/kappa): the double quotient rounded to float is the correctly
  // rounded float reciprocal (53 >= 2*24 + 2).
  prm.kappa_rcp = (float)(1.0 / (double)A.kappa);
  prm.nc_rcp = (float)(1.0 / (double)(float)A.nc);
  prm.nr_rcp = (float)(1.0 / (double)(float)A.nr);
  prm.max_iters = A.max_iters;
  prm.stop_every = A.stop_every;
  prm.stop_le = A.stop_le;
  prm.res2_stop = res2_threshold(A.eps, A.mode == MODE_QR && !A.stop_le);
  prm.nbands = pl.nbands; prm.P = pl.P; prm.Wt = pl.wt; prm.nsb = pl.nsb;
  prm.band_h = pl.band_h;
  prm.ns = pl.ns;
  prm.p2_smem = pl.p2_smem;
  prm.p2_cap_r = pl.p2_cap_r;
  prm.p2_cap_c = pl.p2_cap_c;
  for (size_t k = 0; k < pl.bounds.size(); ++k) prm.gbounds[k] = pl.bounds[k];
  prm.rowpart = (float*)(ws + pl.off_rowpart);
  prm.colpart = (float*)(ws + pl.off_colpart);
  prm.cta_sum = (float2*)(ws + pl.off_sum);
  prm.cta_obj = (float2*)(ws + pl.off_obj);
  prm.cta_res = (float2*)(ws + pl.off_res);
  prm.bar = (unsigned int*)(ws + pl.off_ctrl);
  prm.abort_flag = (int*)(ws + pl.off_ctrl + 64);
  prm.stats = (DeviceStats*)(ws + pl.off_stats);
  // DROT_TIMER_CTA: the CTA whose stage times the result record reports
  // (default 0; a profiling knob).
  prm.timer_cta = getenv("DROT_TIMER_CTA") ? atoi(getenv("DROT_TIMER_CTA")) : 0;
  if (prm.timer_cta < 0 || prm.timer_cta >= pl.grid) prm.timer_cta = 0;
  prm.timeout_ns = barrier_timeout_ns();
  prm.stall_cta = stall_cta_hook();

  if (cudaMemsetAsync(ws, 0, 512, A.stream) != cudaSuccess) return DROT_ERR_CUDA;
  if (repack) {
    const size_t esz = A.ctype == DROT_C_F32 ? sizeof(float) : 2;
    const size_t padr = (size_t)(ldp - A.nr);
    if ((padr && (cudaMemset2DAsync(cpad + A.nr * esz, ldp * esz, 0, padr * esz, A.nc,
                                    A.stream) != cudaSuccess ||
                  cudaMemset2DAsync(xpad + A.nr, ldp * sizeof(float), 0, padr * sizeof(float),
                                    A.nc, A.stream) != cudaSuccess)) ||
        cudaMemcpy2DAsync(cpad, ldp * esz, A.c, A.nr * esz, A.nr * esz, A.nc,
                          cudaMemcpyDeviceToDevice, A.stream) != cudaSuccess ||
        cudaMemcpy2DAsync(xpad, ldp * sizeof(float), A.x, A.nr * sizeof(float),
                          A.nr * sizeof(float), A.nc, cudaMemcpyDeviceToDevice,
                          A.stream) != cudaSuccess)
      return DROT_ERR_CUDA;
  }
  SolveFn fn = kernel_for(A.mode, pl.vec, pl.kv, pl.tma, pl.ctype);
  if (pl.smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)pl.smem) != cudaSuccess)
    return DROT_ERR_CUDA;
  void* args[] = {(void*)&prm};
  if (cudaLaunchCooperativeKernel((const void*)fn, dim3(pl.grid), dim3(pl.threads), args,
                                  pl.smem, A.stream) != cudaSuccess) {
    cudaGetLastError();
    return DROT_ERR_CUDA;
  }
  if (repack && cudaMemcpy2DAsync(A.x, A.nr * sizeof(float), xpad, ldp * sizeof(float),
                                  A.nr * sizeof(float), A.nc, cudaMemcpyDeviceToDevice,
                                  A.stream) != cudaSuccess)
    return DROT_ERR_CUDA;
  if (result) return read_stats(ws, result, A.stream);
  return DROT_OK;
}

static int init_state(int nr, int nc, float s, int warm, const float* p, const float* q,
                      float* x, float* a, float* b, float* phi1, float* phi2, float* alpha,
                      cudaStream_t st) {
  if (nr <= 0 || nc <= 0 || !x || !a || !b || !phi1 || !phi2 || !alpha)
    return DROT_ERR_INVALID_ARG;
  const int th = 256;
  auto blocks = [](long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); };
  if (warm) {
    // core/drot_qr.hpp:322-331: _k = 1*s*n*m - 2; phi1 = (_k+2)/n/(m+n); ...
    const float n = (float)nr, m = (float)nc;
    float k = 1.0f * s;
    k = k * n;
    k = k * m;
    k = k - 2.0f;
    float t = (k + 2.0f) / n;
    const float v_phi1 = t / (m + n);
    t = (k + 2.0f) / m;
    const float v_phi2 = t / (m + n);
    const float v_a = (k + 1.0f) / n;
    const float v_b = (k + 1.0f) / m;
    const float v_alpha = k + 1.0f;
    if (cudaMemsetAsync(x, 0, sizeof(float) * (size_t)nr * nc, st) != cudaSuccess)
      return DROT_ERR_CUDA;
    fill_kernel<<<blocks(nr), th, 0, st>>>(phi1, nr, v_phi1);
    fill_kernel<<<blocks(nc), th, 0, st>>>(phi2, nc, v_phi2);
    fill_kernel<<<blocks(nr), th, 0, st>>>(a, nr, v_a);
    fill_kernel<<<blocks(nc), th, 0, st>>>(b, nc, v_b);
    fill_kernel<<<1, 32, 0, st>>>(alpha, 1, v_alpha);
  } else {
    if (!p || !q) return DROT_ERR_INVALID_ARG;
    outer_kernel<<<blocks((long long)nr * nc), th, 0, st>>>(x, p, q, nr, nc);
    fill_kernel<<<blocks(nr), th, 0, st>>>(phi1, nr, 0.0f);
    fill_kernel<<<blocks(nc), th, 0, st>>>(phi2, nc, 0.0f);
    fill_kernel<<<blocks(nr), th, 0, st>>>(a, nr, 0.0f);
    fill_kernel<<<blocks(nc), th, 0, st>>>(b, nc, 0.0f);
    fill_kernel<<<1, 32, 0, st>>>(alpha, 1, 0.0f);
  }
  return cudaGetLastError() == cudaSuccess ? DROT_OK : DROT_ERR_CUDA;
}

// State region used by the operator-style entry points: a, b, phi1, phi2, alpha.
struct StateLayout {
  size_t off_a, off_b, off_phi1, off_phi2, off_alpha, total;
};

static StateLayout state_layout(size_t base, int nr, int nc) {
  StateLayout L;
  size_t off = align_up(base);
  L.off_a = off; off = align_up(off + sizeof(float) * nr);
  L.off_b = off; off = align_up(off + sizeof(float) * nc);
  L.off_phi1 = off; off = align_up(off + sizeof(float) * nr);
  L.off_phi2 = off; off = align_up(off + sizeof(float) * nc);
  L.off_alpha = off; off = align_up(off + sizeof(float));
  L.total = off;
  return L;
}

static thread_local int g_last_status = DROT_OK;

}  // namespace drot

using namespace drot;

// ---------------------------------------------------------------------------
// extern "C" entry points
// ---------------------------------------------------------------------------

extern "C" {

const char* drot_status_string(int status) {
  switch (status) {
    case DROT_OK: return "ok";
    case DROT_ERR_INVALID_ARG: return "invalid argument";
    case DROT_ERR_CUDA: return "CUDA runtime error";
    case DROT_ERR_BARRIER_TIMEOUT: return "device grid barrier timed out";
    case DROT_ERR_UNSUPPORTED: return "unsupported shape";
    case DROT_ERR_WORKSPACE: return "workspace too small or misaligned";
    default: return "unknown status";
  }
}

int drot_last_status(void) { return g_last_status; }

int drot_q_get_work_size_update_x(int n_rows, int n_cols) {
  // core/drot_qr.hpp:236-239
  const int l2 = (int)round(log2(std::max(n_rows, n_cols) * 0.002793 + 3.480));
  return (int)exp2((double)std::min(std::max(l2, 2), 6));
}

int drot_gl_get_work_size_update_x(int n_rows, int n_cols) {
  // core/drot_glr.hpp:357-360 (same heuristic)
  return drot_q_get_work_size_update_x(n_rows, n_cols);
}

int drot_gl_group_bounds(int n_rows, int n_groups, int* bounds) {
  if (n_rows <= 0 || n_groups <= 0 || !bounds) return DROT_ERR_INVALID_ARG;
  group_bounds(n_rows, n_groups, bounds);
  return DROT_OK;
}

int drot_set_launch_choice(int mode, int n_rows, int n_cols, int n_groups, int c_dtype,
                           const drot_launch_choice* choice) {
  if ((mode != MODE_QR && mode != MODE_GL) || n_rows < 0 || n_cols < 0 ||
      (n_rows == 0) != (n_cols == 0) || (mode == MODE_GL && n_rows > 0 && n_groups <= 0) ||
      (c_dtype != DROT_C_F32 && c_dtype != DROT_C_BF16))
    return DROT_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DROT_ERR_CUDA;
  const ChoiceKey key = {dev, mode, n_rows, n_cols, (mode == MODE_GL && n_rows > 0) ? n_groups : 0,
                         c_dtype};
  LaunchChoice ch;
  if (choice) {
    const drot_launch_choice& c = *choice;
    const bool kv_ok = c.vectors_per_lane == 0 || c.vectors_per_lane == 1 ||
                       c.vectors_per_lane == 2 || c.vectors_per_lane == 4 ||
                       (mode == MODE_GL && c.vectors_per_lane == 8);
    if (!kv_ok || (c.warps_per_cta != 0 && (c.warps_per_cta < 4 || c.warps_per_cta > 16)) ||
        (c.data_path != 0 && c.data_path != 1) || c.ctas_per_sm < 0 || c.ctas_per_sm > 2)
      return DROT_ERR_INVALID_ARG;
    ch.kv = c.vectors_per_lane;
    ch.warps = c.warps_per_cta;
    ch.tma = c.data_path;
    ch.ctas = c.ctas_per_sm;
    if (n_rows > 0) {
      // the pinned shape must plan (on the path it names, when it can run there)
      Plan pl;
      int rc = make_plan(mode, n_rows, n_cols, n_groups, 4, ch.tma != 0, pl, c_dtype, nullptr,
                         ch);
      if (rc != DROT_OK && ch.tma) rc = make_plan(mode, n_rows, n_cols, n_groups, 4, false, pl,
                                                  c_dtype, nullptr, ch);
      if (rc != DROT_OK) return rc;
    }
  }
  std::lock_guard<std::mutex> lk(g_choice_mu);
  for (size_t k = 0; k < g_choices.size(); ++k)
    if (g_choices[k].first == key) {
      g_choices.erase(g_choices.begin() + k);
      break;
    }
  if (choice) g_choices.emplace_back(key, ch);
  return DROT_OK;
}

int drot_clear_launch_choices(void) {
  std::lock_guard<std::mutex> lk(g_choice_mu);
  g_choices.clear();
  return DROT_OK;
}

int drot_init_state(int n_rows, int n_cols, float step_size, int warm, const float* p,
                    const float* q, float* x, float* a, float* b, float* phi1, float* phi2,
                    float* alpha, drot_stream_t stream) {
  return init_state(n_rows, n_cols, step_size, warm, p, q, x, a, b, phi1, phi2, alpha,
                    (cudaStream_t)stream);
}

size_t drot_qr_workspace_bytes(int n_rows, int n_cols) {
  return solve_ws_bytes(MODE_QR, n_rows, n_cols, 0);
}

size_t drot_gl_workspace_bytes(int n_rows, int n_cols, int n_groups) {
  return solve_ws_bytes(MODE_GL, n_rows, n_cols, n_groups);
}

int drot_qr_solve_ex(const void* c, int c_dtype, const float* p, const float* q, int n_rows,
                     int n_cols, float step_size, float scale, int max_iters, float eps,
                     float* x, float* a, float* b, float* phi1, float* phi2, float* alpha,
                     void* workspace, size_t workspace_bytes, drot_result* result,
                     drot_stream_t stream) {
  SolveArgs A = {MODE_QR, c, c_dtype, p, q, n_rows, n_cols, 0, step_size, scale, 0.0f,
                 max_iters, eps, x, a, b, phi1, phi2, alpha, workspace, workspace_bytes,
                 (cudaStream_t)stream};
  if (!(scale > 0.0f)) return DROT_ERR_INVALID_ARG;
  return run_solve(A, result);
}

int drot_qr_solve(const float* c, const float* p, const float* q, int n_rows, int n_cols,
                  float step_size, float scale, int max_iters, float eps, float* x, float* a,
                  float* b, float* phi1, float* phi2, float* alpha, void* workspace,
                  size_t workspace_bytes, drot_result* result, drot_stream_t stream) {
  return drot_qr_solve_ex(c, DROT_C_F32, p, q, n_rows, n_cols, step_size, scale, max_iters, eps,
                          x, a, b, phi1, phi2, alpha, workspace, workspace_bytes, result, stream);
}

int drot_gl_solve_ex(const void* c, int c_dtype, const float* p, const float* q, int n_rows,
                     int n_cols, int n_groups, float step_size, float lambda, int max_iters,
                     float eps, float* x, float* a, float* b, float* phi1, float* phi2,
                     float* alpha, void* workspace, size_t workspace_bytes, drot_result* result,
                     drot_stream_t stream) {
  if (n_groups <= 0) return DROT_ERR_INVALID_ARG;
  SolveArgs A = {MODE_GL, c, c_dtype, p, q, n_rows, n_cols, n_groups, step_size, 1.0f, lambda,
                 max_iters, eps, x, a, b, phi1, phi2, alpha, workspace, workspace_bytes,
                 (cudaStream_t)stream};
  return run_solve(A, result);
}

int drot_gl_solve(const float* c, const float* p, const float* q, int n_rows, int n_cols,
                  int n_groups, float step_size, float lambda, int max_iters, float eps,
                  float* x, float* a, float* b, float* phi1, float* phi2, float* alpha,
                  void* workspace, size_t workspace_bytes, drot_result* result,
                  drot_stream_t stream) {
  return drot_gl_solve_ex(c, DROT_C_F32, p, q, n_rows, n_cols, n_groups, step_size, lambda,
                          max_iters, eps, x, a, b, phi1, phi2, alpha, workspace, workspace_bytes,
                          result, stream);
}

static bool valid_bounds(int nr, int G, const int* b) {
  if (!b || G <= 0 || G > kMaxGroups || b[0] != 0 || b[G] != nr) return false;
  for (int g = 0; g < G; ++g)
    if (b[g + 1] <= b[g]) return false;
  return true;
}

size_t drot_np_workspace_bytes(int mode, int n_rows, int n_cols, int n_groups,
                               const int* bounds) {
  if (n_rows <= 0 || n_cols <= 0) return 0;
  if (mode == MODE_QR) return solve_ws_bytes(MODE_QR, n_rows, n_cols, 0);
  if (mode != MODE_GL || !valid_bounds(n_rows, n_groups, bounds)) return 0;
  return solve_ws_bytes(MODE_GL, n_rows, n_cols, n_groups, bounds);
}

int drot_np_solve(int mode, const void* c, int c_dtype, const float* p, const float* q,
                  int n_rows, int n_cols, int n_groups, const int* bounds, float step_size,
                  float scale_or_lambda, int max_iters, float eps, float* x, float* a, float* b,
                  float* phi1, float* phi2, float* alpha, void* workspace,
                  size_t workspace_bytes, drot_result* result, drot_stream_t stream) {
  if (mode == MODE_QR) {
    SolveArgs A = {MODE_QR, c, c_dtype, p, q, n_rows, n_cols, 0, step_size, scale_or_lambda,
                   0.0f, max_iters, eps, x, a, b, phi1, phi2, alpha, workspace,
                   workspace_bytes, (cudaStream_t)stream};
    A.stop_every = 1;
    A.stop_le = 1;
    return run_solve(A, result);
  }
  if (mode != MODE_GL || !valid_bounds(n_rows, n_groups, bounds)) return DROT_ERR_INVALID_ARG;
  SolveArgs A = {MODE_GL, c, c_dtype, p, q, n_rows, n_cols, n_groups, step_size, 1.0f,
                 scale_or_lambda, max_iters, eps, x, a, b, phi1, phi2, alpha, workspace,
                 workspace_bytes, (cudaStream_t)stream};
  A.bounds = bounds;
  return run_solve(A, result);
}

int drot_read_result(const void* workspace, drot_result* result, drot_stream_t stream) {
  if (!workspace || !result) return DROT_ERR_INVALID_ARG;
  return read_stats(workspace, result, (cudaStream_t)stream);
}

// Operator-style workspace: the dual state, then the solve's workspace.
size_t drot_quadratic_drot_workspace_bytes(int n_rows, int n_cols) {
  const size_t sw = solve_ws_bytes(MODE_QR, n_rows, n_cols, 0);
  if (sw == 0) return 0;
  return state_layout(0, n_rows, n_cols).total + sw;
}

size_t drot_group_lasso_drot_workspace_bytes(int n_rows, int n_cols, int n_class) {
  const size_t sw = solve_ws_bytes(MODE_GL, n_rows, n_cols, n_class);
  if (sw == 0) return 0;
  return state_layout(0, n_rows, n_cols).total + sw;
}

int drot_quadratic_drot_ex(const void* c, int c_dtype, const float* p, const float* q,
                           int n_rows, int n_cols, float rho, float r_weight, int max_iters,
                           float eps, float* x, void* workspace, size_t workspace_bytes,
                           drot_result* result, drot_stream_t stream) {
  if (n_rows <= 0 || n_cols <= 0 || !workspace) return DROT_ERR_INVALID_ARG;
  const size_t sc = scratch_bytes(MODE_QR, n_rows, n_cols, 0);
  if (sc == 0) return DROT_ERR_UNSUPPORTED;
  const StateLayout L = state_layout(0, n_rows, n_cols);
  if (workspace_bytes < L.total + sc) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  // pytorch/src/qr_drot_cuda_kernel.cu:100-102
  const float s = rho / ((float)n_rows + (float)n_cols);
  float t = s * r_weight;
  t = t * (float)(n_rows + n_cols);
  const float kappa = 1.0f + t;
  float *a = (float*)(ws + L.off_a), *b = (float*)(ws + L.off_b);
  float *phi1 = (float*)(ws + L.off_phi1), *phi2 = (float*)(ws + L.off_phi2);
  float* alpha = (float*)(ws + L.off_alpha);
  int rc = init_state(n_rows, n_cols, s, 1, p, q, x, a, b, phi1, phi2, alpha,
                      (cudaStream_t)stream);
  if (rc != DROT_OK) return rc;
  return drot_qr_solve_ex(c, c_dtype, p, q, n_rows, n_cols, s, kappa, max_iters, eps, x, a, b,
                          phi1, phi2, alpha, ws + L.total, workspace_bytes - L.total, result,
                          stream);
}

int drot_quadratic_drot(const float* c, const float* p, const float* q, int n_rows, int n_cols,
                        float rho, float r_weight, int max_iters, float eps, float* x,
                        void* workspace, size_t workspace_bytes, drot_result* result,
                        drot_stream_t stream) {
  return drot_quadratic_drot_ex(c, DROT_C_F32, p, q, n_rows, n_cols, rho, r_weight, max_iters,
                                eps, x, workspace, workspace_bytes, result, stream);
}

int drot_group_lasso_drot_ex(const void* c, int c_dtype, const float* p, const float* q,
                             int n_rows, int n_cols, int n_class, float rho, float r_weight,
                             int max_iters, float eps, float* x, void* workspace,
                             size_t workspace_bytes, drot_result* result, drot_stream_t stream) {
  if (n_rows <= 0 || n_cols <= 0 || n_class <= 0 || !workspace) return DROT_ERR_INVALID_ARG;
  const size_t sc = scratch_bytes(MODE_GL, n_rows, n_cols, n_class);
  if (sc == 0) return DROT_ERR_UNSUPPORTED;
  const StateLayout L = state_layout(0, n_rows, n_cols);
  if (workspace_bytes < L.total + sc) return DROT_ERR_WORKSPACE;
  char* ws = (char*)workspace;
  // pytorch/src/glr_drot_cuda_kernel.cu:255-257
  const float s = rho / ((float)n_rows + (float)n_cols);
  const float lambda = (float)((double)r_weight * sqrt((double)(n_rows / n_class)));
  float *a = (float*)(ws + L.off_a), *b = (float*)(ws + L.off_b);
  float *phi1 = (float*)(ws + L.off_phi1), *phi2 = (float*)(ws + L.off_phi2);
  float* alpha = (float*)(ws + L.off_alpha);
  int rc = init_state(n_rows, n_cols, s, 1, p, q, x, a, b, phi1, phi2, alpha,
                      (cudaStream_t)stream);
  if (rc != DROT_OK) return rc;
  return drot_gl_solve_ex(c, c_dtype, p, q, n_rows, n_cols, n_class, s, lambda, max_iters, eps,
                          x, a, b, phi1, phi2, alpha, ws + L.total, workspace_bytes - L.total,
                          result, stream);
}

int drot_group_lasso_drot(const float* c, const float* p, const float* q, int n_rows,
                          int n_cols, int n_class, float rho, float r_weight, int max_iters,
                          float eps, float* x, void* workspace, size_t workspace_bytes,
                          drot_result* result, drot_stream_t stream) {
  return drot_group_lasso_drot_ex(c, DROT_C_F32, p, q, n_rows, n_cols, n_class, rho, r_weight,
                                  max_iters, eps, x, workspace, workspace_bytes, result, stream);
}

// Host-buffer wrappers ------------------------------------------------------

static float* wrapper_impl(int mode, const float* hc, const float* hp, const float* hq,
                           int nr, int nc, int G, float s, float r_weight, int max_iters,
                           float eps, float* dur_ms, float* prep_ms, int* n_iter,
                           float* objective, int warm, int return_x) {
  g_last_status = DROT_OK;
  if (!hc || !hp || !hq || nr <= 0 || nc <= 0 || (mode == MODE_GL && G <= 0)) {
    g_last_status = DROT_ERR_INVALID_ARG;
    return nullptr;
  }
  const size_t mat = sizeof(float) * (size_t)nr * nc;
  const size_t sw = mode == MODE_QR ? solve_ws_bytes(MODE_QR, nr, nc, 0)
                                    : solve_ws_bytes(MODE_GL, nr, nc, G);
  if (sw == 0) {
    g_last_status = DROT_ERR_UNSUPPORTED;
    return nullptr;
  }
  const StateLayout L = state_layout(0, nr, nc);  // the state, then the solve's workspace
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventRecord(e0, 0);
  cudaEventSynchronize(e0);
  float *c = nullptr, *p = nullptr, *q = nullptr, *x = nullptr;
  char* ws = nullptr;
  int rc = DROT_OK;
  float* out = nullptr;
  drot_result res;
  memset(&res, 0, sizeof(res));
  if (cudaMalloc(&c, mat) != cudaSuccess || cudaMalloc(&x, mat) != cudaSuccess ||
      cudaMalloc(&p, sizeof(float) * nr) != cudaSuccess ||
      cudaMalloc(&q, sizeof(float) * nc) != cudaSuccess ||
      cudaMalloc(&ws, L.total + sw) != cudaSuccess) {
    rc = DROT_ERR_CUDA;
  }
  if (rc == DROT_OK &&
      (cudaMemcpy(c, hc, mat, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(p, hp, sizeof(float) * nr, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(q, hq, sizeof(float) * nc, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = DROT_ERR_CUDA;
  float *a = (float*)(ws + L.off_a), *b = (float*)(ws + L.off_b);
  float *phi1 = (float*)(ws + L.off_phi1), *phi2 = (float*)(ws + L.off_phi2);
  float* alpha = (float*)(ws + L.off_alpha);
  if (rc == DROT_OK) rc = init_state(nr, nc, s, warm, p, q, x, a, b, phi1, phi2, alpha, 0);
  cudaEventRecord(e1, 0);
  cudaEventSynchronize(e1);
  if (rc == DROT_OK) {
    if (mode == MODE_QR) {
      // core/drot_qr.hpp:262: scale = 1 + step_size * T(n_rows + n_cols) * r_weight
      float t = s * (float)(nr + nc);
      t = t * r_weight;
      const float kappa = 1.0f + t;
      rc = drot_qr_solve(c, p, q, nr, nc, s, kappa, max_iters, eps, x, a, b, phi1, phi2, alpha,
                         ws + L.total, sw, &res, 0);
    } else {
      // core/drot_glr.hpp:385: lambda = r_weight / sqrt(n_rows / NGROUPS)
      const float lambda = (float)((double)r_weight / sqrt((double)(nr / G)));
      rc = drot_gl_solve(c, p, q, nr, nc, G, s, lambda, max_iters, eps, x, a, b, phi1, phi2,
                         alpha, ws + L.total, sw, &res, 0);
    }
  }
  cudaEventRecord(e2, 0);
  cudaEventSynchronize(e2);
  if (dur_ms) cudaEventElapsedTime(dur_ms, e1, e2);
  if (prep_ms) cudaEventElapsedTime(prep_ms, e0, e1);
  if (rc == DROT_OK) {
    if (n_iter) *n_iter = res.n_iter;
    if (objective && res.objective_valid) *objective = res.objective;
    if (return_x) {
      out = (float*)malloc(mat);
      if (!out || cudaMemcpy(out, x, mat, cudaMemcpyDeviceToHost) != cudaSuccess) {
        free(out);
        out = nullptr;
        rc = DROT_ERR_CUDA;
      }
    }
  }
  cudaFree(c);
  cudaFree(x);
  cudaFree(p);
  cudaFree(q);
  cudaFree(ws);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  g_last_status = rc;
  return out;
}

float* drot_qr_wrapper(const float* c, const float* p, const float* q, int n_rows, int n_cols,
                       float step_size, float r_weight, int max_iters, float eps,
                       float* dur_in_ms, float* prep_dur_in_ms, int* n_iter, float* objective,
                       int use_warmup_init, int return_x) {
  return wrapper_impl(MODE_QR, c, p, q, n_rows, n_cols, 0, step_size, r_weight, max_iters, eps,
                      dur_in_ms, prep_dur_in_ms, n_iter, objective, use_warmup_init, return_x);
}

float* drot_gl_wrapper(const float* c, const float* p, const float* q, int n_rows, int n_cols,
                       int n_groups, float step_size, float r_weight, int max_iters, float eps,
                       float* dur_in_ms, float* prep_dur_in_ms, int* n_iter, float* objective,
                       int use_warmup_init, int return_x) {
  return wrapper_impl(MODE_GL, c, p, q, n_rows, n_cols, n_groups, step_size, r_weight,
                      max_iters, eps, dur_in_ms, prep_dur_in_ms, n_iter, objective,
                      use_warmup_init, return_x);
}

void drot_free_host(float* ptr) { free(ptr); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Solve without any device allocation
// ---------------------------------------------------------------------------
//
// Some callers cannot allocate device memory when they call the solver: a
// latency-critical loop in which cudaMalloc / cudaFree would synchronise the
// whole device, or a host (a plugin, a caller in another language) whose
// device memory is owned by a different allocator that it may not bypass.
// For them drot_quadratic_drot_noalloc keeps the solver's workspace (partial
// sums, barrier words, result record and the dual state) in a fixed array in
// the library's own device memory.  Every GPU that loads the library holds
// this array until the process exits.

namespace drot {

// Workspace of the allocation-free entry point, one per device.
static __device__ __align__(256) unsigned char g_noalloc_ws[DROT_NOALLOC_WORKSPACE_BYTES];

// The array's name in host code is only a host-side handle; the kernels need
// its device address, which the runtime gives per device.  Looked up on every
// call, with the call's device current: the lookup is a host-side table read
// once the library's device code is loaded, and no address is kept that a
// cudaDeviceReset (a new context, possibly a new address) could leave stale.
static int noalloc_workspace(void** out) {
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_ws) != cudaSuccess || !ptr) {
    cudaGetLastError();
    return DROT_ERR_CUDA;
  }
  *out = ptr;
  return DROT_OK;
}

}  // namespace drot

extern "C" int drot_quadratic_drot_noalloc(const float* c, const float* p, const float* q,
                                           int n_rows, int n_cols, float rho, float r_weight,
                                           int max_iters, float eps, float* x,
                                           drot_result* result, drot_stream_t stream) {
  if (!c || !p || !q || !x || n_rows <= 0 || n_cols <= 0 || max_iters < 0)
    return DROT_ERR_INVALID_ARG;
  // Size check first: nothing is launched for a problem that does not fit.
  // The minimum (without the aligned copies of unaligned columns, which the
  // solve takes when the rest of the array holds them).
  const size_t sc = scratch_bytes(MODE_QR, n_rows, n_cols, 0);
  if (sc == 0) return DROT_ERR_UNSUPPORTED;
  const size_t need = state_layout(0, n_rows, n_cols).total + sc;
  if (need > (size_t)DROT_NOALLOC_WORKSPACE_BYTES) return DROT_ERR_WORKSPACE;
  void* ws = nullptr;
  const int rc = noalloc_workspace(&ws);
  if (rc != DROT_OK) return rc;
  // drot_quadratic_drot clears the barrier words, writes the warm start into
  // the dual state and every partial before it is read, so nothing left in
  // the array by an earlier call is used.
  return drot_quadratic_drot(c, p, q, n_rows, n_cols, rho, r_weight, max_iters, eps, x, ws,
                             (size_t)DROT_NOALLOC_WORKSPACE_BYTES, result, stream);
}
