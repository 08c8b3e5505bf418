#!/usr/bin/env python
"""Benchmark of the GB300 DROT solver.

Headline workload (one step = one full solve):
  quadratic-regularised DROT, m = n = 3000, C ~ U[0,1) float32, p, q ~
  Dirichlet(1), r_weight (alpha) = 1e-3, rho = 2, warm start, stop at a
  relative marginal residual ||(X1-p, X^T1-q)||_2 / ||(p;q)||_2 < 1e-4.
  Metric: solves/s (whole job).

  value  solves with C, p, q resident in HBM, through reg_drot.solve_qr (the
         drop-in operator's C-ABI entry point); L2 flushed between solves.
  e2e    the same solve through the host-buffer C-ABI wrapper
         (drot_qr_wrapper, the reference's quadratic_regularizer_drot_wrapper):
         device allocation, H2D of C/p/q, solve, D2H of X per step.
  roofline  the solve kernel: algorithmic bytes (12 B/element on iterations
         that read C, 8 B on the others, 12 B for the final unfold) over its
         measured time, against the measured HBM copy bandwidth.
  cpu_baseline  the oracle (C restatement of the reference loop, OpenMP on all
         host cores) timed on a bounded number of iterations of the same
         solve and scaled to the iterations a solve takes.

`--impl reference` times that CPU implementation alone (the reference's
solver is CUDA and its CPU implementation is numpy; neither runs on the GPU
host, so the oracle port stands in for it).

Multi-GPU: the solve does not shard; N ranks run N independent replicas.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "regularized-drot_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N = 3000
ALPHA = 1e-3
RHO = 2.0
REL_EPS = 1e-4
SEED = 1234
# DR iterations one solve of this workload takes (measured on the GPU solver;
# the CPU restatement runs the same iteration map).  Used to scale the
# bounded CPU samples to a full solve.
ITERS_PER_SOLVE = 113831
WORKLOAD = (f"QR-DROT {N}x{N}, C~U[0,1) fp32, p,q~Dirichlet(1), alpha={ALPHA}, rho={RHO}, "
            f"warm start, stop at relative marginal residual {REL_EPS}")
METRIC = f"solves/s at relative marginal error {REL_EPS} (QR-DROT {N}x{N}, alpha={ALPHA})"
L2_FLUSH_BYTES = 512 << 20


def make_problem(n, seed=SEED):
    rng = np.random.default_rng(seed)
    c = rng.random((n, n), dtype=np.float32)
    p = rng.dirichlet(np.ones(n)).astype(np.float32)
    q = rng.dirichlet(np.ones(n)).astype(np.float32)
    eps = REL_EPS * math.sqrt(float((p.astype(np.float64) ** 2).sum() +
                                    (q.astype(np.float64) ** 2).sum()))
    return c, p, q, eps


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic_per_iteration():
    """DRAM bytes per DR iteration of the solve kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "drot_solve_qr_3000.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_iteration:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


# --------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------- CPU legs

def cpu_sample(budget_s=12.0, threads=None):
    """Time the oracle on a bounded number of iterations of the workload."""
    from oracle import oracle as O
    c, p, q, eps = make_problem(N)  # c is [n_cols, n_rows], the operator's layout
    s = O.step_size(RHO, N, N)
    kappa = O.qr_scale(s, ALPHA, N, N, "torch")
    threads = threads or O.lib().oracle_max_threads()
    O.qr_solve(c, p, q, s, kappa, 2, eps, threads=threads)  # page in, spin up threads
    iters, spent = 0, 0.0
    chunk = 10
    while spent < budget_s:
        t0 = time.perf_counter()
        O.qr_solve(c, p, q, s, kappa, chunk, eps, threads=threads)
        spent += time.perf_counter() - t0
        iters += chunk
        chunk = min(chunk * 2, 400)
    per_iter = spent / iters
    value = 1.0 / (per_iter * ITERS_PER_SOLVE)
    return {"value": value, "unit": "solves/s", "cores": int(threads), "kind": "port",
            "sample": (f"{iters} DR iterations of the {N}x{N} QR solve from the warm start "
                       f"(FP32 oracle, {threads} OpenMP threads, {spent:.1f} s), scaled to the "
                       f"{ITERS_PER_SOLVE} iterations of a full solve"),
            "s_per_iteration": per_iter}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    for _ in range(args.warmup):
        cpu_sample(budget_s=0.5)
    vals = [cpu_sample(budget_s=10.0) for _ in range(args.steps)]
    value = statistics.median(v["value"] for v in vals)
    base = dict(vals[0])
    base["value"] = value
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_rows": N, "n_cols": N, "alpha": ALPHA, "rho": RHO,
                   "rel_eps": REL_EPS, "seed": SEED},
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU legs

def e2e_wrapper(c, p, q, eps, steps):
    """Solves through drot_qr_wrapper with pinned host buffers (host in, host out)."""
    import torch
    from reg_drot import _lib
    L = _lib.lib()
    ct = torch.from_numpy(c).pin_memory()  # column-major n_rows x n_cols
    pt = torch.from_numpy(p).pin_memory()
    qt = torch.from_numpy(q).pin_memory()
    s = float(np.float32(RHO) / (np.float32(N) + np.float32(N)))
    dur, prep = ctypes.c_float(), ctypes.c_float()
    nit, obj = ctypes.c_int(), ctypes.c_float()

    def once():
        ptr = L.drot_qr_wrapper(ct.data_ptr(), pt.data_ptr(), qt.data_ptr(), N, N, s, ALPHA,
                                10 ** 9, eps, ctypes.byref(dur), ctypes.byref(prep),
                                ctypes.byref(nit), ctypes.byref(obj), 1, 1)
        if not ptr:
            raise RuntimeError(f"drot_qr_wrapper failed: {_lib.status_string(L.drot_last_status())}")
        L.drot_free_host(ptr)

    once()
    t0 = time.perf_counter()
    for _ in range(steps):
        once()
    wall = time.perf_counter() - t0
    return {"value": steps / wall, "unit": "solves/s",
            "h2d_bytes_per_step": (N * N + 2 * N) * 4, "d2h_bytes_per_step": N * N * 4,
            "n_iter": nit.value, "wall_s_per_step": wall / steps}


def hbm_point(dev, flush):
    """QR at 10000^2 (X + C = 800 MB, beyond L2) for a fixed iteration count."""
    import torch
    import reg_drot
    n, iters = 10000, 400
    c, p, q, _ = make_problem(n)
    cd = torch.from_numpy(c).to(dev)
    pd = torch.from_numpy(p).to(dev)
    qd = torch.from_numpy(q).to(dev)
    x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10, 0.0)
    times = []
    for _ in range(3):
        flush.zero_()
        torch.cuda._sleep(20_000_000)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, iters, 0.0, out=x, workspace=ws)
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b) / 1e3)
    t = min(times)
    it = info["iters_run"]
    nbytes = float(n) * n * (12 * ((it + 1) // 2) + 8 * (it // 2))
    ph = [v / it for v in info["phase_ms"]]
    del cd, x, ws
    return {"workload": f"QR-DROT {n}x{n}, {iters} iterations (X + C = 800 MB, HBM resident)",
            "us_per_iteration": t / it * 1e6, "achieved_GBps": nbytes / t / 1e9,
            "phase_us_per_iteration_cta0": [round(v * 1e3, 2) for v in ph]}


def config_points(dev, flush):
    """The other single-instance configurations: QR 1000^2 on N(0, I_2) clouds
    (the reference's CPU-runnable case; GPU solve and the oracle solve on the
    host cores), and the 3000^2 workload at alpha 1e-2 and 1e-4 and with the
    cost stored in BF16 (alpha 1e-3)."""
    import torch
    import reg_drot
    from oracle import oracle as O
    out = {}

    def timed(fn):
        fn()
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        r = fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / 1e3, r

    rng = np.random.default_rng(SEED)
    xs = rng.normal(size=(1000, 2))
    yt = rng.normal(size=(1000, 2))
    C = ((yt[:, None, :] - xs[None, :, :]) ** 2).sum(-1)
    C = (C / C.max()).astype(np.float32)
    p1 = np.full(1000, 1e-3, np.float32)
    eps1 = REL_EPS * math.sqrt(2 * 1000 * 1e-6)
    c1, pp1 = torch.from_numpy(C).to(dev), torch.from_numpy(p1).to(dev)
    t, (x, info, _) = timed(lambda: reg_drot.solve_qr(c1, pp1, pp1, RHO, ALPHA, 10 ** 6, eps1))
    t0 = time.perf_counter()
    o = O.quadratic_drot(C, p1, p1, RHO, ALPHA, 10 ** 6, eps1)
    t_cpu = time.perf_counter() - t0
    out["config1_qr_1000_clouds"] = {
        "workload": "QR-DROT 1000x1000, C = sq. Euclidean of N(0,I_2) clouds / max, uniform "
                    f"marginals, alpha={ALPHA}, relative eps {REL_EPS}",
        "gpu_s_per_solve": t, "n_iter": info["n_iter"], "cpu_oracle_s_per_solve": t_cpu,
        "cpu_oracle_n_iter": o["n_iter"], "cpu_threads": int(O.lib().oracle_max_threads())}
    c, p, q, eps = make_problem(N, SEED)
    cd, pd, qd = (torch.from_numpy(a).to(dev) for a in (c, p, q))
    for alpha in (1e-2, 1e-4):
        t, (x, info, _) = timed(lambda: reg_drot.solve_qr(cd, pd, qd, RHO, alpha, 10 ** 7, eps))
        out[f"config2_qr_3000_alpha_{alpha:g}"] = {
            "s_per_solve": t, "n_iter": info["n_iter"], "converged": info["converged"],
            "objective": info["objective_f64"], "residual": info["residual"]}
    cb = cd.to(torch.bfloat16)
    t, (x, info, _) = timed(lambda: reg_drot.solve_qr(cb, pd, qd, RHO, ALPHA, 10 ** 7, eps))
    out["config2_qr_3000_bf16_cost"] = {
        "s_per_solve": t, "n_iter": info["n_iter"], "converged": info["converged"],
        "objective": info["objective_f64"], "residual": info["residual"],
        "note": "the solve of the BF16-rounded cost (FP32 iterates)"}
    return out


def gl_da_point(dev, gl_weight=1e-3):
    """Group-lasso domain-adaptation solve (1500 source x 1000 target, 2 classes)."""
    import reg_drot  # noqa: F401
    from reg_drot import _lib
    L = _lib.lib()
    times, iters = [], []
    for seed in range(5):
        rng = np.random.default_rng(1234 + seed)
        ns, nt = 1500, 1000
        ys = np.repeat([0, 1], ns // 2)
        xs = rng.normal(size=(ns, 2)) + np.where(ys[:, None] == 0, -2.0, 2.0) * np.array([1.0, 0.0])
        A = np.eye(2) + 0.3 * rng.normal(size=(2, 2))
        b = rng.normal(size=2)
        yt = np.repeat([0, 1], nt // 2)
        xt0 = rng.normal(size=(nt, 2)) + np.where(yt[:, None] == 0, -2.0, 2.0) * np.array([1.0, 0.0])
        xt = xt0 @ A.T + b
        C = ((xs[:, None, :] - xt[None, :, :]) ** 2).sum(-1)
        C = (C / C.max()).astype(np.float32)          # [n_rows=source, n_cols=target]
        cm = np.ascontiguousarray(C.T)                # column-major n_rows x n_cols
        p = np.full(ns, 1.0 / ns, np.float32)
        q = np.full(nt, 1.0 / nt, np.float32)
        s = float(np.float32(RHO) / (np.float32(ns) + np.float32(nt)))
        dur, prep = ctypes.c_float(), ctypes.c_float()
        nit, obj = ctypes.c_int(), ctypes.c_float()
        for rep in range(2):
            ptr = L.drot_gl_wrapper(cm.ctypes.data, p.ctypes.data, q.ctypes.data, ns, nt, 2, s,
                                    gl_weight, 20000, 1e-4, ctypes.byref(dur), ctypes.byref(prep),
                                    ctypes.byref(nit), ctypes.byref(obj), 1, 0)
        times.append(dur.value / 1e3)
        iters.append(nit.value)
    return {"workload": f"GL-DROT domain adaptation 1500 src x 1000 tgt, 2 classes, GL weight {gl_weight:g} "
                        "(C++ wrapper convention), eps 1e-4, rho 2, 20000 max iterations",
            "median_solve_s": statistics.median(times), "median_iterations": statistics.median(iters),
            "published_v100_median_s": 0.0619 if gl_weight == 1e-3 else None}


BATCH_INSTANCES = 256
BATCH_MIN, BATCH_MAX = 64, 2048


def make_batch_problem(dev, n_inst=BATCH_INSTANCES, seed=SEED):
    """Batched workload: n_inst instances, m, n ~ U{64..2048} independent,
    C = squared Euclidean distances of N(0, I_8) point clouds (max-normalised
    per instance), uniform marginals; eps_k = REL_EPS * ||(p_k; q_k)||_2."""
    import torch
    rng = np.random.default_rng(seed)
    shapes = [(int(a), int(b)) for a, b in rng.integers(BATCH_MIN, BATCH_MAX + 1, size=(n_inst, 2))]
    g = torch.Generator(device=dev).manual_seed(seed)
    costs, ps, qs, eps = [], [], [], []
    for (m, n) in shapes:
        xs = torch.randn(m, 8, generator=g, device=dev)
        yt = torch.randn(n, 8, generator=g, device=dev)
        c = (yt * yt).sum(1, keepdim=True) + (xs * xs).sum(1)[None, :] - 2.0 * (yt @ xs.T)
        c = c.clamp_min_(0.0)
        costs.append(c / c.max())                      # [n_cols = n, n_rows = m]
        ps.append(torch.full((m,), 1.0 / m))
        qs.append(torch.full((n,), 1.0 / n))
        eps.append(REL_EPS * math.sqrt(1.0 / m + 1.0 / n))
    return shapes, costs, ps, qs, eps


def batched_point(dev, flush, single_sample=16):
    """The batched solver on the 256-instance workload (FP32 and BF16-stored
    C), one CUDA-graph replay per solve of the whole batch, against solving
    the same instances one at a time with reg_drot.solve_qr."""
    import torch
    import reg_drot
    from reg_drot.batch import QRBatch
    shapes, costs, ps, qs, eps = make_batch_problem(dev)
    elems = np.array([m * n for m, n in shapes], dtype=np.float64)
    out = {"workload": (f"batched QR-DROT, {len(shapes)} instances, m,n ~ U{{{BATCH_MIN}..{BATCH_MAX}}}, "
                        f"C = sq. Euclidean of N(0,I_8) clouds / max, uniform marginals, "
                        f"alpha={ALPHA}, rho={RHO}, relative eps {REL_EPS}"),
           "elements": int(elems.sum())}
    peak, _ = measured_peak()
    for name, dtype in (("fp32", torch.float32), ("bf16_c", torch.bfloat16)):
        B = QRBatch(shapes, RHO, ALPHA, eps, device=dev)
        c = B.pack_c(costs, dtype=dtype)
        p, q = B.pack_marginals(ps, qs)
        cpt = B.autotune(c, p, q, iters=200)
        x = B.empty_x()
        graph = B.capture(c, p, q, x, 10 ** 6)
        graph.replay()
        times = []
        for _ in range(3):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            graph.replay()
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b) / 1e3)
        info = B.results()
        it = np.array([r["n_iter"] for r in info], dtype=np.float64)
        cb = 2 if dtype == torch.bfloat16 else 4
        # even iterations read C (cb bytes) + X and write X, odd ones X only,
        # plus the unfold pass (C + X read, X write).
        nbytes = float((elems * ((8 + cb) * np.ceil(it / 2) + 8 * np.floor(it / 2) + 8 + cb)).sum())
        t = statistics.median(times)
        out[name] = {"solves_per_s": len(shapes) / t, "s_per_batch": t, "cols_per_tile": cpt,
                     "converged": int(sum(r["converged"] for r in info)),
                     "n_iter_min_median_max": [int(it.min()), float(np.median(it)), int(it.max())],
                     "achieved_GBps": nbytes / t / 1e9, "frac_of_measured_hbm": nbytes / t / 1e9 / peak}
        del B, c, x, graph
    # The same instances one solve at a time (a sample, every 16th instance).
    ks = list(range(0, len(shapes), max(1, len(shapes) // single_sample)))
    t_sum = 0.0
    for k in ks:
        cd, pd, qd = costs[k].contiguous(), ps[k].to(dev), qs[k].to(dev)
        xk, ik, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 6, eps[k])
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        xk, ik, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 6, eps[k], out=xk, workspace=ws)
        b.record()
        b.synchronize()
        t_sum += a.elapsed_time(b) / 1e3
    out["per_instance_solves_per_s"] = len(ks) / t_sum
    out["per_instance_sample"] = f"{len(ks)} instances (every {len(shapes) // len(ks)}th), one solve each"
    out["speedup_fp32_vs_per_instance"] = out["fp32"]["solves_per_s"] / out["per_instance_solves_per_s"]
    return out


DIFF_INSTANCES = 64
DIFF_MIN, DIFF_MAX = 512, 4096
DIFF_DIM = 16
DIFF_SCALE = 1.0 / (4 * DIFF_DIM)  # C = |x - y|^2 / 64: mean cost 0.5 for N(0, I_16) clouds


def differentiable_point(dev, n_inst=DIFF_INSTANCES, gl_inst=4, single_sample=8, gl_iters=500):
    """Differentiable OT loss: point clouds x_k (m x 16), y_k (n x 16) ~ N(0, 1),
    m, n ~ U{512..4096}; C_k = |x - y|^2 / 64 on the tensor cores; loss =
    sum_k <C_k, X_k*> + w ||X_k*||_F^2 (w fixed random); one step = cost +
    batched QR solve (relative eps 1e-4, alpha 1e-3) + backward (implicit
    adjoint + cost chain rule) for all instances.  GL part: the same loss with
    the group-lasso plan (2 classes, lambda weight 1e-3) and the checkpointed
    unrolled adjoint on the first `gl_inst` instances, `gl_iters` iterations
    each (the GL solve does not reach the relative 1e-4 stop on these clouds
    within 20000 iterations; the adjoint's cost is linear in the iterations)."""
    import torch
    import reg_drot
    from reg_drot.autograd import batch_quadratic_drot_fn, group_lasso_drot_fn
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost, sqeuclidean_cost
    rng = np.random.default_rng(SEED + 5)
    shapes = [(int(a), int(b)) for a, b in rng.integers(DIFF_MIN, DIFF_MAX + 1, size=(n_inst, 2))]
    g = torch.Generator(device=dev).manual_seed(SEED + 5)
    x_cat = torch.randn(sum(m for m, _ in shapes), DIFF_DIM, generator=g, device=dev,
                        requires_grad=True)
    y_cat = torch.randn(sum(n for _, n in shapes), DIFF_DIM, generator=g, device=dev,
                        requires_grad=True)
    w = float(torch.rand(1, generator=torch.Generator().manual_seed(SEED)).item())
    eps = [REL_EPS * math.sqrt(1.0 / m + 1.0 / n) for m, n in shapes]
    B = QRBatch(shapes, RHO, ALPHA, eps, device=dev)
    p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                            [torch.full((n,), 1.0 / n) for _, n in shapes])
    with torch.no_grad():
        B.autotune(packed_sqeuclidean_cost(B, x_cat, y_cat, DIFF_SCALE), p, q, iters=100)

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def step():
        x_cat.grad = None
        y_cat.grad = None
        e0 = ev()
        c = packed_sqeuclidean_cost(B, x_cat, y_cat, DIFF_SCALE)
        e1 = ev()
        X = batch_quadratic_drot_fn(B, c, p, q, 10 ** 6)
        e2 = ev()
        loss = (c * X).sum() + w * (X * X).sum()
        loss.backward()
        e3 = ev()
        e3.synchronize()
        return (e0.elapsed_time(e1) / 1e3, e1.elapsed_time(e2) / 1e3, e2.elapsed_time(e3) / 1e3,
                X.grad_fn, float(loss.detach()))

    step()  # warm-up
    t_cost, t_fwd, t_bwd, fn, loss = step()
    it = np.array([r["n_iter"] for r in fn.info])
    total = t_cost + t_fwd + t_bwd
    out = {"workload": (f"differentiable QR-DROT loss, {n_inst} instances, m,n ~ U{{{DIFF_MIN}..{DIFF_MAX}}}, "
                        f"x,y ~ N(0,I_{DIFF_DIM}), C = |x-y|^2/64 (tcgen05 split-TF32 GEMM), "
                        f"alpha={ALPHA}, relative eps {REL_EPS}, loss = sum <C,X*> + w|X*|^2"),
           "elements": int(sum(m * n for m, n in shapes)),
           "qr": {"s_per_step": total, "solves_with_grad_per_s": n_inst / total,
                  "cost_s": t_cost, "forward_s": t_fwd, "backward_s": t_bwd,
                  "converged": int(sum(r["converged"] for r in fn.info)),
                  "n_iter_min_median_max": [int(it.min()), float(np.median(it)), int(it.max())],
                  "cg_iters_min_median_max": [int(min(fn.cg_iters)), float(np.median(fn.cg_iters)),
                                              int(max(fn.cg_iters))],
                  "loss": loss}}
    # plain per-instance FP32 solves, forward only (sample)
    ks = list(range(0, n_inst, max(1, n_inst // single_sample)))
    t_single = 0.0
    with torch.no_grad():
        for k in ks:
            m, n = shapes[k]
            xo = sum(a for a, _ in shapes[:k])
            yo = sum(b for _, b in shapes[:k])
            ck = sqeuclidean_cost(x_cat[xo:xo + m].detach(), y_cat[yo:yo + n].detach(), DIFF_SCALE)
            pk, qk = torch.full((m,), 1.0 / m, device=dev), torch.full((n,), 1.0 / n, device=dev)
            xk, _, ws = reg_drot.solve_qr(ck, pk, qk, RHO, ALPHA, 10 ** 6, eps[k])
            e0 = ev()
            reg_drot.solve_qr(ck, pk, qk, RHO, ALPHA, 10 ** 6, eps[k], out=xk, workspace=ws)
            e1 = ev()
            e1.synchronize()
            t_single += e0.elapsed_time(e1) / 1e3
    out["per_instance_forward_only_solves_per_s"] = len(ks) / t_single
    out["per_instance_sample"] = f"{len(ks)} instances, reg_drot.solve_qr forward only"
    # GL with the unrolled adjoint, one instance at a time
    gl_times, gl_iters_run = [], []
    for k in range(gl_inst):
        m, n = shapes[k]
        xo = sum(a for a, _ in shapes[:k])
        yo = sum(b for _, b in shapes[:k])
        xk = x_cat[xo:xo + m].detach().clone().requires_grad_(True)
        yk = y_cat[yo:yo + n].detach().clone().requires_grad_(True)
        pk, qk = torch.full((m,), 1.0 / m, device=dev), torch.full((n,), 1.0 / n, device=dev)
        for rep in range(2):
            e0 = ev()
            ck = sqeuclidean_cost(xk, yk, DIFF_SCALE)
            Xk = group_lasso_drot_fn(ck, pk, qk, 2, RHO, ALPHA, gl_iters, eps[k])
            ((ck * Xk).sum() + w * (Xk * Xk).sum()).backward()
            e1 = ev()
            e1.synchronize()
        gl_times.append(e0.elapsed_time(e1) / 1e3)
        gl_iters_run.append(Xk.grad_fn.info["n_iter"])
    out["gl"] = {"instances": gl_inst, "s_per_instance_with_grad": statistics.mean(gl_times),
                 "iterations": gl_iters_run, "segment": 32,
                 "ms_per_iteration_with_grad": 1e3 * sum(gl_times) / sum(gl_iters_run)}
    return out


def max_over_ranks(values, dist, device):
    """Element-wise maximum of per-rank timings (the slowest replica sets the
    job's time); identity without a process group."""
    import torch
    if not dist:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def replica_throughput(world, steps, slowest_total_s):
    """Whole-job solves/s of `world` independent replicas, each doing `steps`
    solves, timed by the slowest replica (weak scaling: no collective on the
    solve path)."""
    return world * steps / slowest_total_s


def run_gpu(args):
    import torch
    import reg_drot

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    c, p, q, eps = make_problem(N, SEED)
    cd = torch.from_numpy(c).to(dev)
    pd = torch.from_numpy(p).to(dev)
    qd = torch.from_numpy(q).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 9, eps)
    for _ in range(max(args.warmup - 1, 0)):
        flush.zero_()
        x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 9, eps, out=x, workspace=ws)
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        # A short GPU-side wait ahead of the first timed step: the host
        # enqueues every step while it runs, so a host stall cannot leave the
        # GPU idle inside the timed events.
        torch.cuda._sleep(100_000_000)
        for i in range(args.steps):
            flush.zero_()
            starts[i].record()
            x, _, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 9, eps, out=x,
                                         workspace=ws, sync=False)
            ends[i].record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    info = reg_drot.read_result(ws)
    step_s = [a.elapsed_time(b) / 1e3 for a, b in zip(starts, ends)]
    total = sum(step_s)
    total, wall = max_over_ranks([total, wall], dist, dev)
    value = replica_throughput(world, args.steps, total)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    it = info["iters_run"]
    n_even = (it + 1) // 2
    kernel_bytes = float(N) * N * (12 * n_even + 8 * (it - n_even) + (12 if info["converged"] else 0))
    kernel_s = total / args.steps
    peak, peak_kind = measured_peak()
    achieved = kernel_bytes / kernel_s / 1e9
    traffic_it = profile_traffic_per_iteration()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic_it * it if traffic_it is not None else None,
                "algorithmic_bytes_per_launch": kernel_bytes,
                "note": ("X + C = 72 MB stays L2-resident across the iterations of a solve; "
                         "the 10000^2 point in extra.hbm_point is the HBM-resident case")}

    e2e = e2e_wrapper(c, p, q, eps, args.steps)
    extra = {"hbm_point": hbm_point(dev, flush), "gl_da": gl_da_point(dev),
             "gl_da_weight_5e-3": gl_da_point(dev, 5e-3), "configs": config_points(dev, flush),
             "batched": batched_point(dev, flush), "differentiable": differentiable_point(dev)}
    cpu = cpu_sample(budget_s=12.0) if world == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_rows": N, "n_cols": N, "alpha": ALPHA, "rho": RHO,
                   "rel_eps": REL_EPS, "eps_abs": eps, "seed": SEED,
                   "l2": "flushed (512 MB write) before every timed solve",
                   "parallelism": f"replicas x{world}"},
        "iterations_per_solve": it, "iterations_per_s": it / kernel_s,
        "converged": info["converged"], "residual": info["residual"],
        "phase_ms_per_solve_cta0": info["phase_ms"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")},
        "e2e_detail": {"n_iter": e2e["n_iter"], "wall_s_per_step": e2e["wall_s_per_step"]},
        "gpu_launches": 6 * args.steps,
        "clocks": clk.summary(),
        "wall_s_timed_region": wall,
        "extra": extra,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_diff_case(n_inst, iters):
    """Profiler case: the differentiable workload's first n_inst instances,
    one launch each of the cost kernel, the batched solve (iters iterations)
    and the adjoint CG (--case diff:n_inst:iters)."""
    import warnings
    import torch
    from reg_drot.autograd import batch_quadratic_drot_fn
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    warnings.simplefilter("ignore")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(SEED + 5)
    shapes = [(int(a), int(b)) for a, b in rng.integers(DIFF_MIN, DIFF_MAX + 1, size=(n_inst, 2))]
    g = torch.Generator(device=dev).manual_seed(SEED + 5)
    x = torch.randn(sum(m for m, _ in shapes), DIFF_DIM, generator=g, device=dev, requires_grad=True)
    y = torch.randn(sum(n for _, n in shapes), DIFF_DIM, generator=g, device=dev, requires_grad=True)
    B = QRBatch(shapes, RHO, ALPHA, [REL_EPS * math.sqrt(1.0 / m + 1.0 / n) for m, n in shapes],
                device=dev, cols_per_tile=256)
    p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                            [torch.full((n,), 1.0 / n) for _, n in shapes])
    c = packed_sqeuclidean_cost(B, x, y, DIFF_SCALE)
    X = batch_quadratic_drot_fn(B, c, p, q, iters)
    ((c * X).sum() + 0.5 * (X * X).sum()).backward()
    torch.cuda.synchronize()
    print(json.dumps({"case": f"diff:{n_inst}:{iters}", "elements": sum(m * n for m, n in shapes),
                      "cg_iters": X.grad_fn.cg_iters[:4]}), flush=True)
    return 0


def run_batch_timeline():
    """Timeline of one solve of the batched workload (256 instances): CTA 0's
    device clock at four points of every iteration (QRBatch.iteration_log),
    summarised per iteration range as mean stage times (--case batchlog)."""
    import torch
    from reg_drot.batch import QRBatch
    dev = torch.device("cuda", 0)
    shapes, costs, ps, qs, eps = make_batch_problem(dev)
    B = QRBatch(shapes, RHO, ALPHA, eps, device=dev)
    c = B.pack_c(costs)
    p, q = B.pack_marginals(ps, qs)
    cpt = B.autotune(c, p, q, iters=200)
    x = B.empty_x()
    B.launch(c, p, q, x, 10 ** 6)
    times, _ = B.iteration_log(30000, cpt)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    B.launch(c, p, q, x, 10 ** 6)
    b.record()
    b.synchronize()
    B.iteration_log(0, cpt)
    info = B.results()
    it = np.array([r["n_iter"] for r in info])
    elems = np.array([m * n for m, n in shapes], dtype=np.float64)
    n = min(int(it.max()) - 1, 30000)
    t = times[:n].cpu().numpy().astype(np.float64) / 1e3  # us
    total = np.append(np.diff(t[:, 0]), np.nan)
    rest = np.append(t[1:, 0] - t[:-1, 3], np.nan)
    rows = []
    edges = [0, 2000, 3000, 4000, 6000, 10000, n]
    for lo, hi in zip(edges[:-1], edges[1:]):
        if hi <= lo:
            continue
        sl = slice(lo, hi)
        ev = np.arange(lo, hi) % 2 == 0
        rows.append({"iterations": [lo, hi],
                     "active_elements_M": float(elems[it > lo].sum() / 1e6),
                     "us_per_iteration": float(np.nanmean(total[sl])),
                     "fused_update_us": float(np.mean(t[sl, 1] - t[sl, 0])),
                     "barrier1_wait_us": float(np.mean(t[sl, 2] - t[sl, 1])),
                     "dual_update_us": float(np.mean(t[sl, 3] - t[sl, 2])),
                     "rest_even_us": float(np.nanmean(rest[sl][ev])),
                     "rest_odd_us": float(np.nanmean(rest[sl][~ev])),
                     "seconds": float(np.nansum(total[sl]) / 1e6)})
    print(json.dumps({"case": "batchlog", "cols_per_tile": cpt, "tiles": B.tiles(cpt),
                      "s_per_batch": a.elapsed_time(b) / 1e3,
                      "n_iter_max": int(it.max()), "ranges": rows}), flush=True)
    return 0


def run_case(spec):
    """One solve of the headline workload at size n for a fixed iteration count
    (for profiler captures): --case n:iters[:gl][:bf16]; --case diff:n_inst:iters
    for the differentiable workload's kernels; --case batchlog for the
    batched solver's per-iteration timeline."""
    import torch
    import reg_drot
    parts = spec.split(":")
    if parts[0] == "batchlog":
        return run_batch_timeline()
    if parts[0] == "diff":
        return run_diff_case(int(parts[1]), int(parts[2]))
    n, iters = int(parts[0]), int(parts[1])
    dev = torch.device("cuda", 0)
    c, p, q, _ = make_problem(n)
    cd, pd, qd = (torch.from_numpy(a).to(dev) for a in (c, p, q))
    if "bf16" in parts[2:]:
        cd = cd.to(torch.bfloat16)
    if "gl" in parts[2:]:
        x, info, _ = reg_drot.solve_gl(cd, pd, qd, 2, RHO, ALPHA, iters, 0.0)
    else:
        x, info, _ = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, iters, 0.0)
    torch.cuda.synchronize()
    print(json.dumps({"case": spec, "iters_run": info["iters_run"],
                      "phase_ms": info["phase_ms"]}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--case", default=None,
                    help="n:iters[:gl][:bf16] -- one fixed-length solve; diff:n_inst:iters -- "
                         "cost, batched solve and adjoint of the differentiable workload; "
                         "for profiler captures")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
