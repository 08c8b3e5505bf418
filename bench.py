#!/usr/bin/env python
"""Benchmark of the GB300 DROT solver.

Headline -- the metric "solves/s at marginal error 1e-4, batched + adjoint
against the plain solver; X-update HBM GB/s against the peak".  One step =
forward + backward of the differentiable OT loss over one batch:

  64 quadratic-regularised DROT instances, m, n ~ U{512..4096}, points
  x (m x 16), y (n x 16) ~ N(0, 1) (numpy default_rng(1239)), C = |x - y|^2
  / 64 built on the tensor cores, uniform p, q, alpha = 1e-3, rho = 2, warm
  start, every instance stopped at its relative marginal residual 1e-4
  (||(X1 - p, X^T1 - q)||_2 / ||(p; q)||_2); loss = sum_k <C_k, X_k> +
  w ||X_k||_F^2 with a fixed random w; backward = the implicit adjoint
  (support masks, batched Jacobi-PCG) and the chain rule to x and y.
  Seeded synthetic clouds stand in for the reference's data.

  value        instances solved with gradient per second: 64 x steps over
               the device time of the steps (CUDA events; point clouds
               resident in HBM; the solve streams 3.0 GB of X and C per
               iteration, far beyond L2, and L2 is flushed before every step).
  e2e          the same step through the public API from pinned host point
               clouds: H2D of x and y, the step, D2H of dL/dx, dL/dy and the
               loss, by wall clock.
  plain        the same 64 instances one at a time with the drop-in
               operator's entry point (reg_drot.solve_qr: FP32, forward
               only); batched_over_plain = value / plain.
  roofline     batch_solve_kernel, the dominant kernel of the step:
               algorithmic bytes of its launch (12 B per element on the
               iterations that read C, 8 B on the others, 12 B for the final
               unfold) over its measured time, against the measured HBM copy
               bandwidth; x_update_10000 inside it: the single-instance fused
               X-update at 10000^2 (X + C = 800 MB, HBM resident), 400
               iterations.
  cpu_baseline the oracle (C restatement of the reference loop, OpenMP on
               every host core) solving instances of the same workload one
               at a time to the same stop -- forward only: the reference has
               no backward.

`--impl reference` times that CPU implementation alone.  The reference's own
CPU solver is numpy, whose sources do not reach the GPU host; the oracle port
stands in for it (on the reference's CPU-runnable 1000^2 case the numpy
solver takes 47.0 ms per iteration and the port 0.54 ms on the same 8 cores:
oracle/time_reference_numpy.py).

Multi-GPU: the instances are independent and a step does not shard; N ranks
run N independent replicas (weak scaling).
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

ALPHA = 1e-3
RHO = 2.0
REL_EPS = 1e-4
SEED = 1234
N = 3000              # the dense single-instance workload (extra.qr_3000)
L2_FLUSH_BYTES = 512 << 20
MAX_ITERS = 10 ** 6

DIFF_INSTANCES = 64
DIFF_MIN, DIFF_MAX = 512, 4096
DIFF_DIM = 16
DIFF_SCALE = 1.0 / (4 * DIFF_DIM)  # C = |x - y|^2 / 64: mean cost 0.5 for N(0, I_16) clouds
DIFF_SEED = SEED + 5

WORKLOAD = (f"differentiable QR-DROT loss, {DIFF_INSTANCES} instances, m,n ~ U{{{DIFF_MIN}..{DIFF_MAX}}}, "
            f"x,y ~ N(0,I_{DIFF_DIM}), C = |x-y|^2/64 (tcgen05 split-TF32), alpha={ALPHA}, "
            f"rho={RHO}, uniform marginals, relative eps {REL_EPS}, loss = sum <C,X*> + w|X*|^2, "
            "forward + backward per step")
METRIC = (f"solves/s at marginal error {REL_EPS:g}, batched forward+backward "
          f"({DIFF_INSTANCES} differentiable QR-DROT instances)")
CONFIG = {"workload": WORKLOAD, "instances": DIFF_INSTANCES, "m_n_range": [DIFF_MIN, DIFF_MAX],
          "dim": DIFF_DIM, "alpha": ALPHA, "rho": RHO, "rel_eps": REL_EPS, "seed": DIFF_SEED,
          "l2": "flushed (512 MB write) before every timed step; X + C = 3.0 GB streamed per iteration"}


def diff_workload(seed=DIFF_SEED):
    """Shapes, concatenated point clouds (host, float32), the loss weight w
    and the absolute stop tolerance of every instance."""
    rng = np.random.default_rng(seed)
    shapes = [(int(a), int(b)) for a, b in
              rng.integers(DIFF_MIN, DIFF_MAX + 1, size=(DIFF_INSTANCES, 2))]
    xs = rng.standard_normal((sum(m for m, _ in shapes), DIFF_DIM), dtype=np.float32)
    ys = rng.standard_normal((sum(n for _, n in shapes), DIFF_DIM), dtype=np.float32)
    w = float(rng.random())
    eps = [REL_EPS * math.sqrt(1.0 / m + 1.0 / n) for m, n in shapes]
    return shapes, xs, ys, w, eps


def instance_slices(shapes):
    xo = yo = 0
    out = []
    for m, n in shapes:
        out.append((slice(xo, xo + m), slice(yo, yo + n)))
        xo += m
        yo += n
    return out


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


def profile_value(name, key):
    """A `key: value` line of a committed ncu summary under profiles/."""
    try:
        for line in open(os.path.join(REPO, "profiles", name)):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except (OSError, ValueError):
        pass
    return None


def solve_bytes(shapes, info, cbytes=4):
    """Algorithmic bytes of one batched solve launch: per instance, elements
    x (12 B on the iterations that read C, 8 B on the others, 12 B for the
    final unfold of a converged instance) with cbytes-byte C."""
    tot = 0.0
    for (m, n), r in zip(shapes, info):
        t = int(r["iters_run"])
        tot += float(m) * n * ((8 + cbytes) * ((t + 1) // 2) + 8 * (t // 2) +
                               ((8 + cbytes) if r["converged"] else 0))
    return tot


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

def cpu_cost(xk, yk):
    """C = |x - y|^2 / 64 of one instance ([n, m] float32, FP64 arithmetic)."""
    x = xk.astype(np.float64)
    y = yk.astype(np.float64)
    c = (y * y).sum(1)[:, None] + (x * x).sum(1)[None, :] - 2.0 * (y @ x.T)
    return (np.maximum(c, 0.0) * DIFF_SCALE).astype(np.float32)


def cpu_solve_instance(k, shapes, xs, ys, eps, threads=None):
    """The oracle (FP32 restatement of the reference loop) solving instance k
    of the headline workload to its stop; returns (seconds, n_iter)."""
    from oracle import oracle as O
    m, n = shapes[k]
    sx, sy = instance_slices(shapes)[k]
    c = cpu_cost(xs[sx], ys[sy])
    p = np.full(m, 1.0 / m, np.float32)
    q = np.full(n, 1.0 / n, np.float32)
    t0 = time.perf_counter()
    o = O.quadratic_drot(c, p, q, RHO, ALPHA, MAX_ITERS, eps[k], threads=threads)
    return time.perf_counter() - t0, int(o["n_iter"])


def cpu_sample(budget_s=15.0):
    """cpu_baseline: instances of the headline workload solved one at a time
    by the oracle on every host core, in workload order, until budget_s."""
    from oracle import oracle as O
    shapes, xs, ys, _, eps = diff_workload()
    threads = int(O.lib().oracle_max_threads())
    small = int(np.argmin([m * n for m, n in shapes]))
    cpu_solve_instance(small, shapes, xs, ys, eps, threads)  # page in, spin up threads
    spent, done, iters = 0.0, 0, []
    while spent < budget_s and done < len(shapes):
        t, it = cpu_solve_instance(done, shapes, xs, ys, eps, threads)
        spent += t
        iters.append(it)
        done += 1
    return {"value": done / spent, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": (f"instances 0..{done - 1} of the {len(shapes)} solved to their stop one at "
                       f"a time by the FP32 oracle ({threads} OpenMP threads, {spent:.1f} s, "
                       f"{sum(iters)} iterations); forward only -- the reference has no backward")}


def run_reference(args):
    """The reference arm: the oracle port solving instances of the headline
    workload one at a time on the host cores, one full solve per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    shapes, xs, ys, _, eps = diff_workload()
    threads = int(O.lib().oracle_max_threads())
    small = int(np.argmin([m * n for m, n in shapes]))
    for _ in range(args.warmup):
        cpu_solve_instance(small, shapes, xs, ys, eps, threads)
    times, iters = [], []
    for i in range(args.steps):
        t, it = cpu_solve_instance(i % len(shapes), shapes, xs, ys, eps, threads)
        times.append(t)
        iters.append(it)
    total = sum(times)
    value = args.steps / total
    sample = (f"one full solve per step: instances 0..{min(args.steps, len(shapes)) - 1} of the "
              f"{len(shapes)} (warm-up: the smallest), FP32 oracle on {threads} OpenMP threads, "
              f"{sum(iters)} iterations in {total:.1f} s; forward only -- the reference has no "
              "backward")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": CONFIG,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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


# --------------------------------------------------------------------------- GPU legs

class DiffStep:
    """The headline step on one device: plan, marginals and the step."""

    def __init__(self, dev, shapes, eps, w):
        import torch
        from reg_drot.batch import QRBatch
        self.dev = dev
        self.shapes = shapes
        self.w = w
        self.B = QRBatch(shapes, RHO, ALPHA, eps, device=dev)
        self.p, self.q = self.B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                                               [torch.full((n,), 1.0 / n) for _, n in shapes])

    def autotune(self, x, y):
        import torch
        from reg_drot.cost import packed_sqeuclidean_cost
        with torch.no_grad():
            return self.B.autotune(packed_sqeuclidean_cost(self.B, x, y, DIFF_SCALE),
                                   self.p, self.q, iters=100)

    def run(self, x, y, events=None):
        """cost -> batched solve -> loss -> backward; x, y leaves with
        requires_grad.  events: four CUDA events recorded around the stages.
        Returns (loss, the solve's autograd node)."""
        from reg_drot.autograd import batch_quadratic_drot_fn
        from reg_drot.cost import packed_sqeuclidean_cost
        if events:
            events[0].record()
        c = packed_sqeuclidean_cost(self.B, x, y, DIFF_SCALE)
        if events:
            events[1].record()
        X = batch_quadratic_drot_fn(self.B, c, self.p, self.q, MAX_ITERS)
        if events:
            events[2].record()
        loss = (c * X).sum() + self.w * (X * X).sum()
        loss.backward()
        if events:
            events[3].record()
        return loss.detach(), X.grad_fn


def e2e_point(step, xh, yh, steps):
    """The headline step end to end through the public API: pinned host
    point clouds -> H2D -> step -> D2H of dL/dx, dL/dy and the loss."""
    import torch
    dev = step.dev
    xp = torch.from_numpy(xh).pin_memory()
    yp = torch.from_numpy(yh).pin_memory()
    gxh = torch.empty_like(xp).pin_memory()
    gyh = torch.empty_like(yp).pin_memory()

    def once():
        x = xp.to(dev, non_blocking=True).requires_grad_(True)
        y = yp.to(dev, non_blocking=True).requires_grad_(True)
        loss, _ = step.run(x, y)
        gxh.copy_(x.grad, non_blocking=True)
        gyh.copy_(y.grad, non_blocking=True)
        val = float(loss)  # D2H of the loss; synchronises
        torch.cuda.synchronize(dev)
        return val

    once()
    t0 = time.perf_counter()
    for _ in range(steps):
        once()
    wall = time.perf_counter() - t0
    return {"value": DIFF_INSTANCES * steps / wall, "unit": "solves/s",
            "h2d_bytes_per_step": int(xp.nbytes + yp.nbytes),
            "d2h_bytes_per_step": int(gxh.nbytes + gyh.nbytes + 4), "steps": steps}


def plain_point(dev, shapes, xs, ys, eps, flush):
    """The plain per-instance solver on the headline instances: each solved
    alone with reg_drot.solve_qr (FP32, forward only), L2 flushed before
    each; C from the tensor-core kernel (not timed)."""
    import torch
    import reg_drot
    from reg_drot.cost import sqeuclidean_cost
    t_sum, iters = 0.0, []
    sl = instance_slices(shapes)
    with torch.no_grad():
        for k, (m, n) in enumerate(shapes):
            xk = torch.from_numpy(xs[sl[k][0]]).to(dev)
            yk = torch.from_numpy(ys[sl[k][1]]).to(dev)
            ck = sqeuclidean_cost(xk, yk, DIFF_SCALE)
            pk = torch.full((m,), 1.0 / m, device=dev)
            qk = torch.full((n,), 1.0 / n, device=dev)
            if k == 0:
                reg_drot.solve_qr(ck, pk, qk, RHO, ALPHA, MAX_ITERS, eps[k])  # warm-up
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            _, info, _ = reg_drot.solve_qr(ck, pk, qk, RHO, ALPHA, MAX_ITERS, eps[k])
            b.record()
            b.synchronize()
            t_sum += a.elapsed_time(b) / 1e3
            iters.append(info["n_iter"])
    return {"solves_per_s": len(shapes) / t_sum, "s_total": t_sum,
            "n_iter_min_median_max": [int(min(iters)), float(np.median(iters)), int(max(iters))]}


def qr_3000_point(dev, flush):
    """The dense single-instance workload: QR 3000^2, C ~ U[0,1) float32,
    p, q ~ Dirichlet(1), alpha 1e-3, relative eps 1e-4 (X + C = 72 MB:
    L2-resident for the whole solve)."""
    import torch
    import reg_drot
    c, p, q, eps = make_problem(N, SEED)
    cd, pd, qd = (torch.from_numpy(a).to(dev) for a in (c, p, q))
    x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 9, eps)
    flush.zero_()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    x, info, ws = reg_drot.solve_qr(cd, pd, qd, RHO, ALPHA, 10 ** 9, eps, out=x, workspace=ws)
    b.record()
    b.synchronize()
    t = a.elapsed_time(b) / 1e3
    it = info["iters_run"]
    nbytes = float(N) * N * (12 * ((it + 1) // 2) + 8 * (it // 2) + 12)
    return {"solves_per_s": 1.0 / t, "n_iter": info["n_iter"],
            "us_per_iteration": t / it * 1e6, "algorithmic_GBps": nbytes / t / 1e9,
            "note": "X + C = 72 MB stays in the 129 MB L2 across iterations"}


GL_LAST_K = 64


def diff_gl_point(dev, shapes, xs, ys, w, eps, gl_inst=8, gl_iters=20000):
    """The group-lasso half of the differentiable workload: 2 classes (the
    row halves), GL weight 1e-3 in the C++ wrapper's convention (lambda =
    r / sqrt(m / 2), core/drot_glr.hpp:385, as the domain-adaptation
    benchmark), each solve run to its relative 1e-4 stop, backward = the
    checkpointed unrolled adjoint of the last GL_LAST_K iterations; the first
    gl_inst instances, one at a time."""
    import torch
    from reg_drot.autograd import group_lasso_drot_fn
    from reg_drot.cost import sqeuclidean_cost
    sl = instance_slices(shapes)
    times, iters, conv = [], [], []
    for k in range(gl_inst):
        m, n = shapes[k]
        xk = torch.from_numpy(xs[sl[k][0]]).to(dev).requires_grad_(True)
        yk = torch.from_numpy(ys[sl[k][1]]).to(dev).requires_grad_(True)
        pk, qk = torch.full((m,), 1.0 / m, device=dev), torch.full((n,), 1.0 / n, device=dev)
        for rep in range(2):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            ck = sqeuclidean_cost(xk, yk, DIFF_SCALE)
            Xk = group_lasso_drot_fn(ck, pk, qk, 2, RHO, ALPHA, gl_iters, eps[k],
                                     convention="wrapper", last_k=GL_LAST_K)
            ((ck * Xk).sum() + w * (Xk * Xk).sum()).backward()
            e1.record()
            e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        iters.append(Xk.grad_fn.info["n_iter"])
        conv.append(Xk.grad_fn.info["converged"])
    return {"instances": gl_inst, "solves_with_grad_per_s": gl_inst / sum(times),
            "iterations": iters, "converged": int(sum(conv)), "last_k": GL_LAST_K,
            "lambda_convention": "wrapper"}


def diff_gl_batched(dev, shapes, xs, ys, w, eps, gl_inst, gl_iters=20000, steps=1, cpt=256):
    """The group-lasso half of the differentiable workload through the
    batched solver: the first gl_inst instances in one GLBatch (2 classes,
    the C++ wrapper's threshold), each stopped at its relative 1e-4, packed
    tensor-core cost, backward = the truncated unrolled adjoint of the last
    GL_LAST_K iterations per instance (batch_group_lasso_drot_fn).  Forward
    and backward timed apart (CUDA events)."""
    import torch
    from reg_drot.autograd import batch_group_lasso_drot_fn
    from reg_drot.batch import GLBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    sh = shapes[:gl_inst]
    sl = instance_slices(sh)
    B = GLBatch(sh, 2, RHO, ALPHA, eps[:gl_inst], device=dev, cols_per_tile=cpt,
                convention="wrapper")
    p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in sh],
                            [torch.full((n,), 1.0 / n) for _, n in sh])
    x = torch.from_numpy(xs[:sl[-1][0].stop]).to(dev).requires_grad_(True)
    y = torch.from_numpy(ys[:sl[-1][1].stop]).to(dev).requires_grad_(True)
    fwd, bwd = [], []
    for rep in range(steps + 1):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        c = packed_sqeuclidean_cost(B, x, y, DIFF_SCALE)
        X = batch_group_lasso_drot_fn(B, c, p, q, gl_iters, last_k=GL_LAST_K)
        e[1].record()
        ((c * X).sum() + w * (X * X).sum()).backward()
        e[2].record()
        e[2].synchronize()
        if rep > 0:
            fwd.append(e[0].elapsed_time(e[1]) / 1e3)
            bwd.append(e[1].elapsed_time(e[2]) / 1e3)
    info = X.grad_fn.info
    its = sorted(r["n_iter"] for r in info)
    # GL reads X and C and writes X on every iteration: 12 B per element
    nbytes = sum(12.0 * m * n * r["n_iter"] for (m, n), r in zip(sh, info))
    peak, _ = measured_peak()
    return {"instances": gl_inst, "solves_with_grad_per_s": gl_inst / (min(fwd) + min(bwd)),
            "forward_s": min(fwd), "backward_s": min(bwd),
            "forward_algorithmic_GBps": nbytes / min(fwd) / 1e9,
            "forward_frac_of_measured_hbm": nbytes / min(fwd) / 1e9 / peak,
            "n_iter_min_median_max": [its[0], its[len(its) // 2], its[-1]],
            "converged": int(sum(r["converged"] for r in info)), "last_k": GL_LAST_K,
            "lambda_convention": "wrapper"}


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

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    shapes, xs, ys, w, eps = diff_workload()
    step = DiffStep(dev, shapes, eps, w)
    x = torch.from_numpy(xs).to(dev).requires_grad_(True)
    y = torch.from_numpy(ys).to(dev).requires_grad_(True)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    cpt = step.autotune(x, y)
    for _ in range(args.warmup):
        x.grad = y.grad = None
        flush.zero_()
        step.run(x, y)
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    fn = None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            x.grad = y.grad = None
            flush.zero_()
            _, fn = step.run(x, y, evs[i])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    step_s = [e[0].elapsed_time(e[3]) / 1e3 for e in evs]
    solve_s = [e[1].elapsed_time(e[2]) / 1e3 for e in evs]
    bwd_s = [e[2].elapsed_time(e[3]) / 1e3 for e in evs]
    cost_s = [e[0].elapsed_time(e[1]) / 1e3 for e in evs]
    total = sum(step_s)
    total, wall = max_over_ranks([total, wall], dist, dev)
    value = replica_throughput(world, args.steps * DIFF_INSTANCES, total)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    info = fn.info
    it = np.array([r["iters_run"] for r in info])
    peak, peak_kind = measured_peak()
    kbytes = solve_bytes(shapes, info)
    ksec = statistics.mean(solve_s)
    ratio = profile_value("batch_solve_diff16.md", "traffic_over_algorithmic")
    hbm = hbm_point(dev, flush)
    roofline = {"bound": "hbm", "kernel": "batch_solve_kernel<float>",
                "achieved": kbytes / ksec / 1e9, "peak": peak, "unit": "GB/s",
                "frac": kbytes / ksec / 1e9 / peak, "peak_source": peak_kind,
                "traffic": ratio * kbytes if ratio else None,
                "algorithmic_bytes_per_launch": kbytes,
                "traffic_basis": ("ncu DRAM bytes / algorithmic bytes of a 16-instance capture "
                                  "of the same kernel, times this launch's algorithmic bytes"),
                "x_update_10000": {"achieved": hbm["achieved_GBps"],
                                   "frac": hbm["achieved_GBps"] / peak,
                                   "us_per_iteration": hbm["us_per_iteration"]}}
    e2e = e2e_point(step, xs, ys, min(args.steps, 3))
    plain = plain_point(dev, shapes, xs, ys, eps, flush)
    extra = {"qr_3000": qr_3000_point(dev, flush), "hbm_point": hbm,
             "gl_da": gl_da_point(dev), "gl_da_weight_5e-3": gl_da_point(dev, 5e-3),
             "configs": config_points(dev, flush), "batched_config4": batched_point(dev, flush),
             "diff_gl": {"batched_64": diff_gl_batched(dev, shapes, xs, ys, w, eps, 64),
                         "batched_8": diff_gl_batched(dev, shapes, xs, ys, w, eps, 8),
                         "one_at_a_time_8": diff_gl_point(dev, shapes, xs, ys, w, eps)}}
    cpu = cpu_sample(budget_s=15.0) if world == 1 else None
    cg = fn.cg_iters
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded N(0,1) point clouds)", "config": CONFIG,
        "parallelism": f"replicas x{world}", "cols_per_tile": cpt,
        "clocks": clk.summary(), "wall_s_timed_region": wall,
        # our kernels per step: cost, batch init + solve, adjoint masks + PCG
        "gpu_launches": 5 * args.steps,
        "extra": extra,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "roofline": roofline,
        "stages_s_per_step": {"cost": statistics.mean(cost_s), "forward_solve": ksec,
                              "backward": statistics.mean(bwd_s)},
        "n_iter_min_median_max": [int(it.min()), float(np.median(it)), int(it.max())],
        "cg_iters_min_median_max": [int(min(cg)), float(np.median(cg)), int(max(cg))],
        "converged": int(sum(r["converged"] for r in info)),
        "plain_per_instance": plain,
        "batched_over_plain": value / plain["solves_per_s"],
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_diff_case(n_inst, iters):
    """Profiler case: the headline workload's first n_inst instances, one
    launch each of the cost kernel, the batched solve (iters iterations) and
    the adjoint CG (--case diff:n_inst:iters)."""
    import warnings
    import torch
    from reg_drot.autograd import batch_quadratic_drot_fn
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    warnings.simplefilter("ignore")
    dev = torch.device("cuda", 0)
    shapes, xs, ys, w, eps = diff_workload()
    shapes, eps = shapes[:n_inst], eps[:n_inst]
    sl = instance_slices(shapes)
    x = torch.from_numpy(xs[:sl[-1][0].stop]).to(dev).requires_grad_(True)
    y = torch.from_numpy(ys[:sl[-1][1].stop]).to(dev).requires_grad_(True)
    B = QRBatch(shapes, RHO, ALPHA, eps, device=dev, cols_per_tile=256)
    p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                            [torch.full((n,), 1.0 / n) for _, n in shapes])
    c = packed_sqeuclidean_cost(B, x, y, DIFF_SCALE)
    X = batch_quadratic_drot_fn(B, c, p, q, iters)
    ((c * X).sum() + w * (X * X).sum()).backward()
    torch.cuda.synchronize()
    # the forward launch alone, timed (inputs in HBM, all instances active)
    with torch.no_grad():
        xo = B.empty_x()
        B.launch(c.detach(), p, q, xo, iters)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        B.launch(c.detach(), p, q, xo, iters)
        b.record()
        b.synchronize()
    t = a.elapsed_time(b) / 1e3
    info = B.results()
    nbytes = solve_bytes(shapes, info)
    peak, _ = measured_peak()
    # the cost kernel alone: C bytes written (4 per stored element) per call;
    # each call also reads back its 4-byte status, inside the events
    with torch.no_grad():
        xd, yd = x.detach(), y.detach()
        for _ in range(2):
            packed_sqeuclidean_cost(B, xd, yd, DIFF_SCALE)
        a.record()
        for _ in range(5):
            packed_sqeuclidean_cost(B, xd, yd, DIFF_SCALE)
        b.record()
        b.synchronize()
    t_cost = a.elapsed_time(b) / 1e3 / 5
    cost_bytes = 4 * sum(m * n for m, n in shapes)
    print(json.dumps({"case": f"diff:{n_inst}:{iters}", "elements": sum(m * n for m, n in shapes),
                      "cg_iters": X.grad_fn.cg_iters[:4], "solve_s": t,
                      "us_per_iteration": 1e6 * t / max(1, iters),
                      "achieved_GBps": nbytes / t / 1e9, "frac": nbytes / t / 1e9 / peak,
                      "cost_us": 1e6 * t_cost, "cost_GBps": cost_bytes / t_cost / 1e9,
                      "cost_frac": cost_bytes / t_cost / 1e9 / peak}), flush=True)
    return 0


def run_batch_timeline(workload="config4"):
    """Timeline of one solve of a batched workload (config4: the 256-instance
    batch; diff: the headline's 64 instances; gl: their group-lasso solve):
    CTA 0's device clock at four points of every iteration
    (QRBatch.iteration_log), summarised per iteration range as mean stage
    times (--case batchlog[:diff|:gl])."""
    import torch
    from reg_drot.batch import QRBatch
    dev = torch.device("cuda", 0)
    if workload in ("diff", "gl"):
        from reg_drot.batch import GLBatch
        from reg_drot.cost import packed_sqeuclidean_cost
        shapes, xs, ys, _, eps = diff_workload()
        if workload == "gl":  # the GL half: 2 classes, the C++ wrapper's threshold
            B = GLBatch(shapes, 2, RHO, ALPHA, eps, device=dev, convention="wrapper")
        else:
            B = QRBatch(shapes, RHO, ALPHA, eps, device=dev)
        with torch.no_grad():
            c = packed_sqeuclidean_cost(B, torch.from_numpy(xs).to(dev),
                                        torch.from_numpy(ys).to(dev), DIFF_SCALE)
        p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                                [torch.full((n,), 1.0 / n) for _, n in shapes])
    else:
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
                     # even iterations read C (12 B / element), odd ones do not (8 B)
                     "fused_update_even_us": float(np.mean((t[sl, 1] - t[sl, 0])[ev])),
                     "fused_update_odd_us": float(np.mean((t[sl, 1] - t[sl, 0])[~ev])),
                     "barrier1_wait_us": float(np.mean(t[sl, 2] - t[sl, 1])),
                     "dual_update_us": float(np.mean(t[sl, 3] - t[sl, 2])),
                     "rest_even_us": float(np.nanmean(rest[sl][ev])),
                     "rest_odd_us": float(np.nanmean(rest[sl][~ev])),
                     "seconds": float(np.nansum(total[sl]) / 1e6)})
    slowest = sorted(zip(it.tolist(), shapes), reverse=True)[:8]
    print(json.dumps({"case": f"batchlog:{workload}", "cols_per_tile": cpt, "tiles": B.tiles(cpt),
                      "s_per_batch": a.elapsed_time(b) / 1e3,
                      "n_iter_max": int(it.max()),
                      "slowest": [[n, list(sh)] for n, sh in slowest],
                      "ranges": rows}), flush=True)
    return 0


def run_case(spec):
    """Single cases for profiler captures and one-off measurements:
    n:iters[:gl][:bf16] (one dense solve at a fixed iteration count),
    diff:n_inst:iters (the differentiable workload's kernels),
    batchlog[:diff|:gl] (the batched solver's per-iteration timeline),
    conv:n:alpha[:bf16] (one dense solve to its stop), diffpts:n_inst:iters
    (the point-cloud launch), diffgl:n_inst:iters[:cols_per_tile] (the GL
    batch, every instance active) and glbatch:n_inst[:cols_per_tile] (the GL
    half of the differentiable workload with its gradient)."""
    import torch
    import reg_drot
    parts = spec.split(":")
    if parts[0] == "batchlog":
        return run_batch_timeline(parts[1] if len(parts) > 1 else "config4")
    if parts[0] == "diff":
        return run_diff_case(int(parts[1]), int(parts[2]))
    if parts[0] == "conv":
        # one dense QR solve to relative marginal residual 1e-4: --case
        # conv:n:alpha[:bf16] (C ~ U[0,1), Dirichlet marginals, as configured
        # for the 3000^2 / 10000^2 workloads); the residual is recomputed
        # from X in FP64
        dev = torch.device("cuda", 0)
        n, alpha = int(parts[1]), float(parts[2])
        c, p, q, eps = make_problem(n)
        cd, pd, qd = (torch.from_numpy(a).to(dev) for a in (c, p, q))
        if "bf16" in parts[3:]:
            cd = cd.to(torch.bfloat16)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record()
        x, info, _ = reg_drot.solve_qr(cd, pd, qd, RHO, alpha, 10 ** 7, eps)
        b_.record()
        b_.synchronize()
        xd = x.double()
        resid = torch.sqrt(((pd.double() - xd.sum(0)) ** 2).sum() +
                           ((qd.double() - xd.sum(1)) ** 2).sum()).item()
        pq = float(np.sqrt((p.astype(np.float64) ** 2).sum() + (q.astype(np.float64) ** 2).sum()))
        print(json.dumps({"case": spec, "s_per_solve": a_.elapsed_time(b_) / 1e3,
                          "n_iter": info["n_iter"], "converged": info["converged"],
                          "objective": info["objective_f64"], "residual": info["residual"],
                          "relative_residual_recomputed": resid / pq, "eps_relative": 1e-4}),
              flush=True)
        return 0
    if parts[0] == "diffpts":
        # the first n_inst instances of the differentiable workload through the
        # point-cloud launch (cost recomputed on the tensor cores), iters
        # iterations, every instance active
        from reg_drot.batch import QRBatch
        dev = torch.device("cuda", 0)
        shapes, xs, ys, _, eps = diff_workload()
        n_inst, iters = int(parts[1]), int(parts[2])
        shapes = shapes[:n_inst]
        sl = instance_slices(shapes)
        xd = torch.from_numpy(xs[:sl[-1][0].stop]).to(dev)
        yd = torch.from_numpy(ys[:sl[-1][1].stop]).to(dev)
        B = QRBatch(shapes, RHO, ALPHA, eps[:n_inst], device=dev, cols_per_tile=256)
        p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                                [torch.full((n,), 1.0 / n) for _, n in shapes])
        x = B.empty_x()
        B.launch_points(xd, yd, p, q, x, iters, scale=DIFF_SCALE)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        B.launch_points(xd, yd, p, q, x, iters, scale=DIFF_SCALE)
        b.record()
        b.synchronize()
        t = a.elapsed_time(b) / 1e3
        elems = sum(m * n for m, n in shapes)
        print(json.dumps({"case": spec, "elements": elems, "solve_s": t,
                          "us_per_iteration": 1e6 * t / max(1, iters),
                          "achieved_GBps": 8.0 * elems * iters / t / 1e9}), flush=True)
        return 0
    if parts[0] == "diffgl":
        # the GL half's first n_inst instances in one GLBatch (2 classes, the
        # C++ wrapper's threshold), iters iterations with every instance
        # active (eps 0); the second of two launches timed
        from reg_drot.batch import GLBatch
        from reg_drot.cost import packed_sqeuclidean_cost
        dev = torch.device("cuda", 0)
        shapes, xs, ys, _, _ = diff_workload()
        n_inst, iters = int(parts[1]), int(parts[2])
        cpt = int(parts[3]) if len(parts) > 3 else 256
        shapes = shapes[:n_inst]
        sl = instance_slices(shapes)
        B = GLBatch(shapes, 2, RHO, ALPHA, 0.0, device=dev, cols_per_tile=cpt,
                    convention="wrapper")
        p, q = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in shapes],
                                [torch.full((n,), 1.0 / n) for _, n in shapes])
        c = packed_sqeuclidean_cost(B, torch.from_numpy(xs[:sl[-1][0].stop]).to(dev),
                                    torch.from_numpy(ys[:sl[-1][1].stop]).to(dev), DIFF_SCALE)
        x = B.empty_x()
        B.launch(c, p, q, x, iters)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        B.launch(c, p, q, x, iters)
        b.record()
        b.synchronize()
        t = a.elapsed_time(b) / 1e3
        elems = sum(m * n for m, n in shapes)
        print(json.dumps({"case": spec, "elements": elems, "solve_s": t,
                          "us_per_iteration": 1e6 * t / max(1, iters),
                          "achieved_GBps": 12.0 * elems * iters / t / 1e9}), flush=True)
        return 0
    if parts[0] == "glbatch":
        import warnings
        warnings.simplefilter("ignore")
        dev = torch.device("cuda", 0)
        shapes, xs, ys, w, eps = diff_workload()
        n = int(parts[1])
        cpt = int(parts[2]) if len(parts) > 2 else 256
        out = {"case": spec, "batched": diff_gl_batched(dev, shapes, xs, ys, w, eps, n, cpt=cpt)}
        if n <= 8:
            out["one_at_a_time"] = diff_gl_point(dev, shapes, xs, ys, w, eps, gl_inst=n)
        print(json.dumps(out), flush=True)
        return 0
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
                         "cost, batched solve and adjoint of the headline workload; "
                         "batchlog[:diff] -- per-iteration timeline of a batched solve; "
                         "for profiler captures")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
