"""Experiment drivers of the reference benchmark on the GPU solver.

    python -m reg_drot.cli singleexp_qr  <cmat_path> <n_rows> <n_cols> <rho> <r_weight> <use_warmup_init>
    python -m reg_drot.cli singleexp_glr <cmat_path> <n_rows> <n_cols> <n_groups> <rho> <r_weight> <use_warmup_init>
    python -m reg_drot.cli multiexp_qr   <cmat_dir> <n_rows> <n_cols> <n_tests> <rho> <r_weight>
                                         <use_warmup_init> <eps> <max_iters> <is_benchmark>
    python -m reg_drot.cli multiexp_glr  <cmat_dir> <out_dir> <n_rows> <n_cols> <n_groups> <n_tests>
                                         <rho> <r_weight> <use_warmup_init> <eps> <max_iters> <is_benchmark>

The same positional arguments, input files and outputs as the reference's
executables (core/singleexp_qr.cu, core/singleexp_glr.cu,
core/multiexp_qr.cu, core/multiexp_glr.cu): cost matrices are raw row-major
float32 files (core/utils.hpp:9-24; multi-experiment files are named
cmatrix_<n_rows>_<n_cols>[_<n_groups>]_<index>), marginals are uniform, and
every solve goes through the host-buffer C-ABI wrappers drot_qr_wrapper /
drot_gl_wrapper (the reference's quadratic_regularizer_drot_wrapper /
group_lasso_regularizer_drot_wrapper, so the C++ wrappers' parameter
conventions apply: step = rho / (n_rows + n_cols), QR divisor 1 + step *
(n_rows + n_cols) * r_weight, GL threshold r_weight / sqrt(n_rows /
n_groups)).  A single experiment prints the plan (n_cols lines of n_rows
values), the objective and the iteration count; a multi experiment prints
the mean / std summary (the first run, index 0, is the warm-up the
reference leaves out) or, with is_benchmark, the TSV log rows of runs 1..;
multiexp_glr also writes every plan to <out_dir>/drot-gl_<n_rows>_<n_cols>_<n_groups>_<index>
as n_rows lines of n_cols values (core/utils.hpp:48-61).  Without the full
argument list the drivers use the reference's defaults and say so.
"""
import ctypes
import math
import os
import sys

import numpy as np

from . import formats as F
from ._lib import lib, status_string

EPS = 1e-4
RHO = 2.0
MAX_ITERS = 20000


def _solve(kind, c, n_rows, n_cols, n_groups, rho, r_weight, max_iters, eps, warm, return_x):
    """One solve through the host-buffer wrapper; c is [n_cols, n_rows]."""
    L = lib()
    c = np.ascontiguousarray(c, dtype=np.float32)
    p = np.full(n_rows, 1.0 / n_rows, np.float32)  # 1/(T) n_rows, as the drivers
    q = np.full(n_cols, 1.0 / n_cols, np.float32)
    step = float(np.float32(rho) / np.float32(n_rows + n_cols))
    dur, prep = ctypes.c_float(), ctypes.c_float()
    nit, obj = ctypes.c_int(), ctypes.c_float()
    args = (c.ctypes.data, p.ctypes.data, q.ctypes.data, n_rows, n_cols)
    tail = (float(r_weight), int(max_iters), float(eps), ctypes.byref(dur), ctypes.byref(prep),
            ctypes.byref(nit), ctypes.byref(obj), int(bool(warm)), int(bool(return_x)))
    if kind == "qr":
        ptr = L.drot_qr_wrapper(*args, step, *tail)
    else:
        ptr = L.drot_gl_wrapper(*args, int(n_groups), step, *tail)
    status = L.drot_last_status()
    if status != 0:
        raise RuntimeError(f"{kind} wrapper: {status_string(status)}")
    x = None
    if return_x:
        x = np.ctypeslib.as_array(ptr, shape=(n_cols, n_rows)).copy()
        L.drot_free_host(ptr)
    return x, float(obj.value), int(nit.value), float(dur.value), float(prep.value)


def _mean_std(values):
    """utils::calc_mean_std: mean and population std of values[1:] (all of
    them when there is only one), FP32 as the reference accumulates."""
    v = np.asarray(values, np.float32)
    if v.size == 0:
        return 0.0, 0.0
    off = min(v.size - 1, 1)
    d = v[off:]
    mean = np.float32(0)
    for t in d:
        mean = np.float32(mean + t)
    mean = np.float32(mean / np.float32(d.size))
    var = np.float32(0)
    for t in d:
        var = np.float32(var + np.float32(t - mean) * np.float32(t - mean))
    return float(mean), float(np.float32(math.sqrt(float(var / np.float32(d.size)))))


def save_plan_trans(x, path):
    """A plan ([n_cols, n_rows]) as n_rows lines of n_cols "%.10f " values
    (utils::save_trans)."""
    x = np.asarray(x, dtype=np.float32)
    with open(path, "w") as f:
        for row in x.T:
            f.write("".join("%.10f " % v for v in row) + "\n")


def singleexp(kind, argv, out=sys.stdout):
    need = 6 if kind == "qr" else 7
    path, n_rows, n_cols, n_groups, rho, r_weight, warm = "./data/", 512, 512, 2, RHO, 0.0, True
    if kind == "gl":
        path, n_rows, n_cols = "./tmp/cmatrix.tmp", 2000, 2000
    if len(argv) == need:
        path, n_rows, n_cols = argv[0], int(argv[1]), int(argv[2])
        rest = argv[3:]
        if kind == "gl":
            n_groups, rest = int(rest[0]), rest[1:]
        rho, r_weight, warm = float(rest[0]), float(rest[1]), int(rest[2]) > 0
    else:
        out.write("Expected arguments: <cmat_dir> <n_rows> <n_cols> " +
                  ("<alpha> <q_weight>\n" if kind == "qr" else
                   "<n_groups> <rho> <r_weight> <use_warmup_init> <is_benchmark>\n"))
        out.write("Using default values...\n")
    c = F.load_cost(path, n_rows, n_cols)
    x, obj, nit, _, _ = _solve(kind, c, n_rows, n_cols, n_groups, rho, r_weight, MAX_ITERS, EPS,
                               warm, True)
    out.write(F.format_plan(x, obj, nit))
    return 0


def multiexp(kind, argv, out=sys.stdout):
    need = 10 if kind == "qr" else 12
    cdir, odir = ("./data/", None) if kind == "qr" else ("./class/", "./tmp/")
    n_rows, n_cols, n_groups, n_tests = (512, 512, 2, 1) if kind == "qr" else (2000, 2000, 2, 10)
    rho, r_weight, warm, eps, max_iters, bench = RHO, 0.0, True, EPS, MAX_ITERS, 0
    if len(argv) == need:
        a = list(argv)
        cdir = a.pop(0)
        if kind == "gl":
            odir = a.pop(0)
        n_rows, n_cols = int(a.pop(0)), int(a.pop(0))
        if kind == "gl":
            n_groups = int(a.pop(0))
        n_tests = int(a.pop(0))
        rho, r_weight, warm = float(a.pop(0)), float(a.pop(0)), int(a.pop(0)) > 0
        eps, max_iters, bench = float(a.pop(0)), int(float(a.pop(0))), int(a.pop(0))
    else:
        out.write("Expected arguments: <cmat_dir> " + ("<out_dir> " if kind == "gl" else "") +
                  "<n_rows> <n_cols> " + ("<n_groups> " if kind == "gl" else "") +
                  "<n_tests> <alpha> <q_weight> <use_warmup_init> <eps> <max_iters> "
                  "<is_benchmark>\n")
        out.write("Using default values...\n")
    step = float(np.float32(rho) / np.float32(n_rows + n_cols))
    if bench == 0:
        out.write(f"n_rows: {n_rows}, n_cols: {n_cols}, n_tests: {n_tests}\n")
        out.write("step_size: %.8f, %s: %.8f\n" % (step, "q_weight" if kind == "qr" else "r_weight",
                                                   r_weight))
    runs = []
    for idx in range(n_tests):
        stem = f"cmatrix_{n_rows}_{n_cols}_" + (f"{n_groups}_" if kind == "gl" else "") + str(idx)
        c = F.load_cost(os.path.join(cdir, stem), n_rows, n_cols)
        x, obj, nit, dur, prep = _solve(kind, c, n_rows, n_cols, n_groups, rho, r_weight, max_iters,
                                        eps, warm, kind == "gl")
        if kind == "gl":
            save_plan_trans(x, os.path.join(odir, f"drot-gl_{n_rows}_{n_cols}_{n_groups}_{idx}"))
        runs.append((dur, prep, nit, obj))
    if bench == 0:
        out.write("R Weight = %.4f, # Tests = %d\n" % (r_weight, n_tests - 1))
        md, sd = _mean_std([r[0] for r in runs])
        out.write("\tTime (ms)               = %12.8f (std = %.8f)\n" % (md, sd))
        mi, si = _mean_std([r[2] for r in runs])
        out.write("\t# Iteration             = %12.8f (std = %.8f)\n" % (mi, si))
        mo, so = _mean_std([r[3] for r in runs])
        out.write("\tObjective               = %12.8f (std = %.8f)\n" % (mo, so))
        out.write("\tTime Per Iteration (ms) = %12.8f\n" % (md / mi if mi else float("inf")))
        mp, sp = _mean_std([r[1] for r in runs])
        out.write("\tPreperation Time (ms)   = %12.8f (std = %.8f)\n" % (mp, sp))
    else:
        out.write(F.log_header("gl_drot" if kind == "gl" else "quad_drot") + "\n")
        for idx in range(1, n_tests):
            dur, _, nit, obj = runs[idx]
            out.write(F.log_row(idx, n_rows, n_cols, eps, warm,
                                float(np.float32(step) * np.float32(n_rows + n_cols)), r_weight,
                                max_iters, dur, obj, nit,
                                n_class=n_groups if kind == "gl" else None) + "\n")
    return 0


COMMANDS = {
    "singleexp_qr": lambda a, o: singleexp("qr", a, o),
    "singleexp_glr": lambda a, o: singleexp("gl", a, o),
    "multiexp_qr": lambda a, o: multiexp("qr", a, o),
    "multiexp_glr": lambda a, o: multiexp("gl", a, o),
}


def main(argv=None, out=sys.stdout):
    argv = sys.argv[1:] if argv is None else list(argv)
    if not argv or argv[0] not in COMMANDS:
        out.write("usage: python -m reg_drot.cli {" + ",".join(COMMANDS) + "} <arguments>\n")
        return 2
    return COMMANDS[argv[0]](argv[1:], out)


if __name__ == "__main__":
    sys.exit(main())
