"""Autotuner of the single-instance solver's launch shape.

The reference sizes its launches with a fixed heuristic of the matrix size
(core/drot_qr.hpp:236-239, _q_get_work_size_update_x; the same for GL,
core/drot_glr.hpp:357-360).  Here the planner has defaults (four 128-bit
vectors per lane, two 8-warp CTAs per SM, register loads) and
``tune`` times the alternatives on the caller's own data -- vectors per
lane, warps per CTA, the TMA bulk-copy ring with one or two CTAs per SM --
and pins the fastest for that problem shape on the current device
(drot_set_launch_choice).  Later solves of the same shape use it.  The
candidates differ only in how the FP32 row and column partial sums are
grouped, so a tuned solve agrees with the default one to FP32 rounding.

    best, timings = reg_drot.tune("qr", c, p, q, rho=2.0, r_weight=1e-3)
    x, info, ws = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, max_iters, eps)
"""
import ctypes

import torch

from ._lib import DrotLaunchChoice, check, lib

MODES = {"qr": 0, "gl": 1}


def _choice(kv, warps, path, ctas):
    return DrotLaunchChoice(int(kv), int(warps), int(path), int(ctas))


def pin(kind, n_rows, n_cols, n_class=0, *, c_dtype=torch.float32, vectors_per_lane=0,
        warps_per_cta=0, data_path=0, ctas_per_sm=0, device=None):
    """Pin a launch shape for one problem shape (n_rows = n_cols = 0: every
    shape of this kind and cost type without its own entry)."""
    ch = _choice(vectors_per_lane, warps_per_cta, data_path, ctas_per_sm)
    dt = 1 if c_dtype == torch.bfloat16 else 0
    with torch.cuda.device(device if device is not None else torch.cuda.current_device()):
        check(lib().drot_set_launch_choice(MODES[kind], int(n_rows), int(n_cols), int(n_class), dt,
                                           ctypes.byref(ch)), "set_launch_choice")


def unpin(kind, n_rows, n_cols, n_class=0, *, c_dtype=torch.float32, device=None):
    """Remove a pinned launch shape."""
    dt = 1 if c_dtype == torch.bfloat16 else 0
    with torch.cuda.device(device if device is not None else torch.cuda.current_device()):
        check(lib().drot_set_launch_choice(MODES[kind], int(n_rows), int(n_cols), int(n_class), dt,
                                           None), "set_launch_choice")


def clear():
    """Remove every pinned launch shape."""
    check(lib().drot_clear_launch_choices(), "clear_launch_choices")


def _candidates(kind, aligned, fp32):
    kvs = (1, 2, 4) if kind == "qr" else (1, 2, 4, 8)
    out = [dict(vectors_per_lane=kv, warps_per_cta=w, data_path=0, ctas_per_sm=0)
           for kv in kvs for w in (4, 8, 16)]
    if aligned and fp32:
        out += [dict(vectors_per_lane=kv, warps_per_cta=w, data_path=1, ctas_per_sm=ct)
                for kv in kvs for w in (8, 16) for ct in (1, 2)]
    return out


def tune(kind, c, p, q, rho, r_weight, n_class=1, iters=200, repeats=2, stream=None):
    """Times ``iters`` DR iterations (the stop test off) of every candidate
    launch shape on (c, p, q), ``repeats`` times each after one warm-up, and
    pins the fastest for this shape and cost type.  Returns (the pinned
    shape as a dict, [(shape dict, seconds per iteration), ...])."""
    from . import solve_gl, solve_qr
    if kind not in MODES:
        raise RuntimeError("kind must be 'qr' or 'gl'")
    n_cols, n_rows = c.shape
    aligned = n_rows % 4 == 0 and c.data_ptr() % 16 == 0
    fp32 = c.dtype == torch.float32
    iters = max(2, int(iters) // 2 * 2)
    ws, out, timings = None, None, []

    def run():
        nonlocal ws, out
        if kind == "qr":
            out, _, ws = solve_qr(c, p, q, rho, r_weight, iters, 0.0, out=out, workspace=ws,
                                  stream=stream, sync=False)
        else:
            out, _, ws = solve_gl(c, p, q, n_class, rho, r_weight, iters, 0.0, out=out,
                                  workspace=ws, stream=stream, sync=False)

    g = int(n_class) if kind == "gl" else 0
    s = torch.cuda.current_stream(c.device) if stream is None else stream
    with torch.cuda.device(c.device):
        for cand in _candidates(kind, aligned, fp32):
            try:
                pin(kind, n_rows, n_cols, g, c_dtype=c.dtype, **cand)
            except RuntimeError:
                continue  # this shape cannot be planned with the candidate
            run()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(repeats):
                run()
            e1.record(s)
            e1.synchronize()
            timings.append((cand, e0.elapsed_time(e1) / 1e3 / (repeats * iters)))
        if not timings:
            unpin(kind, n_rows, n_cols, g, c_dtype=c.dtype)
            raise RuntimeError("no launch shape could be planned for this problem")
        best = min(timings, key=lambda t: t[1])[0]
        pin(kind, n_rows, n_cols, g, c_dtype=c.dtype, **best)
    return best, timings


__all__ = ["tune", "pin", "unpin", "clear"]
