"""reg_drot -- GB300 Douglas-Rachford optimal transport (drop-in module).

Same module name and operator signatures as the reference PyTorch extension
(WangZesen/Regularized-DROT, pytorch/src/drot_cuda.cpp:26-62):

    quadratic_drot(c, p, q, rho, r_weight, max_iters, eps) -> x
    group_lasso_drot(c, p, q, n_class, rho, r_weight, max_iters, eps) -> x

``c`` is a contiguous float32 CUDA tensor of shape [M, N] with N = p.numel()
(the reference's n_rows, the contiguous axis) and M = q.numel().  The plan
``x`` has the shape of ``c``.  Invalid inputs raise RuntimeError with the
reference's messages.  The solve runs on the current CUDA stream of c's
device in one persistent kernel; like the reference, the operators return
after the solve has finished.

Beyond the reference: ``solve_qr`` / ``solve_gl`` return the solve record
(iterations, objective, residual, convergence) next to x, and accept
``stream`` and pre-allocated ``out`` / ``workspace`` tensors.
"""
import ctypes

import torch

from ._lib import DrotError, DrotResult, check, lib, status_string  # noqa: F401

__all__ = ["quadratic_drot", "group_lasso_drot", "solve_qr", "solve_gl", "DrotError",
           "group_bounds", "workspace_bytes", "tune"]


C_F32, C_BF16 = 0, 1  # DROT_C_F32 / DROT_C_BF16 of drot_gb300.h


def _check_input(t, name, allow_bf16=False):
    # CHECK_CUDA / CHECK_CONTIGUOUS of pytorch/src/drot_cuda.cpp:22-24
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if t.dtype != torch.float32 and not (allow_bf16 and t.dtype == torch.bfloat16):
        raise RuntimeError(f"expected scalar type Float but found {t.dtype} for {name}")


def _check_shapes(c, p, q):
    n_rows = p.numel()
    n_cols = q.numel()
    # qr_drot_cuda_kernel.cu:154-155 / glr_drot_cuda_kernel.cu:313-314
    if c.dim() != 2:
        raise RuntimeError("c must be a 2-D tensor [q.numel(), p.numel()]")
    if c.size(0) != n_cols:
        raise RuntimeError("C.size(0) does not match with q.numel()")
    if c.size(1) != n_rows:
        raise RuntimeError("C.size(1) does not match with p.numel()")
    for t, name in ((p, "p"), (q, "q")):
        if t.device != c.device:
            raise RuntimeError(f"{name} must be on the same device as c")
    return n_rows, n_cols


def _stream_handle(device, stream):
    s = torch.cuda.current_stream(device) if stream is None else stream
    return s.cuda_stream


def workspace_bytes(kind, n_rows, n_cols, n_class=1, device=None):
    """Bytes of the operator workspace for ``kind`` in {"qr", "gl"} on ``device``."""
    with torch.cuda.device(device if device is not None else torch.cuda.current_device()):
        if kind == "qr":
            return int(lib().drot_quadratic_drot_workspace_bytes(n_rows, n_cols))
        return int(lib().drot_group_lasso_drot_workspace_bytes(n_rows, n_cols, n_class))


def _alloc(kind, c, n_rows, n_cols, n_class, out, workspace):
    nbytes = workspace_bytes(kind, n_rows, n_cols, n_class, c.device)
    if nbytes == 0:
        raise DrotError(4, "workspace_bytes")
    if workspace is None or workspace.numel() * workspace.element_size() < nbytes:
        workspace = torch.empty(nbytes + 256, dtype=torch.uint8, device=c.device)
    ptr = workspace.data_ptr()
    pad = (-ptr) % 256
    if out is None:
        out = torch.empty(c.shape, dtype=torch.float32, device=c.device)
    else:
        _check_input(out, "out")
        if out.shape != c.shape or out.device != c.device:
            raise RuntimeError("out must have the shape and device of c")
    return out, workspace, ptr + pad, workspace.numel() * workspace.element_size() - pad


def solve_qr(c, p, q, rho, r_weight, max_iters, eps, *, out=None, workspace=None,
             stream=None, sync=True):
    """Quadratic-regularised DROT; returns (x, info, workspace).

    ``info`` is the solve record (n_iter, iters_run, converged, status,
    objective, objective_f64, residual).  With ``sync=False`` the call
    returns right after enqueueing the solve on ``stream`` and ``info`` is
    None; read the record later with ``read_result(workspace)``.  ``c`` may
    be float32 or bfloat16 (BF16-stored cost, FP32 iterates; x is float32).
    """
    _check_input(c, "c", allow_bf16=True)
    for t, n in ((p, "p"), (q, "q")):
        _check_input(t, n)
    n_rows, n_cols = _check_shapes(c, p, q)
    x, ws, wptr, wbytes = _alloc("qr", c, n_rows, n_cols, 1, out, workspace)
    res = DrotResult()
    with torch.cuda.device(c.device):
        rc = lib().drot_quadratic_drot_ex(
            c.data_ptr(), C_BF16 if c.dtype == torch.bfloat16 else C_F32,
            p.data_ptr(), q.data_ptr(), n_rows, n_cols, float(rho),
            float(r_weight), int(max_iters), float(eps), x.data_ptr(), wptr, wbytes,
            ctypes_byref(res) if sync else None, _stream_handle(c.device, stream))
    check(rc, "quadratic_drot")
    return x, (res.as_dict() if sync else None), ws


def solve_gl(c, p, q, n_class, rho, r_weight, max_iters, eps, *, out=None, workspace=None,
             stream=None, sync=True):
    """Group-lasso-regularised DROT; returns (x, info, workspace).  ``c`` may
    be float32 or bfloat16."""
    _check_input(c, "c", allow_bf16=True)
    for t, n in ((p, "p"), (q, "q")):
        _check_input(t, n)
    n_rows, n_cols = _check_shapes(c, p, q)
    if int(n_class) <= 0:
        raise RuntimeError("n_class must be positive")
    x, ws, wptr, wbytes = _alloc("gl", c, n_rows, n_cols, int(n_class), out, workspace)
    res = DrotResult()
    with torch.cuda.device(c.device):
        rc = lib().drot_group_lasso_drot_ex(
            c.data_ptr(), C_BF16 if c.dtype == torch.bfloat16 else C_F32,
            p.data_ptr(), q.data_ptr(), n_rows, n_cols, int(n_class), float(rho),
            float(r_weight), int(max_iters), float(eps), x.data_ptr(), wptr, wbytes,
            ctypes_byref(res) if sync else None, _stream_handle(c.device, stream))
    check(rc, "group_lasso_drot")
    return x, (res.as_dict() if sync else None), ws


def read_result(workspace, stream=None):
    """Solve record of the last solve that used ``workspace`` (waits for the stream)."""
    ptr = workspace.data_ptr()
    ptr += (-ptr) % 256
    res = DrotResult()
    rc = lib().drot_read_result(ptr, ctypes_byref(res), _stream_handle(workspace.device, stream))
    check(rc, "read_result")
    return res.as_dict()


def quadratic_drot(c, p, q, rho, r_weight, max_iters, eps):
    """Transport plan of the quadratic-regularised OT problem (reference signature)."""
    _check_input(c, "c")
    x, _, _ = solve_qr(c, p, q, rho, r_weight, max_iters, eps)
    return x


def group_lasso_drot(c, p, q, n_class, rho, r_weight, max_iters, eps):
    """Transport plan of the group-lasso-regularised OT problem (reference signature)."""
    _check_input(c, "c")
    x, _, _ = solve_gl(c, p, q, n_class, rho, r_weight, max_iters, eps)
    return x


def group_bounds(n_rows, n_class):
    """Row boundaries of the n_class contiguous groups the GL solver uses."""
    arr = (ctypes.c_int * (n_class + 1))()
    check(lib().drot_gl_group_bounds(n_rows, n_class, arr), "group_bounds")
    return list(arr)


ctypes_byref = ctypes.byref


def tune(kind, c, p, q, rho, r_weight, n_class=1, iters=200, repeats=2, stream=None):
    """Autotune the launch shape of this problem shape (reg_drot.autotune.tune)."""
    from .autotune import tune as _tune
    return _tune(kind, c, p, q, rho, r_weight, n_class, iters, repeats, stream)
