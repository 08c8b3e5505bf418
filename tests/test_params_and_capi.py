"""CPU: parameter mapping known answers, the C ABI surface, host-side errors.

Nothing here launches GPU work: the library is loaded and its host-only
paths (argument checks, parameter helpers) are exercised.
"""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "drot_gb300.h")

f32 = np.float32


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(drot_[a-z0-9_]+)\s*\(", text)))


# --------------------------------------------------------------------------- parameters

@pytest.mark.parametrize("nr,nc,rho", [(1000, 1000, 2.0), (1500, 1000, 2.0), (3, 2, 1.7),
                                       (10000, 10000, 2.0), (5000, 1000, 0.5)])
def test_step_size_matches_float32_restatement(nr, nc, rho):
    # pytorch/src/qr_drot_cuda_kernel.cu:100
    expect = f32(rho) / (f32(nr) + f32(nc))
    assert O.step_size(rho, nr, nc) == float(expect)


@pytest.mark.parametrize("r", [0.0, 1e-5, 1e-3, 1e-2, 10.0])
def test_qr_divisor_conventions(r):
    nr, nc = 1000, 3000
    s = f32(2.0) / (f32(nr) + f32(nc))
    torch_conv = f32(1.0) + (s * f32(r)) * f32(nr + nc)      # qr_drot_cuda_kernel.cu:102
    wrap_conv = f32(1.0) + (s * f32(nr + nc)) * f32(r)       # drot_qr.hpp:262
    assert O.qr_scale(float(s), r, nr, nc, "torch") == float(torch_conv)
    assert O.qr_scale(float(s), r, nr, nc, "wrapper") == float(wrap_conv)


@pytest.mark.parametrize("nr,G", [(1500, 2), (1001, 3), (5000, 10), (7, 2), (2, 2)])
def test_gl_lambda_conventions(nr, G):
    r = 1e-3
    # glr_drot_cuda_kernel.cu:257 (multiply) vs drot_glr.hpp:385 (divide), integer n_rows / G.
    assert O.gl_lambda(r, nr, G, "torch") == float(f32(float(f32(r)) * math.sqrt(nr // G)))
    assert O.gl_lambda(r, nr, G, "wrapper") == float(f32(float(f32(r)) / math.sqrt(nr // G)))


def _bounds_restated(nr, G):
    off = 0.49 if -(-nr // G) <= 256 else 0.49999
    per = f32(nr) / f32(G)
    return [int(float(per * f32(k)) + off) for k in range(G + 1)]


@pytest.mark.parametrize("nr,G,expect", [
    (1500, 2, [0, 750, 1500]),
    (1001, 3, [0, 334, 667, 1001]),
    (2, 2, [0, 1, 2]),
    (2, 3, [0, 1, 1, 2]),
    (5000, 10, [500 * k for k in range(11)]),
    (511, 2, [0, 255, 511]),
])
def test_group_bounds_known_answers(nr, G, expect):
    assert list(O.group_bounds(nr, G)) == expect
    assert _bounds_restated(nr, G) == expect


@pytest.mark.parametrize("nr,G", [(999, 4), (3001, 7), (257, 1), (4097, 16), (300, 256)])
def test_group_bounds_cover_rows(nr, G):
    b = list(O.group_bounds(nr, G))
    assert b == _bounds_restated(nr, G)
    assert b[0] == 0 and b[-1] == nr and all(b[i] <= b[i + 1] for i in range(G))


def test_warm_start_constants():
    nr, nc = 1000, 1000
    s = f32(2.0) / (f32(nr) + f32(nc))
    k = ((f32(1.0) * s) * f32(nr)) * f32(nc) - f32(2.0)
    w = O.warm_start(float(s), nr, nc)
    assert w["phi1"] == ((k + f32(2)) / f32(nr)) / (f32(nc) + f32(nr))
    assert w["phi2"] == ((k + f32(2)) / f32(nc)) / (f32(nc) + f32(nr))
    assert w["a"] == (k + f32(1)) / f32(nr)
    assert w["b"] == (k + f32(1)) / f32(nc)
    assert w["alpha"] == k + f32(1)
    # phi1 + phi2 = s: the warm start's first prox input is the constant s.
    assert abs(float(w["phi1"]) + float(w["phi2"]) - float(s)) < 1e-9


# --------------------------------------------------------------------------- C ABI

def test_library_exports_every_header_symbol(solver_lib):
    names = header_functions()
    assert len(names) >= 18
    from reg_drot import _lib
    missing = [n for n in names if not hasattr(solver_lib, n)]
    assert not missing, missing
    assert sorted(_lib.SIGNATURES) == names


def test_work_size_heuristic_matches_reference_table(solver_lib):
    # core/drot_qr.hpp:236-239
    for n, expect in [(64, 4), (1000, 8), (1500, 8), (2048, 8), (3000, 16), (4096, 16),
                      (10000, 32)]:
        assert solver_lib.drot_q_get_work_size_update_x(n, 1) == expect
        assert solver_lib.drot_gl_get_work_size_update_x(1, n) == expect


def test_library_group_bounds_match_oracle(solver_lib):
    for nr, G in [(1500, 2), (1001, 3), (2, 3), (5000, 10), (777, 5)]:
        arr = (ctypes.c_int * (G + 1))()
        assert solver_lib.drot_gl_group_bounds(nr, G, arr) == 0
        assert list(arr) == list(O.group_bounds(nr, G))
    assert solver_lib.drot_gl_group_bounds(10, 0, None) == 1


def test_status_strings(solver_lib):
    from reg_drot import _lib
    assert _lib.status_string(0) == "ok"
    assert "barrier" in _lib.status_string(3)
    assert _lib.status_string(99) == "unknown status"


def test_invalid_arguments_are_rejected_before_any_device_work(solver_lib):
    from reg_drot._lib import DrotResult
    res = DrotResult()
    rc = solver_lib.drot_qr_solve(None, None, None, 10, 10, 0.1, 1.0, 10, 1e-4, None, None, None,
                                  None, None, None, None, 0, ctypes.byref(res), None)
    assert rc == 1
    rc = solver_lib.drot_gl_solve(None, None, None, 10, 10, 0, 0.1, 1.0, 10, 1e-4, None, None,
                                  None, None, None, None, None, 0, ctypes.byref(res), None)
    assert rc == 1
    out = solver_lib.drot_qr_wrapper(None, None, None, 0, 0, 0.1, 0.0, 10, 1e-4, None, None,
                                     None, None, 1, 1)
    assert not out
    assert solver_lib.drot_last_status() == 1


def test_operator_rejects_host_tensors():
    torch = pytest.importorskip("torch")
    import reg_drot
    c = torch.rand(3, 2)
    p = torch.ones(2) / 2
    q = torch.ones(3) / 3
    with pytest.raises(RuntimeError, match="must be a CUDA tensor"):
        reg_drot.quadratic_drot(c, p, q, 2.0, 1e-2, 100, 1e-4)
    with pytest.raises(RuntimeError, match="must be a CUDA tensor"):
        reg_drot.group_lasso_drot(c, p, q, 2, 2.0, 1e-2, 100, 1e-4)


def test_batch_plan_rejects_bad_descriptors_on_the_host(solver_lib):
    from reg_drot._lib import DrotBatchInstance
    h = ctypes.c_void_p()
    good = dict(n_rows=100, n_cols=50, ld=100, c_offset=0, x_offset=0, p_offset=0, q_offset=0,
                rho=2.0, r_weight=1e-3, eps=1e-4)
    bad = [dict(ld=99), dict(ld=102), dict(n_rows=0), dict(n_cols=-1), dict(c_offset=2),
           dict(x_offset=6), dict(rho=0.0), dict(r_weight=-1.0), dict(p_offset=-1)]
    for change in bad:
        arr = (DrotBatchInstance * 2)()
        for d in arr:
            for k, v in good.items():
                setattr(d, k, v)
        for k, v in change.items():
            setattr(arr[1], k, v)
        assert solver_lib.drot_batch_plan_create(2, arr, 128, ctypes.byref(h)) == 1, change
        assert not h.value
    assert solver_lib.drot_batch_plan_create(0, None, 128, ctypes.byref(h)) == 1
    assert solver_lib.drot_batch_plan_workspace_bytes(None) == 0
    assert solver_lib.drot_batch_plan_tiles(None) == 0
    solver_lib.drot_batch_plan_destroy(None)
    assert solver_lib.drot_qr_batch_launch(None, None, 0, None, None, None, 10, None, 0,
                                           None) == 1
    # the profile log needs a plan, and buffers whenever cap > 0
    assert solver_lib.drot_batch_set_iteration_log(None, None, None, 0) == 1
    assert solver_lib.drot_batch_set_iteration_log(None, None, None, -1) == 1


def test_cost_and_adjoint_reject_bad_arguments_on_the_host(solver_lib):
    from reg_drot._lib import DrotAdjointInstance, DrotCostInstance
    arr = (DrotCostInstance * 1)()
    arr[0].m, arr[0].n, arr[0].ld = 10, 10, 10
    assert solver_lib.drot_sqeuclidean_cost(0, arr, None, None, 16, 1.0, 1, None, None) == 1
    assert solver_lib.drot_sqeuclidean_cost(1, arr, 4, 16, 16, 1.0, 1, 16, None) == 1  # x misaligned
    assert solver_lib.drot_sqeuclidean_cost(1, arr, 16, 16, 12, 1.0, 1, 16, None) == 4  # dim 12
    adj = (DrotAdjointInstance * 1)()
    adj[0].n_rows, adj[0].n_cols, adj[0].ld, adj[0].step_size = 10, 10, 9, 0.1
    adj[0].lambda_ = 2.0
    assert solver_lib.drot_qr_adjoint_workspace_bytes(1, adj) == 0  # ld < n_rows
    assert solver_lib.drot_qr_adjoint_solve(1, adj, None, None, 1e-6, 10, None, 0, None, None) == 1
    assert solver_lib.drot_qr_adjoint_grad(1, adj, None, None, None, None, None, None, 0,
                                           None) == 1
    adj[0].ld, adj[0].lambda_ = 10, 0.0
    assert solver_lib.drot_qr_adjoint_workspace_bytes(1, adj) == 0  # lambda must be > 0


def test_batch_tuning_is_checked_on_the_host(solver_lib):
    from reg_drot._lib import DrotBatchTuning
    names = [n for n, _ in DrotBatchTuning._fields_]
    keep = DrotBatchTuning(*([-1] * len(names)))
    assert solver_lib.drot_batch_set_tuning(ctypes.byref(keep)) == 0
    for name, value in [("prefetch_distance", 9), ("fine_cols", 0), ("item_lines", 0),
                        ("finest_item_lines", 0), ("level_quarters", 5000),
                        ("tail_quarters", 5000), ("fine_cols", 5000)]:
        t = DrotBatchTuning(*([-1] * len(names)))
        setattr(t, name, value)
        assert solver_lib.drot_batch_set_tuning(ctypes.byref(t)) == 1, (name, value)
    assert solver_lib.drot_batch_set_tuning(None) == 0  # the defaults again
    assert solver_lib.drot_batch_resume(None, None, 0, None, None, None, 1, None, 0, None) == 1


def test_gl_adjoint_batch_plan_is_checked_on_the_host(solver_lib):
    from reg_drot._lib import DrotGlAdjointBatchInstance
    good = dict(n_rows=300, n_cols=200, ld=300, n_groups=3, x_offset=0, c_offset=0,
                row_offset=0, col_offset=0, step_size=0.004, lambda_=1e-3)
    bad = [dict(ld=299), dict(n_groups=0), dict(n_groups=301), dict(x_offset=-4),
           dict(row_offset=-1), dict(col_offset=2 ** 31 - 10), dict(step_size=0.0),
           dict(lambda_=-1.0), dict(n_cols=0)]
    h = ctypes.c_void_p()
    for change in bad:
        arr = (DrotGlAdjointBatchInstance * 2)()
        for d in arr:
            for k, v in good.items():
                setattr(d, k, v)
        for k, v in change.items():
            setattr(arr[1], k, v)
        assert solver_lib.drot_gl_adjoint_batch_plan_create(2, arr, ctypes.byref(h)) == 1, change
        assert not h.value
    arr = (DrotGlAdjointBatchInstance * 2)()
    for d in arr:
        for k, v in good.items():
            setattr(d, k, v)
    arr[1].row_offset, arr[1].col_offset = 300, 200
    assert solver_lib.drot_gl_adjoint_batch_plan_create(2, arr, ctypes.byref(h)) == 0
    assert solver_lib.drot_gl_adjoint_batch_workspace_bytes(h) > 0
    assert solver_lib.drot_gl_adjoint_batch_setup(h, arr, None, 0, None, None, None, None,
                                                  None, None, 0, None) == 1
    assert solver_lib.drot_gl_adjoint_batch_step(h, None, None, None, None, 0, None) == 1
    solver_lib.drot_gl_adjoint_batch_plan_destroy(h)
    assert solver_lib.drot_gl_adjoint_batch_workspace_bytes(None) == 0


def test_gl_batch_plan_is_checked_on_the_host(solver_lib):
    """drot_gl_batch_plan_create refuses, before any device work, a class
    count outside 1..n_rows, a negative threshold, a non-positive rho
    (status 1), and a class whose rows from the 16-byte boundary below its
    first row exceed the 4096 rows the launch stages (status 4: 8194 rows
    in two classes of 4097)."""
    from reg_drot._lib import DrotGlBatchInstance
    good = dict(n_rows=300, n_cols=200, ld=300, n_groups=3, c_offset=0, x_offset=0,
                p_offset=0, q_offset=0, rho=2.0, lambda_=1e-3, eps=1e-4)
    h = ctypes.c_void_p()
    for change, status in [(dict(n_groups=0), 1), (dict(n_groups=301), 1),
                           (dict(rho=0.0), 1), (dict(lambda_=-1.0), 1),
                           (dict(n_rows=8194, ld=8196, n_groups=2), 4)]:
        arr = (DrotGlBatchInstance * 2)()
        for d in arr:
            for k, v in good.items():
                setattr(d, k, v)
        for k, v in change.items():
            setattr(arr[1], k, v)
        assert solver_lib.drot_gl_batch_plan_create(2, arr, 128, ctypes.byref(h)) == status, change
        assert not h.value
