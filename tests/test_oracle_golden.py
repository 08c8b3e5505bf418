"""CPU: the oracle against the reference's own numpy implementation.

The golden vectors in tests/golden/npdrot_golden.npz were produced by
tests/golden/gen_golden.py, which imports the reference numpy solver
(numpy/npdrot/solver.py, proximal.py) and records its iterates from the
CUDA reference's cold start (init = p q^T) and, for uniform marginals, its
warm start (init = s * ones).  The FP64 oracle must reproduce those iterates
to rounding (1e-12 relative), which pins its iteration map, warm start,
parameter mapping and GL group shrink to the reference.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "npdrot_golden.npz"))
MANIFEST = json.loads(bytes(GOLD["manifest"]).decode())
ITER_CASES = [m for m in MANIFEST if m["kind"] in ("qr", "gl")]
FIXED_CASES = [m for m in MANIFEST if m["kind"] == "qr_fixedpoint"]


def _inputs(m):
    key = m["inputs"]
    return GOLD[key + "/C"], GOLD[key + "/p"], GOLD[key + "/q"]


def _state64(m, p, q):
    nr, nc, s = m["nr"], m["nc"], m["s"]
    warm = m["start"] == "warm"
    st = O.initial_state(nr, nc, s, p, q, warm=warm, dtype=np.float64)
    if warm:
        # The FP64 restatement of the warm start (core/drot_qr.hpp:322-331).
        k = s * nr * nc - 2.0
        st["phi1"][:] = (k + 2.0) / nr / (nr + nc)
        st["phi2"][:] = (k + 2.0) / nc / (nr + nc)
        st["a"][:] = (k + 1.0) / nr
        st["b"][:] = (k + 1.0) / nc
        st["alpha"][:] = k + 1.0
    return st


def _run64(m, T, C, p, q):
    nr, nc, s = m["nr"], m["nc"], m["s"]
    st0 = _state64(m, p, q)
    if m["kind"] == "qr":
        kappa = 1.0 + s * m["r_weight"] * (nr + nc)
        st = O.qr_solve(C, p, q, s, kappa, T, -1.0, state=st0, dtype=np.float64, threads=1)
        x = st["x"]
        if (T - 1) % 2 == 0:
            # The last iteration was even: X holds X^ - sC (core/kernel_qr.hpp:241-242).
            x = x + s * C
    else:
        st = O.gl_solve(C, p, q, np.array(m["bounds"]), s, m["lam"], T, -1.0, state=st0,
                        dtype=np.float64, threads=1, norm_eps=0.0)
        x = st["x"]
    return x, st


@pytest.mark.parametrize("case", ITER_CASES, ids=[m["name"] for m in ITER_CASES])
def test_oracle_iterates_match_reference_numpy(case):
    C, p, q = _inputs(case)
    x, _ = _run64(case, case["T"], C, p, q)
    ref = GOLD[case["name"] + "/x"]
    assert x.shape == ref.shape
    err = np.abs(x - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("case", [m for m in ITER_CASES if m["T"] == 40 and m["nr"] <= 64],
                         ids=lambda m: m["name"])
def test_oracle_residual_sequence_matches_reference_numpy(case):
    """The per-iteration absolute marginal residual equals numpy's r_primal log."""
    C, p, q = _inputs(case)
    resid = GOLD[case["name"] + "/resid"]
    # GL checks every iteration; QR reports its residual on even iterations only.
    for t in range(1, len(resid) + 1):
        if case["kind"] == "qr" and (t - 1) % 2 == 1:
            continue
        _, st = _run64(case, t, C, p, q)
        assert abs(st["residual"] - resid[t - 1]) <= 1e-12 * max(1.0, resid[t - 1]) + 1e-15


@pytest.mark.parametrize("case", FIXED_CASES, ids=[m["name"] for m in FIXED_CASES])
def test_oracle_fixed_point_matches_reference_numpy(case):
    """Non-uniform marginals: both solvers reach the unique QR solution."""
    name = case["name"]
    C, p, q = GOLD[name + "/C"], GOLD[name + "/p"], GOLD[name + "/q"]
    nr, nc, s = case["nr"], case["nc"], case["s"]
    kappa = 1.0 + s * case["r_weight"] * (nr + nc)
    st0 = O.initial_state(nr, nc, s, p, q, warm=False, dtype=np.float64)
    st = O.qr_solve(C, p, q, s, kappa, 400000, 1e-13, state=st0, dtype=np.float64, threads=1)
    ref = GOLD[name + "/x"]
    assert np.abs(st["x"] - ref).max() / np.abs(ref).max() < 1e-9
    # Both stop at the same iteration count (numpy counts loop passes).
    assert abs(st["n_iter"] - case["iters"]) <= 2


def test_fp32_oracle_tracks_fp64():
    """The FP32 restatement stays within FP32 rounding of the FP64 one."""
    rng = np.random.default_rng(3)
    nr, nc = 150, 90
    C = rng.random((nc, nr)).astype(np.float32)
    p = np.full(nr, 1.0 / nr, np.float32)
    q = np.full(nc, 1.0 / nc, np.float32)
    a = O.quadratic_drot(C, p, q, 2.0, 1e-2, 20000, 1e-4, dtype=np.float32)
    b = O.quadratic_drot(C, p, q, 2.0, 1e-2, 20000, 1e-4, dtype=np.float64)
    assert abs(a["n_iter"] - b["n_iter"]) <= 2
    assert np.abs(a["x"] - b["x"]).max() <= 1e-4 * np.abs(b["x"]).max()
    assert abs(a["objective"] - b["objective"]) <= 1e-5 * abs(b["objective"])


def test_oracle_thread_count_does_not_change_fp32_iterates_beyond_rounding():
    rng = np.random.default_rng(4)
    nr, nc = 64, 48
    C = rng.random((nc, nr)).astype(np.float32)
    p = np.full(nr, 1.0 / nr, np.float32)
    q = np.full(nc, 1.0 / nc, np.float32)
    a = O.group_lasso_drot(C, p, q, 2, 2.0, 1e-2, 5000, 1e-4, threads=1)
    b = O.group_lasso_drot(C, p, q, 2, 2.0, 1e-2, 5000, 1e-4, threads=4)
    assert a["n_iter"] == b["n_iter"]
    assert np.abs(a["x"] - b["x"]).max() <= 1e-6 * np.abs(a["x"]).max()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_oracle_stopped_at_its_own_stop_is_the_converged_solve(dtype):
    """quadratic_drot_at (the QR loop stopped as though the test passed at a
    given even iteration) reproduces the loop's own converged result when
    given the iteration the loop stopped at, bit for bit, and otherwise the
    state a later stop would return."""
    rng = np.random.default_rng(8)
    nr, nc = 120, 70
    C = (rng.random((nc, nr)) + 1e-3).astype(np.float32)
    C /= C.max()
    p = rng.dirichlet(np.ones(nr)).astype(np.float32)
    q = rng.dirichlet(np.ones(nc)).astype(np.float32)
    o = O.quadratic_drot(C, p, q, 2.0, 1e-2, 20000, 1e-4, dtype=dtype)
    assert (o["n_iter"] - 1) % 2 == 0 and o["residual"] < 1e-4
    a = O.quadratic_drot_at(C, p, q, 2.0, 1e-2, o["n_iter"], dtype=dtype)
    assert np.array_equal(a["x"], o["x"])
    assert a["objective"] == o["objective"] and a["residual"] == o["residual"]
    assert a["n_iter"] == o["n_iter"]
    assert O.quadratic_drot_matching(o["n_iter"], o, C, p, q, 2.0, 1e-2, dtype=dtype) is o
    later = O.quadratic_drot_at(C, p, q, 2.0, 1e-2, o["n_iter"] + 2, dtype=dtype)
    assert later["n_iter"] == o["n_iter"] + 2 and later["residual"] < o["residual"]
    with pytest.raises(ValueError):
        O.quadratic_drot_at(C, p, q, 2.0, 1e-2, o["n_iter"] + 1, dtype=dtype)
