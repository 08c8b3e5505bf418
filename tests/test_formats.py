"""CPU: the reference's benchmark data formats and the W2 domain-adaptation
evaluation (reg_drot.formats).

* Cost files: reg_drot.formats.load_cost against a loop restating
  core/utils.hpp:9-24 (raw row-major n_rows x n_cols -> column-major), and
  save/load round trips.
* Plan text and experiment logs: the single-experiment layout
  (core/singleexp_qr.cu:46-53) and the multi-experiment TSV schema
  (core/multiexp_qr.cu:85-89, multiexp_glr.cu:92-98) round-trip.
* W2 evaluation (benchmark/utils/compute_w2_dist.py:59-94) with the FP64
  oracle standing in for the GPU solver: a plan that maps every target
  point to itself gives a distance near 0 (the solver stops on the marginal
  residual, as the reference's); for equal-size uniform groups the
  unregularised OT cost is an assignment, so scipy's exact assignment pins
  the total.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from reg_drot import formats as F


def test_load_cost_matches_reference_reader(tmp_path):
    rng = np.random.default_rng(3)
    n_rows, n_cols = 7, 5
    values = rng.random(n_rows * n_cols).astype(np.float32)  # row-major file
    path = os.path.join(tmp_path, "c.bin")
    values.tofile(path)
    # utils::load: out[col * n_rows + row] = values[row * n_cols + col]
    out = np.empty(n_rows * n_cols, dtype=np.float32)
    for col in range(n_cols):
        for row in range(n_rows):
            out[col * n_rows + row] = values[row * n_cols + col]
    c = F.load_cost(path, n_rows, n_cols)
    assert c.shape == (n_cols, n_rows) and c.dtype == np.float32
    assert np.array_equal(c.reshape(-1), out)
    # and back
    path2 = os.path.join(tmp_path, "c2.bin")
    F.save_cost(path2, c)
    assert np.fromfile(path2, dtype=np.float32).tobytes() == values.tobytes()


def test_load_cost_rejects_short_files(tmp_path):
    path = os.path.join(tmp_path, "short.bin")
    np.zeros(10, dtype=np.float32).tofile(path)
    with pytest.raises(ValueError):
        F.load_cost(path, 4, 3)


def test_plan_text_round_trip():
    rng = np.random.default_rng(5)
    x = (rng.random((3, 4)) * 1e-3).astype(np.float32)  # [n_cols, n_rows]
    text = F.format_plan(x, 0.125, 77)
    lines = text.split("\n")
    assert len(lines) == 3 + 2 + 1  # n_cols rows, objective, n_iter, final newline
    assert lines[0] == "".join("%.10f " % v for v in x[0])
    assert lines[3] == "0.1250000000" and lines[4] == "77"
    x2, obj, it = F.parse_plan(text)
    assert np.allclose(x2, x, rtol=0, atol=1e-10) and obj == 0.125 and it == 77


def test_plan_rows_reader(tmp_path):
    path = os.path.join(tmp_path, "plan.txt")
    with open(path, "w") as f:
        f.write("0.5 0.25 \n0.125 1.0 \n")
    assert np.array_equal(F.load_plan_rows(path), np.array([[0.5, 0.25], [0.125, 1.0]], np.float32))


def test_experiment_log_schema_round_trip():
    qr = F.log_header("quad_drot")
    gl = F.log_header("gl_drot")
    assert qr.split("\t")[:4] == ["test_index", "method", "n", "m"]
    assert gl.split("\t")[4] == "n_class" and len(gl.split("\t")) == len(qr.split("\t")) + 1
    rows = [F.log_row(1, 1000, 800, 1e-4, True, 2.0, 1e-3, 20000, 35.5, 0.0123, 2851),
            F.log_row(2, 1000, 800, 1e-4, True, 2.0, 1e-3, 20000, 36.0, 0.0124, 2853)]
    grow = F.log_row(1, 1500, 1000, 1e-4, True, 2.0, 1e-3, 20000, 4.0, 0.5, 257, n_class=2)
    text = "\n".join([qr] + rows + [gl, grow]) + "\n"
    recs = F.parse_log(text)
    assert len(recs) == 3
    assert recs[0]["method"] == "quad_drot" and recs[0]["n"] == 1000 and recs[0]["n_iteration"] == 2851
    assert recs[0]["runtime_ms_per_iteration"] == pytest.approx(35.5 / 2851, rel=1e-6)
    assert recs[2]["method"] == "gl_drot" and recs[2]["n_class"] == 2 and recs[2]["rho"] == 2.0
    # the reference prints 8 decimals
    assert rows[0].split("\t")[4] == "0.00010000"


def _oracle_solver(c, p, q):
    o = O.quadratic_drot(np.asarray(c, np.float32), np.asarray(p, np.float32),
                         np.asarray(q, np.float32), F.W2_RHO, 0.0, F.W2_MAX_ITERS, F.W2_EPS)
    return o["x"]


def _clouds(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(n // 2, 2)) + np.array([2.0, 0.0])
    b = rng.normal(size=(n - n // 2, 2)) - np.array([2.0, 0.0])
    return np.concatenate([a, b]).astype(np.float32)


def test_w2_of_an_identity_plan_is_near_zero():
    # The adapted points are the target points themselves, so the exact W2
    # is 0.  The solver stops on the marginal residual alone (2e-6, as the
    # reference), where the plan is feasible but not yet exactly optimal, so
    # the distance is small rather than 0: compare with a shuffled plan.
    n = 24
    xt = _clouds(n, 1)
    plan = np.eye(n, dtype=np.float32) / n
    assert np.allclose(F.adapt_target_domain(xt, plan, np.ones(n, np.float32) / n), xt, atol=1e-5)
    total, norm = F.group_w2_distance(xt, plan, 2, solver=_oracle_solver)
    shuffled = plan[np.random.default_rng(4).permutation(n)]
    total_s, _ = F.group_w2_distance(xt, shuffled, 2, solver=_oracle_solver)
    assert 0.0 <= total < 0.01 * total_s and norm >= 0.0


def test_w2_matches_exact_assignment():
    from scipy.optimize import linear_sum_assignment
    n = 24
    xt = _clouds(n, 2)
    rng = np.random.default_rng(9)
    perm = rng.permutation(n)
    # a plan that sends target point perm[k] to source k, plus a small spread
    plan = np.full((n, n), 0.02 / (n * n), dtype=np.float32)
    plan[perm, np.arange(n)] += 0.98 / n
    p = np.ones(n, np.float32) / n
    adapted = F.adapt_target_domain(xt, plan, p)
    total, _ = F.group_w2_distance(xt, plan, 2, solver=_oracle_solver)
    expect = 0.0
    for g in range(2):
        s, t = round(n / 2 * g), round(n / 2 * (g + 1))
        c = ((adapted[s:t, None, :].astype(np.float64) - xt[None, s:t, :]) ** 2).sum(-1)
        r, k = linear_sum_assignment(c)
        expect += c[r, k].sum() / (t - s)
    assert total == pytest.approx(expect, rel=1e-3)
