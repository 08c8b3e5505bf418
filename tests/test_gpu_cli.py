"""GPU: the experiment drivers (reg_drot.cli) on raw cost files.

They mirror the reference's executables (core/singleexp_qr.cu,
core/singleexp_glr.cu, core/multiexp_qr.cu, core/multiexp_glr.cu): the same
arguments, file names and outputs, solving through the host-buffer C-ABI
wrappers.  Checked: the single-experiment plan text against the oracle with
the C++ wrappers' parameters (X within 1e-5 relative), the benchmark TSV rows
(one per run after the warm-up run 0) and the written GL plans.
"""
import io
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


def _cost(nr, nc, seed):
    rng = np.random.default_rng(seed)
    c = rng.random((nc, nr)).astype(np.float32) + 1e-3
    return c / c.max()


def test_singleexp_qr_prints_the_wrapper_solve(tmp_path, solver_lib):
    from reg_drot import cli, formats as F
    nr, nc = 300, 200
    c = _cost(nr, nc, 1)
    path = str(tmp_path / "cmatrix.tmp")
    F.save_cost(path, c)
    buf = io.StringIO()
    assert cli.main(["singleexp_qr", path, str(nr), str(nc), "2.0", "0.01", "1"], buf) == 0
    x, obj, nit = F.parse_plan(buf.getvalue())
    s = O.step_size(2.0, nr, nc)
    o = O.qr_solve(c, np.full(nr, 1 / nr, np.float32), np.full(nc, 1 / nc, np.float32), s,
                   O.qr_scale(s, 0.01, nr, nc, "wrapper"), cli.MAX_ITERS, cli.EPS)
    assert abs(nit - o["n_iter"]) <= 2
    assert np.linalg.norm(x - o["x"]) <= 2e-5 * np.linalg.norm(o["x"])  # 10-digit text
    assert obj == pytest.approx(o["objective"], rel=1e-4)


def test_multiexp_qr_benchmark_log(tmp_path, solver_lib):
    from reg_drot import cli, formats as F
    nr, nc, n_tests = 256, 128, 3
    for k in range(n_tests):
        F.save_cost(str(tmp_path / f"cmatrix_{nr}_{nc}_{k}"), _cost(nr, nc, 10 + k))
    buf = io.StringIO()
    args = ["multiexp_qr", str(tmp_path), str(nr), str(nc), str(n_tests), "2.0", "0.01", "1",
            "1e-4", "20000", "1"]
    assert cli.main(args, buf) == 0
    rows = F.parse_log(buf.getvalue())
    assert [r["test_index"] for r in rows] == [1, 2]
    for r in rows:
        assert r["method"] == "quad_drot" and r["n"] == nr and r["m"] == nc
        assert r["n_iteration"] > 0 and r["objective"] > 0 and r["runtime_ms"] > 0
    buf = io.StringIO()
    assert cli.main(args[:-1] + ["0"], buf) == 0
    assert "# Tests = 2" in buf.getvalue() and "Time Per Iteration (ms)" in buf.getvalue()


def test_multiexp_glr_writes_plans(tmp_path, solver_lib):
    from reg_drot import cli, formats as F
    nr, nc, G, n_tests = 200, 100, 2, 2
    cdir, odir = tmp_path / "class", tmp_path / "out"
    cdir.mkdir()
    odir.mkdir()
    for k in range(n_tests):
        F.save_cost(str(cdir / f"cmatrix_{nr}_{nc}_{G}_{k}"), _cost(nr, nc, 20 + k))
    buf = io.StringIO()
    assert cli.main(["multiexp_glr", str(cdir), str(odir), str(nr), str(nc), str(G), str(n_tests),
                     "2.0", "0.001", "1", "1e-4", "20000", "1"], buf) == 0
    rows = F.parse_log(buf.getvalue())
    assert len(rows) == 1 and rows[0]["method"] == "gl_drot" and rows[0]["n_class"] == G
    for k in range(n_tests):
        plan = F.load_plan_rows(str(odir / f"drot-gl_{nr}_{nc}_{G}_{k}"))
        assert plan.shape == (nr, nc)                 # n_rows lines of n_cols values
        assert abs(plan.sum() - 1.0) < 1e-3          # a transport plan of unit mass
        assert os.path.getsize(str(odir / f"drot-gl_{nr}_{nc}_{G}_{k}")) > 0
