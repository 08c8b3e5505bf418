"""The header-compatible C++ entry points (include/drot_qr.hpp, drot_glr.hpp).

CPU: a translation unit that includes both headers and instantiates every
template compiles and links against libdrot_gb300.so.
GPU: the same program, run the way the reference's drivers call these entry
points, produces the oracle's iterates.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "native", "compat_run.cpp")
LIBDIR = os.path.join(REPO, "regularized-drot_gb300", "reg_drot")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path, solver_lib):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "compat_run")
    cudalib = os.path.join(CUDA, "lib64")
    if not os.path.isdir(cudalib):
        cudalib = os.path.join(CUDA, "lib")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                           "-I", os.path.join(CUDA, "include"), SRC, "-o", exe,
                           "-L", LIBDIR, "-ldrot_gb300", f"-Wl,-rpath,{LIBDIR}",
                           "-L", cudalib, "-lcudart", f"-Wl,-rpath,{cudalib}"])
    return exe


def test_compat_headers_compile_and_link(tmp_path, solver_lib):
    assert os.path.exists(_build(tmp_path, solver_lib))


@pytest.mark.gpu
def test_compat_entry_points_match_oracle(tmp_path, solver_lib, oracle_mod, cuda):
    O = oracle_mod
    exe = _build(tmp_path, solver_lib)
    nr, nc, G = 300, 180, 3
    rng = np.random.default_rng(77)
    c = (rng.random((nc, nr), dtype=np.float32) + 1e-3)
    c /= c.max()
    p = np.full(nr, 1.0 / nr, np.float32)
    q = np.full(nc, 1.0 / nc, np.float32)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(c.tobytes() + p.tobytes() + q.tobytes())
    out = subprocess.run([exe, str(nr), str(nc), str(G), str(inp), str(tmp_path / "x")],
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines()}
    s = O.step_size(2.0, nr, nc)
    # wrapper convention: scale = 1 + s*(m+n)*r (core/drot_qr.hpp:262)
    o = O.qr_solve(c, p, q, s, O.qr_scale(s, 1e-2, nr, nc, "wrapper"), 20000, 1e-4)
    for name in ("qrw",):
        x = np.fromfile(tmp_path / f"x_{name}.bin", dtype=np.float32).reshape(nc, nr)
        assert int(lines["qr_wrapper"][0]) == o["n_iter"]
        assert np.linalg.norm(x - o["x"]) <= 1e-5 * np.linalg.norm(o["x"])
    # device loop with the torch divisor convention (scale computed by the caller)
    o2 = O.qr_solve(c, p, q, s, O.qr_scale(s, 1e-2, nr, nc, "torch"), 20000, 1e-4)
    x = np.fromfile(tmp_path / "x_qrd.bin", dtype=np.float32).reshape(nc, nr)
    assert int(lines["qr_device"][0]) == o2["n_iter"]
    assert np.linalg.norm(x - o2["x"]) <= 1e-5 * np.linalg.norm(o2["x"])
    lam = O.gl_lambda(1e-2, nr, G, "wrapper")
    og = O.gl_solve(c, p, q, O.group_bounds(nr, G), s, lam, 20000, 1e-4)
    og64 = O.gl_solve(c, p, q, O.group_bounds(nr, G), s, lam, 20000, 1e-4, dtype=np.float64)
    x = np.fromfile(tmp_path / "x_glw.bin", dtype=np.float32).reshape(nc, nr)
    assert abs(int(lines["gl_wrapper"][0]) - og["n_iter"]) <= max(1, og["n_iter"] // 50)
    ref_err = np.linalg.norm(og["x"] - og64["x"]) / np.linalg.norm(og64["x"])
    err = np.linalg.norm(x - og64["x"]) / np.linalg.norm(og64["x"])
    assert err <= max(1e-5, 2 * ref_err)
