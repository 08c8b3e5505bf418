"""CPU: the state mapping of the numpy-API backend (reg_drot.npdrot).

reg_drot.npdrot runs the reference's numpy loop (numpy/npdrot/solver.py:7-189)
on the device solver by translating regdrot's start from ``init`` into the
device state (initial_state).  Here that translation is checked without a GPU:
the FP64 oracle, started from initial_state(init), reproduces the reference's
own numpy outputs stored in tests/golden (regdrot with max_iters = T - 1 and
its final prox = T device iterations), to 1e-12.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "npdrot_golden.npz")


def _cases():
    z = np.load(GOLD)
    manifest = json.loads(bytes(z["manifest"]).decode())
    return z, [m for m in manifest if m.get("kind") in ("qr", "gl") and m["T"] >= 2]


def test_initial_state_reproduces_numpy_outputs():
    pytest.importorskip("torch")
    from reg_drot.npdrot import initial_state  # host-side numpy; no device work
    z, cases = _cases()
    assert len(cases) >= 20
    for m in cases:
        inp = m["inputs"]
        C = z[f"{inp}/C"]  # [nc, nr]
        p, q = z[f"{inp}/p"], z[f"{inp}/q"]
        nr, nc, T, s = m["nr"], m["nc"], m["T"], m["s"]
        init = np.outer(p, q) if m["start"] == "cold" else np.full((nr, nc), s)
        st = initial_state(init, p, q)
        state = {"x": np.ascontiguousarray(st["x"].T), "a": st["a"], "b": st["b"],
                 "phi1": st["phi1"], "phi2": st["phi2"], "alpha": st["alpha"]}
        if m["kind"] == "qr":
            kappa = 1.0 + s * m["r_weight"] * (nr + nc)
            o = O.qr_solve(C, p, q, s, kappa, T, -1.0, state=state, dtype=np.float64)
            x = o["x"]
            if (T - 1) % 2 == 0:  # the numpy loop never leaves X folded
                x = np.maximum(x + s * C, 0.0)
        else:
            o = O.gl_solve(C, p, q, np.array(m["bounds"], np.int32), s, m["lam"], T, -1.0,
                           state=state, dtype=np.float64, norm_eps=0.0)
            x = o["x"]
        ref = z[f"{m['name']}/x"]
        err = np.abs(x - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (m["name"], err)


@pytest.mark.parametrize("groups,m,expect", [([(0, 3), (3, 7)], 7, [0, 3, 7]),
                                             ([(4, 9), (0, 4)], 9, [0, 4, 9])])
def test_group_pairs_to_bounds(groups, m, expect):
    pytest.importorskip("torch")
    from reg_drot.npdrot import group_bounds_from_pairs
    assert group_bounds_from_pairs(groups, m) == expect
    with pytest.raises(NotImplementedError):
        group_bounds_from_pairs([(0, 3), (4, 7)], 7)
