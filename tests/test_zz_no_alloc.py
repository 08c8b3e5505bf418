"""GPU: the allocation-free entry point against the regular one.

drot_quadratic_drot_noalloc serves callers that may not allocate device
memory when they call the solver (latency-critical loops where cudaMalloc
would synchronise the device, hosts whose device memory belongs to another
allocator): it keeps its workspace in a fixed array inside the library.
This file is collected after every other test file, so a run that stops at
the first failure has run everything else first; it also passes when run
alone in a fresh process.

The check: through the C ABI, two calls in a row on the same inputs give the
result of drot_quadratic_drot (the reg_drot.quadratic_drot entry point) with
its own workspace -- the same iteration count, and X and the objective within
the parity tolerance used for the solver (1e-5 relative); the second call
also shows that what the first left in the shared array does not leak in,
and that it changes neither torch's reserved pool nor the driver's free
device memory (it allocates nothing).
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _problem(nr, nc, seed):
    """Inputs in the style of the reference's own test (pytorch/test.py:436-440)."""
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g) + 1e-3
    c = c / c.max()
    p = torch.ones(nr) / nr
    q = torch.ones(nc) / nc
    return c, p, q


def test_noalloc_matches_regular_entry_point_twice(cuda, solver_lib):
    from reg_drot._lib import DrotResult
    import reg_drot

    L = solver_lib
    for (nr, nc, seed) in ((1000, 700, 3), (517, 1283, 4)):
        c, p, q = (t.to(cuda).contiguous() for t in _problem(nr, nc, seed))
        eps = 1e-4
        x_ref, info_ref, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 20000, eps)
        assert info_ref["converged"] == 1
        stream = torch.cuda.current_stream().cuda_stream
        outs = [torch.full_like(c, float("nan")) for _ in range(2)]
        mem = []
        for call, x in enumerate(outs):
            res = DrotResult()
            rc = L.drot_quadratic_drot_noalloc(c.data_ptr(), p.data_ptr(), q.data_ptr(), nr, nc,
                                               2.0, 1e-3, 20000, eps, x.data_ptr(),
                                               ctypes.byref(res), stream)
            torch.cuda.synchronize()
            # Device memory after the call: torch's pool and the driver's free
            # bytes.  The first call may load the library's device code; from
            # then on a call must not change either.
            mem.append((torch.cuda.memory_reserved(cuda), torch.cuda.mem_get_info(cuda)[0]))
            assert rc == 0, (call, rc)
            assert res.status == 0 and res.converged == 1
            assert res.n_iter == info_ref["n_iter"], (call, res.n_iter, info_ref["n_iter"])
            err = float(torch.linalg.norm(x.double() - x_ref.double()) /
                        torch.linalg.norm(x_ref.double()))
            assert err <= 1e-5, (call, err)
            assert abs(res.objective - info_ref["objective"]) <= 1e-5 * abs(info_ref["objective"])
        assert mem[1] == mem[0], mem


def test_noalloc_rejects_problems_beyond_its_array(cuda, solver_lib):
    from reg_drot._lib import DrotResult

    L = solver_lib
    nr = nc = 60000  # needs more workspace than the fixed array holds
    assert L.drot_quadratic_drot_workspace_bytes(nr, nc) > (16 << 20)
    buf = torch.zeros(16, device=cuda)
    res = DrotResult()
    rc = L.drot_quadratic_drot_noalloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), nr, nc,
                                       2.0, 1e-3, 10, 1e-4, buf.data_ptr(), ctypes.byref(res),
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == 5  # DROT_ERR_WORKSPACE: rejected before any device work
    assert float(buf.abs().sum()) == 0.0
