"""GPU: the batched QR solver (reg_drot.batch.QRBatch, drot_qr_batch_launch).

Per instance the batch runs the iteration of drot_quadratic_drot
(core/drot_qr.hpp:159-234 with the operator's parameters,
pytorch/src/qr_drot_cuda_kernel.cu:100-102), so each instance is checked
against the FP32 oracle with the single-instance parity bars:
  * ||X - X_o||_F <= 1e-5 ||X_o||_F and max|X - X_o| <= 1e-4 max|X_o|,
  * objective within 1e-5 relative,
  * n_iter within one stop check (2 iterations) of the oracle; X and the
    objective are compared on every instance, against the oracle stopped at
    the instance's iteration when the stop moved (oracle.quadratic_drot_at).
The row and column sums are accumulated per tile (FP32 inside a tile, in a
fixed order across tiles), which is a different summation order from the
oracle's FP64 sums -- hence tolerances, not bitwise equality.  Runs of the
same plan are bitwise identical (tiles are taken dynamically, but every tile
writes its own partial slots).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

RTOL_X = 1e-5
RTOL_XMAX = 1e-4
RTOL_OBJ = 1e-5

SHAPES = [(64, 64), (517, 1283), (1000, 700), (129, 2048), (2048, 65), (300, 200), (513, 511),
          (2, 3), (1537, 97)]


def _instance(nr, nc, seed, marg="uniform"):
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g, dtype=torch.float32) + 1e-3
    c = c / c.max()
    if marg == "uniform":
        p = torch.ones(nr) / nr
        q = torch.ones(nc) / nc
    else:
        rng = np.random.default_rng(seed)
        p = torch.from_numpy(rng.dirichlet(np.ones(nr)).astype(np.float32))
        q = torch.from_numpy(rng.dirichlet(np.ones(nc)).astype(np.float32))
    return c, p, q


def _batch(shapes, cuda, rho=2.0, rw=1e-3, eps=1e-4, marg="uniform", cpt=None, dtype=None,
           tuning=None):
    from reg_drot.batch import QRBatch
    insts = [_instance(nr, nc, 100 + k, marg) for k, (nr, nc) in enumerate(shapes)]
    B = QRBatch(shapes, rho, rw, eps, device=cuda, cols_per_tile=cpt, tuning=tuning)
    c = B.pack_c([i[0].to(cuda) for i in insts], dtype=dtype or torch.float32)
    p, q = B.pack_marginals([i[1] for i in insts], [i[2] for i in insts])
    return B, insts, c, p, q


def _assert_close_x(xg, xo, floor=0.0):
    """Relative errors of X; `floor` (the scale of the plan p q^T) stands in
    for ||X_o|| while the warm-started iterate is still (almost) all zero,
    where relative errors of near-zero entries mean nothing."""
    xg = np.asarray(xg, dtype=np.float64)
    xo = np.asarray(xo, dtype=np.float64)
    fro = np.linalg.norm(xg - xo) / max(np.linalg.norm(xo), floor, 1e-300)
    mx = np.abs(xg - xo).max() / max(np.abs(xo).max(), floor, 1e-300)
    assert fro <= RTOL_X and mx <= RTOL_XMAX, (fro, mx)


def _assert_same_solution(rb, xb, rs, xs, ci, pi, qi, rho=2.0, rw=1e-3):
    """A batch instance (record rb, plan xb) against the single-instance
    solver (rs, xs) on the same inputs: equal when both stopped at the same
    iteration; when one stop moved by a check, each against the oracle
    stopped at its own iteration."""
    assert abs(rb["n_iter"] - rs["n_iter"]) <= 2
    if rb["n_iter"] == rs["n_iter"]:
        _assert_close_x(xb.cpu().numpy(), xs.cpu().numpy())
        return
    for r, x in ((rb, xb), (rs, xs)):
        o = O.quadratic_drot_at(ci.numpy(), pi.numpy(), qi.numpy(), rho, rw, r["n_iter"])
        _assert_close_x(x.cpu().numpy(), o["x"])


@pytest.mark.parametrize("cpt", [32, 128, 256])
@pytest.mark.parametrize("marg", ["uniform", "dirichlet"])
def test_batch_converged_matches_oracle(cuda, solver_lib, cpt, marg):
    B, insts, c, p, q = _batch(SHAPES, cuda, marg=marg, cpt=cpt)
    x, info = B.solve(c, p, q, 20000)
    xs = B.unpack(x)
    iters = set()
    for k, (ci, pi, qi) in enumerate(insts):
        o = O.quadratic_drot(ci.numpy(), pi.numpy(), qi.numpy(), 2.0, 1e-3, 20000, 1e-4)
        r = info[k]
        assert r["converged"] == 1, (k, r)
        assert abs(r["n_iter"] - o["n_iter"]) <= 2, (k, r, o["n_iter"])
        iters.add(r["n_iter"])
        o = O.quadratic_drot_matching(r["n_iter"], o, ci.numpy(), pi.numpy(), qi.numpy(),
                                      2.0, 1e-3)
        _assert_close_x(xs[k].cpu().numpy(), o["x"])
        assert abs(r["objective"] - o["objective"]) <= RTOL_OBJ * abs(o["objective"])
        assert r["residual"] < 1e-4
    assert len(iters) > 1  # the instances really stopped at different iterations


@pytest.mark.parametrize("mi", [1, 2, 7, 30, 31])
def test_batch_fixed_iterations_match_oracle(cuda, solver_lib, mi):
    # eps = 0: nothing converges; X after exactly mi iterations (odd mi
    # leaves the folded X, as the reference's loop does).  Around iteration 30
    # the warm-started X of several instances is all zero but for a few tiny
    # entries, so the comparison is scaled by ||p q^T|| there.
    B, insts, c, p, q = _batch(SHAPES, cuda, eps=0.0, cpt=64)
    x, info = B.solve(c, p, q, mi)
    xs = B.unpack(x)
    for k, (ci, pi, qi) in enumerate(insts):
        o = O.quadratic_drot(ci.numpy(), pi.numpy(), qi.numpy(), 2.0, 1e-3, mi, 0.0)
        assert info[k]["converged"] == 0 and info[k]["n_iter"] == mi + 1
        assert info[k]["iters_run"] == mi
        floor = float(np.linalg.norm(pi.numpy()) * np.linalg.norm(qi.numpy()))
        _assert_close_x(xs[k].cpu().numpy(), o["x"], floor)


def test_batch_matches_single_instance_solver(cuda, solver_lib):
    import reg_drot
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=128)
    x, info = B.solve(c, p, q, 20000)
    xs = B.unpack(x)
    for k, (ci, pi, qi) in enumerate(insts):
        xr, ir, _ = reg_drot.solve_qr(ci.to(cuda), pi.to(cuda), qi.to(cuda), 2.0, 1e-3, 20000, 1e-4)
        _assert_same_solution(info[k], xs[k], ir, xr, ci, pi, qi)


def test_batch_deterministic_and_padding_ignored(cuda, solver_lib):
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=64)
    x1, i1 = B.solve(c, p, q, 20000)
    x1 = x1.clone()
    # Rows between n_rows and ld are the caller's: fill them with NaN.
    c2 = c.clone()
    for k, (nr, nc) in enumerate(SHAPES):
        ld, off = B.lds[k], B.offsets[k]
        if ld > nr:
            c2[off:off + ld * nc].view(nc, ld)[:, nr:] = float("nan")
    x2, i2 = B.solve(c2, p, q, 20000)
    for k in range(len(SHAPES)):
        assert torch.equal(B.view(x1, k), B.view(x2, k)), k
        assert i1[k] == i2[k]


def test_batch_cuda_graph_replay(cuda, solver_lib):
    B, insts, c, p, q = _batch(SHAPES[:5], cuda, cpt=128)
    x_ref, i_ref = B.solve(c, p, q, 20000)
    x_ref = x_ref.clone()
    x = B.empty_x()
    g = B.capture(c, p, q, x, 20000)
    for _ in range(2):
        x.fill_(float("nan"))
        g.replay()
        info = B.results()
        for k in range(B.n):
            assert torch.equal(B.view(x, k), B.view(x_ref, k)), k
        assert info == i_ref


def test_batch_autotune_picks_a_candidate(cuda, solver_lib):
    from reg_drot.batch import TILE_CANDIDATES
    B, insts, c, p, q = _batch(SHAPES, cuda)
    x, info = B.solve(c, p, q, 20000)
    assert B.cols_per_tile in TILE_CANDIDATES
    assert all(r["converged"] == 1 for r in info)


def test_batch_bf16_cost(cuda, solver_lib):
    # BF16-stored C, FP32 iterates: the oracle runs on the rounded cost.
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=128, dtype=torch.bfloat16)
    x, info = B.solve(c, p, q, 20000)
    xs = B.unpack(x)
    for k, (ci, pi, qi) in enumerate(insts):
        cr = ci.to(torch.bfloat16).float().numpy()
        o = O.quadratic_drot(cr, pi.numpy(), qi.numpy(), 2.0, 1e-3, 20000, 1e-4)
        assert abs(info[k]["n_iter"] - o["n_iter"]) <= 2
        o = O.quadratic_drot_matching(info[k]["n_iter"], o, cr, pi.numpy(), qi.numpy(), 2.0, 1e-3)
        _assert_close_x(xs[k].cpu().numpy(), o["x"])


def test_batch_rejects_bad_buffers(cuda, solver_lib):
    B, insts, c, p, q = _batch(SHAPES[:3], cuda, cpt=64)
    with pytest.raises(RuntimeError):
        B.solve(c[:-1], p, q, 10)
    with pytest.raises(RuntimeError):
        B.solve(c, p[:-1], q, 10)
    with pytest.raises(RuntimeError):
        B.solve(c.double(), p, q, 10)


def test_batch_with_more_tiles_than_ctas(cuda, solver_lib):
    # More tiles than CTAs (12 instances x 2-3 bands x 16 chunks of 64
    # columns > 304), so CTAs take several tiles per iteration from the
    # counter and instances leave the list at different iterations.  Every
    # instance must still match the single-instance solver.
    import reg_drot
    shapes = [(600 + 80 * k, 1024) for k in range(12)]
    B, insts, c, p, q = _batch(shapes, cuda, cpt=64, marg="dirichlet")
    assert B.tiles(64) > 304
    x, info = B.solve(c, p, q, 20000)
    xs = B.unpack(x)
    for k, (ci, pi, qi) in enumerate(insts):
        xr, ir, _ = reg_drot.solve_qr(ci.to(cuda), pi.to(cuda), qi.to(cuda), 2.0, 1e-3, 20000, 1e-4)
        assert info[k]["converged"] == 1
        _assert_same_solution(info[k], xs[k], ir, xr, ci, pi, qi)
    assert len({r["n_iter"] for r in info}) > 1


@pytest.mark.parametrize("tuning", [{"finest_cols": 0},
                                    {"finest_cols": 0, "level_quarters": 0, "tail_quarters": 0},
                                    {"prefetch_distance": 0, "item_lines": 256},
                                    {"fine_cols": 64, "finest_cols": 16, "level_quarters": 64},
                                    {"tail_quarters": 0},
                                    {"tail_quarters": 4096, "level_quarters": 0}])
def test_batch_tile_levels_match_oracle(cuda, solver_lib, tuning):
    # The default plan moves to 128-column and then 32-column tiles (with
    # 64-line dual items) as instances converge, and puts the smallest
    # instances on the finer levels from the start; these plans stop at the
    # fine level, keep the coarse tiles throughout, use short dual items
    # without the prefetch, move early to narrower levels, keep every
    # instance on the base level, or put every instance on the finest level
    # while the base level stays coarse.  Every schedule must give the
    # oracle's solution.
    B, insts, c, p, q = _batch(SHAPES, cuda, marg="dirichlet", cpt=256, tuning=tuning)
    x, info = B.solve(c, p, q, 20000)
    xs = B.unpack(x)
    for k, (ci, pi, qi) in enumerate(insts):
        o = O.quadratic_drot(ci.numpy(), pi.numpy(), qi.numpy(), 2.0, 1e-3, 20000, 1e-4)
        assert info[k]["converged"] == 1
        assert abs(info[k]["n_iter"] - o["n_iter"]) <= 2, (k, info[k], o["n_iter"])
        o = O.quadratic_drot_matching(info[k]["n_iter"], o, ci.numpy(), pi.numpy(), qi.numpy(),
                                      2.0, 1e-3)
        _assert_close_x(xs[k].cpu().numpy(), o["x"])


def test_batch_iteration_log(cuda, solver_lib):
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=128)
    times, tiles = B.iteration_log(100000, 128)
    x, info = B.solve(c, p, q, 20000)
    n = max(r["iters_run"] for r in info)
    t = times[:n].cpu().numpy()
    assert (t > 0).all()
    assert (np.diff(t, axis=1) >= 0).all() and (t[1:, 0] >= t[:-1, 3]).all()
    a = tiles[:n].cpu().numpy()
    assert a[0] == B.tiles(128) and (np.diff(a) <= 0).all()
    B.iteration_log(0, 128)
