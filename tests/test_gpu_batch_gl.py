"""GPU: the batched group-lasso solver (reg_drot.batch.GLBatch,
drot_gl_batch_plan_create + drot_qr_batch_launch).

Per instance the batch runs the GL loop of reg_drot.group_lasso_drot
(core/drot_glr.hpp:242-355 with the operator's parameters,
pytorch/src/glr_drot_cuda_kernel.cu:255-257): the classes' row ranges of the
reference kernels, the shrink max(1 - lambda / (||Y_g|| + 1e-9), 0), the stop
test on every iteration (residual <= eps), n_iter = iterations run.  The bars
are those of the single-instance GL parity tests: the group shrink amplifies
FP32 rounding in groups it nearly zeroes, so X and the objective must be as
close to the FP64 oracle as the FP32 restatement of the reference is (within
max(1e-5, 2 x the FP32 oracle's error)), with the stop within
max(1, n_iter / 50) iterations of the FP32 oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

# (n_rows, n_cols, n_class): small classes (one 128-row step), classes
# starting off a 16-byte boundary (1001 / 3, 750 / ...), tall classes
# (1500, 2048 rows: several 512-row steps per column), wide panels.
SHAPES = [(60, 40, 2), (300, 200, 3), (1001, 200, 3), (1500, 1000, 2), (4096, 300, 2),
          (100, 1100, 5), (513, 511, 4)]


def _instance(nr, nc, seed):
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g) + 1e-3
    c = c / c.max()
    return c, torch.ones(nr) / nr, torch.ones(nc) / nc


def _batch(shapes, cuda, rw=1e-3, eps=1e-4, cpt=None, dtype=torch.float32, convention="operator"):
    from reg_drot.batch import GLBatch
    insts = [_instance(nr, nc, 300 + k) for k, (nr, nc, _) in enumerate(shapes)]
    B = GLBatch([(nr, nc) for nr, nc, _ in shapes], [g for _, _, g in shapes], 2.0, rw, eps,
                device=cuda, cols_per_tile=cpt, convention=convention)
    c = B.pack_c([i[0].to(cuda) for i in insts], dtype=dtype)
    p, q = B.pack_marginals([i[1] for i in insts], [i[2] for i in insts])
    return B, insts, c, p, q


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("cpt", [64, 256])
def test_gl_batch_converged_matches_fp64_oracle(cuda, solver_lib, cpt):
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=cpt)
    x, info = B.solve(c, p, q, 20000)
    for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(SHAPES, insts)):
        s = O.step_size(2.0, nr, nc)
        lam = B.lambdas[k]
        bnd = O.group_bounds(nr, G)
        o32 = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), bnd, s, lam, 20000, 1e-4)
        o64 = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), bnd, s, lam, 20000, 1e-4,
                         dtype=np.float64)
        r = info[k]
        assert r["converged"] == 1, (k, r)
        assert abs(r["n_iter"] - o32["n_iter"]) <= max(1, o32["n_iter"] // 50), (k, r, o32["n_iter"])
        ref = _rel(o32["x"], o64["x"])
        err = _rel(B.view(x, k).cpu().numpy(), o64["x"])
        assert err <= max(1e-5, 2.0 * ref), (k, err, ref)
        ref_obj = abs(o32["objective"] - o64["objective"])
        assert abs(r["objective"] - o64["objective"]) <= max(1e-5 * abs(o64["objective"]),
                                                             2.0 * ref_obj), k
        assert r["residual"] <= 1e-4 * 1.0001


@pytest.mark.parametrize("mi", [1, 2, 7])
def test_gl_batch_fixed_iterations_match_oracle(cuda, solver_lib, mi):
    B, insts, c, p, q = _batch(SHAPES, cuda, eps=0.0, cpt=128)
    x, info = B.solve(c, p, q, mi)
    for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(SHAPES, insts)):
        s = O.step_size(2.0, nr, nc)
        o = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), O.group_bounds(nr, G), s,
                       B.lambdas[k], mi, 0.0)
        assert info[k]["converged"] == 0 and info[k]["n_iter"] == mi == o["n_iter"]
        floor = float(np.linalg.norm(pi.numpy()) * np.linalg.norm(qi.numpy()))
        xg = B.view(x, k).cpu().numpy().astype(np.float64)
        assert np.linalg.norm(xg - o["x"]) <= 1e-5 * max(np.linalg.norm(o["x"]), floor), k


def test_gl_batch_matches_single_instance_solver(cuda, solver_lib):
    """Two FP32 solves of the same GL problem in different summation orders:
    each is within max(1e-5, 2 x the FP32 oracle's error) of the FP64
    solution (test above), and that error reaches ~1e-4 on these inputs (the
    shrink amplifies rounding in groups it nearly zeroes), so they agree to
    3e-4."""
    import reg_drot
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=128)
    x, info = B.solve(c, p, q, 20000)
    for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(SHAPES, insts)):
        xs, i1, _ = reg_drot.solve_gl(ci.to(cuda), pi.to(cuda), qi.to(cuda), G, 2.0, 1e-3, 20000,
                                      1e-4)
        assert abs(info[k]["n_iter"] - i1["n_iter"]) <= max(1, i1["n_iter"] // 50), k
        if info[k]["n_iter"] == i1["n_iter"]:
            assert _rel(B.view(x, k).cpu().numpy(), xs.cpu().numpy()) <= 3e-4, k


def test_gl_batch_wrapper_convention_and_bf16_cost(cuda, solver_lib):
    # the C++ wrapper's threshold r / sqrt(n / G) and BF16-stored C (the FP32
    # solve of the rounded cost): against the oracle on that cost
    B, insts, c, p, q = _batch(SHAPES[:4], cuda, cpt=128, dtype=torch.bfloat16,
                               convention="wrapper")
    x, info = B.solve(c, p, q, 20000)
    for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(SHAPES[:4], insts)):
        assert B.lambdas[k] == pytest.approx(1e-3 / np.sqrt(nr // G), rel=1e-6)
        cr = ci.to(torch.bfloat16).float().numpy()
        s = O.step_size(2.0, nr, nc)
        bnd = O.group_bounds(nr, G)
        o32 = O.gl_solve(cr, pi.numpy(), qi.numpy(), bnd, s, B.lambdas[k], 20000, 1e-4)
        o64 = O.gl_solve(cr, pi.numpy(), qi.numpy(), bnd, s, B.lambdas[k], 20000, 1e-4,
                         dtype=np.float64)
        assert info[k]["converged"] == 1
        ref = _rel(o32["x"], o64["x"])
        assert _rel(B.view(x, k).cpu().numpy(), o64["x"]) <= max(1e-5, 2.0 * ref), k


def test_gl_batch_ignores_padding_rows(cuda, solver_lib):
    """Rows between n_rows and ld belong to the caller: NaN there changes
    neither the plans nor any reported figure (the objective included)."""
    B, insts, c, p, q = _batch(SHAPES, cuda, cpt=64)
    x1, i1 = B.solve(c, p, q, 20000)
    x1 = x1.clone()
    c2 = c.clone()
    padded = 0
    for k, (nr, nc, _) in enumerate(SHAPES):
        ld, off = B.lds[k], B.offsets[k]
        if ld > nr:
            c2[off:off + ld * nc].view(nc, ld)[:, nr:] = float("nan")
            padded += 1
    assert padded >= 2
    x2, i2 = B.solve(c2, p, q, 20000)
    for k in range(len(SHAPES)):
        assert torch.equal(B.view(x1, k), B.view(x2, k)), k
        assert i1[k] == i2[k], k


def test_gl_batch_graph_replay_and_determinism(cuda, solver_lib):
    B, insts, c, p, q = _batch(SHAPES[:5], cuda, cpt=64)
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


def test_gl_batch_largest_staged_classes_match_oracle(cuda, solver_lib):
    """Classes at the staging limit of 4096 rows from the 16-byte boundary
    below their first row: one 4096-row class, and classes of 4093 rows of
    which the second starts at row 4093 (staged from row 4092).  The plan's
    shared staging then admits one CTA per SM.  Fixed iteration counts
    against the FP32 oracle, then a converged solve against the FP64 one."""
    shapes = [(4096, 80, 1), (8186, 40, 2), (300, 200, 3)]
    for mi in (2, 7):
        B, insts, c, p, q = _batch(shapes, cuda, eps=0.0, cpt=64)
        x, info = B.solve(c, p, q, mi)
        for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(shapes, insts)):
            s = O.step_size(2.0, nr, nc)
            o = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), O.group_bounds(nr, G), s,
                           B.lambdas[k], mi, 0.0)
            assert info[k]["n_iter"] == mi == o["n_iter"]
            floor = float(np.linalg.norm(pi.numpy()) * np.linalg.norm(qi.numpy()))
            xg = B.view(x, k).cpu().numpy().astype(np.float64)
            assert np.linalg.norm(xg - o["x"]) <= 1e-5 * max(np.linalg.norm(o["x"]), floor), k
    B, insts, c, p, q = _batch(shapes, cuda, cpt=64)
    x, info = B.solve(c, p, q, 20000)
    for k, ((nr, nc, G), (ci, pi, qi)) in enumerate(zip(shapes, insts)):
        s = O.step_size(2.0, nr, nc)
        bnd = O.group_bounds(nr, G)
        o32 = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), bnd, s, B.lambdas[k], 20000, 1e-4)
        o64 = O.gl_solve(ci.numpy(), pi.numpy(), qi.numpy(), bnd, s, B.lambdas[k], 20000, 1e-4,
                         dtype=np.float64)
        assert info[k]["converged"] == 1, (k, info[k])
        ref = _rel(o32["x"], o64["x"])
        assert _rel(B.view(x, k).cpu().numpy(), o64["x"]) <= max(1e-5, 2.0 * ref), k


def test_gl_batch_rejects_classes_taller_than_its_staging(cuda, solver_lib):
    from reg_drot.batch import GLBatch
    B = GLBatch([(9000, 64)], 2, 2.0, 1e-3, 1e-4, device=cuda, cols_per_tile=64)
    c = torch.zeros(B.total, device=cuda)
    p, q = B.pack_marginals([torch.ones(9000) / 9000], [torch.ones(64) / 64])
    with pytest.raises(RuntimeError):
        B.solve(c, p, q, 10)


def test_gl_batch_gradient_is_the_truncated_adjoint_at_the_solution(cuda, solver_lib):
    """batch_group_lasso_drot_fn: batched GL forward to the stop, then per
    instance the unrolled adjoint of last_k iterations taken from the state
    the solve stopped at (held fixed).  Reference: the FP64 unrolled map of
    the same last_k iterations from that same state (oracle.adjoint
    .gl_unrolled, pinned to the oracle's GL loop), differentiated by torch
    autograd.  1e-4 relative, as the single-instance unrolled adjoint."""
    from oracle import adjoint as A
    from reg_drot.autograd import batch_group_lasso_drot_fn
    shapes = [(60, 40, 2), (300, 200, 3), (513, 300, 2)]
    B, insts, c, p, q = _batch(shapes, cuda, cpt=64)
    K = 40
    cl = c.clone().requires_grad_(True)
    pl = p.clone().requires_grad_(True)
    ql = q.clone().requires_grad_(True)
    x = batch_group_lasso_drot_fn(B, cl, pl, ql, 20000, last_k=K, segment=16)
    assert all(r["converged"] == 1 for r in x.grad_fn.info)
    state = [{k: v.double().cpu() for k, v in st.items()} for st in x.grad_fn.state]
    rng = np.random.default_rng(5)
    W = torch.tensor(rng.normal(size=x.shape), dtype=torch.float32, device=cuda)
    (x * W).sum().backward()
    prow = pcol = 0
    for k, (nr, nc, G) in enumerate(shapes):
        ck = torch.tensor(B.view(c, k).cpu().numpy(), dtype=torch.float64, requires_grad=True)
        pk = p[prow:prow + nr].double().cpu().requires_grad_(True)
        qk = q[pcol:pcol + nc].double().cpu().requires_grad_(True)
        st = dict(state[k], x=B.view(x.detach(), k).double().cpu())
        X = A.gl_unrolled(ck, pk, qk, G, 2.0, 1e-3, K, state=st, lam=B.lambdas[k])
        (X * B.view(W, k).double().cpu()).sum().backward()
        e_c = _rel(B.view(cl.grad, k).cpu().numpy(), ck.grad.numpy())
        e_p = _rel(pl.grad[prow:prow + nr].cpu().numpy(), pk.grad.numpy())
        e_q = _rel(ql.grad[pcol:pcol + nc].cpu().numpy(), qk.grad.numpy())
        assert e_c <= 1e-4 and e_p <= 1e-4 and e_q <= 1e-4, (k, e_c, e_p, e_q)
        # K more steps from the saved state stay near the plan (measured
        # 0.3-1.8 %); a state that is not the solve's (wrong alpha or duals)
        # moves X by O(1)
        assert _rel(X.detach().numpy(), st["x"].numpy()) <= 5e-2
        prow += nr
        pcol += nc


def test_gl_batch_gradient_does_not_depend_on_the_checkpoint_spacing(cuda, solver_lib):
    """The recomputation from checkpoints is deterministic (the same batched
    iterations from the same states), so any checkpoint spacing gives the
    same gradient bit for bit."""
    from reg_drot.autograd import batch_group_lasso_drot_fn
    shapes = [(60, 40, 2), (300, 200, 3), (513, 300, 2)]
    grads = []
    for seg in (7, 16, 40):
        B, insts, c, p, q = _batch(shapes, cuda, cpt=64)
        cl = c.clone().requires_grad_(True)
        pl = p.clone().requires_grad_(True)
        ql = q.clone().requires_grad_(True)
        x = batch_group_lasso_drot_fn(B, cl, pl, ql, 20000, last_k=40, segment=seg)
        W = torch.linspace(-1.0, 1.0, x.numel(), device=cuda).view_as(x)
        (x * W).sum().backward()
        grads.append((cl.grad.clone(), pl.grad.clone(), ql.grad.clone()))
    for g in grads[1:]:
        for a, b in zip(grads[0], g):
            assert torch.equal(a, b)
