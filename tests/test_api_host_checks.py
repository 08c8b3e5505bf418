"""CPU: host-side argument checks of the Python APIs beyond the reference's
operators (they raise before any device work, so they run without a GPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_cost_rejects_host_tensors_and_bad_dims():
    from reg_drot.cost import sqeuclidean_cost
    with pytest.raises(RuntimeError, match="CUDA tensor"):
        sqeuclidean_cost(torch.zeros(4, 16), torch.zeros(4, 16))


def test_qrbatch_rejects_bad_shapes_and_devices():
    from reg_drot.batch import QRBatch
    with pytest.raises(RuntimeError):
        QRBatch([], 2.0, 1e-3, 1e-4, device="cuda:0")
    with pytest.raises(RuntimeError):
        QRBatch([(0, 3)], 2.0, 1e-3, 1e-4, device="cuda:0")
    with pytest.raises(RuntimeError):
        QRBatch([(4, 3)], 2.0, 1e-3, 1e-4, device="cpu")
    with pytest.raises(RuntimeError):
        QRBatch([(4, 3), (5, 6)], [2.0], 1e-3, 1e-4, device="cuda:0")  # one rho per instance
    with pytest.raises(RuntimeError):
        QRBatch([(4, 3)], 2.0, 1e-3, 1e-4, device="cuda:0", band_rows=256)


def test_qrbatch_packing_layout():
    from reg_drot.batch import QRBatch
    B = QRBatch([(5, 3), (8, 2), (1, 1)], 2.0, 1e-3, 1e-4, device="cuda:0")
    # ld = n_rows rounded up to 4; blocks start on 32-element boundaries
    assert B.lds == [8, 8, 4]
    assert B.offsets == [0, 32, 64]
    assert B.total == 96 and B.total_rows == 14 and B.total_cols == 6


def test_autograd_rejects_zero_regularisation():
    from reg_drot.autograd import quadratic_drot_fn
    with pytest.raises(RuntimeError, match="r_weight > 0"):
        quadratic_drot_fn(torch.zeros(3, 2), torch.ones(2) / 2, torch.ones(3) / 3, 2.0, 0.0, 10,
                          1e-4)


def test_gl_autograd_rejects_bad_unroll_settings():
    """last_k and the checkpoint spacing must be positive (a zero spacing
    would recompute nothing); checked before the solve starts."""
    from reg_drot.autograd import batch_group_lasso_drot_fn, group_lasso_drot_fn
    c, p, q = torch.zeros(3, 2), torch.ones(2) / 2, torch.ones(3) / 3
    for kw in (dict(last_k=0), dict(segment=0), dict(segment=-3)):
        with pytest.raises(RuntimeError, match="positive"):
            group_lasso_drot_fn(c, p, q, 1, 2.0, 1e-3, 10, 1e-4, **kw)
        with pytest.raises(RuntimeError, match="positive"):
            batch_group_lasso_drot_fn(None, c.view(-1), p, q, 10, **kw)


def test_npdrot_rejects_unsupported_arguments():
    from reg_drot import npdrot
    C = np.asfortranarray(np.random.default_rng(0).random((4, 3)))
    p = np.full(4, 0.25)
    q = np.full(3, 1 / 3)
    with pytest.raises(NotImplementedError):
        npdrot.quaddrot(np.outer(p, q), C, p, q, 1.0, callbacks={"f": lambda *a, **k: 0.0})
    with pytest.raises(AssertionError):
        npdrot.quaddrot(np.outer(p, q), np.ascontiguousarray(C), p, q, 1.0)
    with pytest.raises(NotImplementedError):
        npdrot.l1l2drot(np.outer(p, q), C, p, q, 1.0, groups=[(0, 2)])
