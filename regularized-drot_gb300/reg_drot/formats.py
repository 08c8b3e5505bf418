"""The reference's benchmark data formats and its W2 domain-adaptation
evaluation, around the GPU solver.

* Cost files (core/utils.hpp:9-24): raw float32, an n_rows x n_cols matrix
  in row-major order.  ``load_cost`` returns it in the solver's layout, a
  [n_cols, n_rows] array whose flat order is the column-major matrix that
  ``utils::load`` hands to the solver (element (i, j) at j * n_rows + i);
  ``save_cost`` writes that layout back.
* Plan text (core/singleexp_qr.cu:46-53, singleexp_glr.cu:42-49): X as n_cols
  lines of n_rows values ("%.10f "), then the objective and the iteration
  count, one per line.  ``format_plan`` / ``parse_plan``; ``load_plan_rows``
  reads a file of plan rows only, as benchmark/utils/compute_w2_dist.py:49-57.
* Experiment logs (core/multiexp_qr.cu:85-89, multiexp_glr.cu:92-98): a
  tab-separated header and one row per run after the first; ``log_header``,
  ``log_row``, ``parse_log``.
* Within-class W2 distance of an adapted target domain
  (benchmark/utils/compute_w2_dist.py:59-94): ``adapt_target_domain`` and
  ``group_w2_distance``.  The per-group OT problems are solved by the GPU
  solver (reg_drot.quadratic_drot, r_weight 0, rho 2, 50000 iterations,
  eps 2e-6, as the reference) unless a ``solver`` is passed.

The CLI drivers themselves (core/*exp_*.cu) are not reproduced.
"""
import numpy as np

QR_LOG_FIELDS = ("test_index", "method", "n", "m", "eps", "use_warmup_init", "rho", "r_weight",
                 "max_iters", "runtime_ms", "objective", "n_iteration", "runtime_ms_per_iteration")
GL_LOG_FIELDS = ("test_index", "method", "n", "m", "n_class", "eps", "use_warmup_init", "rho",
                 "r_weight", "max_iters", "runtime_ms", "objective", "n_iteration",
                 "runtime_ms_per_iteration")

W2_RHO = 2.0
W2_MAX_ITERS = 50000
W2_EPS = 2e-6


# ---------------------------------------------------------------- cost files
def load_cost(path, n_rows, n_cols):
    """[n_cols, n_rows] float32 cost (the solver's layout) from a raw
    row-major n_rows x n_cols float32 file.  A short file raises."""
    raw = np.fromfile(path, dtype=np.float32, count=n_rows * n_cols)
    if raw.size != n_rows * n_cols:
        raise ValueError(f"{path}: expected {n_rows * n_cols} float32 values, found {raw.size}")
    return np.ascontiguousarray(raw.reshape(n_rows, n_cols).T)


def save_cost(path, c):
    """Writes a [n_cols, n_rows] cost as the raw row-major n_rows x n_cols file."""
    c = np.asarray(c, dtype=np.float32)
    if c.ndim != 2:
        raise ValueError("cost must be a 2-D [n_cols, n_rows] array")
    np.ascontiguousarray(c.T).tofile(path)


# ---------------------------------------------------------------- plan text
def format_plan(x, objective, n_iter):
    """The single-experiment output: x ([n_cols, n_rows], the solver's
    layout) as n_cols lines of n_rows "%.10f " values, then the objective and
    the iteration count."""
    x = np.asarray(x, dtype=np.float32)
    lines = ["".join("%.10f " % v for v in row) for row in x]
    lines.append("%.10f" % float(np.float32(objective)))
    lines.append("%d" % int(n_iter))
    return "\n".join(lines) + "\n"


def parse_plan(text):
    """(x [n_cols, n_rows] float32, objective, n_iter) from ``format_plan``'s text."""
    rows = [ln.strip(" ") for ln in text.strip("\n").split("\n")]
    if len(rows) < 3:
        raise ValueError("plan text needs X rows, the objective and the iteration count")
    x = np.array([[float(v) for v in r.split(" ") if v] for r in rows[:-2]], dtype=np.float32)
    return x, float(rows[-2]), int(rows[-1])


def load_plan_rows(path):
    """Plan rows of a text file (space-separated floats per line) as a
    float32 array, the reader of the W2 evaluation."""
    mat = []
    with open(path) as f:
        for line in f:
            line = line.strip(" \n")
            if line:
                mat.append([float(v) for v in line.split(" ") if v])
    return np.array(mat, dtype=np.float32)


# ---------------------------------------------------------------- logs
def log_header(method="quad_drot"):
    return "\t".join(GL_LOG_FIELDS if method == "gl_drot" else QR_LOG_FIELDS)


def log_row(test_index, n_rows, n_cols, eps, use_warmup_init, rho, r_weight, max_iters,
            runtime_ms, objective, n_iteration, n_class=None):
    """One run in the experiment-log schema (quad_drot, or gl_drot when n_class
    is given); numbers formatted as the reference's printf."""
    head = [str(int(test_index)), "gl_drot" if n_class is not None else "quad_drot",
            str(int(n_rows)), str(int(n_cols))]
    if n_class is not None:
        head.append(str(int(n_class)))
    per_it = float(np.float32(runtime_ms) / np.float32(n_iteration)) if n_iteration else float("inf")
    tail = ["%.8f" % eps, str(int(bool(use_warmup_init))), "%.8f" % rho, "%.8f" % r_weight,
            str(int(max_iters)), "%.8f" % runtime_ms, "%.8f" % objective, str(int(n_iteration)),
            "%.8f" % per_it]
    return "\t".join(head + tail)


def parse_log(text):
    """Records (dicts) of every table in an experiment log: a header line
    starts a table, the lines after it are its rows."""
    out, fields = [], None
    ints = {"test_index", "n", "m", "n_class", "use_warmup_init", "max_iters", "n_iteration"}
    for line in text.splitlines():
        if not line.strip():
            continue
        parts = line.split("\t")
        if parts[0] == "test_index":
            fields = parts
            continue
        if fields is None:
            continue
        rec = {}
        for k, v in zip(fields, parts):
            rec[k] = v if k == "method" else (int(v) if k in ints else float(v))
        out.append(rec)
    return out


# ---------------------------------------------------------------- W2 distance
def adapt_target_domain(xt, plan, p):
    """Barycentric map of compute_w2_dist.py:59-63: plan [n_t, n_s] (rows the
    target points xt), p the uniform source weights; returns plan^T xt / scale
    with scale = (column sums of the plan + p) / 2."""
    plan = np.asarray(plan, dtype=np.float32)
    scale = plan.sum(axis=0) + np.asarray(p, dtype=np.float32)
    scale = scale / np.float32(2)
    return (plan.T @ np.asarray(xt, dtype=np.float32)) / scale.reshape(-1, 1)


def _sq_dist(a, b):
    """Squared Euclidean distances |a_i - b_j|^2 ([len(a), len(b)])."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return ((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)


def _gpu_solver(c, p, q):
    import torch

    import reg_drot
    dev = torch.device("cuda", torch.cuda.current_device())
    x = reg_drot.quadratic_drot(torch.tensor(c, dtype=torch.float32, device=dev),
                                torch.tensor(p, dtype=torch.float32, device=dev),
                                torch.tensor(q, dtype=torch.float32, device=dev),
                                W2_RHO, 0.0, W2_MAX_ITERS, W2_EPS)
    return x.cpu().numpy()


def group_w2_distance(xt, plan, n_group, solver=None):
    """(total, normalised) within-class W2 distance between the target points
    xt and the source domain adapted by the plan (compute_w2_dist.py:65-94).
    Per group g: rows [round(N g / G), round(N (g+1) / G)) of xt and of the
    adapted points; C = squared distances / max (FP32, [adapted, target]);
    the unregularised OT plan X of C (``solver(c, p, q)``, default the GPU
    solver) must meet the residual 2 * eps; obj_g = <C, X> * max(C); the
    normalised sum divides obj_g by the group's mean distance to its centre
    times the adapted group size."""
    xt = np.asarray(xt, dtype=np.float32)
    plan = np.asarray(plan, dtype=np.float32)
    solver = solver or _gpu_solver
    p_src = np.ones(plan.shape[1], dtype=np.float32) / np.float32(plan.shape[1])
    adapted = adapt_target_domain(xt, plan, p_src)
    total = norm = 0.0
    for g in range(n_group):
        s = round(xt.shape[0] / n_group * g)
        t = round(xt.shape[0] / n_group * (g + 1))
        a_s = round(adapted.shape[0] / n_group * g)
        a_t = round(adapted.shape[0] / n_group * (g + 1))
        c = _sq_dist(adapted[a_s:a_t], xt[s:t])
        c_max = c.max()
        c = (c / c_max).astype(np.float32)
        p = np.ones(t - s, dtype=np.float32) / np.float32(t - s)
        q = np.ones(a_t - a_s, dtype=np.float32) / np.float32(a_t - a_s)
        x = np.asarray(solver(c, p, q), dtype=np.float32)
        res = np.sqrt(np.square(x.sum(0) - p).sum() + np.square(x.sum(1) - q).sum())
        if not res < 2 * W2_EPS:
            raise RuntimeError(f"group {g}: marginal residual {res} above {2 * W2_EPS}")
        grp = xt[s:t]
        dist_norm = np.mean(np.sqrt(np.sum(np.square(grp - grp.mean(axis=0)), axis=1)))
        obj = float((c * x).sum()) * c_max
        total += obj
        norm += obj / (dist_norm * (a_t - a_s))
    return total, norm


__all__ = ["load_cost", "save_cost", "format_plan", "parse_plan", "load_plan_rows",
           "log_header", "log_row", "parse_log", "adapt_target_domain", "group_w2_distance",
           "QR_LOG_FIELDS", "GL_LOG_FIELDS"]
