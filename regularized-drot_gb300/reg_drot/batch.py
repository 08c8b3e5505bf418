"""Batched quadratic-regularised DROT: many instances, one persistent launch.

The reference solves one problem per call (pytorch/src/drot_cuda.cpp:26-44;
its callers loop, e.g. benchmark/utils/compute_w2_dist.py:86).  ``QRBatch``
solves a list of independent instances of different shapes together: per
instance the iteration, warm start, stop test and iteration count of
``reg_drot.quadratic_drot``, each instance stopping on its own.

Instances are packed into flat buffers.  Instance k's cost ``c_k`` (a
[n_cols, n_rows] tensor, the layout of the reference operator) occupies
``n_cols`` columns of ``ld_k = n_rows`` rounded up to 4 elements, starting at
a 32-element boundary of the packed C buffer; its plan X has the same place
in the packed X buffer; p_k and q_k are concatenated.

    B = QRBatch([(nr, nc), ...], rho=2.0, r_weight=1e-3, eps=1e-4)
    c = B.pack_c(list_of_costs)            # float32 or bfloat16
    p, q = B.pack_marginals(ps, qs)
    x, info = B.solve(c, p, q, max_iters)  # info: list of per-instance dicts
    plans = B.unpack(x)                    # [n_cols, n_rows] views

``solve(..., sync=False)`` only enqueues device work (an init kernel and one
cooperative launch), so it can be captured in a CUDA graph
(``B.capture(c, p, q, x, max_iters)``).  ``cols_per_tile=None`` picks the tile
width by timing short runs of each candidate on the caller's data.
"""
import ctypes
import threading

import torch

from ._lib import (DrotBatchInstance, DrotBatchResult, DrotBatchTuning, DrotError,
                   DrotGlBatchInstance, check, lib)

C_F32, C_BF16 = 0, 1
TILE_CANDIDATES = (32, 64, 128, 256)
_ALIGN = 32  # elements between instance blocks (128 bytes of FP32)


_TUNING_FIELDS = ("fine_cols", "finest_cols", "item_lines", "finest_item_lines",
                  "level_quarters", "prefetch_distance", "tail_quarters")
_tuning_lock = threading.Lock()
_tuning = {}


def _apply_tuning(t):
    v = DrotBatchTuning(*(int(t.get(f, -1)) for f in _TUNING_FIELDS))
    check(lib().drot_batch_set_tuning(ctypes.byref(v)), "drot_batch_set_tuning")


def set_tuning(**fields):
    """Tile-level shape of the batch plans created afterwards (process-wide;
    drot_batch_set_tuning).  Fields left out or below 0 keep the default:
    fine_cols 128, finest_cols 32 (0: no third level), item_lines 1024,
    finest_item_lines 64, level_quarters 8 (0: keep the coarse tiles),
    prefetch_distance 1 (0: off), tail_quarters 4 (the smallest instances on
    finer tiles at the end of each iteration; 0: off).  ``set_tuning()``
    restores the defaults.
    Plans already built keep theirs; a batch built with ``tuning=`` uses its
    own."""
    bad = set(fields) - set(_TUNING_FIELDS)
    if bad:
        raise RuntimeError(f"unknown tuning fields {sorted(bad)}")
    global _tuning
    with _tuning_lock:
        _apply_tuning(fields)
        _tuning = dict(fields)


def _create_plan(fn, tuning, *args):
    """fn(*args) with the batch's own tuning in force (the process-wide one
    restored after)."""
    with _tuning_lock:
        if tuning is None:
            return fn(*args)
        _apply_tuning(tuning)
        try:
            return fn(*args)
        finally:
            _apply_tuning(_tuning)


def _as_list(v, n, name):
    if isinstance(v, (list, tuple)):
        if len(v) != n:
            raise RuntimeError(f"{name} needs one value per instance")
        return [float(t) for t in v]
    return [float(v)] * n


class QRBatch:
    """A fixed set of instance shapes and parameters, planned once."""

    def __init__(self, shapes, rho, r_weight, eps, *, device=None, cols_per_tile=None,
                 band_rows=512, tuning=None):
        shapes = [(int(a), int(b)) for a, b in shapes]
        if not shapes:
            raise RuntimeError("QRBatch needs at least one instance")
        self.shapes = shapes
        self.n = len(shapes)
        device = torch.device("cuda" if device is None else device)
        if device.type != "cuda":
            raise RuntimeError("QRBatch runs on a CUDA device")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        rho = _as_list(rho, self.n, "rho")
        r_weight = _as_list(r_weight, self.n, "r_weight")
        eps = _as_list(eps, self.n, "eps")
        desc = (DrotBatchInstance * self.n)()
        off = prow = pcol = 0
        self.offsets, self.lds = [], []
        for k, (nr, nc) in enumerate(shapes):
            if nr <= 0 or nc <= 0:
                raise RuntimeError("instance shapes must be positive")
            ld = (nr + 3) // 4 * 4
            d = desc[k]
            d.n_rows, d.n_cols, d.ld = nr, nc, ld
            d.c_offset = d.x_offset = off
            d.p_offset, d.q_offset = prow, pcol
            d.rho, d.r_weight, d.eps = rho[k], r_weight[k], eps[k]
            self.offsets.append(off)
            self.lds.append(ld)
            off += (ld * nc + _ALIGN - 1) // _ALIGN * _ALIGN
            prow += nr
            pcol += nc
        self.total = off
        self.total_rows, self.total_cols = prow, pcol
        self._desc = desc
        self.rho, self.r_weight, self.eps = rho, r_weight, eps
        self._plans = {}
        self._ws = None
        self._ws_plan = None
        self.cols_per_tile = cols_per_tile
        if band_rows not in (128, 512):
            raise RuntimeError("band_rows must be 128 or 512")
        self.band_rows = band_rows  # 512 (default; point-cloud launches need it) or 128
        if tuning is not None and set(tuning) - set(_TUNING_FIELDS):
            raise RuntimeError(f"unknown tuning fields {sorted(set(tuning) - set(_TUNING_FIELDS))}")
        self.tuning = None if tuning is None else dict(tuning)  # tile levels (set_tuning)

    # ------------------------------------------------------------------ packing
    def pack_c(self, costs, dtype=torch.float32):
        """Packed C buffer from [n_cols, n_rows] costs (padding rows zero)."""
        buf = torch.zeros(self.total, dtype=dtype, device=self.device)
        for k, c in enumerate(costs):
            nr, nc = self.shapes[k]
            if tuple(c.shape) != (nc, nr):
                raise RuntimeError(f"cost {k} must have shape [{nc}, {nr}]")
            self.view(buf, k).copy_(c)
        return buf

    def pack_marginals(self, ps, qs):
        p = torch.cat([t.reshape(-1).float() for t in ps]).to(self.device).contiguous()
        q = torch.cat([t.reshape(-1).float() for t in qs]).to(self.device).contiguous()
        if p.numel() != self.total_rows or q.numel() != self.total_cols:
            raise RuntimeError("marginal sizes do not match the instance shapes")
        return p, q

    def view(self, buf, k):
        """[n_cols, n_rows] view of instance k inside a packed buffer."""
        nr, nc = self.shapes[k]
        ld, off = self.lds[k], self.offsets[k]
        return buf[off:off + ld * nc].view(nc, ld)[:, :nr]

    def unpack(self, buf):
        return [self.view(buf, k) for k in range(self.n)]

    def empty_x(self):
        return torch.empty(self.total, dtype=torch.float32, device=self.device)

    # ------------------------------------------------------------------ plans
    def _plan(self, cols_per_tile):
        cpt = int(cols_per_tile)
        if cpt not in self._plans:
            h = ctypes.c_void_p()
            with torch.cuda.device(self.device):
                check(_create_plan(lib().drot_batch_plan_create_ex, self.tuning, self.n,
                                   self._desc, cpt, self.band_rows, ctypes.byref(h)),
                      "batch_plan_create")
            self._plans[cpt] = h
        return self._plans[cpt]

    def workspace_for(self, cols_per_tile, stream=None):
        """Workspace holding the plan's uploaded descriptors (reused while the
        tile width stays the same)."""
        h = self._plan(cols_per_tile)
        nbytes = int(lib().drot_batch_plan_workspace_bytes(h))
        if self._ws is None or self._ws.numel() < nbytes + 256:
            self._ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.device)
            self._ws_plan = None
        ptr = self._ws.data_ptr()
        ptr += (-ptr) % 256
        if self._ws_plan != cols_per_tile:
            s = torch.cuda.current_stream(self.device) if stream is None else stream
            check(lib().drot_batch_upload(h, ptr, nbytes, s.cuda_stream), "batch_upload")
            self._ws_plan = cols_per_tile
        return h, ptr, nbytes

    def tiles(self, cols_per_tile):
        return int(lib().drot_batch_plan_tiles(self._plan(cols_per_tile)))

    def iteration_log(self, cap, cols_per_tile=None):
        """Profile the next launches with tile width ``cols_per_tile``: returns
        (times [cap, 4] int64, active_tiles [cap] int32) device tensors that
        each launch fills, for iterations it < cap, with CTA 0's device clock
        (ns) at the start of the iteration, after its fused-update tiles,
        after the first grid barrier and after its dual-update items, and the
        coarse tiles of unconverged instances at the start
        (drot_batch_set_iteration_log).  cap = 0 switches it off."""
        cpt = cols_per_tile or self.cols_per_tile or 128
        times = torch.zeros(max(cap, 1), 4, dtype=torch.int64, device=self.device)
        tiles = torch.zeros(max(cap, 1), dtype=torch.int32, device=self.device)
        check(lib().drot_batch_set_iteration_log(self._plan(cpt), times.data_ptr(),
                                                 tiles.data_ptr(), int(cap)),
              "batch_set_iteration_log")
        self._log = (times, tiles) if cap > 0 else None  # keeps the buffers alive
        return times, tiles

    # ------------------------------------------------------------------ solve
    def _check(self, c, p, q, x):
        if c.device != self.device or c.dim() != 1 or c.numel() != self.total or \
                c.dtype not in (torch.float32, torch.bfloat16) or not c.is_contiguous():
            raise RuntimeError("c must be the packed cost buffer (pack_c)")
        if p.numel() != self.total_rows or q.numel() != self.total_cols or \
                p.dtype != torch.float32 or q.dtype != torch.float32 or \
                not p.is_contiguous() or not q.is_contiguous() or \
                p.device != self.device or q.device != self.device:
            raise RuntimeError("p, q must be the packed marginals (pack_marginals)")
        if x.numel() != self.total or x.dtype != torch.float32 or x.device != self.device or \
                not x.is_contiguous():
            raise RuntimeError("x must be a packed float32 buffer (empty_x)")

    def launch(self, c, p, q, x, max_iters, cols_per_tile=None, stream=None):
        """Enqueue warm start + solve on ``stream``; device work only."""
        cpt = cols_per_tile or self.cols_per_tile or 128
        h, ptr, nbytes = self.workspace_for(cpt, stream)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        rc = lib().drot_qr_batch_launch(h, c.data_ptr(),
                                        C_BF16 if c.dtype == torch.bfloat16 else C_F32,
                                        p.data_ptr(), q.data_ptr(), x.data_ptr(), int(max_iters),
                                        ptr, nbytes, s.cuda_stream)
        check(rc, "qr_batch_launch")

    def launch_points(self, x_cat, y_cat, p, q, x, max_iters, scale=1.0, cols_per_tile=None,
                      stream=None):
        """Enqueue a point-cloud solve: instance k's cost is scale * |x_i - y_j|^2
        of its points (x_cat, y_cat: every instance's points concatenated in
        order, [rows, dim] / [cols, dim] float32, dim 8 or 16), recomputed in
        the fused update instead of read from memory."""
        if self.band_rows != 512:
            raise RuntimeError("point-cloud solves need a QRBatch with 512-row bands (the default)")
        for t, name, n in ((x_cat, "x_cat", self.total_rows), (y_cat, "y_cat", self.total_cols)):
            if t.device != self.device or t.dtype != torch.float32 or t.dim() != 2 or \
                    t.size(0) != n or t.size(1) not in (8, 16) or not t.is_contiguous():
                raise RuntimeError(f"{name} must be a contiguous float32 [{n}, 8 or 16] tensor")
        if x_cat.size(1) != y_cat.size(1):
            raise RuntimeError("x_cat and y_cat must have the same dimension")
        cpt = cols_per_tile or self.cols_per_tile or 512
        h, ptr, nbytes = self.workspace_for(cpt, stream)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        rc = lib().drot_qr_batch_launch_points(h, x_cat.data_ptr(), y_cat.data_ptr(), x_cat.size(1),
                                               float(scale), p.data_ptr(), q.data_ptr(),
                                               x.data_ptr(), int(max_iters), ptr, nbytes,
                                               s.cuda_stream)
        check(rc, "qr_batch_launch_points")

    def solve_points(self, x_cat, y_cat, p, q, max_iters, scale=1.0, *, out=None, stream=None,
                     sync=True):
        """solve() with the cost recomputed from point clouds (launch_points)."""
        x = self.empty_x() if out is None else out
        with torch.cuda.device(self.device):
            if self.cols_per_tile is None:
                self.cols_per_tile = 512
            self.launch_points(x_cat.detach(), y_cat.detach(), p, q, x, max_iters, scale,
                               stream=stream)
            info = self.results(stream) if sync else None
        return x, info

    def results(self, stream=None):
        """Per-instance records of the last launch (waits for the stream)."""
        out = (DrotBatchResult * self.n)()
        h, ptr, _ = self.workspace_for(self._ws_plan or self.cols_per_tile or 128, stream)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        rc = lib().drot_batch_results(h, ptr, out, s.cuda_stream)
        check(rc, "batch_results")
        return [{name: getattr(r, name) for name, _ in r._fields_} for r in out]

    def duals(self):
        """(phi1, phi2) after the last launch: copies of the packed final duals
        (instance k's rows / columns at its p / q offsets)."""
        h, ptr, _ = self.workspace_for(self._ws_plan or self.cols_per_tile or 128)
        f1, f2 = ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().drot_batch_state(h, ptr, ctypes.byref(f1), ctypes.byref(f2)), "batch_state")
        base = self._ws.data_ptr()
        o1, o2 = f1.value - base, f2.value - base
        phi1 = self._ws[o1:o1 + 4 * self.total_rows].view(torch.float32).clone()
        phi2 = self._ws[o2:o2 + 4 * self.total_cols].view(torch.float32).clone()
        return phi1, phi2

    def state(self, info=None):
        """Per-instance copies of the final solver state after the last launch:
        dicts (x, a, b, phi1, phi2, alpha) with x in the [n_cols, n_rows]
        layout -- the state drot_gl_solve / drot_qr_solve continue from.
        info: the launch's results (their iters_run give alpha's parity)."""
        info = self.results() if info is None else info
        h, ptr, _ = self.workspace_for(self._ws_plan or self.cols_per_tile or 128)
        vp = [ctypes.c_void_p() for _ in range(5)]
        check(lib().drot_batch_state_ex(h, ptr, *[ctypes.byref(v) for v in vp]), "batch_state_ex")
        base = self._ws.data_ptr()

        def vec(ptr_v, off, n):
            o = ptr_v.value - base + 4 * off
            return self._ws[o:o + 4 * n].view(torch.float32).clone()
        out, prow, pcol = [], 0, 0
        for k, (nr, nc) in enumerate(self.shapes):
            par = int(info[k]["iters_run"]) & 1
            out.append({"a": vec(vp[0], prow, nr), "b": vec(vp[1], pcol, nc),
                        "phi1": vec(vp[2], prow, nr), "phi2": vec(vp[3], pcol, nc),
                        "alpha": vec(vp[4], par * self.n + k, 1)})
            prow += nr
            pcol += nc
        return out

    def step_sizes(self):
        """s = rho / (n_rows + n_cols) of every instance (FP32, as the solver)."""
        import numpy as np
        return [float(np.float32(r) / (np.float32(nr) + np.float32(nc)))
                for r, (nr, nc) in zip(self.rho, self.shapes)]

    def autotune(self, c, p, q, iters=40, candidates=TILE_CANDIDATES):
        """Times ``iters`` iterations per tile width on the caller's data and
        keeps the fastest (the widths differ only in the order of the FP32
        partial sums)."""
        x = self.empty_x()
        best = None
        for cpt in candidates:
            self.launch(c, p, q, x, iters, cpt)  # warm-up (plan upload, caches)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(2):
                self.launch(c, p, q, x, iters, cpt)
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1)
            if best is None or t < best[0]:
                best = (t, cpt)
        self.cols_per_tile = best[1]
        return best[1]

    def solve(self, c, p, q, max_iters, *, out=None, stream=None, sync=True):
        """Solve every instance; returns (x, info list or None)."""
        x = self.empty_x() if out is None else out
        self._check(c, p, q, x)
        with torch.cuda.device(self.device):
            if self.cols_per_tile is None:
                self.autotune(c, p, q)
            self.launch(c, p, q, x, max_iters, stream=stream)
            info = self.results(stream) if sync else None
        return x, info

    def capture(self, c, p, q, x, max_iters, stream=None):
        """A CUDA graph of the whole solve (warm start included); replay it
        with ``g.replay()`` and read ``results()`` afterwards."""
        self._check(c, p, q, x)
        if self.cols_per_tile is None:
            self.autotune(c, p, q)
        cpt = self.cols_per_tile
        self.workspace_for(cpt)  # upload outside the capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(c, p, q, x, max_iters, cpt, torch.cuda.current_stream(self.device))
        g.drot_workspace = self._ws  # the graph reads this workspace
        return g

    def __del__(self):
        try:
            for h in self._plans.values():
                lib().drot_batch_plan_destroy(h)
        except Exception:
            pass
        self._plans = {}


class GLBatch(QRBatch):
    """Many group-lasso instances in one persistent launch
    (drot_gl_batch_plan_create): per instance the loop of
    reg_drot.group_lasso_drot -- n_class contiguous row classes with the
    reference's boundaries, the stop test on every iteration (residual <=
    eps), n_iter = iterations run, X never folded.  The threshold is
    r_weight * sqrt(n_rows // n_class) (convention="operator", the PyTorch
    operator) or r_weight / sqrt(n_rows // n_class) (convention="wrapper",
    the C++ wrapper).  Packing, launch, capture and results as QRBatch;
    classes of at most 4096 rows; cost matrices only (no point launches)."""

    def __init__(self, shapes, n_class, rho, r_weight, eps, *, device=None, cols_per_tile=None,
                 convention="operator", tuning=None):
        super().__init__(shapes, rho, r_weight, eps, device=device, cols_per_tile=cols_per_tile,
                         tuning=tuning)
        from .autograd import gl_step_and_lambda
        self.n_class = [int(v) for v in (n_class if isinstance(n_class, (list, tuple))
                                         else [n_class] * self.n)]
        if len(self.n_class) != self.n:
            raise RuntimeError("n_class needs one value per instance")
        self.convention = convention
        self.lambdas = [gl_step_and_lambda(self.rho[k], self.r_weight[k], nr, nc,
                                           self.n_class[k], convention)[1]
                        for k, (nr, nc) in enumerate(self.shapes)]
        desc = (DrotGlBatchInstance * self.n)()
        for k, (nr, nc) in enumerate(self.shapes):
            src, d = self._desc[k], desc[k]
            d.n_rows, d.n_cols, d.ld, d.n_groups = nr, nc, src.ld, self.n_class[k]
            d.c_offset, d.x_offset = src.c_offset, src.x_offset
            d.p_offset, d.q_offset = src.p_offset, src.q_offset
            d.rho, d.lambda_, d.eps = src.rho, self.lambdas[k], src.eps
        self._gl_desc = desc

    def _plan(self, cols_per_tile):
        cpt = int(cols_per_tile)
        if cpt not in self._plans:
            h = ctypes.c_void_p()
            with torch.cuda.device(self.device):
                check(_create_plan(lib().drot_gl_batch_plan_create, self.tuning, self.n,
                                   self._gl_desc, cpt, ctypes.byref(h)),
                      "gl_batch_plan_create")
            self._plans[cpt] = h
        return self._plans[cpt]

    def state_views(self):
        """Views (aliasing the workspace of the last launch) of the packed
        state: a, phi1 (all rows), b, phi2 (all columns) and alpha [2, n]
        by iteration parity (drot_batch_state_ex)."""
        if self._ws_plan is None:
            raise RuntimeError("no launch yet")
        h, ptr, _ = self.workspace_for(self._ws_plan)
        vp = [ctypes.c_void_p() for _ in range(5)]
        check(lib().drot_batch_state_ex(h, ptr, *[ctypes.byref(v) for v in vp]), "batch_state_ex")
        base = self._ws.data_ptr()

        def view(pv, n):
            o = pv.value - base
            return self._ws[o:o + 4 * n].view(torch.float32)
        return {"a": view(vp[0], self.total_rows), "b": view(vp[1], self.total_cols),
                "phi1": view(vp[2], self.total_rows), "phi2": view(vp[3], self.total_cols),
                "alpha": view(vp[4], 2 * self.n).view(2, self.n)}

    def resume(self, c, p, q, x, n_iters, stream=None):
        """Enqueue n_iters more iterations of every instance from the state in
        the workspace (state_views(); alpha in parity slot 0) and the plans in
        x, the stop test off (drot_batch_resume); alpha ends in slot 0."""
        if self._ws_plan is None:
            raise RuntimeError("no launch yet")
        h, ptr, nbytes = self.workspace_for(self._ws_plan)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        check(lib().drot_batch_resume(h, c.data_ptr(),
                                      C_BF16 if c.dtype == torch.bfloat16 else C_F32,
                                      p.data_ptr(), q.data_ptr(), x.data_ptr(), int(n_iters),
                                      ptr, nbytes, s.cuda_stream), "batch_resume")

    def launch_points(self, *args, **kwargs):
        raise RuntimeError("GLBatch solves cost matrices only")

    solve_points = launch_points


__all__ = ["QRBatch", "GLBatch", "DrotError", "TILE_CANDIDATES", "set_tuning"]
