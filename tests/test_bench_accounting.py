"""CPU: the byte accounting behind bench.py's roofline.

achieved = algorithmic bytes of the batched solve's launch / its time, and
traffic = that launch's algorithmic bytes x the DRAM-over-algorithmic ratio
of a committed ncu capture.  Checked here: the per-instance byte count of a
QR launch (12 B per element on the iterations that read C, 8 B on the
others, 12 B for a converged instance's final unfold; BF16 C: 10 B), the
ratio line of the capture summary, and the workload's stop tolerances.
"""
import math
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_solve_bytes_counts_even_odd_and_unfold():
    shapes = [(3, 5), (7, 2)]
    info = [{"iters_run": 4, "converged": 1}, {"iters_run": 3, "converged": 0}]
    # (3 x 5): iterations 0, 2 read C (12 B), 1, 3 do not (8 B), + unfold
    # (7 x 2): iterations 0, 2 read C, 1 does not, no unfold
    want = 15 * (2 * 12 + 2 * 8 + 12) + 14 * (2 * 12 + 1 * 8)
    assert bench.solve_bytes(shapes, info) == want
    # BF16-stored C: 2 bytes of C per element
    want16 = 15 * (2 * 10 + 2 * 8 + 10) + 14 * (2 * 10 + 1 * 8)
    assert bench.solve_bytes(shapes, info, cbytes=2) == want16


def test_traffic_ratio_comes_from_the_committed_capture():
    ratio = bench.profile_value("batch_solve_diff16.md", "traffic_over_algorithmic")
    assert ratio is not None and 0.9 < ratio < 1.2
    assert bench.profile_value("batch_solve_gl_diff16.md", "traffic_over_algorithmic") is not None
    assert bench.profile_value("no_such_summary.md", "traffic_over_algorithmic") is None


def test_workload_stop_is_relative_1e4_of_the_marginals():
    shapes, xs, ys, w, eps = bench.diff_workload()
    assert len(shapes) == bench.DIFF_INSTANCES
    assert all(bench.DIFF_MIN <= m <= bench.DIFF_MAX and bench.DIFF_MIN <= n <= bench.DIFF_MAX
               for m, n in shapes)
    assert xs.shape == (sum(m for m, _ in shapes), bench.DIFF_DIM)
    assert ys.shape == (sum(n for _, n in shapes), bench.DIFF_DIM)
    for (m, n), e in zip(shapes, eps):
        # uniform marginals: ||(p; q)||_2 = sqrt(1/m + 1/n)
        assert math.isclose(e, bench.REL_EPS * math.sqrt(1.0 / m + 1.0 / n), rel_tol=1e-12)
    # the same seed gives the same workload
    shapes2, xs2, _, w2, _ = bench.diff_workload()
    assert shapes2 == shapes and w2 == w and (xs2 == xs).all()
