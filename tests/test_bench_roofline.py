"""The bench line's roofline object (CPU): the PageRank degree-bin kernels of
an iteration count as one launch, timed by the library's fork-to-join
`pagerank_iteration` span when the profile has it (the bins overlap, so
their summed kernel times would overstate the iteration), else by the sum of
the bin kernels; shares are of the step's time."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N, M = 16_777_216, 520_761_746
PER_ITER = 4 * (N + 1) + 8 * M + 8 * N


def profile(with_span):
    p = {"k_expand_sssp": (89, 20.0), "k_bottom_up": (183, 17.0), "k_pr_small": (20, 1.9),
         "k_pr_mid": (20, 21.3), "k_pr_big": (20, 28.1), "k_pr_chunks": (20, 9.4), "k_pr_long": (20, 15.9),
         "k_pr_init": (1, 0.1), "k_pr_bin_count": (1, 0.2)}
    if with_span:
        p["pagerank_iteration"] = (20, 28.4)
    return p


def test_span_times_the_iteration():
    import bench
    r = bench.roofline(profile(True), N, M, 1, [], None, 93.0)
    assert r["kernel"] == "pagerank_spmv"
    assert r["avg_launch_ms"] == pytest.approx(28.4 / 20)
    assert r["achieved"] == pytest.approx(PER_ITER / (28.4 / 20 / 1e3) / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["share_of_step"] == pytest.approx(28.4 / 93.0)
    assert set(r["kernels"]) == {"k_pr_small", "k_pr_mid", "k_pr_big", "k_pr_chunks", "k_pr_long"}


def test_without_span_the_bins_are_summed():
    import bench
    r = bench.roofline(profile(False), N, M, 1, [], None, 100.0)
    assert r["kernel"] == "pagerank_spmv"
    assert r["avg_launch_ms"] == pytest.approx((1.9 + 21.3 + 28.1 + 9.4 + 15.9) / 20)


def test_another_kernel_can_dominate():
    import bench
    p = profile(True)
    p["k_expand_sssp"] = (89, 40.0)
    r = bench.roofline(p, N, M, 1, [], None, 100.0)
    assert r["kernel"] == "k_expand_sssp" and r["achieved"] is None
    assert r["share_of_step"] == pytest.approx(0.4)
