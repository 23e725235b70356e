"""The project's own OpenMP host grid join (oracle/hostjoin.c), timed by the
benchmark as an indexed CPU baseline: on seeded inputs its pair count equals
the brute-force oracle's, and a sampled run joins exactly the candidate
pairs of the sampled home bins."""
import numpy as np
import pytest

from oracle import oracle as O
from mistic import workloads as W


@pytest.mark.parametrize("case", ["uniform", "susy", "gauss90", "grid_ties", "dups"])
def test_host_join_count_equals_brute_force(case):
    rng = np.random.default_rng(7)
    if case == "uniform":
        x, eps, k = rng.random((20000, 8)), 0.12, 6
    elif case == "susy":
        x, eps, k = W.gen_susy_like(30000, seed=3), 0.03, 6
    elif case == "gauss90":
        x, eps, k = rng.normal(size=(5000, 90)), 9.0, 8
    elif case == "grid_ties":
        x, eps, k = np.floor(rng.random((3000, 3)) * 10), 1.0, 3
    else:
        x = rng.random((4000, 5))
        x[2000:2400] = x[:400]
        x, eps, k = x, 1e-9, 4
    ref = O.brute_pairs(x, eps)
    r = O.host_join(x, eps, O.pca_far_points(x, k))
    assert r["pairs"] == len(ref)
    assert r["cand_sampled"] == r["cand_all"] >= r["pairs"]


def test_host_join_sample_covers_its_home_bins():
    x = W.gen_susy_like(20000, seed=5)
    rp = O.pca_far_points(x, 6)
    full = O.host_join(x, 0.03, rp)
    parts = [O.host_join(x, 0.03, rp, home_stride=4) for _ in range(1)]
    s = parts[0]
    assert s["cand_all"] == full["cand_all"] and 0 < s["cand_sampled"] < full["cand_all"]
    assert s["pairs"] <= full["pairs"]
