"""The GPU FP64 brute force (mistic_bruteforce_rows, a subsample oracle at
scale): its per-row counts against the oracle on small inputs, then used at
full size to check the join's neighbour table on a sample of rows, where the
O(n^2) CPU brute force cannot run."""
import numpy as np
import pytest

from oracle import oracle as O

from mistic import workloads as W

pytestmark = pytest.mark.gpu


def _row_counts(pairs, n):
    c = np.zeros(n, dtype=np.int64)
    np.add.at(c, pairs[:, 0], 1)
    np.add.at(c, pairs[:, 1], 1)
    return c


@pytest.mark.parametrize("d,dtype", [(1, np.float64), (5, np.float64), (18, np.float64), (33, np.float32),
                                     (384, np.float32)])
def test_counts_match_oracle(handle, d, dtype):
    rng = np.random.default_rng(d)
    x = rng.normal(size=(3000, d)).astype(dtype)
    eps = float(np.sqrt(d) * 0.45)
    ref = _row_counts(O.brute_pairs(x, eps), 3000)
    got = handle.bruteforce_rows(x, eps, 0, 3000)
    assert np.array_equal(got, ref)
    part = handle.bruteforce_rows(x, eps, 1234, 2000)
    assert np.array_equal(part, ref[1234:2000])


def test_ties_and_duplicates(handle):
    x = np.random.default_rng(1).integers(0, 4, size=(2000, 3)).astype(np.float64)
    for eps in (0.0, 1.0, 2.0 ** 0.5):
        assert np.array_equal(handle.bruteforce_rows(x, eps, 0, 2000), _row_counts(O.brute_pairs(x, eps), 2000))


@pytest.mark.parametrize("which", ["msd90_full", "susy18_1m"])
def test_neighbour_table_degrees_at_scale(handle, which):
    if which == "msd90_full":
        wl = W.msd90()
    else:
        x = W.gen_susy_like(1_000_000)
        wl = W.Workload("susy18:1m", x, 6, float.fromhex(W.EPS_HEX["susy18:5000000"]), 64.0)
    x, n = wl.pts, wl.n
    r = handle.selfjoin(x, wl.k, wl.eps, csr="host")
    deg = np.diff(r.csr_offsets.astype(np.int64)) - 1  # minus the self edge
    rows = np.sort(np.random.default_rng(7).choice(n, size=512, replace=False))
    for lo, hi in ((rows[0], rows[0] + 256), (n - 256, n)):  # two contiguous blocks
        got = handle.bruteforce_rows(x, wl.eps, int(lo), int(hi))
        assert np.array_equal(got, deg[lo:hi])
    for i in rows[:64]:  # scattered rows
        assert handle.bruteforce_rows(x, wl.eps, int(i), int(i) + 1)[0] == deg[i]
    assert int(r.csr_offsets[-1]) == r.pairs_ordered_incl_self
