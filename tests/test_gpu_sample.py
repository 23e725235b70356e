"""mistic_opts.home_sample: a fixed sample of the join at full density (the
home points of about 1 in S groups of 512 points of every bin, each joined
with all its candidates).  The sample must be the same in every mode -- the
benchmark compares mixed precision with plain FP64 on it -- and its pairs
must be pairs of the full join."""
import numpy as np
import pytest

from helpers import canon
from oracle import oracle as O

from mistic import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("x,k,eps", [
    (W.gen_susy_like(60000, seed=21), 6, 0.03),
    (np.random.default_rng(22).normal(size=(20000, 90)), 8, 9.0),
])
def test_sample_is_identical_across_modes_and_inside_the_full_join(handle, x, k, eps):
    ref = O.brute_pairs(x, eps)
    full = set(map(tuple, ref.tolist()))
    S = 4
    out = {}
    for mode in ("fp64", "fp32", "bf16", "tf32"):
        r = handle.selfjoin(x, k, eps, mode=mode, pairs="host", sort_pairs=True, home_sample=S)
        out[mode] = r
    base = out["fp64"]
    assert 0 < base.pairs_ij < len(ref)
    for mode, r in out.items():
        assert np.array_equal(r.pairs, base.pairs), mode
        assert r.candidates == base.candidates, mode
    assert set(map(tuple, base.pairs.tolist())) <= full
    rall = handle.selfjoin(x, k, eps, mode="fp64")
    assert 0.05 * rall.candidates < base.candidates < 0.6 * rall.candidates
    # S = 1 is the whole join
    r1 = handle.selfjoin(x, k, eps, pairs="host", sort_pairs=True, home_sample=1)
    assert np.array_equal(canon(r1.pairs), ref)
