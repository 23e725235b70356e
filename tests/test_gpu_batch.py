"""Batches of independent self-joins (mistic_batch_selfjoin): every
instance of a mixed-dimension batch must give the oracle's pair set --
fused (every instance's work units drained by shared persistent launches,
captured as one CUDA graph, or issued directly) and one pipeline per
instance (concurrently on worker streams, or one after another)."""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

from mistic import workloads as W

pytestmark = pytest.mark.gpu


def _instances(count, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(200, 3000))
        d = int(rng.choice([2, 8, 18, 32, 57, 90]))
        x = W.gen_clusters(n, d, int(rng.integers(1, 8)), seed=seed * 1000 + i, eig_lo=1e-2)
        eps = W.calibrate_eps(x.astype(np.float64), float(rng.choice([4.0, 16.0])), sample=min(n, 1500), seed=i)
        out.append((x, min(6, d), eps))
    return out


@pytest.mark.parametrize("fused,graph", [("1", "1"), ("1", "0"), ("0", "1")])
@pytest.mark.parametrize("streams", ["8", "1"])
def test_batch_matches_oracle(handle, monkeypatch, streams, fused, graph):
    monkeypatch.setenv("MISTIC_BATCH_STREAMS", streams)
    monkeypatch.setenv("MISTIC_BATCH_FUSED", fused)
    monkeypatch.setenv("MISTIC_BATCH_GRAPH", graph)
    inst = _instances(24)
    res = handle.batch_selfjoin(inst, pairs="host", sort_pairs=True)
    assert len(res) == len(inst)
    for (x, k, eps), r in zip(inst, res):
        ref = O.brute_pairs(x, eps)
        assert r.n == x.shape[0] and r.d == x.shape[1]
        assert r.pairs_ij == len(ref)
        assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


@pytest.mark.parametrize("pairs", ["none", "host"])
def test_fused_batch_with_tensor_core_units(handle, monkeypatch, pairs):
    """Instances large enough for tensor-core units (d = 18, 32, 90) next to
    small ones (d = 2): counts and pair sets per instance."""
    monkeypatch.setenv("MISTIC_BATCH_FUSED", "1")
    rng = np.random.default_rng(9)
    inst = []
    for i, (n, d) in enumerate([(40000, 18), (500, 2), (20000, 90), (3000, 8), (25000, 32), (800, 57)]):
        x = W.gen_clusters(n, d, 3, seed=500 + i, eig_lo=1e-2)
        eps = W.calibrate_eps(x.astype(np.float64), 16.0, sample=min(n, 2000), seed=i)
        inst.append((x, min(6, d), eps))
    res = handle.batch_selfjoin(inst, pairs=pairs, sort_pairs=True)
    assert sum(r.n_units_tc for r in res) > 0
    for (x, k, eps), r in zip(inst, res):
        ref = O.brute_pairs(x, eps)
        assert r.pairs_ij == len(ref)
        assert r.pairs_ordered_incl_self == 2 * len(ref) + x.shape[0]
        if pairs == "host":
            assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_batch_reports_the_failing_instance(handle):
    inst = _instances(6, seed=4)
    x, k, _ = inst[3]
    inst[3] = (x, k, -1.0)  # negative ε is an invalid argument
    import mistic
    from mistic import _lib as L
    with pytest.raises(mistic.MisticError) as e:
        handle.batch_selfjoin(inst, pairs="host")
    assert e.value.status == L.ERR_INVALID_ARG and "eps" in str(e.value)
    # the handle stays usable
    r = handle.batch_selfjoin(inst[:3], pairs="host", sort_pairs=True)
    for (x, k, eps), q in zip(inst[:3], r):
        assert np.array_equal(q.pairs, O.brute_pairs(x, eps))
