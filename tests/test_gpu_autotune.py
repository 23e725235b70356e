"""The autotuner: the tensor-core bin threshold (and, for long rows, the
operand precision) timed on a sample of the work on the first call for a
shape, written to the tune cache file, and reused.  Results stay exact
whatever it picks."""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

from mistic import workloads as W

pytestmark = pytest.mark.gpu


def test_tuner_writes_and_reuses_the_cache(handle, monkeypatch, tmp_path):
    cache = tmp_path / "tune.tsv"
    monkeypatch.setenv("MISTIC_TUNE_CACHE", str(cache))
    x = W.gen_susy_like(80000, seed=31)
    eps = 0.03
    ref = O.brute_pairs(x, eps)
    r1 = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True, autotune=1)
    assert r1.tuned and r1.tc_min_bin >= 1
    assert np.array_equal(r1.pairs, ref), diff_pairs(r1.pairs, ref)
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].startswith("v4 d=18")
    key, tc_min, prec, ms = lines[0].split("\t")
    assert int(tc_min) == r1.tc_min_bin and int(prec) == 0 and float(ms) > 0
    r2 = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True, autotune=1)
    assert r2.tuned and r2.tc_min_bin == r1.tc_min_bin
    assert len(cache.read_text().strip().splitlines()) == 1  # reused, not re-measured
    assert np.array_equal(r2.pairs, ref)
    r3 = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True, autotune=-1)
    assert not r3.tuned
    assert np.array_equal(r3.pairs, ref)


def test_tuner_long_rows_precision_choice(handle, monkeypatch, tmp_path):
    """Unit-norm 256-d rows with a wide eps: both operand precisions are
    candidates; the pick is cached and the pair set is exact."""
    cache = tmp_path / "tune.tsv"
    monkeypatch.setenv("MISTIC_TUNE_CACHE", str(cache))
    rng = np.random.default_rng(78)
    x = rng.normal(size=(6000, 256)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    x[3000:] = x[:3000] + rng.normal(scale=0.04, size=(3000, 256)).astype(np.float32)
    eps = 1.0
    ref = O.brute_pairs(x, eps)
    r = handle.selfjoin(x, 8, eps, pairs="host", sort_pairs=True, autotune=1)
    assert r.tuned and r.tc_operands in ("split-bf16", "bf16")
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
    key, tc_min, prec, ms = cache.read_text().strip().splitlines()[0].split("\t")
    assert "tcw" in key and int(prec) == (1 if r.tc_operands == "bf16" else 0)
