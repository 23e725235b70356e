"""Orchestration guards that turn would-be wrong results into errors.

- The join's work lists address neighbour bins and units with 32-bit
  offsets.  Their totals are also summed in 64 bits; a total the 32-bit
  offsets cannot hold makes the call fail with MISTIC_ERR_TOO_LARGE instead of
  wrapping and silently dropping candidate pairs.  MISTIC_TEST_WORKLIST_LIMIT
  lowers the limit so that an ordinary input crosses it.
- The join runs again when its band list (pairs left to the FP64 decision)
  or its self-sized pair buffer overflowed.  If the last pass still
  overflowed, the call fails with MISTIC_ERR_INTERNAL rather than return
  counts nothing was decided for.  MISTIC_TEST_JOIN_ATTEMPTS=1 with a 1-entry
  band list (MISTIC_BAND_CAP=1) forces that exit.
- Coordinates near 1e300 overflow the FP64 reference-point distances; the
  affected key fields are dropped and the join stays exact.
"""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

import mistic
from mistic import _lib as L
from mistic import workloads as W

pytestmark = pytest.mark.gpu


def test_worklist_beyond_32bit_offsets_is_an_error(handle, monkeypatch):
    x = np.random.default_rng(31).random((20000, 18))
    eps = 0.62
    r = handle.selfjoin(x, 6, eps)
    assert r.n_units + r.n_units_tc > 50 and r.n_bin_pairs > 50
    monkeypatch.setenv("MISTIC_TEST_WORKLIST_LIMIT", "50")
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 6, eps, pairs="host")
    assert e.value.status == L.ERR_TOO_LARGE
    monkeypatch.delenv("MISTIC_TEST_WORKLIST_LIMIT")
    r2 = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True)
    ref = O.brute_pairs(x, eps)
    assert np.array_equal(r2.pairs, ref), diff_pairs(r2.pairs, ref)


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_last_join_pass_must_be_complete(handle, monkeypatch, mode):
    x = W.gen_susy_like(30000, seed=4)
    eps = 0.03
    r = handle.selfjoin(x, 6, eps, mode=mode)
    assert r.band_pairs > 1
    monkeypatch.setenv("MISTIC_BAND_CAP", "1")
    monkeypatch.setenv("MISTIC_TEST_JOIN_ATTEMPTS", "1")
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 6, eps, mode=mode)
    assert e.value.status == L.ERR_INTERNAL
    # with the regular number of passes the overflow is absorbed by a rerun
    monkeypatch.delenv("MISTIC_TEST_JOIN_ATTEMPTS")
    r2 = handle.selfjoin(x, 6, eps, mode=mode, pairs="host", sort_pairs=True)
    ref = O.brute_pairs(x, eps)
    assert np.array_equal(r2.pairs, ref), diff_pairs(r2.pairs, ref)


@pytest.mark.parametrize("mode", ["auto", "fp64"])
def test_coordinates_near_fp64_overflow(handle, mode):
    rng = np.random.default_rng(12)
    x = rng.random((3000, 3))
    x[100:120] = 1e300
    x[200:204] = -1e300
    eps = 0.02
    ref = O.brute_pairs(x, eps)
    r = handle.selfjoin(x, 4, eps, mode=mode, pairs="host", sort_pairs=True)
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
