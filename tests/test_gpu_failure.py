"""Failure detection without a GPU fault: a bounded device wait that runs out
must come back as MISTIC_ERR_TIMEOUT, and the handle must stay usable.

MISTIC_TEST_TC_STALL=1 makes the tensor-core join's MMA warp signal nothing
(a flag nothing sets), with a short wait limit: the epilogue's wait expires,
every warp role leaves its loop, tensor memory is released and the kernel
returns.  No trap, assert, bad address or endless loop is involved."""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

import mistic
from mistic import _lib as L
from mistic import workloads as W

pytestmark = pytest.mark.gpu


def test_tensor_core_wait_timeout_is_reported(handle, monkeypatch):
    x = W.gen_susy_like(20000, seed=9)
    eps = 0.03
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")
    monkeypatch.setenv("MISTIC_TEST_TC_STALL", "1")
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 6, eps, mode="bf16")
    assert e.value.status == L.ERR_TIMEOUT
    monkeypatch.delenv("MISTIC_TEST_TC_STALL")
    r = handle.selfjoin(x, 6, eps, mode="bf16", pairs="host", sort_pairs=True)
    ref = O.brute_pairs(x, eps)
    assert r.n_units_tc > 0
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
