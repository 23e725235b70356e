"""Failure detection without a GPU fault: a bounded device wait that runs out
must come back as MISTIC_ERR_TIMEOUT, and the handle must stay usable.

MISTIC_TEST_TC_STALL=1 makes the tensor-core joins' MMA warp signal nothing
(a flag nothing sets), with a short wait limit: the epilogue's (and, in the
long-row kernel, the producers') waits expire, every warp role leaves its
loop, copies in flight are waited for, tensor memory is released and the
kernel returns.  No trap, assert, bad address or endless loop is involved."""
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


def test_long_row_wait_timeout_is_reported(handle, monkeypatch):
    """The K-chunked kernel (d = 384): the producer that issues a contiguous
    group's TMA tiles alone finds its stage never freed, gives up, and every
    producer leaves at its next shared wait."""
    wl = W.tiny384(3000)
    x, eps = wl.pts, wl.eps
    monkeypatch.setenv("MISTIC_TEST_TC_STALL", "1")
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 2, eps, mode="bf16")
    assert e.value.status == L.ERR_TIMEOUT
    monkeypatch.delenv("MISTIC_TEST_TC_STALL")
    r = handle.selfjoin(x, 2, eps, mode="bf16", pairs="host", sort_pairs=True)
    ref = O.brute_pairs(x, eps)
    assert r.tc_kernel == "k-chunked" and r.n_units_tc > 0
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
