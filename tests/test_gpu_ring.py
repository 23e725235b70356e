"""Streamed pair ring (mistic_opts.ring_capacity): pairs pass through a
device ring of a few thousand entries; each time it fills, the join stops
claiming work units, the ring is drained to the host and the join resumes
from its cursor.  The pair set must be exactly the oracle's -- no pair lost
or repeated -- across many passes, for the CUDA-core, short-row and
long-row tensor-core kernels, and through a host callback."""
import ctypes

import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

import mistic
from mistic import _lib as L
from mistic import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["auto", "fp32", "fp64"])
def test_ring_low_dimensional_sample(handle, mode):
    x = W.gen_susy_like(60000, seed=44)
    eps = 0.03
    ref = O.brute_pairs(x, eps)
    assert len(ref) > 20 * 4096
    r = handle.selfjoin(x, 6, eps, mode=mode, pairs="host", sort_pairs=True, ring_capacity=4096)
    assert r.ring_passes > 10
    assert r.pairs_ij == len(ref)
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


@pytest.mark.parametrize("mode", ["bf16", "tf32"])
def test_ring_384_dimensional(handle, mode):
    """Long rows on the K-chunked tensor-core kernel: 3,000 pairs of near
    duplicates among unit-norm 384-d rows, so a unit (at most 256 home rows,
    one neighbour each) never holds more than 256 pairs and a ring of 512
    needs several passes."""
    rng = np.random.default_rng(46)
    x = rng.normal(size=(6000, 384)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    x[3000:] = x[:3000] + rng.normal(scale=0.01, size=(3000, 384)).astype(np.float32)
    eps = 0.3
    ref = O.brute_pairs(x, eps)
    assert len(ref) == 3000
    r = handle.selfjoin(x, 8, eps, mode=mode, pairs="host", sort_pairs=True, ring_capacity=512)
    assert r.n_units_tc > 0 and r.ring_passes > 1
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_ring_to_a_host_sink(handle):
    x = np.random.default_rng(45).random((30000, 8))
    eps = 0.3
    ref = O.brute_pairs(x, eps)
    assert len(ref) > 10 * 3000
    got = []
    SINK = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64, ctypes.c_void_p)

    def sink(p, cnt, user):
        got.append(np.ctypeslib.as_array(p, shape=(int(cnt) * 2,)).copy().reshape(-1, 2))

    cb = SINK(sink)
    o = handle.opts(ring_capacity=3000)
    o.pair_sink = ctypes.cast(cb, ctypes.c_void_p)
    raw = handle.selfjoin_raw(x.ctypes.data, x.shape[0], 8, L.F64, 6, eps, o)
    r = handle.to_result(raw)
    assert r.pairs is None and r.pairs_ij == len(ref) and r.ring_passes > 1
    allp = np.concatenate(got)
    assert all(len(g) <= 3000 for g in got)
    from helpers import canon
    assert np.array_equal(canon(allp), ref)


def test_ring_smaller_than_one_unit_is_an_error(handle):
    x = np.ones((400, 3))  # one bin, one unit of 79,800 pairs
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 2, 0.5, pairs="host", ring_capacity=1000)
    assert e.value.status == L.ERR_PAIR_OVERFLOW
    r = handle.selfjoin(x, 2, 0.5, pairs="host", ring_capacity=100000)
    assert r.pairs_ij == 400 * 399 // 2
