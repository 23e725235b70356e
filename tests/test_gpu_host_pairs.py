"""Host pair lists written by the join kernels straight into pinned host
memory (where the CPU-GPU link is coherent: GB300 with a Grace host) hold the
same pair set as the device list copied to the host after the join, and as
the oracle: every join kernel (CUDA-core FP64 and FP32, short-row and
long-row tensor core), the band decisions appended after the join, and a
first pass whose pair buffer overflows and runs again with a larger one."""
import numpy as np
import pytest

from helpers import canon, diff_pairs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _handles(monkeypatch):
    import mistic
    monkeypatch.setenv("MISTIC_HOST_PAIRS", "1")
    direct = mistic.Handle(0)  # reads MISTIC_HOST_PAIRS when it is created
    monkeypatch.setenv("MISTIC_HOST_PAIRS", "0")
    copied = mistic.Handle(0)
    return direct, copied


@pytest.mark.parametrize("n,d,k,mode,kernel", [
    (12_000, 6, 6, "fp64", None),
    (12_000, 18, 6, "fp32", None),
    (12_000, 18, 2, "bf16", "short-rows"),
    (6_000, 90, 2, "bf16", None),
    (4_000, 200, 2, "tf32", "k-chunked"),
    (4_000, 384, 2, "bf16", "k-chunked"),
])
def test_direct_host_pairs_match_oracle(monkeypatch, n, d, k, mode, kernel):
    from mistic import workloads as W
    x = W.gen_clusters(n, d, 12, seed=n + d)
    eps = W.calibrate_eps(x, 12.0, sample=min(n, 3000), seed=1)
    ref = O.brute_pairs(x, eps)
    assert len(ref) > 1000
    direct, copied = _handles(monkeypatch)
    try:
        for _ in range(2):  # the second call reuses the pinned block
            r = direct.selfjoin(x, k, eps, mode=mode, pairs="host")
            assert r.pairs_ij == len(ref)
            got = canon(r.pairs)
            assert np.array_equal(got, ref), diff_pairs(got, ref)
        if kernel is not None:
            assert r.tc_kernel == kernel
        rc = copied.selfjoin(x, k, eps, mode=mode, pairs="host")
        assert np.array_equal(canon(rc.pairs), ref)
        # a sorted list or a CSR table needs the device list: same pairs
        rs = direct.selfjoin(x, k, eps, mode=mode, pairs="host", sort_pairs=True)
        assert np.array_equal(rs.pairs, ref)
    finally:
        direct.close()
        copied.close()


def test_direct_host_pairs_after_overflow(monkeypatch):
    """More pairs than the first pass's buffer (2^20 for this n): the join
    runs again into a larger pinned block; the next call starts with it."""
    rng = np.random.default_rng(5)
    x = rng.random((120_000, 5))
    from mistic import workloads as W
    eps = W.calibrate_eps(x, 40.0, sample=4000, seed=2)
    direct, copied = _handles(monkeypatch)
    try:
        rc = copied.selfjoin(x, 4, eps, pairs="host", sort_pairs=True)
        assert rc.pairs_ij > (1 << 20) * 1.5
        for _ in range(2):
            r = direct.selfjoin(x, 4, eps, pairs="host")
            assert r.pairs_ij == rc.pairs_ij
            assert np.array_equal(canon(r.pairs), rc.pairs)
    finally:
        direct.close()
        copied.close()
