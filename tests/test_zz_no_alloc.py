"""mistic_selfjoin_noalloc: the entry point for callers that cannot allocate
device memory (a pool allocator owns it all, or cudaMalloc's implicit
synchronisation is not acceptable on their path).

It is called through the C ABI on device inputs with a caller-owned device
pair buffer, twice in a row (the second call reuses the static scratch
that the first left behind), and its pair set must equal the regular
mistic_selfjoin's bit for bit, the tolerance of every parity test here.
This file sorts last so that a first-failure run has run everything else."""
import ctypes

import numpy as np
import pytest

from helpers import canon

from mistic import _lib as L

pytestmark = pytest.mark.gpu


class _DevView:
    def __init__(self, ptr, count):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<i4",
                                         "data": (ptr, False), "version": 3}


def _noalloc(lib, torch, xt, n, d, dt, eps, cap):
    buf = torch.zeros((cap,), dtype=torch.int64, device="cuda")
    cnt = ctypes.c_uint64(0)
    torch.cuda.synchronize()
    st = lib.mistic_selfjoin_noalloc(ctypes.c_void_p(xt.data_ptr()), n, d, dt, eps,
                                     ctypes.c_void_p(buf.data_ptr()), cap, ctypes.byref(cnt), None)
    return st, int(cnt.value), buf


@pytest.mark.parametrize("dtype,d,eps", [("f64", 18, 0.75), ("f32", 33, 5.0)])
def test_noalloc_matches_selfjoin_twice(handle, dtype, d, eps):
    torch = pytest.importorskip("torch")
    lib = L.load()
    rng = np.random.default_rng(77 + d)
    x = rng.random((6000, d)) if dtype == "f64" else rng.normal(size=(6000, d)).astype(np.float32)
    n = x.shape[0]
    dt = L.F64 if dtype == "f64" else L.F32
    ref = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True)
    assert ref.pairs_ij > 0
    xt = torch.from_numpy(x).cuda()
    for _ in range(2):
        st, cnt, buf = _noalloc(lib, torch, xt, n, d, dt, eps, ref.pairs_ij + 16)
        assert st == L.OK, lib.mistic_strerror(st)
        assert cnt == ref.pairs_ij
        got = buf[:cnt].cpu().numpy().view(np.uint32).reshape(-1, 2)
        assert (got[:, 0] < got[:, 1]).all()
        assert np.array_equal(canon(got), ref.pairs)


def test_noalloc_limits_and_overflow(handle):
    torch = pytest.importorskip("torch")
    lib = L.load()
    x = np.random.default_rng(3).random((3000, 4))
    xt = torch.from_numpy(x).cuda()
    ref = handle.selfjoin(x, 3, 0.1)
    st, cnt, _ = _noalloc(lib, torch, xt, 3000, 4, L.F64, 0.1, 5)
    assert st == L.ERR_PAIR_OVERFLOW and cnt == ref.pairs_ij
    cnt = ctypes.c_uint64(0)
    # beyond the stated scratch limit: rejected before any device work
    big_n = L.NOALLOC_SCRATCH_BYTES // (4 * 4) + 1
    assert lib.mistic_selfjoin_noalloc(ctypes.c_void_p(xt.data_ptr()), big_n, 4, L.F64, 0.1, None, 0,
                                       ctypes.byref(cnt), None) == L.ERR_TOO_LARGE
    assert lib.mistic_selfjoin_noalloc(ctypes.c_void_p(xt.data_ptr()), 10, L.NOALLOC_MAX_D + 1, L.F64, 0.1,
                                       None, 0, ctypes.byref(cnt), None) == L.ERR_TOO_LARGE
