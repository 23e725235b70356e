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


def _pairs_of(buf, cnt):
    got = buf[:cnt].cpu().numpy().view(np.uint32).reshape(-1, 2)
    assert (got[:, 0] < got[:, 1]).all()
    return canon(got)


@pytest.mark.parametrize("case", ["max_d", "tiny_eps", "huge_offsets"])
def test_noalloc_edge_cases_against_oracle(handle, case):
    """d at MISTIC_NOALLOC_MAX_D, and the two inputs on which the FP32 filter
    cannot be used (eps^2 below 1e-28; row offsets beyond FLT_MAX), where every
    candidate is decided in FP64: the pair set must equal the oracle's and the
    regular entry point's."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    lib = L.load()
    rng = np.random.default_rng(11)
    if case == "max_d":
        d = int(L.NOALLOC_MAX_D)
        x = rng.random((1500, d))
        x[700:710] = x[0:10] + 1e-3  # a few close pairs
        eps = 0.05
    elif case == "tiny_eps":
        d = 5
        x = rng.random((2000, d))
        x[1000:1040] = x[0:40]  # exact duplicates: distance 0
        eps = 1e-15
    else:
        d = 3
        x = rng.random((2000, d))
        x[100:120] = 1e300  # twenty identical far rows, row 0 near the origin
        eps = 0.02
    ref = O.brute_pairs(x, eps)
    assert len(ref) > 0
    assert np.array_equal(handle.selfjoin(x, 4, eps, pairs="host", sort_pairs=True).pairs, ref)
    xt = torch.from_numpy(x).cuda()
    for _ in range(2):
        st, cnt, buf = _noalloc(lib, torch, xt, x.shape[0], d, L.F64, eps, len(ref) + 16)
        assert st == L.OK, lib.mistic_strerror(st)
        assert cnt == len(ref)
        assert np.array_equal(_pairs_of(buf, cnt), ref)


def test_noalloc_rejects_non_finite_and_allocates_nothing(handle):
    """A NaN in row 0 (which every FP32 row is taken relative to) is rejected
    as the regular entry point rejects it; and a second call leaves the
    device's free memory exactly where the first left it."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    lib = L.load()
    x = np.random.default_rng(5).random((4000, 18))
    eps = 0.75
    ref = O.brute_pairs(x, eps)
    xt = torch.from_numpy(x).cuda()
    buf = torch.zeros((len(ref) + 16,), dtype=torch.int64, device="cuda")
    cnt = ctypes.c_uint64(0)

    def call(pts):
        torch.cuda.synchronize()
        return lib.mistic_selfjoin_noalloc(ctypes.c_void_p(pts.data_ptr()), x.shape[0], 18, L.F64, eps,
                                           ctypes.c_void_p(buf.data_ptr()), len(ref) + 16, ctypes.byref(cnt),
                                           None)

    assert call(xt) == L.OK and cnt.value == len(ref)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert call(xt) == L.OK and cnt.value == len(ref)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.array_equal(_pairs_of(buf, cnt.value), ref)
    bad = xt.clone()
    bad[0, 3] = float("nan")
    assert call(bad) == L.ERR_NOT_FINITE
    import mistic
    with pytest.raises(mistic.MisticError) as ei:
        handle.selfjoin(bad.cpu().numpy(), 6, eps)
    assert ei.value.status == L.ERR_NOT_FINITE
