"""ORACLE — test infrastructure only.

ctypes binding of oracle/brute.c, the CPU restatement of the reference's
brute-force ε-self-join (src/utils.cu:285-317 of bwd29/self-join-MiSTIC).
Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, no GPU)."""
    srcs = [os.path.join(_HERE, f) for f in ("brute.c", "hostjoin.c", "Makefile")]
    if force or not os.path.exists(_LIB) or any(os.path.getmtime(_LIB) < os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        u64, u32, i32, dbl, vp = (ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_void_p)
        L.oracle_brute_pairs.restype = u64
        L.oracle_brute_pairs.argtypes = [vp, i32, u64, u32, dbl,
                                         ctypes.POINTER(ctypes.POINTER(u32)),
                                         ctypes.POINTER(u64), i32]
        L.oracle_query_pairs.restype = u64
        L.oracle_query_pairs.argtypes = [vp, i32, u64, u32, dbl, vp, u64,
                                         ctypes.POINTER(ctypes.POINTER(u32)), i32]
        L.oracle_brute_count_ordered.restype = u64
        L.oracle_brute_count_ordered.argtypes = [vp, i32, u64, u32, dbl, i32]
        L.oracle_brute_count_rows.restype = u64
        L.oracle_brute_count_rows.argtypes = [vp, i32, u64, u32, dbl, u64, u64, i32]
        L.oracle_sqdist.restype = dbl
        L.oracle_sqdist.argtypes = [vp, i32, u64, u64, u32]
        L.oracle_max_threads.restype = i32
        L.hostjoin_count.restype = u64
        L.hostjoin_count.argtypes = [vp, u64, u32, vp, i32, dbl, u64, i32, ctypes.POINTER(u64),
                                     ctypes.POINTER(u64), ctypes.POINTER(dbl), ctypes.POINTER(dbl),
                                     ctypes.POINTER(u64)]
        L.oracle_free.argtypes = [vp]
        _lib = L
    return _lib


def _prep(pts: np.ndarray):
    if pts.dtype == np.float32:
        a = np.ascontiguousarray(pts, dtype=np.float32)
        return a, 1
    a = np.ascontiguousarray(pts, dtype=np.float64)
    return a, 0


def _take_pairs(ptr, count: int) -> np.ndarray:
    if count == 0:
        lib().oracle_free(ptr)
        return np.zeros((0, 2), dtype=np.uint32)
    arr = np.ctypeslib.as_array(ptr, shape=(count * 2,)).copy().reshape(count, 2)
    lib().oracle_free(ptr)
    return arr


def brute_pairs(pts: np.ndarray, eps: float, threads: int = 0,
                want_ambig: bool = False):
    """Canonical (i<j, sorted) pair array of the brute-force join, plus the
    count of pairs within 4 ulp of eps*eps when requested."""
    a, dt = _prep(pts)
    n, d = a.shape
    p = ctypes.POINTER(ctypes.c_uint32)()
    amb = ctypes.c_uint64(0)
    cnt = lib().oracle_brute_pairs(a.ctypes.data, dt, n, d, float(eps),
                                   ctypes.byref(p),
                                   ctypes.byref(amb) if want_ambig else None,
                                   threads)
    pairs = _take_pairs(p, int(cnt))
    if want_ambig:
        return pairs, int(amb.value)
    return pairs


def query_pairs(pts: np.ndarray, eps: float, queries, threads: int = 0) -> np.ndarray:
    """All pairs (min, max) involving the given rows, same predicate."""
    a, dt = _prep(pts)
    n, d = a.shape
    q = np.ascontiguousarray(np.sort(np.asarray(queries, dtype=np.uint32)))
    p = ctypes.POINTER(ctypes.c_uint32)()
    cnt = lib().oracle_query_pairs(a.ctypes.data, dt, n, d, float(eps),
                                   q.ctypes.data, q.size, ctypes.byref(p), threads)
    return _take_pairs(p, int(cnt))


def count_ordered(pts: np.ndarray, eps: float, threads: int = 0) -> int:
    """The reference's brute_force number: ordered pairs incl. self."""
    a, dt = _prep(pts)
    n, d = a.shape
    return int(lib().oracle_brute_count_ordered(a.ctypes.data, dt, n, d, float(eps), threads))


def count_rows(pts: np.ndarray, eps: float, i0: int, i1: int, threads: int = 0) -> int:
    a, dt = _prep(pts)
    n, d = a.shape
    return int(lib().oracle_brute_count_rows(a.ctypes.data, dt, n, d, float(eps), i0, i1, threads))


def sqdist(pts: np.ndarray, i: int, j: int) -> float:
    a, dt = _prep(pts)
    return float(lib().oracle_sqdist(a.ctypes.data, dt, i, j, a.shape[1]))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def pca_far_points(pts: np.ndarray, k: int, sample: int = 8192, seed: int = 0) -> np.ndarray:
    """k reference points for the host grid join: the sample mean moved well
    outside the data along the sample's top-k principal axes (far points make
    the distance fields nearly linear projections)."""
    x = np.asarray(pts, dtype=np.float64)
    rng = np.random.default_rng(seed)
    s = x[rng.choice(x.shape[0], size=min(sample, x.shape[0]), replace=False)] if x.shape[0] > sample else x
    mu = s.mean(axis=0)
    c = s - mu
    _, _, vt = np.linalg.svd(c, full_matrices=False)
    span = float(np.max(np.linalg.norm(c, axis=1))) if c.size else 1.0
    k = min(k, vt.shape[0])
    return np.ascontiguousarray(mu + 10.0 * max(span, 1e-300) * vt[:k], dtype=np.float64)


def host_join(pts: np.ndarray, eps: float, rps: np.ndarray, home_stride: int = 1, threads: int = 0) -> dict:
    """The project's own OpenMP host grid join (oracle/hostjoin.c): unordered
    pairs of the joined home bins (every `home_stride`-th), their candidate
    pairs and those of all bins, and the seconds of the index build with the
    neighbour enumeration and of the sampled distance work."""
    x = np.ascontiguousarray(pts, dtype=np.float64)
    r = np.ascontiguousarray(rps, dtype=np.float64)
    cs, ca, nb = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
    si, sj = ctypes.c_double(0), ctypes.c_double(0)
    p = lib().hostjoin_count(x.ctypes.data, x.shape[0], x.shape[1], r.ctypes.data, r.shape[0], float(eps),
                             int(home_stride), threads, ctypes.byref(cs), ctypes.byref(ca), ctypes.byref(si),
                             ctypes.byref(sj), ctypes.byref(nb))
    return {"pairs": int(p), "cand_sampled": int(cs.value), "cand_all": int(ca.value), "s_index": si.value,
            "s_join": sj.value, "bins": int(nb.value)}
