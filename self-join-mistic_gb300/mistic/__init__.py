"""Python host interface of the GB300 ε-self-join (libmistic.so).

This mirrors the reference's data path (bwd29/self-join-MiSTIC
src/main.cu:20-182): points, d, k reference points and ε in; the number of
ordered pairs including self pairs ("Total results Set Size",
src/launcher.cu:3513), the unordered pair count and optionally the canonical
pair list out.  All work happens in the CUDA library; this module only moves
arguments across the C ABI.  There is no CPU fallback: a missing or unloadable
library raises.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

__all__ = ["MisticError", "JoinResult", "Handle", "selfjoin", "read_points", "convert_text"]

MODES = {"auto": L.MODE_AUTO, "fp64": L.MODE_FP64, "fp32": L.MODE_FP32, "bf16": L.MODE_BF16,
         "tf32": L.MODE_TF32}
RP_MODES = {"pca": L.RP_PCA, "box": L.RP_BOX, "user": L.RP_USER, "scored": L.RP_SCORED}


class MisticError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mistic error {status}: {msg}")
        self.status = status


@dataclass
class JoinResult:
    n: int
    d: int
    k_used: int
    pairs_ij: int
    pairs_ordered_incl_self: int
    candidates: int
    band_pairs: int
    ulp_ambiguous: int
    n_bins: int
    n_bin_pairs: int
    n_units: int
    n_units_tc: int
    tc_tiles: int
    tc_cells: int
    mode_used: str
    ms: dict
    kernel_launches: int
    pairs: np.ndarray | None = None          # (P, 2) uint32 host array
    csr_offsets: np.ndarray | None = None    # (n + 1,) uint64, host CSR table
    csr_nbrs: np.ndarray | None = None       # (offsets[n],) uint32
    device_pairs: int | None = None          # device pointer when pairs="device"
    tc_operands: str = "none"                # tensor-core operands: none, split-bf16, bf16, tf32
    tc_min_bin: int = 0                      # smallest home bin on the tensor cores
    tuned: bool = False                      # threshold / operands from the autotuner
    ring_passes: int = 0                     # ring mode: join passes
    ring_units_redone: int = 0               # ring mode: units run again after the ring filled
    tc_kernel: str = "none"                  # tensor-core join: none, short-rows, k-chunked
    extra: dict = field(default_factory=dict)


def _check(lib, h, status: int) -> None:
    if status != L.OK:
        msg = lib.mistic_last_error(h) if h else lib.mistic_strerror(status)
        raise MisticError(status, (msg or b"").decode(errors="replace"))


class Handle:
    """One library handle: a device, a CUDA stream and cached buffers."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = L.load()
        h = ctypes.c_void_p()
        st = self.lib.mistic_create(ctypes.byref(h), device, ctypes.c_void_p(stream) if stream else None)
        if st != L.OK:
            raise MisticError(st, self.lib.mistic_strerror(st).decode())
        self.h = h

    def close(self) -> None:
        if self.h:
            self.lib.mistic_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def opts(self, mode="auto", rp="pca", seed=0, pairs="none", sort_pairs=False,
             pair_capacity=0, input_on_device=False, check_finite=True, timing=True,
             rp_user=None, pair_buffer=None, csr="none", home_sample=0, autotune=0,
             ring_capacity=0) -> L.Opts:
        o = L.Opts()
        self.lib.mistic_opts_init(ctypes.byref(o))
        o.mode = MODES[mode]
        o.rp_mode = RP_MODES[rp]
        o.seed = seed
        o.pairs = {"none": L.PAIRS_NONE, "host": L.PAIRS_HOST, "device": L.PAIRS_DEVICE}[pairs]
        o.sort_pairs = 1 if sort_pairs else 0
        o.pair_capacity = pair_capacity
        if pair_buffer is not None:
            o.pair_buffer = ctypes.cast(ctypes.c_void_p(pair_buffer), ctypes.POINTER(ctypes.c_uint32))
        o.input_on_device = 1 if input_on_device else 0
        o.check_finite = 1 if check_finite else 0
        o.timing = 1 if timing else 0
        o.csr = {"none": L.PAIRS_NONE, "host": L.PAIRS_HOST, "device": L.PAIRS_DEVICE}[csr]
        o.home_sample = home_sample
        o.autotune = autotune
        o.ring_capacity = ring_capacity
        if rp_user is not None:
            self._rp_keep = np.ascontiguousarray(rp_user, dtype=np.float64)
            o.rp_user = self._rp_keep.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        return o

    def selfjoin_raw(self, ptr: int, n: int, d: int, dtype: int, k: int, eps: float,
                     opts: L.Opts) -> L.Result:
        """Call mistic_selfjoin on a raw pointer (host or device per opts)."""
        r = L.Result()
        st = self.lib.mistic_selfjoin(self.h, ctypes.c_void_p(ptr), n, d, dtype, k, float(eps),
                                      ctypes.byref(opts), ctypes.byref(r))
        if st != L.OK:
            self.lib.mistic_result_free(ctypes.byref(r))
        _check(self.lib, self.h, st)
        return r

    def to_result(self, r: L.Result, keep_device: bool = False) -> JoinResult:
        pairs = None
        dev = None
        if r.pairs and not r.pairs_on_device:
            cnt = int(r.pairs_len)
            pairs = (np.ctypeslib.as_array(r.pairs, shape=(cnt * 2,)).copy().reshape(cnt, 2)
                     if cnt else np.zeros((0, 2), np.uint32))
        elif r.pairs and r.pairs_on_device:
            dev = ctypes.cast(r.pairs, ctypes.c_void_p).value
        csr_off = csr_nb = None
        if r.csr_offsets and not r.csr_on_device:
            n1 = int(r.n) + 1
            csr_off = np.ctypeslib.as_array(r.csr_offsets, shape=(n1,)).copy()
            tot = int(csr_off[-1])
            csr_nb = (np.ctypeslib.as_array(r.csr_nbrs, shape=(tot,)).copy() if tot
                      else np.zeros((0,), np.uint32))
        ms = {k: getattr(r, "ms_" + k) for k in
              ("total", "h2d", "prep", "keys", "sort", "bins", "enum", "join", "d2h", "join_simt",
               "join_tc", "wall")}
        out = JoinResult(
            n=r.n, d=r.d, k_used=r.k_used, pairs_ij=r.pairs_ij,
            pairs_ordered_incl_self=r.pairs_ordered_incl_self, candidates=r.candidates,
            band_pairs=r.band_pairs, ulp_ambiguous=r.ulp_ambiguous, n_bins=r.n_bins,
            n_bin_pairs=r.n_bin_pairs, n_units=r.n_units, n_units_tc=r.n_units_tc,
            tc_tiles=r.tc_tiles, tc_cells=r.tc_cells,
            mode_used={0: "auto", 1: "fp64", 2: "fp32", 3: "bf16", 4: "tf32"}.get(r.mode_used, "?"),
            ms=ms, kernel_launches=r.kernel_launches, pairs=pairs, device_pairs=dev,
            csr_offsets=csr_off, csr_nbrs=csr_nb,
            tc_operands={0: "none", 1: "split-bf16", 2: "bf16", 3: "tf32"}.get(r.tc_operands, "?"),
            tc_min_bin=r.tc_min_bin, tuned=bool(r.tuned), ring_passes=r.ring_passes,
            ring_units_redone=r.ring_units_redone,
            tc_kernel={0: "none", 1: "short-rows", 2: "k-chunked"}.get(r.tc_kernel, "?"))
        if not keep_device or not r.pairs_on_device:
            self.lib.mistic_result_free(ctypes.byref(r))
        else:
            out.extra["_raw"] = r
        return out

    def selfjoin(self, pts: np.ndarray, k: int, eps: float, **kw) -> JoinResult:
        """ε-self-join of a host (n, d) float64/float32 array."""
        a = np.ascontiguousarray(pts)
        if a.dtype == np.float64:
            dt = L.F64
        elif a.dtype == np.float32:
            dt = L.F32
        else:
            a = a.astype(np.float64)
            dt = L.F64
        if a.ndim != 2:
            raise ValueError("points must be a 2-D array")
        n, d = a.shape
        o = self.opts(**kw)
        r = self.selfjoin_raw(a.ctypes.data if n else 0, n, d, dt, k, eps, o)
        return self.to_result(r)

    def batch_selfjoin(self, instances, **kw) -> list[JoinResult]:
        """mistic_batch_selfjoin over [(pts, k, eps), ...] host arrays; one
        result per instance, in order."""
        arrs, inst = [], (L.Instance * max(1, len(instances)))()
        for i, (pts, k, eps) in enumerate(instances):
            a = np.ascontiguousarray(pts)
            if a.dtype not in (np.float64, np.float32):
                a = a.astype(np.float64)
            arrs.append(a)
            inst[i].pts = a.ctypes.data if a.shape[0] else None
            inst[i].n, inst[i].d = a.shape
            inst[i].dtype = L.F64 if a.dtype == np.float64 else L.F32
            inst[i].k, inst[i].eps = k, float(eps)
        res = (L.Result * max(1, len(instances)))()
        o = self.opts(**kw)
        st = self.lib.mistic_batch_selfjoin(self.h, inst, len(instances), ctypes.byref(o), res)
        if st != L.OK:
            for i in range(len(instances)):
                self.lib.mistic_result_free(ctypes.byref(res[i]))
        _check(self.lib, self.h, st)
        return [self.to_result(res[i]) for i in range(len(instances))]

    def bruteforce_rows(self, pts, eps: float, row0: int, row1: int, on_device_ptr: int | None = None,
                        n: int | None = None, d: int | None = None, dtype: int | None = None) -> np.ndarray:
        """FP64 brute-force neighbour counts (self excluded) of rows
        [row0, row1) against all rows, on the GPU (mistic_bruteforce_rows).
        `pts` is a host array, or pass on_device_ptr with n, d, dtype."""
        out = np.zeros(max(0, row1 - row0), dtype=np.uint32)
        if on_device_ptr is None:
            a = np.ascontiguousarray(pts)
            if a.dtype not in (np.float64, np.float32):
                a = a.astype(np.float64)
            n, d = a.shape
            dtype = L.F64 if a.dtype == np.float64 else L.F32
            ptr, dev = a.ctypes.data, 0
        else:
            ptr, dev = on_device_ptr, 1
        st = self.lib.mistic_bruteforce_rows(self.h, ctypes.c_void_p(ptr), n, d, dtype, float(eps), row0, row1, dev,
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        _check(self.lib, self.h, st)
        return out

    def free_result(self, jr: JoinResult) -> None:
        raw = jr.extra.pop("_raw", None)
        if raw is not None:
            self.lib.mistic_result_free(ctypes.byref(raw))


def selfjoin(pts: np.ndarray, k: int, eps: float, device: int = 0, **kw) -> JoinResult:
    """One-shot ε-self-join (creates and destroys a handle)."""
    with Handle(device) as h:
        return h.selfjoin(pts, k, eps, **kw)


def read_points(path: str, d: int, dtype: str = "f64") -> np.ndarray:
    """Read a raw point file through the library's reader."""
    lib = L.load()
    p = ctypes.c_void_p()
    n = ctypes.c_uint64()
    dt = L.F64 if dtype == "f64" else L.F32
    st = lib.mistic_read_points(path.encode(), d, dt, ctypes.byref(p), ctypes.byref(n))
    if st != L.OK:
        raise MisticError(st, lib.mistic_strerror(st).decode())
    npdt = np.float64 if dt == L.F64 else np.float32
    cnt = int(n.value) * d
    if cnt:
        buf = (ctypes.c_char * (cnt * np.dtype(npdt).itemsize)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=npdt).copy().reshape(int(n.value), d)
    else:
        arr = np.zeros((0, d), dtype=npdt)
    lib.mistic_free_host(p)
    return arr


def convert_text(text_path: str, bin_path: str) -> int:
    """Text -> raw FP64 point file (the reference's toBin behaviour, see
    mistic_convert_text); returns the number of values written."""
    lib = L.load()
    n = ctypes.c_uint64()
    st = lib.mistic_convert_text(text_path.encode(), bin_path.encode(), ctypes.byref(n))
    if st != L.OK:
        raise MisticError(st, lib.mistic_strerror(st).decode())
    return int(n.value)
