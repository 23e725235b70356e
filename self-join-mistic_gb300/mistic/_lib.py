"""ctypes binding of libmistic.so (include/mistic.h).

The structures below mirror the C declarations field for field; the test
suite checks their sizes against the library's own view (opts.struct_size).
No fallback exists: if the library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

u32, u64, i32, dbl, vp = (ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32,
                          ctypes.c_double, ctypes.c_void_p)

# enum values (include/mistic.h)
OK = 0
ERR_INVALID_ARG, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_TOO_LARGE = 1, 2, 3, 4
ERR_NOT_FINITE, ERR_PAIR_OVERFLOW, ERR_TIMEOUT, ERR_NO_DEVICE = 5, 6, 7, 8
ERR_IO, ERR_INTERNAL = 9, 10
F64, F32 = 0, 1
MODE_AUTO, MODE_FP64, MODE_FP32, MODE_BF16, MODE_TF32 = 0, 1, 2, 3, 4
RP_PCA, RP_BOX, RP_USER, RP_SCORED = 0, 1, 2, 3
PAIRS_NONE, PAIRS_HOST, PAIRS_DEVICE = 0, 1, 2

#: every symbol include/mistic.h declares
EXPORTS = (
    "mistic_abi_version", "mistic_opts_init", "mistic_create", "mistic_destroy",
    "mistic_selfjoin", "mistic_batch_selfjoin", "mistic_read_points",
    "mistic_free_host", "mistic_result_free", "mistic_strerror",
    "mistic_last_error", "mistic_selfjoin_noalloc", "mistic_convert_text", "mistic_bruteforce_rows",
    "mistic_tc_gram_probe",
)

#: scratch limits of mistic_selfjoin_noalloc (include/mistic.h)
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024
NOALLOC_MAX_D = 128


class Opts(ctypes.Structure):
    _fields_ = [
        ("struct_size", u32),
        ("mode", i32),
        ("rp_mode", i32),
        ("rp_user", ctypes.POINTER(dbl)),
        ("seed", u64),
        ("input_on_device", i32),
        ("pairs", i32),
        ("sort_pairs", i32),
        ("pair_capacity", u64),
        ("pair_buffer", ctypes.POINTER(u32)),
        ("check_finite", i32),
        ("timing", i32),
        ("csr", i32),
        ("home_sample", u32),
        ("autotune", i32),
        ("ring_capacity", u64),
        ("pair_sink", vp),
        ("sink_user", vp),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("n", u64),
        ("d", u32), ("k_used", u32),
        ("pairs_ij", u64),
        ("pairs_ordered_incl_self", u64),
        ("candidates", u64),
        ("band_pairs", u64),
        ("ulp_ambiguous", u64),
        ("n_bins", u64),
        ("n_bin_pairs", u64),
        ("n_units", u64),
        ("n_units_tc", u64),
        ("tc_tiles", u64),
        ("tc_cells", u64),
        ("pairs", ctypes.POINTER(u32)),
        ("pairs_len", u64),
        ("pairs_on_device", i32),
        ("mode_used", i32),
        ("ms_total", dbl), ("ms_h2d", dbl), ("ms_prep", dbl), ("ms_keys", dbl),
        ("ms_sort", dbl), ("ms_bins", dbl), ("ms_enum", dbl), ("ms_join", dbl),
        ("ms_d2h", dbl),
        ("ms_join_simt", dbl), ("ms_join_tc", dbl),
        ("ms_wall", dbl),
        ("kernel_launches", u32),
        ("csr_offsets", ctypes.POINTER(u64)),
        ("csr_nbrs", ctypes.POINTER(u32)),
        ("csr_on_device", i32),
        ("tc_operands", i32),
        ("tc_min_bin", u32),
        ("tuned", i32),
        ("ring_passes", u32),
        ("ring_units_redone", u64),
        ("tc_kernel", i32),
        ("_owner", vp),
    ]


class Instance(ctypes.Structure):
    _fields_ = [
        ("pts", vp),
        ("n", u64),
        ("d", u32),
        ("dtype", i32),
        ("k", u32),
        ("eps", dbl),
    ]


_lib = None


def load(build_if_needed: bool = True) -> ctypes.CDLL:
    """Load libmistic.so (building it first when stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_needed:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libmistic.so not found at {path}; run the build first")
    L = ctypes.CDLL(path)
    L.mistic_abi_version.restype = ctypes.c_int
    L.mistic_opts_init.argtypes = [ctypes.POINTER(Opts)]
    L.mistic_opts_init.restype = None
    L.mistic_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, vp]
    L.mistic_create.restype = ctypes.c_int
    L.mistic_destroy.argtypes = [vp]
    L.mistic_destroy.restype = ctypes.c_int
    L.mistic_selfjoin.argtypes = [vp, vp, u64, u32, ctypes.c_int, u32, dbl,
                                  ctypes.POINTER(Opts), ctypes.POINTER(Result)]
    L.mistic_selfjoin.restype = ctypes.c_int
    L.mistic_batch_selfjoin.argtypes = [vp, ctypes.POINTER(Instance), u32,
                                        ctypes.POINTER(Opts), ctypes.POINTER(Result)]
    L.mistic_batch_selfjoin.restype = ctypes.c_int
    L.mistic_read_points.argtypes = [ctypes.c_char_p, u32, ctypes.c_int,
                                     ctypes.POINTER(vp), ctypes.POINTER(u64)]
    L.mistic_read_points.restype = ctypes.c_int
    L.mistic_bruteforce_rows.argtypes = [vp, vp, u64, u32, ctypes.c_int, dbl, u64, u64, ctypes.c_int,
                                         ctypes.POINTER(u32)]
    L.mistic_bruteforce_rows.restype = ctypes.c_int
    L.mistic_convert_text.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(u64)]
    L.mistic_convert_text.restype = ctypes.c_int
    L.mistic_free_host.argtypes = [vp]
    L.mistic_free_host.restype = None
    L.mistic_result_free.argtypes = [ctypes.POINTER(Result)]
    L.mistic_result_free.restype = None
    L.mistic_strerror.argtypes = [ctypes.c_int]
    L.mistic_strerror.restype = ctypes.c_char_p
    L.mistic_last_error.argtypes = [vp]
    L.mistic_last_error.restype = ctypes.c_char_p
    L.mistic_selfjoin_noalloc.argtypes = [vp, u64, u32, ctypes.c_int, dbl, vp, u64,
                                          ctypes.POINTER(u64), vp]
    L.mistic_selfjoin_noalloc.restype = ctypes.c_int
    L.mistic_tc_gram_probe.argtypes = [ctypes.c_int, vp, vp, u32, vp]
    L.mistic_tc_gram_probe.restype = ctypes.c_int
    _lib = L
    return L
