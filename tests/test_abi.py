"""The C ABI: library loads, exports every declared symbol, structure layout
and host-side error paths (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT

import mistic
from mistic import _lib as L


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mistic.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mistic_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    decl = declared_functions()
    assert len(decl) >= 10
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) == set(L.EXPORTS)


def test_abi_version_and_opts_layout():
    lib = L.load()
    assert lib.mistic_abi_version() == 2
    o = L.Opts()
    lib.mistic_opts_init(ctypes.byref(o))
    assert o.struct_size == ctypes.sizeof(L.Opts)
    assert o.mode == L.MODE_AUTO and o.rp_mode == L.RP_PCA and o.check_finite == 1


def test_strerror_covers_all_codes():
    lib = L.load()
    for s in range(11):
        assert lib.mistic_strerror(s) not in (None, b"unknown status")
    assert lib.mistic_strerror(99) == b"unknown status"


def test_read_points_roundtrip(tmp_path):
    x = np.arange(30, dtype=np.float64).reshape(10, 3)
    p = tmp_path / "x.bin"
    x.tofile(p)
    with open(p, "ab") as f:  # trailing partial row is ignored like the reference
        f.write(b"\0" * 8)
    y = mistic.read_points(str(p), 3)
    assert np.array_equal(x, y)
    z = mistic.read_points(str(p), 3, "f32")
    assert z.shape == ((10 * 3 * 8 + 8) // 4 // 3, 3)


def test_read_points_errors(tmp_path):
    with pytest.raises(mistic.MisticError) as e:
        mistic.read_points(str(tmp_path / "missing.bin"), 3)
    assert e.value.status == L.ERR_IO


def test_null_arguments_rejected():
    lib = L.load()
    assert lib.mistic_create(None, 0, None) == L.ERR_INVALID_ARG
    assert lib.mistic_destroy(None) == L.ERR_INVALID_ARG
    r = L.Result()
    assert lib.mistic_selfjoin(None, None, 0, 3, 0, 1, 1.0, None, ctypes.byref(r)) == L.ERR_INVALID_ARG


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device path")
def test_create_without_device_reports_no_device():
    lib = L.load()
    h = ctypes.c_void_p()
    assert lib.mistic_create(ctypes.byref(h), 0, None) == L.ERR_NO_DEVICE
