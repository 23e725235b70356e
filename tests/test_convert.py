"""The text -> binary converter (mistic_convert_text, CLI --to-bin) against
the behaviour of the reference's toBin tool (toCSV.cpp:52-85): numbers
separated by commas and/or white space, raw FP64 out, stop at the first
token that is not a number.  Where oracle/build_ref.sh compiled the
reference's own toCSV.cpp (oracle/_ref/ref_tobin), outputs are compared
byte for byte.  Host only."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

import mistic
from mistic import _lib as L

REF_TOBIN = os.path.join(ROOT, "oracle", "_ref", "ref_tobin")

CASES = {
    "csv": "1.5, 2, -3e-2\n4, 5, 6\n",
    "csv_no_space": "1,2,3\n4,5,6\n",
    "spaces": "1 2 3\n\t4   5\n6\n",
    "trailing_comma": "1, 2, 3,\n4, 5, 6,\n",
    "header_stops": "x,y,z\n1,2,3\n",
    "stop_mid": "1, 2, 3\n4, oops, 6\n",
    "space_before_comma": "1 ,2, 3\n",
    "double_comma": "1,,2\n",
    "semicolon": "1;2;3\n",
    "empty": "",
    "exponents_hex": "1e300, -2.5E-300, 0x1p-3, 7\n",
}
EXPECT = {
    "csv": [1.5, 2, -3e-2, 4, 5, 6],
    "csv_no_space": [1, 2, 3, 4, 5, 6],
    "spaces": [1, 2, 3, 4, 5, 6],
    "trailing_comma": [1, 2, 3, 4, 5, 6],
    "header_stops": [],
    "stop_mid": [1, 2, 3, 4],
    "space_before_comma": [1],
    "double_comma": [1],
    "semicolon": [1],
    "empty": [],
    "exponents_hex": [1e300, -2.5e-300, 0.125, 7],
}


def _convert(tmp_path, text, name="in.txt"):
    src = tmp_path / name
    src.write_text(text)
    out = tmp_path / (name + ".bin")
    n = mistic.convert_text(str(src), str(out))
    v = np.fromfile(out, dtype="<f8")
    assert len(v) == n
    return v


@pytest.mark.parametrize("case", sorted(CASES))
def test_cases(tmp_path, case):
    assert np.array_equal(_convert(tmp_path, CASES[case]), np.array(EXPECT[case], dtype=np.float64))


@pytest.mark.parametrize("case", sorted(CASES))
def test_same_bytes_as_reference_tool(tmp_path, case):
    if not os.path.exists(REF_TOBIN):
        pytest.skip("the reference's toCSV.cpp was not built here (oracle/build_ref.sh)")
    src = tmp_path / "in.txt"
    src.write_text(CASES[case])
    subprocess.run([REF_TOBIN, str(src), str(tmp_path / "ref.bin")], capture_output=True, check=True)
    mistic.convert_text(str(src), str(tmp_path / "ours.bin"))
    assert (tmp_path / "ours.bin").read_bytes() == (tmp_path / "ref.bin").read_bytes()


def test_large_file_is_split_and_truncated_in_order(tmp_path):
    """Tens of MB: parsed in several chunks; a bad token in the middle ends
    the output exactly there, as the sequential tool would."""
    rng = np.random.default_rng(0)
    x = rng.normal(size=(400_000, 10))
    lines = [", ".join(repr(float(v)) for v in row) for row in x]
    cut = 250_000
    lines[cut] = "1.0, 2.0, junk, 3.0"
    text = "\n".join(lines) + "\n"
    assert len(text) > 30e6
    v = _convert(tmp_path, text, "big.txt")
    want = np.concatenate([x[:cut].ravel(), [1.0, 2.0]])
    assert np.array_equal(v, want)
    if os.path.exists(REF_TOBIN):
        subprocess.run([REF_TOBIN, str(tmp_path / "big.txt"), str(tmp_path / "ref.bin")], capture_output=True,
                       check=True)
        assert np.array_equal(np.fromfile(tmp_path / "ref.bin", dtype="<f8"), v)


def test_read_back_as_points(tmp_path):
    x = np.random.default_rng(1).random((100, 7))
    (tmp_path / "p.csv").write_text("\n".join(",".join(repr(float(v)) for v in r) for r in x))
    n = mistic.convert_text(str(tmp_path / "p.csv"), str(tmp_path / "p.bin"))
    assert n == 700
    assert np.array_equal(mistic.read_points(str(tmp_path / "p.bin"), 7), x)


def test_cli_to_bin(tmp_path):
    from mistic import build as B
    if not os.path.exists(B.CLI):
        pytest.skip("CLI not built")
    (tmp_path / "a.txt").write_text("1, 2, 3, 4\n")
    r = subprocess.run([B.CLI, "--to-bin", str(tmp_path / "a.txt"), str(tmp_path / "a.bin")], capture_output=True,
                       text=True, check=True)
    assert "4" in r.stdout
    assert np.array_equal(np.fromfile(tmp_path / "a.bin", dtype="<f8"), [1, 2, 3, 4])


def test_errors(tmp_path):
    with pytest.raises(mistic.MisticError) as e:
        mistic.convert_text(str(tmp_path / "missing.txt"), str(tmp_path / "o.bin"))
    assert e.value.status == L.ERR_IO
    lib = L.load()
    assert lib.mistic_convert_text(None, None, None) == L.ERR_INVALID_ARG
