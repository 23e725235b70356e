"""Adversarial pairs around the tensor-core joins' error band.

The tensor-core joins accept a pair outright when its fast value is below
eps^2 minus the pair's error bound E, reject it above eps^2 plus E, and send
everything in between to the FP64 predicate.  A bound that is too small
would show up as a pair just outside eps (exact s a little above eps^2)
accepted, or one just inside rejected.  These cases build thousands of pairs
whose exact squared distance sits at eps^2 (1 + delta) for delta swept
log-uniformly over +-[1e-7, 0.3] -- every multiple of E from well inside the
band to well outside it -- and place them far from the unit's centring row
(|a'| + |q'| up to the size where E reaches the 0.1 eps^2 cap, beyond which a
column is decided entirely in FP64).  Every pair set must equal the
oracle's bit for bit, for the short-row kernel (d = 18, 90) and the K-chunked
kernel (d = 384, and d = 90 routed to it).
"""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def shell_case(d: int, n_pairs: int, rho_max: float, seed: int):
    """Rows in dims 2..d-1 (dims 0 and 1 are zero, so two far reference
    points on those axes put every row in one or two bins); row 128 t is the
    origin (the centring row of every unit chunk); eps = 1."""
    rng = np.random.default_rng(seed)
    free = d - 2
    rows = []
    for i in range(n_pairs):
        rho = rho_max * rng.random() ** 0.5
        w = rng.normal(size=free)
        w *= rho / np.linalg.norm(w)
        u = rng.normal(size=free)
        u /= np.linalg.norm(u)
        delta = np.sign(rng.random() - 0.5) * 10.0 ** rng.uniform(-7, np.log10(0.3))
        rows.append(w)
        rows.append(w + np.sqrt(1.0 + delta) * u)
    x = np.zeros((len(rows) + len(rows) // 127 + 2, d))
    j = 0
    for r in range(x.shape[0]):
        if r % 128 == 0 or j >= len(rows):
            continue  # the origin
        x[r, 2:] = rows[j]
        j += 1
    # a few rows at the largest radius: every unit's max |a'| is near rho_max
    x[1::257, 2:] *= rho_max / np.maximum(np.linalg.norm(x[1::257, 2:], axis=1, keepdims=True), 1e-9)
    rps = np.zeros((2, d))
    rps[0, 0] = rps[1, 1] = 1e4
    return x, rps


@pytest.mark.parametrize("prec", ["auto", "bf16", "tf32"])
@pytest.mark.parametrize("rho_max", [4.0, 12.0, 30.0])
@pytest.mark.parametrize("d", [18, 90, 384])
def test_pairs_around_the_band(handle, monkeypatch, d, rho_max, prec):
    """prec: the library's choice in BF16 mode (split for short rows; split
    or single bf16 for d = 384), single bf16 forced on the K-chunked kernel
    (d = 384 only), or TF32 mode."""
    if prec == "bf16" and d != 384:
        pytest.skip("single bf16 operands exist on the K-chunked kernel only")
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")  # every home bin on the tensor cores
    monkeypatch.setenv("MISTIC_TC_WIDE", "0")    # d = 90 on the short-row kernel
    if prec == "bf16":
        monkeypatch.setenv("MISTIC_TC_PREC", "bf16")
    x, rps = shell_case(d, 1500, rho_max, seed=d * 100 + int(rho_max))
    eps = 1.0
    ref = O.brute_pairs(x, eps)
    r = handle.selfjoin(x, 2, eps, mode="tf32" if prec == "tf32" else "bf16", rp="user", rp_user=rps,
                        pairs="host", sort_pairs=True)
    assert r.n_units_tc > 0 and r.tc_tiles > 0
    assert r.band_pairs > 0
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


@pytest.mark.parametrize("rho_max", [4.0, 12.0])
def test_pairs_around_the_band_medium_rows_on_the_k_chunked_kernel(handle, monkeypatch, rho_max):
    """d = 90 on the K-chunked kernel (globally centred rows, prepared once):
    the same shells around eps^2, pair sets bit-identical to the oracle's."""
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")
    monkeypatch.setenv("MISTIC_TC_WIDE", "1")
    x, rps = shell_case(90, 1500, rho_max, seed=9000 + int(rho_max))
    ref = O.brute_pairs(x, 1.0)
    r = handle.selfjoin(x, 2, 1.0, mode="bf16", rp="user", rp_user=rps, pairs="host", sort_pairs=True)
    assert r.n_units_tc > 0 and r.tc_tiles > 0
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
