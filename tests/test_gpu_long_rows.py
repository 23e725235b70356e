"""GPU parity of the long-row tensor-core join (d + 2 > 128: K-chunked
tcgen05 tiles over rows split once into bf16 hi/lo) against the oracle.
Pair sets must be bit-identical to the FP64 predicate of src/utils.cu:296-309."""
import numpy as np
import pytest

from helpers import diff_pairs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run(h, x, k, eps, **kw):
    kw.setdefault("pairs", "host")
    kw.setdefault("sort_pairs", True)
    return h.selfjoin(x, k, eps, **kw)


def _eps_for_mean(x, mean):
    """ε giving about `mean` neighbours per point (bisection on a sample)."""
    from mistic import workloads as W
    return W.calibrate_eps(x, mean, sample=min(len(x), 3000), seed=1)


@pytest.mark.parametrize("k", [2, 8])
def test_tiny_shaped_384(handle, k):
    """384-d clustered FP32 rows (the 5M x 384 workload's shape at 8k points):
    few reference points give bins of hundreds of rows (two 128-row home
    chunks per unit, several 256-column groups per segment)."""
    from mistic import workloads as W
    wl = W.tiny384(8000)
    x, eps = wl.pts, wl.eps
    ref = O.brute_pairs(x, eps)
    for mode in ("bf16", "auto"):
        r = run(handle, x, k, eps, mode=mode)
        assert r.mode_used == "bf16"
        assert r.n_units_tc > 0 and r.tc_tiles > 0
        assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
        assert r.pairs_ordered_incl_self == 2 * len(ref) + len(x)


@pytest.mark.parametrize("d", [127, 130, 200, 257])
def test_padded_k_and_all_bins_on_tensor_cores(handle, monkeypatch, d):
    """K not a multiple of the 32-wide chunk (zero padding), every home bin on
    the tensor cores, many small bins (windows of 256 neighbour bins)."""
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")
    rng = np.random.default_rng(d)
    x = rng.normal(size=(3000, d)).astype(np.float32)
    x[1500:] = x[:1500] + rng.normal(scale=0.3, size=(1500, d)).astype(np.float32)  # near pairs
    eps = float(np.sqrt(2 * d) * 0.3)
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 6, eps, mode="bf16")
    assert r.n_units == 0 and r.n_units_tc > 0
    assert len(ref) > 1000
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_fp64_input_duplicates_and_ties(handle, monkeypatch):
    """FP64 rows with exact duplicates and pairs at exactly ε (integer grid):
    the band decides every tie as the reference predicate does."""
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")
    rng = np.random.default_rng(3)
    base = rng.integers(0, 3, size=(600, 150)).astype(np.float64)
    x = np.concatenate([base, base[:200], base[:50] + np.eye(150)[:50]])
    eps = 1.0
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 4, eps, mode="bf16")
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
    assert r.ulp_ambiguous > 0


def test_band_overflow_and_csr(handle, monkeypatch):
    """A band list far too short reruns the join; the CSR table matches."""
    from mistic import workloads as W
    x = W.tiny384(5000).pts
    eps = _eps_for_mean(x, 16)
    ref = O.brute_pairs(x, eps)
    monkeypatch.setenv("MISTIC_BAND_CAP", "2")
    r = handle.selfjoin(x, 4, eps, mode="bf16", pairs="host", sort_pairs=True, csr="host")
    assert r.band_pairs > 2
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
    deg = np.bincount(ref.ravel().astype(np.int64), minlength=len(x)) + 1
    assert np.array_equal(np.diff(r.csr_offsets.astype(np.int64)), deg)


def test_repeat_calls_same_handle(handle):
    """Two calls in a row on one handle (arena reuse, persistent CTAs) agree."""
    from mistic import workloads as W
    x = W.tiny384(4000).pts
    eps = _eps_for_mean(x, 8)
    a = run(handle, x, 3, eps, mode="bf16")
    b = run(handle, x, 3, eps, mode="bf16")
    assert np.array_equal(a.pairs, b.pairs)
    assert np.array_equal(a.pairs, O.brute_pairs(x, eps))


@pytest.mark.parametrize("prec", ["split", "bf16", "tf32"])
@pytest.mark.parametrize("d", [130, 384])
def test_operand_precisions(handle, monkeypatch, prec, d):
    """The K-chunked join at each operand precision: split bf16 (3 products),
    single bf16 (forced here; the library picks it only when its bound leaves
    a narrow band) and tf32 (MISTIC_MODE_TF32).  Exact pair sets in all."""
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", "1")
    rng = np.random.default_rng(d + 7)
    x = rng.normal(size=(3000, d)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    x[1500:] = x[:1500] + rng.normal(scale=0.25 / np.sqrt(d), size=(1500, d)).astype(np.float32)
    eps = 0.3
    ref = O.brute_pairs(x, eps)
    assert len(ref) > 1000
    if prec != "tf32":
        monkeypatch.setenv("MISTIC_TC_PREC", prec)
    r = run(handle, x, 4, eps, mode="tf32" if prec == "tf32" else "bf16")
    assert r.mode_used == ("tf32" if prec == "tf32" else "bf16")
    assert r.n_units == 0 and r.n_units_tc > 0
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


@pytest.mark.parametrize("d", [8, 18, 57, 90])
def test_tf32_mode_short_rows(handle, d):
    """TF32 mode runs every tensor-core unit on the K-chunked kernel, short
    rows included (globally centred rows; columns whose bound is too wide go
    to FP64): exact pair sets."""
    rng = np.random.default_rng(40 + d)
    x = rng.normal(size=(6000, d))
    eps = float(np.sqrt(d) * 0.35)
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 6, eps, mode="tf32")
    assert r.mode_used == "tf32"
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_single_bf16_is_picked_for_wide_bands(handle):
    """Unit-norm rows with eps comparable to their spread: the single-bf16
    bound stays within eps^2 / 20, so AUTO runs a third of the tensor work;
    the band is decided in FP64 and the pair set is exact."""
    rng = np.random.default_rng(77)
    x = rng.normal(size=(5000, 256)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    x[2500:] = x[:2500] + rng.normal(scale=0.04, size=(2500, 256)).astype(np.float32)
    eps = 1.0
    # single bf16 fits the cap here: |a| + |q| <= 2 + noise, eps^2 = 1
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 8, eps)
    assert r.mode_used == "bf16"
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
