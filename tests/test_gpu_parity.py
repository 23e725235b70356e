"""GPU parity: the CUDA join through the C ABI against the oracle and the
reference's pinned counts.  Bit-exact pair sets are required: the result of
every mode is the FP64 predicate of src/utils.cu:296-309."""
import numpy as np
import pytest

from helpers import canon, case_input, diff_pairs, input_sha, pairs_sha
from oracle import oracle as O

import mistic
from mistic import _lib as L

pytestmark = pytest.mark.gpu

MODES = ["auto", "fp64", "fp32", "bf16", "tf32"]


def run(h, x, k, eps, **kw):
    kw.setdefault("pairs", "host")
    kw.setdefault("sort_pairs", True)
    return h.selfjoin(x, k, eps, **kw)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("idx", range(15))
def test_golden_case(handle, golden, idx, mode):
    c = golden[idx]
    x = case_input(c)
    eps = float.fromhex(c["eps_hex"])
    r = run(handle, x, c["k"], eps, mode=mode)
    if input_sha(x) == c["input_sha256"]:
        assert r.pairs_ordered_incl_self == c["ref_ordered_incl_self"]
        assert pairs_sha(r.pairs) == c["oracle_pairs_sha256"], diff_pairs(r.pairs, O.brute_pairs(x, eps))
    else:
        ref = O.brute_pairs(x, eps)
        assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
    assert r.pairs_ij == len(r.pairs)
    assert r.ulp_ambiguous == c["ulp_ambiguous"]


@pytest.mark.parametrize("mode", MODES)
def test_uniform_100k_full_size(handle, golden_full, mode):
    """The uniform workload at full size (n = 100,000, d = 18): the reference's
    own brute-force count and the oracle's pair-list hash, in every mode."""
    c = golden_full[0]
    x = case_input(c)
    assert input_sha(x) == c["input_sha256"]
    r = run(handle, x, c["k"], float.fromhex(c["eps_hex"]), mode=mode)
    assert r.pairs_ordered_incl_self == c["ref_ordered_incl_self"] == 3293520
    assert r.pairs_ij == c["oracle_pairs_ij"]
    assert pairs_sha(r.pairs) == c["oracle_pairs_sha256"]
    assert r.ulp_ambiguous == c["ulp_ambiguous"]


@pytest.mark.parametrize("rp", ["pca", "box", "scored"])
@pytest.mark.parametrize("k", [1, 3, 6, 8, 16])
def test_reference_point_choices_agree(handle, rp, k):
    rng = np.random.default_rng(100 + k)
    x = rng.normal(size=(3000, 10))
    eps = 1.1
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, k, eps, rp=rp)
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_scored_reference_points_prune_like_the_reference(handle):
    """The reference's per-layer scoring (MISTIC_RP_SCORED): exact pair set,
    and no more candidate pairs than seeded box points leave."""
    from mistic import workloads as W
    x = W.gen_susy_like(40000, seed=12)
    eps = 0.03
    ref = O.brute_pairs(x, eps)
    scored = run(handle, x, 6, eps, rp="scored")
    box = run(handle, x, 6, eps, rp="box")
    assert np.array_equal(scored.pairs, ref), diff_pairs(scored.pairs, ref)
    assert scored.candidates <= box.candidates


def test_user_reference_points(handle):
    rng = np.random.default_rng(5)
    x = rng.random((2500, 4))
    rps = rng.random((3, 4)) * 3 - 1
    eps = 0.08
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 3, eps, rp="user", rp_user=rps)
    assert np.array_equal(r.pairs, ref)


@pytest.mark.parametrize("mode", ["auto", "fp64"])
def test_medium_uniform18(handle, mode):
    x = np.random.default_rng(21).random((20000, 18))
    eps = 0.62
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 6, eps, mode=mode)
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)
    assert r.candidates >= r.pairs_ij


@pytest.mark.parametrize("tc_min", ["1", "16", "100000"])
def test_tensor_core_split_points(handle, monkeypatch, tc_min):
    """Every home bin on the tensor cores (1), the default split (16), none (huge)."""
    monkeypatch.setenv("MISTIC_TC_MIN_BIN", tc_min)
    from mistic import workloads as W
    for x, k, eps in ((W.gen_susy_like(30000, seed=6), 6, 0.03),
                      (np.random.default_rng(4).normal(size=(6000, 90)), 8, 9.0),
                      (np.random.default_rng(5).random((5000, 3)), 3, 0.02)):
        ref = O.brute_pairs(x, eps)
        r = run(handle, x, k, eps, mode="bf16")
        assert r.mode_used == "bf16"
        if tc_min == "1":
            assert r.n_units == 0 and r.n_units_tc > 0
        if tc_min == "100000":
            assert r.n_units_tc == 0
        assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_modes_agree_and_band_is_small(handle):
    from mistic import workloads as W
    x = W.gen_susy_like(60000, seed=4)
    eps = 0.03
    a = run(handle, x, 6, eps, mode="fp32")
    b = run(handle, x, 6, eps, mode="fp64")
    c = run(handle, x, 6, eps, mode="bf16")
    assert np.array_equal(a.pairs, b.pairs) and np.array_equal(c.pairs, b.pairs)
    assert a.mode_used == "fp32" and b.mode_used == "fp64" and c.mode_used == "bf16"
    assert run(handle, x, 6, eps).mode_used == "bf16"  # AUTO at d = 18
    assert a.band_pairs < 0.01 * a.candidates + 1000


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_band_list_overflow_reruns(handle, monkeypatch, mode):
    """A band list far too short for the band pairs: the join runs again with
    a longer list and the pair set stays exact."""
    from mistic import workloads as W
    x = W.gen_susy_like(30000, seed=9)
    eps = 0.03
    ref = O.brute_pairs(x, eps)
    monkeypatch.setenv("MISTIC_BAND_CAP", "2")
    r = run(handle, x, 6, eps, mode=mode)
    assert r.band_pairs > 2
    assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_f32_input_uses_widened_predicate(handle):
    x = np.random.default_rng(8).normal(size=(4000, 33)).astype(np.float32)
    eps = 5.0
    ref = O.brute_pairs(x, eps)
    for mode in ("auto", "fp64"):
        r = run(handle, x, 5, eps, mode=mode)
        assert np.array_equal(r.pairs, ref), diff_pairs(r.pairs, ref)


def test_counts_only_and_repeat_calls(handle):
    x = np.random.default_rng(9).random((5000, 6))
    eps = 0.1
    ref = O.brute_pairs(x, eps)
    for _ in range(3):
        r = handle.selfjoin(x, 4, eps)
        assert r.pairs is None and r.pairs_ij == len(ref)
        assert r.pairs_ordered_incl_self == 2 * len(ref) + 5000


def test_unsorted_pairs_are_same_set(handle):
    x = np.random.default_rng(10).random((6000, 3))
    eps = 0.05
    ref = O.brute_pairs(x, eps)
    r = run(handle, x, 3, eps, sort_pairs=False)
    assert np.array_equal(canon(r.pairs), ref)
    assert (r.pairs[:, 0] < r.pairs[:, 1]).all()


def test_edge_sizes(handle):
    for n in (0, 1):
        r = handle.selfjoin(np.zeros((n, 4)), 3, 1.0, pairs="host")
        assert r.pairs_ij == 0 and r.pairs_ordered_incl_self == n
    r = run(handle, np.zeros((2, 4)), 3, 0.0)
    assert r.pairs_ij == 1 and r.pairs.tolist() == [[0, 1]]
    x = np.ones((300, 5))
    r = run(handle, x, 4, 0.0)
    assert r.pairs_ij == 300 * 299 // 2


def test_invalid_inputs(handle):
    x = np.random.default_rng(1).random((100, 3))
    bad = x.copy()
    bad[7, 1] = np.nan
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(bad, 2, 0.1)
    assert e.value.status == L.ERR_NOT_FINITE
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 17, 0.1)
    assert e.value.status == L.ERR_INVALID_ARG
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 2, -1.0)
    assert e.value.status == L.ERR_INVALID_ARG
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin(x, 2, float("inf"))
    assert e.value.status == L.ERR_INVALID_ARG
    # the handle stays usable after errors
    r = handle.selfjoin(x, 2, 0.1)
    assert r.pairs_ij == len(O.brute_pairs(x, 0.1))


def test_caller_capacity_overflow_reports_status(handle):
    x = np.random.default_rng(2).random((3000, 2))
    eps = 0.05
    ref = O.brute_pairs(x, eps)
    o = handle.opts(pairs="host", pair_capacity=10)
    with pytest.raises(mistic.MisticError) as e:
        handle.selfjoin_raw(x.ctypes.data, 3000, 2, L.F64, 2, eps, o)
    assert e.value.status == L.ERR_PAIR_OVERFLOW


class _DevView:
    """Exposes a raw device buffer to torch via __cuda_array_interface__."""

    def __init__(self, ptr, count):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<i4",
                                         "data": (ptr, False), "version": 3}


def test_device_input_and_device_pairs(handle):
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(11).random((8000, 9))
    eps = 0.3
    ref = O.brute_pairs(x, eps)
    t = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    o = handle.opts(pairs="device", sort_pairs=True, input_on_device=True)
    raw = handle.selfjoin_raw(t.data_ptr(), 8000, 9, L.F64, 6, eps, o)
    jr = handle.to_result(raw, keep_device=True)
    assert jr.device_pairs and jr.pairs_ij == len(ref)
    dev = torch.as_tensor(_DevView(jr.device_pairs, 2 * jr.pairs_ij), device="cuda")
    host = dev.cpu().numpy().view(np.uint32).reshape(-1, 2)
    handle.free_result(jr)
    assert np.array_equal(host, ref)


def _csr_reference(ref_pairs, n):
    """Neighbour table of the reference (include/utils.cuh:33-41): every row's
    neighbours ascending, the row itself included."""
    src = np.concatenate([ref_pairs[:, 0], ref_pairs[:, 1], np.arange(n, dtype=np.uint32)]).astype(np.int64)
    dst = np.concatenate([ref_pairs[:, 1], ref_pairs[:, 0], np.arange(n, dtype=np.uint32)]).astype(np.int64)
    order = np.lexsort((dst, src))
    offs = np.zeros(n + 1, dtype=np.uint64)
    offs[1:] = np.cumsum(np.bincount(src, minlength=n))
    return offs, dst[order].astype(np.uint32)


@pytest.mark.parametrize("mode", ["auto", "fp32", "fp64"])
def test_csr_neighbour_table(handle, mode):
    x = np.random.default_rng(31).random((6000, 7))
    eps = 0.18
    ref = O.brute_pairs(x, eps)
    offs, nbrs = _csr_reference(ref, 6000)
    r = handle.selfjoin(x, 5, eps, mode=mode, csr="host", pairs="host", sort_pairs=True)
    assert np.array_equal(r.pairs, ref)
    assert np.array_equal(r.csr_offsets, offs)
    assert np.array_equal(r.csr_nbrs, nbrs)
    assert int(r.csr_offsets[-1]) == r.pairs_ordered_incl_self


def test_csr_device_and_edges(handle):
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(32).normal(size=(4000, 12))
    eps = 2.5
    ref = O.brute_pairs(x, eps)
    offs, nbrs = _csr_reference(ref, 4000)
    o = handle.opts(csr="device")
    raw = handle.selfjoin_raw(x.ctypes.data, 4000, 12, L.F64, 6, eps, o)
    import ctypes
    op = ctypes.cast(raw.csr_offsets, ctypes.c_void_p).value
    npp = ctypes.cast(raw.csr_nbrs, ctypes.c_void_p).value
    assert raw.csr_on_device == 1
    d_off = torch.as_tensor(_DevView(op, 2 * 4001), device="cuda").cpu().numpy().view(np.uint64)
    d_nbr = torch.as_tensor(_DevView(npp, len(nbrs)), device="cuda").cpu().numpy().view(np.uint32)
    handle.lib.mistic_result_free(ctypes.byref(raw))
    assert np.array_equal(d_off, offs) and np.array_equal(d_nbr, nbrs)
    for n in (0, 1):
        r = handle.selfjoin(np.zeros((n, 3)), 2, 1.0, csr="host")
        assert r.csr_offsets.tolist() == list(range(n + 1)) and r.csr_nbrs.tolist() == list(range(n))
