"""Large host inputs (>= 128 MB) reach the device either through a kernel that
reads the caller's pageable array directly (where the GPU uses the host's
page tables: GB300 with a Grace host) or through the handle's pinned staging
ring (several host threads copying 8 MB chunks, each chunk's DMA issued
behind the previous use of its slot).  On both paths the pair set must be
the one the same join produces from a device-resident copy of the rows, on
the first call and on the next ones, including a ragged last chunk."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", ["host_reads", "staging_ring"])
@pytest.mark.parametrize("n,d", [(1_200_001, 14), (2_100_003, 8)])
def test_staged_host_input_matches_device_input(monkeypatch, path, n, d):
    torch = pytest.importorskip("torch")
    import mistic
    monkeypatch.setenv("MISTIC_HOST_READS", "1" if path == "host_reads" else "0")
    rng = np.random.default_rng(n)
    x = rng.random((n, d))
    assert x.nbytes >= 128 << 20 and x.nbytes % (8 << 20) != 0
    from mistic import _lib as L
    from mistic import workloads as W
    eps = W.calibrate_eps(x, 4.0, sample=3000, seed=1)
    xt = torch.from_numpy(x).cuda()
    handle = mistic.Handle(0)  # reads MISTIC_HOST_READS when it is created
    rd = handle.to_result(handle.selfjoin_raw(xt.data_ptr(), n, d, L.F64, 6, eps,
                                              handle.opts(input_on_device=True, pairs="host",
                                                          sort_pairs=True)))
    assert rd.pairs_ij > 1000
    for _ in range(2):
        rh = handle.selfjoin(x, 6, eps, pairs="host", sort_pairs=True)
        assert rh.pairs_ij == rd.pairs_ij
        assert np.array_equal(rh.pairs, rd.pairs)
    # the caller may reuse the array once the call has returned
    x[:] = 0.0
    rz = handle.selfjoin(x[:1000], 2, 0.5, pairs="none")
    assert rz.pairs_ij == 1000 * 999 // 2
    handle.close()
