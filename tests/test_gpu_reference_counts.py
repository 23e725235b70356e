"""Full-size parity against the reference's own GPU join: on the 5M x 18
SUSY-shaped and the 515,345 x 90 MSD-shaped workloads (seeded generators,
fixed hex epsilons) the library's ordered pair count including self pairs
equals the 'Total results Set Size' the reference's build printed for the same
points on a GB300 (tests/golden/reference_gpu_counts.json)."""
import json
import os

import pytest

ROOT = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(ROOT, "golden", "reference_gpu_counts.json")) as f:
    REF = json.load(f)


@pytest.mark.parametrize("case", REF["cases"], ids=[c["workload"] for c in REF["cases"]])
def test_fixture_matches_the_workload_definitions(case):
    from mistic import workloads as W
    assert W.EPS_HEX[f"{case['workload']}:{case['n']}"] == case["eps_hex"]
    assert (case["ref_ordered_incl_self"] - case["n"]) % 2 == 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", REF["cases"], ids=[c["workload"] for c in REF["cases"]])
def test_count_equals_the_reference_gpu_build(handle, case):
    from mistic import workloads as W
    wl = getattr(W, case["workload"])(case["n"])
    assert wl.pts.shape == (case["n"], case["d"]) and wl.k == case["k"]
    assert float(wl.eps).hex() == case["eps_hex"]
    r = handle.selfjoin(wl.pts, wl.k, wl.eps, pairs="none")
    assert r.pairs_ordered_incl_self == case["ref_ordered_incl_self"]
    assert r.pairs_ij == (case["ref_ordered_incl_self"] - case["n"]) // 2
