"""Generates tests/golden/golden.json: parity pins for the ε-self-join.

For every case the seeded input is regenerated here, written as the
reference's raw FP64 file, and joined by
  - the reference's own CPU brute force (src/utils.cu:285-317 of
    bwd29/self-join-MiSTIC, compiled from its unmodified source by
    oracle/build_ref.sh into oracle/_ref/ref_brute), giving the ordered
    pair count including self pairs; and
  - the oracle (oracle/brute.c), giving the canonical i<j pair list, whose
    SHA-256 is stored.
The fixture keeps only seeds, sizes, ε (hex), the input's SHA-256 and the
results, so it stays small; tests regenerate the inputs and check the input
hash before trusting a pin.

Run from the repository root (needs the reference tree; not run by tests):
    oracle/build_ref.sh && python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "self-join-mistic_gb300"))

from mistic import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ref_brute")


def gen_case(c: dict) -> np.ndarray:
    """Regenerates a case's points (shared with the tests)."""
    g, n, d, seed = c["gen"], c["n"], c["d"], c["seed"]
    if g == "uniform":
        return W.gen_uniform(n, d, seed)
    if g == "susy":
        return W.gen_susy_like(n, seed=seed)
    if g == "msd":
        return W.gen_msd_like(n, d, seed)
    if g == "clusters":
        return W.gen_clusters(n, d, c.get("clusters", 8), seed, normalise=c.get("normalise", False), rank=32)
    if g == "clusters_norm":
        return W.gen_clusters(n, d, c.get("clusters", 8), seed, zipf=1.1, normalise=True, rank=32)
    if g == "grid":
        rng = np.random.default_rng(seed)
        return rng.integers(0, c.get("side", 4), size=(n, d)).astype(np.float64)
    if g == "dups":
        rng = np.random.default_rng(seed)
        base = rng.random((max(1, n // 8), d))
        return base[rng.integers(0, base.shape[0], size=n)]
    if g == "offset":  # data far from the origin: large coordinates, small ε
        rng = np.random.default_rng(seed)
        return 1e6 + rng.random((n, d))
    raise ValueError(g)


def input_sha(x: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def pairs_sha(p: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(p, dtype=np.uint32).tobytes()).hexdigest()


CASES = [
    dict(name="uniform18_n2000", gen="uniform", n=2000, d=18, seed=0, k=6, target=32.0),
    dict(name="uniform2_n3000", gen="uniform", n=3000, d=2, seed=1, k=2, target=16.0),
    dict(name="uniform5_n2500_k3", gen="uniform", n=2500, d=5, seed=4, k=3, target=8.0),
    dict(name="susy18_n3000", gen="susy", n=3000, d=18, seed=2, k=6, target=64.0),
    dict(name="msd90_n1500", gen="msd", n=1500, d=90, seed=3, k=8, target=16.0),
    dict(name="clusters32_f32_n2000", gen="clusters", n=2000, d=32, seed=5, k=6, target=16.0, f32=True),
    dict(name="clusters57_f32_n1200", gen="clusters", n=1200, d=57, seed=6, k=6, target=4.0, f32=True),
    dict(name="tiny384_f32_n1000", gen="clusters_norm", n=1000, d=384, seed=7, k=8, target=16.0,
         f32=True, clusters=20),
    dict(name="grid3_ties_eps1", gen="grid", n=1500, d=3, seed=8, k=3, eps=1.0, side=6),
    dict(name="grid4_ties_eps_sqrt2", gen="grid", n=1200, d=4, seed=9, k=4, eps=2.0 ** 0.5, side=5),
    dict(name="dups7_n1600", gen="dups", n=1600, d=7, seed=10, k=4, target=32.0),
    dict(name="dups7_eps0", gen="dups", n=1600, d=7, seed=10, k=4, eps=0.0),
    dict(name="offset6_n2000", gen="offset", n=2000, d=6, seed=11, k=4, target=8.0),
    dict(name="uniform18_k0", gen="uniform", n=1000, d=18, seed=12, k=0, target=16.0),
    dict(name="uniform1_n4000", gen="uniform", n=4000, d=1, seed=13, k=1, target=8.0),
]


# Full-size cases (the uniform workload: n = 100,000, d = 18, U[0,1) from seed 0,
# ε calibrated to 32 mean neighbours).  `--full` (re)computes only these and
# keeps the small cases; the reference's brute force takes about 30 s here.
FULL_CASES = [
    dict(name="c1_uniform18_n100000", gen="uniform", n=100000, d=18, seed=0, k=6, eps_hex="0x1.c37b06bdae65ep-1"),
]


def pin(c: dict) -> dict:
    x = gen_case(c)
    if c.get("f32"):
        x = x.astype(np.float32)
    if "eps_hex" in c:
        eps = float.fromhex(c["eps_hex"])
    else:
        eps = c["eps"] if "eps" in c else W.calibrate_eps(x.astype(np.float64), c["target"])
    x64 = x.astype(np.float64)
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        path = f.name
    W.write_bin(path, x64)
    r = subprocess.run([REF, path, str(c["d"]), repr(float(eps))], capture_output=True, text=True, check=True)
    os.unlink(path)
    ref = json.loads(r.stdout.strip().splitlines()[-1])
    pairs, amb = O.brute_pairs(x, eps, want_ambig=True)
    rec = dict(c)
    rec.update(eps_hex=float(eps).hex(), input_sha256=input_sha(x), ref_ordered_incl_self=ref["ordered_incl_self"],
               oracle_pairs_ij=int(len(pairs)), oracle_pairs_sha256=pairs_sha(pairs), ulp_ambiguous=int(amb))
    assert 2 * len(pairs) + c["n"] == ref["ordered_incl_self"], (c["name"], len(pairs), ref)
    print(c["name"], len(pairs), ref["ordered_incl_self"], "amb", amb, flush=True)
    return rec


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/ref_brute missing: run oracle/build_ref.sh first")
    path = os.path.join(HERE, "golden.json")
    if "--full" in sys.argv:
        with open(path) as f:
            g = json.load(f)
        g["full_size"] = [pin(c) for c in FULL_CASES]
        with open(path, "w") as f:
            json.dump(g, f, indent=1)
        return
    out = []
    for c in CASES:
        out.append(pin(c))
    g = {"generator": "tests/golden/make_golden.py",
         "reference_binary": "oracle/_ref/ref_brute (src/utils.cu:285-317, unmodified)", "cases": out}
    if os.path.exists(path):
        with open(path) as f:
            old = json.load(f)
        if "full_size" in old:
            g["full_size"] = old["full_size"]
    with open(path, "w") as f:
        json.dump(g, f, indent=1)


if __name__ == "__main__":
    main()
