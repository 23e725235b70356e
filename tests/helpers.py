"""Helpers shared by the tests: golden-case inputs and pair-set comparison."""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

from make_golden import gen_case, input_sha, pairs_sha  # noqa: E402,F401


def case_input(c):
    x = gen_case(c)
    if c.get("f32"):
        x = x.astype(np.float32)
    return x


def canon(p: np.ndarray) -> np.ndarray:
    """Canonical pair array: rows (i, j), i < j, sorted by (i, j)."""
    p = np.asarray(p, dtype=np.uint32).reshape(-1, 2)
    lo = np.minimum(p[:, 0], p[:, 1])
    hi = np.maximum(p[:, 0], p[:, 1])
    key = (lo.astype(np.uint64) << np.uint64(32)) | hi.astype(np.uint64)
    key.sort()
    out = np.empty((key.size, 2), dtype=np.uint32)
    out[:, 0] = (key >> np.uint64(32)).astype(np.uint32)
    out[:, 1] = (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    return out


def diff_pairs(a: np.ndarray, b: np.ndarray, limit: int = 5) -> str:
    ka = set(map(tuple, canon(a).tolist()))
    kb = set(map(tuple, canon(b).tolist()))
    return f"only-left {sorted(ka - kb)[:limit]} only-right {sorted(kb - ka)[:limit]}"
