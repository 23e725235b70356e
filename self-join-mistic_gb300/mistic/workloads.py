"""Seeded synthetic point sets for the ε-self-join workloads, and ε calibration.

The reference measures on real datasets (SUSY 5,000,000x18, MSD 515,345x90,
TINY 5,000,000x384) that are not shipped with it.  These generators produce
seeded stand-ins with the same shapes and comparable value distributions:

  uniform18     n=100,000  d=18  FP64  i.i.d. U[0,1)^18, seed 0, k=6, 32 nbrs
  susy18        n=5,000,000 d=18 FP64  8 lognormal(sigma=0.8) raw columns plus
                10 seeded nonlinear combinations of them with N(0,0.05) noise,
                every column min-max scaled to [0,1]; k=6, 64 nbrs
  msd90         n=515,345  d=90  FP64  correlated Gaussian (random orthogonal
                basis, spectrum i^-1.2), column-standardised; k=8, 16 nbrs
  batch2000     2,000 independent instances, n log-uniform in [1e3, 2e5],
                d in {2,8,18,32,57,90}, FP32 anisotropic Gaussian mixtures
  tiny384       n=5,000,000 d=384 FP32, 1,000 Zipf(1.1)-sized Gaussian
                clusters, each with a full-rank covariance R diag(eig) R^T
                (R a random rotation, the 384 eigenvalues log-uniform in
                [1e-3, 1]), L2-normalised; k=8, 16 nbrs

ε is calibrated by bisection on a seeded 10,000-point sample: the mean
neighbour count of the full set is estimated as (n-1)/(|S|-1) times the mean
within-sample FP64 neighbour count (self excluded), and ε is bisected in FP64
for 60 iterations to the smallest value whose estimate reaches the target.
The calibrated ε is stored as a hex float so every implementation uses the
identical value.

The reference reads a raw little-endian FP64 row-major file whose row count
is bytes/8/d (src/main.cu:42-50); `write_bin`/`read_bin` follow that format.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------- file format


def write_bin(path: str, pts: np.ndarray) -> None:
    """Write points as the reference's input file: raw little-endian FP64,
    row-major, no header (src/main.cu:42-50)."""
    np.ascontiguousarray(pts, dtype="<f8").tofile(path)


def read_bin(path: str, d: int, dtype: str = "<f8") -> np.ndarray:
    """Read a raw row-major point file; n = bytes / itemsize / d, any trailing
    partial row is ignored exactly as the reference's integer division does
    (src/main.cu:50)."""
    raw = np.fromfile(path, dtype=dtype)
    n = raw.size // d
    return raw[: n * d].reshape(n, d)


# ---------------------------------------------------------------- generators


def gen_uniform(n: int = 100_000, d: int = 18, seed: int = 0) -> np.ndarray:
    """i.i.d. U[0,1)^d from numpy PCG64 with the given seed."""
    return np.random.default_rng(seed).random((n, d))


def gen_susy_like(n: int = 5_000_000, d_raw: int = 8, d_derived: int = 10,
                  seed: int = 2) -> np.ndarray:
    """Heavy-tailed positive raw features plus nonlinear derived features,
    each column min-max normalised to [0,1] (SUSY-shaped, d = 18)."""
    rng = np.random.default_rng(seed)
    spec_rng = np.random.default_rng(seed + 1000)
    spec = [tuple(spec_rng.choice(d_raw, size=3, replace=False)) for _ in range(d_derived)]
    x = np.empty((n, d_raw + d_derived), dtype=np.float64)
    chunk = 1 << 18
    for r0 in range(0, n, chunk):  # chunked: bounded temporaries
        m = min(chunk, n - r0)
        raw = rng.lognormal(mean=0.0, sigma=0.8, size=(m, d_raw))
        noise = rng.normal(0.0, 0.05, size=(m, d_derived))
        out = x[r0:r0 + m]
        out[:, :d_raw] = raw
        for t, (a, b, c) in enumerate(spec):
            kind = t % 3
            if kind == 0:      # product
                v = raw[:, a] * raw[:, b]
            elif kind == 1:    # ratio
                v = raw[:, a] / (raw[:, b] + 0.5)
            else:              # sqrt of a sum of squares
                v = np.sqrt(raw[:, a] ** 2 + raw[:, b] ** 2 + raw[:, c] ** 2)
            out[:, d_raw + t] = v + noise[:, t]
    lo = x.min(axis=0)
    hi = x.max(axis=0)
    x -= lo
    x /= (hi - lo)
    return x


def gen_msd_like(n: int = 515_345, d: int = 90, seed: int = 3) -> np.ndarray:
    """Correlated Gaussian: random orthogonal basis times a spectrum decaying
    as i^-1.2, then column-standardised (MSD-shaped, d = 90)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(d, d)))
    scale = np.arange(1, d + 1, dtype=np.float64) ** -0.6  # sqrt of i^-1.2
    z = rng.normal(size=(n, d)) * scale
    x = z @ q.T
    x = (x - x.mean(axis=0)) / x.std(axis=0)
    return x


def gen_clusters(n: int, d: int, n_clusters: int, seed: int,
                 zipf: float | None = None, normalise: bool = False,
                 eig_lo: float = 1e-3, eig_hi: float = 1.0,
                 dtype=np.float32, rank: int | None = None) -> np.ndarray:
    """Gaussian mixture: cluster c has covariance R_c diag(eig_c) R_c^T with
    R_c a random rotation (QR of a Gaussian matrix) and eig_c log-uniform in
    [eig_lo, eig_hi].  rank=None: full rank (all d eigenvalues); rank=r: the
    rotation spans a random min(d, r)-dimensional subspace and every point
    gets isotropic noise of variance eig_lo on top.  Cluster sizes Zipf(zipf) when given, else
    multinomial with random weights."""
    rng = np.random.default_rng(seed)
    if zipf is not None:
        w = 1.0 / np.arange(1, n_clusters + 1, dtype=np.float64) ** zipf
    else:
        w = rng.random(n_clusters) + 0.1
    w /= w.sum()
    sizes = rng.multinomial(n, w)
    out = np.empty((n, d), dtype=dtype)
    pos = 0
    centres = rng.normal(size=(n_clusters, d))
    r = d if rank is None else min(d, rank)
    for c in range(n_clusters):
        m = int(sizes[c])
        if m == 0:
            continue
        basis, _ = np.linalg.qr(rng.normal(size=(d, r)))
        eig = np.exp(rng.uniform(math.log(eig_lo), math.log(eig_hi), size=r))
        z = rng.normal(size=(m, r)) * np.sqrt(eig)
        pts = centres[c] * 0.5 + z @ basis.T
        if rank is not None:
            pts += rng.normal(scale=math.sqrt(eig_lo), size=(m, d))
        out[pos:pos + m] = pts
        pos += m
    perm = rng.permutation(n)
    out = out[perm]
    if normalise:  # row L2 norms in FP64 (same bits as np.linalg.norm), in chunks
        for r0 in range(0, n, 1 << 16):
            blk = out[r0:r0 + (1 << 16)].astype(np.float64)
            nrm = np.sqrt(np.add.reduce(blk * blk, axis=1, keepdims=True))
            out[r0:r0 + (1 << 16)] = (blk / nrm).astype(dtype)
    return out


def gen_clusters_device(n: int, d: int, n_clusters: int, seed: int, zipf: float = 1.1,
                        eig_lo: float = 1e-3, eig_hi: float = 1.0, device: str = "cuda"):
    """The generator of gen_clusters at full rank (Zipf cluster sizes, a
    random rotation times d log-uniform eigenvalues per cluster, rows
    L2-normalised), drawn with a seeded torch generator on the GPU so that a
    5M x 384 set takes seconds instead of many minutes.  Returns an FP32
    host array.  The values differ from gen_clusters (another random
    stream); ε is calibrated on the result."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    w = 1.0 / torch.arange(1, n_clusters + 1, dtype=torch.float64) ** zipf
    sizes = np.random.default_rng(seed).multinomial(n, (w / w.sum()).numpy())
    out = torch.empty((n, d), dtype=torch.float32, device=device)
    centres = torch.randn((n_clusters, d), generator=g, device=device, dtype=torch.float32)
    pos = 0
    for c0 in range(0, n_clusters, 50):  # rotations 50 at a time (batched QR)
        c1 = min(n_clusters, c0 + 50)
        basis, _ = torch.linalg.qr(torch.randn((c1 - c0, d, d), generator=g, device=device, dtype=torch.float32))
        u = torch.rand((c1 - c0, d), generator=g, device=device, dtype=torch.float32)
        eig = torch.exp(math.log(eig_lo) + u * (math.log(eig_hi) - math.log(eig_lo)))
        for c in range(c0, c1):
            m = int(sizes[c])
            if m == 0:
                continue
            z = torch.randn((m, d), generator=g, device=device, dtype=torch.float32) * eig[c - c0].sqrt()
            out[pos:pos + m] = centres[c] * 0.5 + z @ basis[c - c0].T
            pos += m
    out = out[torch.randperm(n, generator=g, device=device)]
    out /= out.double().norm(dim=1, keepdim=True).float()
    host = out.cpu().numpy()
    del out
    torch.cuda.empty_cache()
    return host


# ---------------------------------------------------------------- ε calibration


def _within_sample_sqdist(s: np.ndarray) -> np.ndarray:
    """All unordered i<j squared FP64 distances within the sample, sorted."""
    s = np.ascontiguousarray(s, dtype=np.float64)
    m = s.shape[0]
    nrm = np.einsum("ij,ij->i", s, s)
    out = []
    blk = 1024
    for i0 in range(0, m, blk):
        a = s[i0:i0 + blk]
        g = a @ s.T
        d2 = nrm[i0:i0 + blk, None] + nrm[None, :] - 2.0 * g
        rows = np.arange(i0, min(i0 + blk, m))[:, None]
        mask = np.arange(m)[None, :] > rows
        out.append(d2[mask])
    d2 = np.concatenate(out)
    np.maximum(d2, 0.0, out=d2)
    d2.sort()
    return d2


def calibrate_eps(pts: np.ndarray, target_mean: float, sample: int = 10_000,
                  seed: int = 12345, iters: int = 60) -> float:
    """Bisect ε in FP64 so that the sample-extrapolated mean neighbour count
    (self excluded) reaches `target_mean`."""
    n = pts.shape[0]
    rng = np.random.default_rng(seed)
    m = min(sample, n)
    idx = np.sort(rng.choice(n, size=m, replace=False))
    d2 = _within_sample_sqdist(pts[idx])
    scale = (n - 1) / max(m - 1, 1)

    def est(eps: float) -> float:
        cnt = np.searchsorted(d2, eps * eps, side="right")  # unordered pairs
        return 2.0 * cnt / m * scale

    lo, hi = 0.0, float(math.sqrt(d2[-1])) * 1.0001 + 1e-300
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        if est(mid) >= target_mean:
            hi = mid
        else:
            lo = mid
    return hi


# ---------------------------------------------------------------- configs


@dataclass
class Workload:
    """One self-join instance: points (n x d), reference-point count k, ε."""
    name: str
    pts: np.ndarray
    k: int
    eps: float
    target_mean: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pts.shape[0])

    @property
    def d(self) -> int:
        return int(self.pts.shape[1])


#: ε values calibrated once with calibrate_eps (stored as hex floats so every
#: implementation uses the identical value).  Filled lazily when absent.
EPS_HEX: dict[str, str] = {
    "uniform18:100000": "0x1.c37b06bdae65ep-1",
    "susy18:5000000": "0x1.55e138a251ac5p-7",
    "msd90:515345": "0x1.c5a7e6636d473p+2",
}


def _eps_for(name: str, pts: np.ndarray, target: float) -> float:
    if name in EPS_HEX:
        return float.fromhex(EPS_HEX[name])
    e = calibrate_eps(pts, target)
    EPS_HEX[name] = e.hex()
    return e


def uniform18(n: int = 100_000) -> Workload:
    pts = gen_uniform(n, 18, seed=0)
    key = f"uniform18:{n}"
    return Workload(key, pts, 6, _eps_for(key, pts, 32.0), 32.0)


def susy18(n: int = 5_000_000) -> Workload:
    pts = gen_susy_like(n)
    key = f"susy18:{n}"
    return Workload(key, pts, 6, _eps_for(key, pts, 64.0), 64.0)


def msd90(n: int = 515_345) -> Workload:
    pts = gen_msd_like(n)
    key = f"msd90:{n}"
    return Workload(key, pts, 8, _eps_for(key, pts, 16.0), 16.0)


def tiny384(n: int = 5_000_000) -> Workload:
    """TINY-shaped: FP32, d = 384, 1,000 Zipf(1.1) clusters, L2-normalised
    rows, k = 8, 16 mean neighbours.  Large sets are drawn on the GPU."""
    try:
        import torch
        on_gpu = n >= 200_000 and torch.cuda.is_available()
    except ImportError:
        on_gpu = False
    if on_gpu:
        pts = gen_clusters_device(n, 384, 1000, seed=5)
    else:
        pts = gen_clusters(n, 384, 1000, seed=5, zipf=1.1, normalise=True)
    key = f"tiny384:{n}:{'gpu' if on_gpu else 'np'}"
    return Workload(key, pts, 8, _eps_for(key, pts, 16.0), 16.0)


def _calibrate_eps_device(x, target_mean: float, sample: int, seed: int, iters: int = 60) -> float:
    """calibrate_eps on a device tensor: the same estimator and bisection,
    with the sample's FP64 squared distances computed and sorted on the GPU."""
    import torch
    n = x.shape[0]
    m = min(sample, n)
    g = torch.Generator(device=x.device)
    g.manual_seed(seed)
    idx = torch.sort(torch.randperm(n, generator=g, device=x.device)[:m]).values
    s = x[idx].double()
    nrm = (s * s).sum(dim=1)
    d2 = (nrm[:, None] + nrm[None, :] - 2.0 * (s @ s.T))
    iu = torch.triu_indices(m, m, offset=1, device=x.device)
    d2 = torch.sort(d2[iu[0], iu[1]].clamp_min_(0.0)).values
    scale = (n - 1) / max(m - 1, 1)
    top = float(d2[-1].item()) if d2.numel() else 0.0
    lo, hi = 0.0, math.sqrt(top) * 1.0001 + 1e-300
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        cnt = int(torch.searchsorted(d2, torch.tensor([mid * mid], dtype=torch.float64, device=x.device),
                                     right=True).item())
        if 2.0 * cnt / m * scale >= target_mean:
            hi = mid
        else:
            lo = mid
    return hi


def batch_instances_device(count: int = 2000, seed: int = 7, n_lo: int = 1_000, n_hi: int = 200_000,
                           device: str = "cuda") -> list[Workload]:
    """The instance mix of batch_instances (same n, d, cluster count and
    target per index), with the points drawn and ε calibrated on the GPU so
    that 2,000 instances take seconds.  FP32 host arrays."""
    import torch
    master = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(master.uniform(math.log(n_lo), math.log(n_hi)))))
        d = int(master.choice([2, 8, 18, 32, 57, 90]))
        nc = int(master.integers(1, 51))
        tgt = float(master.choice([4.0, 16.0, 64.0]))
        rng = np.random.default_rng(seed * 100_003 + i)
        w = rng.random(nc) + 0.1
        sizes = rng.multinomial(n, w / w.sum())
        g = torch.Generator(device=device)
        g.manual_seed(seed * 100_003 + i)
        x = torch.empty((n, d), dtype=torch.float32, device=device)
        centres = torch.randn((nc, d), generator=g, device=device)
        r = min(d, 32)
        pos = 0
        for c in range(nc):
            m = int(sizes[c])
            if m == 0:
                continue
            basis, _ = torch.linalg.qr(torch.randn((d, r), generator=g, device=device))
            u = torch.rand((r,), generator=g, device=device)
            eig = torch.exp(math.log(1e-2) + u * (0.0 - math.log(1e-2)))
            z = torch.randn((m, r), generator=g, device=device) * eig.sqrt()
            blk = centres[c] * 0.5 + z @ basis.T
            blk += torch.randn((m, d), generator=g, device=device) * 0.1
            x[pos:pos + m] = blk
            pos += m
        x = x[torch.randperm(n, generator=g, device=device)]
        eps = _calibrate_eps_device(x, tgt, sample=min(n, 4000), seed=i)
        out.append(Workload(f"batch{i}", x.cpu().numpy(), min(6, d), eps, tgt, {"index": i}))
    return out


def batch_instances(count: int = 2000, seed: int = 7, n_lo: int = 1_000,
                    n_hi: int = 200_000) -> list[Workload]:
    """Uneven independent instances: n log-uniform in [n_lo, n_hi], d in
    {2,8,18,32,57,90}, FP32 Gaussian mixtures of 1-50 anisotropic clusters,
    mean neighbour target in {4,16,64}.  Per-instance seeds derive from
    (seed, index)."""
    master = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(master.uniform(math.log(n_lo), math.log(n_hi)))))
        d = int(master.choice([2, 8, 18, 32, 57, 90]))
        nc = int(master.integers(1, 51))
        tgt = float(master.choice([4.0, 16.0, 64.0]))
        pts = gen_clusters(n, d, nc, seed=seed * 100_003 + i, eig_lo=1e-2, rank=32)
        eps = calibrate_eps(pts, tgt, sample=min(n, 4000), seed=i)
        out.append(Workload(f"batch{i}", pts, min(6, d), eps, tgt,
                            {"index": i}))
    return out
