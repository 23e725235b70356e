"""Accuracy of the tensor-core arithmetic the joins' error band relies on.

The band bound of the tensor-core joins (join_tc.cu, join_tcw.cu) allows for
  - the operand rounding (bf16 keeps 8 significant bits, tf32 11; split
    bf16: <= 3.02 * 2^-16 of |a_k||q_k| a product; single bf16:
    2^-7 + 2^-16; tf32 rounded to nearest: 2^-10 + 2^-22), and
  - the FP32 accumulation in tensor memory: an allowance of 2^-19 of the sum
    of |products| per MMA instruction.
The accumulation allowance is not a documented hardware property, so these
tests measure it: mistic_tc_gram_probe issues one 128 x 128 tile exactly as
the joins do, and the result is compared with exact sums (math.fsum of the
exact FP64 products) on random operands with mixed exponents and on operands
built to cancel.  The measured worst case must stay well inside the
allowance; each test prints it.
"""
import ctypes
import math

import numpy as np
import pytest

from mistic import _lib as L

pytestmark = pytest.mark.gpu

ALLOW_PER_INST = 2.0 ** -19


def to_bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to bf16 (nearest even); returns the uint16 bit patterns."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def bf16_val(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def to_tf32(x: np.ndarray) -> np.ndarray:
    """Round FP32 to tf32 (nearest even): FP32 bit patterns with 13 zero low bits."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0xFFF + ((u >> 13) & 1)) >> 13) << 13
    return r.astype(np.uint32).view(np.float32)


def probe(kind: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    lib = L.load()
    K = a.shape[1]
    d = np.zeros((128, 128), np.float32)
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    st = lib.mistic_tc_gram_probe(kind, a.ctypes.data, b.ctypes.data, K, d.ctypes.data)
    assert st == L.OK, lib.mistic_strerror(st)
    return d.astype(np.float64)


def exact_gram(av: np.ndarray, bv: np.ndarray):
    """Exact row x row dot products (fsum of exact FP64 products) and the sums
    of |products|."""
    ex = np.empty((128, 128))
    for i in range(128):
        prod = av[i][None, :] * bv  # exact: <= 48-bit significands
        for j in range(128):
            ex[i, j] = math.fsum(prod[j])
    mag = np.abs(av) @ np.abs(bv).T
    return ex, mag


def operands(rng, K: int, pattern: str):
    if pattern == "mixed":  # random signs and exponents over 2^-8 .. 2^8
        a = rng.normal(size=(128, K)) * np.exp2(rng.integers(-8, 9, size=(128, K)))
        b = rng.normal(size=(128, K)) * np.exp2(rng.integers(-8, 9, size=(128, K)))
    elif pattern == "cancel":  # b's second half cancels its first half against a
        a = rng.normal(size=(128, K))
        a[:, K // 2:] = a[:, :K // 2]
        b = rng.normal(size=(128, K)) * np.exp2(rng.integers(-4, 5, size=(128, K)))
        b[:, K // 2:] = -b[:, :K // 2] * (1 + rng.normal(size=(128, K // 2)) * 2.0 ** -7)
    else:  # "positive": every product positive, magnitudes near 1
        a = rng.random((128, K)) + 0.5
        b = rng.random((128, K)) + 0.5
    return a.astype(np.float32), b.astype(np.float32)


@pytest.mark.parametrize("pattern", ["mixed", "cancel", "positive"])
@pytest.mark.parametrize("K", [32, 96, 256])
def test_bf16_accumulation_error(K, pattern):
    rng = np.random.default_rng(1000 * K + len(pattern))
    a, b = operands(rng, K, pattern)
    ab, bb = to_bf16(a), to_bf16(b)
    d = probe(0, ab, bb)
    ex, mag = exact_gram(bf16_val(ab), bf16_val(bb))
    n_inst = K // 16
    rel = np.abs(d - ex) / np.maximum(mag, 1e-300)
    worst = float(rel.max()) / n_inst
    print(f"bf16 K={K} {pattern}: max error {worst:.3e} of sum|products| per instruction "
          f"(allowance {ALLOW_PER_INST:.3e}, ratio {worst / ALLOW_PER_INST:.4f})")
    assert worst <= ALLOW_PER_INST / 4


@pytest.mark.parametrize("pattern", ["mixed", "cancel", "positive"])
@pytest.mark.parametrize("K", [32, 128])
def test_tf32_accumulation_error(K, pattern):
    rng = np.random.default_rng(7000 * K + len(pattern))
    a, b = operands(rng, K, pattern)
    at, bt = to_tf32(a), to_tf32(b)
    d = probe(1, at, bt)
    ex, mag = exact_gram(at.astype(np.float64), bt.astype(np.float64))
    n_inst = K // 8
    rel = np.abs(d - ex) / np.maximum(mag, 1e-300)
    worst = float(rel.max()) / n_inst
    print(f"tf32 K={K} {pattern}: max error {worst:.3e} of sum|products| per instruction "
          f"(allowance {ALLOW_PER_INST:.3e}, ratio {worst / ALLOW_PER_INST:.4f})")
    assert worst <= ALLOW_PER_INST / 4


def test_tf32_reads_pre_rounded_operands_exactly():
    """Operands already rounded to tf32 lose nothing in the tensor core: with
    one non-zero product per output the tile equals the exact product."""
    rng = np.random.default_rng(3)
    a = to_tf32(rng.normal(size=(128, 8)).astype(np.float32))
    b = np.zeros((128, 8), np.float32)
    b[np.arange(128), np.arange(128) % 8] = to_tf32(rng.normal(size=128).astype(np.float32))
    d = probe(1, a, b)
    ex = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.array_equal(d, ex)


@pytest.mark.parametrize("K", [32, 64])
def test_split_bf16_product_error(K):
    """The joins' split-bf16 product on FP32 operands (hi.hi + hi.lo + lo.hi
    accumulated in one tile, 3 K/16 instructions) against the exact FP64
    Gram of the FP32 values: within the operand allowance 3.02 * 2^-16 plus
    the accumulation allowance."""
    rng = np.random.default_rng(K)
    a, b = operands(rng, K, "mixed")
    ah, bh = to_bf16(a), to_bf16(b)
    al = to_bf16((a.astype(np.float64) - bf16_val(ah)).astype(np.float32))
    bl = to_bf16((b.astype(np.float64) - bf16_val(bh)).astype(np.float32))
    A = np.concatenate([ah, ah, al], axis=1)
    B = np.concatenate([bh, bl, bh], axis=1)
    d = probe(0, A, B)
    ex, mag = exact_gram(a.astype(np.float64), b.astype(np.float64))
    n_inst = 3 * K // 16
    bound = 3.02 * 2.0 ** -16 + n_inst * ALLOW_PER_INST
    rel = float((np.abs(d - ex) / mag).max())
    print(f"split bf16 K={K}: max error {rel:.3e} of sum|a_k||b_k| (bound {bound:.3e})")
    assert rel <= bound


@pytest.mark.parametrize("kind", ["bf16", "tf32"])
def test_single_operand_product_error(kind):
    """Single-operand precisions of the K-chunked join on FP32 values (rows
    rounded once to bf16 or to tf32) against the exact FP64 Gram: within the
    operand allowance (bf16: 2^-7 + 2^-16, tf32: 2^-10 + 2^-22) plus the
    accumulation allowance."""
    K = 64
    rng = np.random.default_rng(11 if kind == "bf16" else 12)
    a, b = operands(rng, K, "mixed")
    if kind == "bf16":
        d = probe(0, to_bf16(a), to_bf16(b))
        n_inst, op = K // 16, 2.0 ** -7 + 2.0 ** -16
    else:
        d = probe(1, to_tf32(a), to_tf32(b))
        n_inst, op = K // 8, 2.0 ** -10 + 2.0 ** -22
    ex, mag = exact_gram(a.astype(np.float64), b.astype(np.float64))
    bound = op + n_inst * ALLOW_PER_INST
    rel = float((np.abs(d - ex) / mag).max())
    print(f"single {kind} K={K}: max error {rel:.3e} of sum|a_k||b_k| (bound {bound:.3e})")
    assert rel <= bound
