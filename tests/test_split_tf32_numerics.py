"""CPU model of the FP32 MLP's split-tf32 products (no GPU needed).

The tensor-core FP32 path rounds every operand to tf32 (10 explicit mantissa bits, round
to nearest with ties away from zero, as cvt.rna.tf32.f32 does), keeps the remainder as a
second tf32 value, and sums three products per pair: hi*hi + hi*lo + lo*hi. This test
restates that split in numpy and checks the claim the kernels rely on: the product is
FP32-accurate (~22 significant bits of each input), while a single tf32 product is not.
"""
import numpy as np


def _rna_tf32(x):
    """float32 -> nearest tf32 value, ties away from zero (low 13 mantissa bits cleared)."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32)
    mag = (b & np.uint32(0x7FFFFFFF)) + np.uint32(0x1000)
    out = (mag & np.uint32(0xFFFFE000)) | (b & np.uint32(0x80000000))
    return out.view(np.float32)


def _split(x):
    hi = _rna_tf32(x)
    lo = _rna_tf32((x - hi).astype(np.float32))
    return hi, lo


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_tf32_rounding_keeps_ten_mantissa_bits():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(10000) * 10.0).astype(np.float32)
    h = _rna_tf32(x)
    assert np.all((h.view(np.uint32) & np.uint32(0x1FFF)) == 0)
    assert np.abs(h - x).max() <= np.abs(x).max() * 2.0 ** -11
    hi, lo = _split(x)
    # hi + lo carries ~22 significant bits of x
    assert np.all(np.abs((hi.astype(np.float64) + lo) - x) <= np.abs(x) * 2.0 ** -21 + 1e-30)


def test_three_term_split_product_is_fp32_accurate():
    rng = np.random.default_rng(1)
    for m, k, n in [(257, 150, 128), (128, 128, 128), (300, 144, 27)]:
        a = rng.standard_normal((m, k)).astype(np.float32)
        b = (rng.standard_normal((k, n)) / np.sqrt(k)).astype(np.float32)
        ah, al = _split(a)
        bh, bl = _split(b)
        # tf32 x tf32 products are exact in float64; sums are rounded like the float32 accumulator.
        d = np.zeros((m, n), dtype=np.float32)
        for kk in range(k):
            t = (np.outer(ah[:, kk], bh[kk]) + np.outer(ah[:, kk], bl[kk]) + np.outer(al[:, kk], bh[kk]))
            d = (d + t.astype(np.float32)).astype(np.float32)
        ref = a.astype(np.float64) @ b.astype(np.float64)
        one_pass = ah.astype(np.float64) @ bh.astype(np.float64)
        fp32 = a @ b  # a float32 GEMM on the host, for scale
        assert _rel(d, ref) < max(3 * _rel(fp32, ref), 1e-6), (m, k, n)  # FP32-level
        assert _rel(one_pass, ref) > 5e-5, (m, k, n)                     # plain tf32 is not
