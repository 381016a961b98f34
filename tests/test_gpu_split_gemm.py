"""The split-precision GEMM engine against FP64 numpy (needs a GB300)."""

import numpy as np
import pytest

from molfdir_gb300 import rotran

pytestmark = pytest.mark.gpu


def scaled_err(c, ref, a, b):
    # error relative to the row/column maxima that set the slice scales
    scale = np.abs(a).max(1)[:, None] * np.abs(b).max(0)[None, :] * a.shape[1]
    return float(np.max(np.abs(c - ref) / scale))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_integer_digits_exact(mode):
    # one-slice-exact operands: small integers times powers of two
    rng = np.random.default_rng(0)
    a = rng.integers(-100, 101, (200, 96)).astype(float) * 2.0 ** -5
    b = rng.integers(-60, 61, (96, 130)).astype(float) * 2.0 ** 3
    c = rotran.split_dgemm(a, b, slices=3, mode=mode)
    assert np.array_equal(c, a @ b)


@pytest.mark.parametrize("slices,bound", [(3, 2e-6), (4, 2e-8), (5, 2e-10), (6, 2e-12)])
@pytest.mark.parametrize("shape", [(128, 128, 64), (300, 257, 800), (77, 513, 1000)])
def test_random_accuracy(slices, bound, shape):
    m, n, k = shape
    rng = np.random.default_rng(slices * 7 + m)
    a = rng.standard_normal((m, k)) * np.exp(rng.uniform(-5, 5, (m, 1)))
    b = rng.standard_normal((k, n)) * np.exp(rng.uniform(-5, 5, (1, n)))
    ref = a @ b
    for mode in (0, 1, 2):
        c = rotran.split_dgemm(a, b, slices=slices, mode=mode)
        err = scaled_err(c, ref, a, b)
        print(f"s={slices} shape={shape} mode={mode}: scaled err {err:.3e}")
        assert err <= bound


# Operands whose three leading base-128 digits sit at their extremes:
# narrow slicing (K <= 819) allows a leading digit of 127, wide slicing
# (deeper GEMMs) keeps every digit within 64.  The third product diagonal
# then reaches (127*63 + 63*63 + 63*127) * 819 = 1.64e7 units (narrow) or
# 3 * 63 * 63 * 1024 = 1.22e7 units (wide), both just below 2^24, which the
# FP32 accumulator must hold exactly.  Every 16th k of B has the third digit
# one lower, so that the 16-deep partial sums of one MMA are odd and a
# dropped unit above 2^24 would show.
def _extreme(d1, d2, d3):
    return d1 / 128 + d2 / 128 ** 2 + d3 / 128 ** 3


@pytest.mark.parametrize("k,lead", [(819, 127), (1024, 63)], ids=["narrow_k819", "wide_k1024"])
@pytest.mark.parametrize("slices", [5, 6])
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_extreme_digits_are_summed_exactly(k, lead, slices, mode, sign):
    """With 5 or 6 slices every digit product of these three-digit values is
    formed, so C = a * sum_k b_k up to the FP32 rounding of the fourth
    accumulator (relative weight 2^-21; a few units in its last place over
    at most 64 adds, below 1e-11 relative).  A leading diagonal summed
    inexactly above 2^24 units would be off by 1e-9 or more."""
    a_val = _extreme(lead, 63, 63)
    a = np.full((128, k), sign * a_val)
    col = np.full(k, a_val)
    col[::16] = _extreme(lead, 63, 62)
    b = np.repeat(col[:, None], 136, axis=1)
    c = rotran.split_dgemm(a, b, slices=slices, mode=mode)
    ref = sign * a_val * float(col.sum())  # exact: 21-bit a, 31-bit sum of 21-bit b
    rel = float(np.max(np.abs(c - ref)) / abs(ref))
    print(f"K={k} s={slices} mode={mode} sign={sign}: relative error {rel:.3e}")
    assert rel <= 4e-11


def test_depth_beyond_the_tested_range_is_refused():
    a = np.ones((8, 1025))
    b = np.ones((1025, 8))
    with pytest.raises(rotran.RotranError) as e:
        rotran.split_dgemm(a, b, slices=5, mode=0)
    assert e.value.code == rotran.RT_ERR_DIM


def test_split_transform_beyond_the_exact_range_is_refused():
    """2 NSC > 1365 (the depth of GEMM2 and GEMM4) is refused on the split
    path with class 3, before any transform."""
    from molfdir_gb300 import synth
    rng = np.random.default_rng(0)
    n, nkr = 700, 2
    qa, qb, itrmo, kra, krb, ikrmo = synth.make_spinors(n, nkr, rng)
    cfg, keep = rotran.make_config(n, 300, nkr, precision=rotran.RT_PREC_SPLIT_BF16, slices=5)
    rt = rotran.Rotran(cfg, keep)
    try:
        with pytest.raises(rotran.RotranError) as e:
            rt.set_coefficients(qa, itrmo, kra, krb, ikrmo)
        assert e.value.code == rotran.RT_ERR_DIM
    finally:
        rt.close()
