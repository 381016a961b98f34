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
