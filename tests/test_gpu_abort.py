"""The split GEMM's abort path, exercised without a fault (needs a GB300).

With RT_TEST_GEMM_NO_COPIES=1 in the environment, every split GEMM launch of
the library issues no tensor copies and limits its waits to 50 ms: the MMA
issuer's wait for operand tiles runs out, the launch stops all its roles
(producer, MMA issuer, epilogue; for the CTA-pair kernel in both CTAs),
drains its MMAs, frees TMEM and returns status 2.  The transform then fails
with class 6, and the same context transforms correctly afterwards.  The
cases below run the default single-CTA kernel; the CTA-pair kernel's abort
path is run in tests/test_gpu_pair_kernel.py."""

import numpy as np
import pytest

from molfdir_gb300 import rotran, synth

pytestmark = pytest.mark.gpu


def test_gemm_abort_reports_class6_and_context_recovers(monkeypatch):
    p = synth.make_problem(12, 20, 10, seed=6)
    with rotran.Rotran.for_problem(p, precision=rotran.RT_PREC_SPLIT_BF16) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        good = rt.result()
        monkeypatch.setenv("RT_TEST_GEMM_NO_COPIES", "1")
        with pytest.raises(rotran.RotranError) as e:
            rt.transform()
        assert e.value.code == rotran.RT_ERR_PROGRAM
        assert "gave up" in str(e.value) and "could not confirm" not in str(e.value)
        monkeypatch.delenv("RT_TEST_GEMM_NO_COPIES")
        rt.transform()
        again = rt.result()
    for a, b in zip(good, again):
        assert np.array_equal(a, b)


def test_split_dgemm_abort_then_correct(monkeypatch):
    """The same through rt_split_dgemm (M = 300, three row tiles)."""
    rng = np.random.default_rng(3)
    a = rng.standard_normal((300, 256))
    b = rng.standard_normal((256, 200))
    monkeypatch.setenv("RT_TEST_GEMM_NO_COPIES", "1")
    with pytest.raises(rotran.RotranError) as e:
        rotran.split_dgemm(a, b, slices=5, mode=1)
    assert e.value.code == rotran.RT_ERR_PROGRAM
    monkeypatch.delenv("RT_TEST_GEMM_NO_COPIES")
    c = rotran.split_dgemm(a, b, slices=5, mode=1)
    ref = a @ b
    scale = np.abs(a).max(1)[:, None] * np.abs(b).max(0)[None, :] * a.shape[1]
    assert float(np.max(np.abs(c - ref) / scale)) <= 1e-11
