"""rt_split_dgemm_noalloc (fixed scratch array, no device allocation) against
rt_split_dgemm mode 2, which slices the same FP64 rows on the device.

Collected last on purpose: it must pass both alone in a fresh process (the
first call does the per-device set-up) and after every other test."""

import numpy as np
import pytest

from molfdir_gb300 import rotran


def operands(m, n, k, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, k)) * np.exp(rng.uniform(-5, 5, (m, 1)))
    b = rng.standard_normal((k, n)) * np.exp(rng.uniform(-5, 5, (1, n)))
    return a, b


def scaled_err(c, ref, a, b):
    scale = np.abs(a).max(1)[:, None] * np.abs(b).max(0)[None, :] * a.shape[1]
    return float(np.max(np.abs(c - ref) / scale))


BOUND = {5: 2e-10, 6: 2e-12}  # the split GEMM tests' bounds


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    results = []
    # two calls in a row sharing the scratch array: a larger product, then a
    # smaller one with another slice count over the left-over contents
    for (m, n, k, s, seed) in [(300, 257, 800, 6, 1), (77, 513, 1000, 5, 2)]:
        a, b = operands(m, n, k, seed)
        da = torch.from_numpy(a).cuda()
        db = torch.from_numpy(b).cuda()
        dc = torch.full((m, n), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rotran.split_dgemm_noalloc(m, n, k, da.data_ptr(), db.data_ptr(), dc.data_ptr(),
                                   slices=s, stream=stream.cuda_stream)
        got = dc.cpu().numpy()
        ref = rotran.split_dgemm(a, b, slices=s, mode=2)
        assert np.isfinite(got).all()
        err_ref = scaled_err(got, ref, a, b)
        err_exact = scaled_err(got, a @ b, a, b)
        print(f"noalloc {m}x{n}x{k} s={s}: vs rt_split_dgemm {err_ref:.3e}, vs FP64 {err_exact:.3e}")
        assert err_ref <= BOUND[s]
        assert err_exact <= BOUND[s]
        results.append((dc, got))
    # the first output is untouched by the second call
    assert np.array_equal(results[0][0].cpu().numpy(), results[0][1])
    # repeated calls take no device memory: the free memory the driver
    # reports is the same right before and right after each call
    for (m, n, k, s, seed) in [(300, 257, 800, 6, 1), (77, 513, 1000, 5, 2)] * 2:
        a, b = operands(m, n, k, seed)
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        dc = torch.empty((m, n), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        rotran.split_dgemm_noalloc(m, n, k, da.data_ptr(), db.data_ptr(), dc.data_ptr(),
                                   slices=s, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == before
        del da, db, dc


def test_noalloc_rejects_sizes_beyond_scratch():
    # returns before any CUDA call, so this runs without a GPU too
    lib = rotran.load()
    for (m, n, k, code) in [(4096, 4096, 512, 3), (64, 64, 2048, 3), (0, 8, 8, 2)]:
        rc = lib.rt_split_dgemm_noalloc(m, n, k, 1, 1, 1, 6, None)
        assert rc == code
        msg = lib.rt_last_error(None).decode()
        assert "rt_split_dgemm_noalloc" in msg
        if (m, n, k) == (4096, 4096, 512):
            assert "50331648" in msg
