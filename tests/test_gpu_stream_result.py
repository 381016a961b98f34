"""Elements streamed into host buffers while the transform runs
(rt_set_result_host) against rt_copy_result and the oracle (needs a GB300).

With host buffers registered, each item chunk's MDCINT elements are copied
to the caller's per-class arrays as soon as the chunk is done, so the last
copies overlap the remaining chunks; the streamed elements must be the ones
rt_copy_result gives, bit for bit, for the Coulomb path, rotran's half
buckets and the Gaunt (Breit) path.  A class buffer that is too small fails
the transform with class 3 and leaves the context usable."""

import numpy as np
import pytest
import torch

import pyoracle
from molfdir_gb300 import rotran, synth
from util import compare_streams

pytestmark = pytest.mark.gpu

SPLIT, FP64 = rotran.RT_PREC_SPLIT_BF16, rotran.RT_PREC_FP64


def pinned_class_buffers(sizes, extra=3):
    """Per-class pinned host arrays (numpy views of pinned torch tensors)."""
    keep, idx, val = [], [], []
    for n in sizes:
        ti = torch.empty((n + extra, 2), dtype=torch.int32).pin_memory()
        tv = torch.empty((n + extra, 2), dtype=torch.float64).pin_memory()
        keep += [ti, tv]
        idx.append(ti.numpy())
        val.append(tv.numpy().view(np.complex128).reshape(-1))
    return keep, idx, val


def streamed(idx, val, sizes):
    return (np.concatenate([a[:n] for a, n in zip(idx, sizes)]),
            np.concatenate([v[:n] for v, n in zip(val, sizes)]))


@pytest.mark.parametrize("precision", [FP64, SPLIT], ids=["fp64", "split"])
@pytest.mark.parametrize("kind", ["coulomb", "half_buckets", "breit"])
def test_streamed_elements_are_the_copied_ones(kind, precision):
    breit = kind == "breit"
    p = synth.make_problem(12, 20, 10, seed=4, breit=breit)
    img = pyoracle.run(p, breit=breit)
    kw = dict(precision=precision, breit=breit, half_buckets=kind == "half_buckets")
    with rotran.Rotran.for_problem(p, **kw) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        hdr, idx, val = rt.result()
        sizes = [int(x) for x in rt.stats().nfinal]
        keep, hidx, hval = pinned_class_buffers(sizes)
        rt.set_result_host(hidx, hval)
        rt.transform()
        assert [int(x) for x in rt.stats().nfinal] == sizes
        assert np.array_equal(rt.headers(), hdr)
        sidx, sval = streamed(hidx, hval, sizes)
        assert np.array_equal(sidx, idx)
        assert np.array_equal(sval.view(np.float64), val.view(np.float64))
        tol = 1e-10 if precision == SPLIT else 1e-12
        err = compare_streams((hdr, sidx, sval), (img.hdr, img.idx, img.val), tol)
        assert err <= tol, err
        del keep


def test_too_small_class_buffer_fails_and_the_context_recovers():
    p = synth.make_problem(12, 20, 10, seed=5)
    with rotran.Rotran.for_problem(p, precision=SPLIT) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        good = rt.result()
        sizes = [int(x) for x in rt.stats().nfinal]
        big = int(np.argmax(sizes))
        small = list(sizes)
        small[big] = sizes[big] // 2
        keep, hidx, hval = pinned_class_buffers(small, extra=0)
        rt.set_result_host(hidx, hval)
        with pytest.raises(rotran.RotranError) as e:
            rt.transform()
        assert e.value.code == rotran.RT_ERR_DIM and f"class {big + 1}" in str(e.value)
        with pytest.raises(rotran.RotranError):   # the failed transform left no result
            rt.result()
        rt.set_result_host()
        rt.transform()
        again = rt.result()
        assert all(np.array_equal(a, b) for a, b in zip(good, again))
        del keep


def test_pageable_buffers_stream_too():
    """Plain numpy arrays work (the copies then do not overlap)."""
    p = synth.make_problem(6, 10, 5, seed=1)
    with rotran.Rotran.for_problem(p, precision=SPLIT) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        hdr, idx, val = rt.result()
        sizes = [int(x) for x in rt.stats().nfinal]
        hidx = [np.empty((n, 2), np.int32) for n in sizes]
        hval = [np.empty(n, np.complex128) for n in sizes]
        rt.set_result_host(hidx, hval)
        rt.transform()
        sidx, sval = streamed(hidx, hval, sizes)
        assert np.array_equal(sidx, idx) and np.array_equal(sval, val)


def test_deferred_copies_complete_before_results_are_reused():
    """Deferred mode: the last copies land by rt_result_host_wait, by a result
    read, or before the next transform writes results again."""
    p = synth.make_problem(12, 20, 10, seed=6)
    with rotran.Rotran.for_problem(p, precision=SPLIT) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        hdr, idx, val = rt.result()
        sizes = [int(x) for x in rt.stats().nfinal]
        keep, hidx, hval = pinned_class_buffers(sizes)
        rt.set_result_host(hidx, hval)
        rt.set_result_host_deferred(True)
        for wait in ("explicit", "headers", "next transform"):
            for x in hidx + hval:
                x.fill(0)
            rt.transform()
            if wait == "explicit":
                rt.result_host_wait()
            elif wait == "headers":
                assert np.array_equal(rt.headers(), hdr)
            else:
                rt.transform()   # waits before its second half, then streams again
                rt.result_host_wait()
            sidx, sval = streamed(hidx, hval, sizes)
            assert np.array_equal(sidx, idx), wait
            assert np.array_equal(sval.view(np.float64), val.view(np.float64)), wait
        rt.set_result_host_deferred(False)
        del keep
