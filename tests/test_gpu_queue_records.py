"""The queued next record set (rt_queue_ao_records_bulk) against plain
record adds and the oracle (needs a GB300).

A transform with a set queued must give the results of the records it
started with, copy the queued set while it runs, and return with the queued
set as the context's records; every other call that touches the records
applies the queue first.  Two problems of the same sizes with different
integrals share one set of spinors (the first problem's)."""

import numpy as np
import pytest
import torch

import pyoracle
from molfdir_gb300 import rotran, synth
from util import compare_streams

pytestmark = pytest.mark.gpu

SPLIT = rotran.RT_PREC_SPLIT_BF16


def pinned(recs):
    cls, its, nts, v, l2, l1 = recs
    keep = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (v, l2, l1)]
    return (cls, nts, its), keep


def queue(rt, recs):
    (cls, nts, its), keep = pinned(recs)
    rt.queue_records_bulk_ptr(cls, nts, its, keep[0].data_ptr(), keep[1].data_ptr(), keep[2].data_ptr())
    return keep


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def problems():
    pa = synth.make_problem(12, 20, 6, seed=1)
    pb = synth.make_problem(12, 20, 6, seed=2)
    ra, rb = pa.flat_records(), pb.flat_records()
    ia = pyoracle.run(pa)
    ib = pyoracle.run(pa, records=rb)   # A's spinors, B's integrals
    return pa, ra, rb, ia, ib


def test_transform_with_a_queued_set(problems):
    pa, ra, rb, ia, ib = problems
    with rotran.Rotran.for_problem(pa, precision=SPLIT) as rt:
        rt.set_problem_coefficients(pa)
        rt.add_records_bulk(ra[0], ra[2], ra[1], ra[3], ra[4], ra[5])
        keep = queue(rt, rb)
        rt.transform()               # A's records; B's copied meanwhile
        got_a = rt.result()
        del keep
        rt.transform()               # B's records now
        got_b = rt.result()
    assert compare_streams(got_a, (ia.hdr, ia.idx, ia.val), 1e-10) <= 1e-10
    assert compare_streams(got_b, (ib.hdr, ib.idx, ib.val), 1e-10) <= 1e-10
    with rotran.Rotran.for_problem(pa, precision=SPLIT) as rt:   # plain adds give the same bits
        rt.set_problem_coefficients(pa)
        rt.add_records_bulk(rb[0], rb[2], rb[1], rb[3], rb[4], rb[5])
        rt.transform()
        assert same(rt.result(), got_b)


def test_other_calls_apply_the_queue_first(problems):
    pa, ra, rb, ia, ib = problems
    n = pa.n
    dens = np.random.default_rng(0).standard_normal((1, 4, n * (n + 1) // 2))
    with rotran.Rotran.for_problem(pa, precision=SPLIT) as rt:
        rt.set_problem_coefficients(pa)
        rt.add_records_bulk(ra[0], ra[2], ra[1], ra[3], ra[4], ra[5])
        keep = queue(rt, rb)
        f, _ = rt.fock_skeleton(dens)            # B's records
        want = pyoracle.fock_skeleton(rb, n, dens, mfil=pa.mfil)
        assert np.abs(f - want).max() <= 1e-12 * np.abs(want).max()
        keep = queue(rt, ra)
        rt.clear_records()                       # applies A, then clears
        del keep
        rt.add_records_bulk(rb[0], rb[2], rb[1], rb[3], rb[4], rb[5])
        rt.transform()
        assert compare_streams(rt.result(), (ib.hdr, ib.idx, ib.val), 1e-10) <= 1e-10


def test_a_larger_set_and_a_failed_transform(problems):
    pa, ra, rb, ia, ib = problems
    cls, its, nts, v, l2, l1 = ra
    # current: the first half of A's records; queued: all of B's
    half = cls.size // 2
    nh = int(nts[:half].sum())
    with rotran.Rotran.for_problem(pa, precision=SPLIT) as rt:
        rt.set_problem_coefficients(pa)
        rt.add_records_bulk(cls[:half], nts[:half], its[:half], v[:nh], l2[:nh], l1[:nh])
        keep = queue(rt, rb)
        rt.transform()
        ref = pyoracle.run(pa, records=(cls[:half], its[:half], nts[:half], v[:nh], l2[:nh], l1[:nh]))
        assert compare_streams(rt.result(), (ref.hdr, ref.idx, ref.val), 1e-10) <= 1e-10
        del keep
        rt.transform()
        assert compare_streams(rt.result(), (ib.hdr, ib.idx, ib.val), 1e-10) <= 1e-10
        # a transform that fails on its current records still makes the queued set current
        bad = l1.copy()
        bad[3] = (pa.n + 2) << 16 | 1
        rt.add_records_bulk(cls, nts, its, v, l2, bad)   # B plus A with a bad label
        keep = queue(rt, rb)
        with pytest.raises(rotran.RotranError):
            rt.transform()
        del keep
        rt.transform()
        assert compare_streams(rt.result(), (ib.hdr, ib.idx, ib.val), 1e-10) <= 1e-10


def test_queued_gaunt_records():
    """The Gaunt transform (file 4 only) with a queued set."""
    pa = synth.make_problem(6, 9, 4, seed=11, breit=True)
    pb = synth.make_problem(6, 9, 4, seed=12, breit=True)
    ra, rb = pa.flat_records(), pb.flat_records()
    ia = pyoracle.run(pa, breit=True)
    ib = pyoracle.run(pa, records=rb, breit=True)
    with rotran.Rotran.for_problem(pa, precision=SPLIT, breit=True) as rt:
        rt.set_problem_coefficients(pa)
        rt.add_records_bulk(ra[0], ra[2], ra[1], ra[3], ra[4], ra[5])
        keep = queue(rt, rb)
        rt.transform()
        got_a = rt.result()
        del keep
        rt.transform()
        got_b = rt.result()
    assert compare_streams(got_a, (ia.hdr, ia.idx, ia.val), 1e-10) <= 1e-10
    assert compare_streams(got_b, (ib.hdr, ib.idx, ib.val), 1e-10) <= 1e-10
