"""Split-precision (BF16 slices on the tensor cores) path vs the FP64 oracle."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import rotran, synth
from util import compare_streams

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-10   # maximum absolute error of the split path


def run(p, precision, **kw):
    with rotran.Rotran.for_problem(p, precision=precision, **kw) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        return rt.result(), rt.stats()


@pytest.mark.parametrize("nl,ns,nkr,mfil,seed", [
    (3, 4, 2, 3, 0), (6, 8, 4, 3, 1), (6, 8, 4, 2, 2), (7, 0, 3, 1, 3), (12, 20, 10, 3, 6)])
def test_split_small(nl, ns, nkr, mfil, seed):
    p = synth.make_problem(nl, ns, nkr, seed=seed, mfil=mfil)
    img = pyoracle.run(p)
    got, st = run(p, rotran.RT_PREC_SPLIT_BF16)
    err = compare_streams(got, (img.hdr, img.idx, img.val), TOL_SPLIT)
    print(f"split max abs err {err:.3e}")
    assert err <= TOL_SPLIT


def test_split_config1_n64_k32():
    p = synth.make_problem(24, 40, 32, seed=0)
    img = pyoracle.run(p)
    got, st = run(p, rotran.RT_PREC_SPLIT_BF16)
    err = compare_streams(got, (img.hdr, img.idx, img.val), TOL_SPLIT)
    rms = float(np.sqrt(np.mean(np.abs(got[2] - img.val) ** 2)))
    print(f"config1 split: max abs err {err:.3e} rms {rms:.3e}")
    assert err <= TOL_SPLIT


@pytest.mark.parametrize("slices", [3, 4, 5, 6])
def test_split_slices_error_decreases(slices):
    p = synth.make_problem(12, 20, 8, seed=21)
    img = pyoracle.run(p)
    got, _ = run(p, rotran.RT_PREC_SPLIT_BF16, slices=slices)
    err = compare_streams(got, (img.hdr, img.idx, img.val), 1e-3, presence_tol=1e-3)
    bound = {3: 1e-5, 4: 1e-7, 5: 1e-9, 6: 1e-12}[slices]
    print(f"slices={slices}: max abs err {err:.3e}")
    assert err <= bound


def test_split_irrep_blocks():
    p = synth.make_problem(10, 14, 5, seed=13, n_irrep=4)
    img = pyoracle.run(p)
    got, _ = run(p, rotran.RT_PREC_SPLIT_BF16)
    assert compare_streams(got, (img.hdr, img.idx, img.val), TOL_SPLIT) <= TOL_SPLIT


def test_split_error_per_integral_class():
    """Max and RMS error of the split path per AO integral class, (LL|LL),
    (SS|LL) and (SS|SS), each transformed alone at the CPU-sized case."""
    p = synth.make_problem(24, 40, 32, seed=0)
    cls, its, nts, v, l2, l1 = p.flat_records()
    ends = np.cumsum(nts)
    starts = ends - nts
    for c, name in ((1, "(LL|LL)"), (2, "(SS|LL)"), (3, "(SS|SS)")):
        sel = np.nonzero(cls == c)[0]
        pieces = [slice(int(starts[r]), int(ends[r])) for r in sel]
        recs = (cls[sel], its[sel], nts[sel], np.concatenate([v[s] for s in pieces]),
                np.concatenate([l2[s] for s in pieces]), np.concatenate([l1[s] for s in pieces]))
        img = pyoracle.run(p, records=recs)
        with rotran.Rotran.for_problem(p, precision=rotran.RT_PREC_SPLIT_BF16) as rt:
            rt.set_problem_coefficients(p)
            rt.add_records_bulk(recs[0], recs[2], recs[1], *recs[3:])
            rt.transform()
            got = rt.result()
        err = compare_streams(got, (img.hdr, img.idx, img.val), TOL_SPLIT)
        same = np.array_equal(got[0], img.hdr) and np.array_equal(got[1], img.idx)
        rms = float(np.sqrt(np.mean(np.abs(got[2] - img.val) ** 2))) if same else float("nan")
        print(f"{name}: max abs err {err:.3e}, rms {rms:.3e}, max |value| "
              f"{float(np.abs(img.val).max()):.3e}")
        assert err <= TOL_SPLIT
