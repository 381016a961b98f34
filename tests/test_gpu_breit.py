"""The Gaunt (Breit) transform on the GPU against the oracle's MDBINT stream
(needs a GB300).

rotran with BREIT = .TRUE. reads only the (SL|SL) Gaunt file (class 4, sign
turned by GETTW), transforms the SL pair blocks with QA and with QB
(TRANS1's Gaunt branch: MTIMHER(-1), MTIMHR2, TRBOUT's three streams), and
in TRANS2 contracts the three streams with QA/QB (MATMUL3, MATMUL7 x2,
MSUMTIM(-1)) before the same OUTPP/PPSYM record stream as MDCINT.  Each
stored element is the sum of two halves that PPSYM adds (the record's own
item and the item OUTPP2 pushes from); for the Gaunt integrals those halves
are not images of each other, so the GPU keeps every item's RL and
assembles the records as PPSYM does.  The record stream must match the
oracle's record for record."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import fortio, rotran, synth
from util import compare_streams

pytestmark = pytest.mark.gpu

TOL = {rotran.RT_PREC_FP64: 1e-12, rotran.RT_PREC_SPLIT_BF16: 1e-10}


def run_gpu(p, precision, **kw):
    with rotran.Rotran.for_problem(p, precision=precision, breit=True, **kw) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        out = rt.result()
        st = rt.stats()
    return out, st


@pytest.mark.parametrize("precision", [rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16], ids=["fp64", "split"])
@pytest.mark.parametrize("nl,ns,nkr,seed", [(3, 4, 2, 0), (4, 6, 3, 2), (5, 7, 4, 3), (6, 10, 5, 1),
                                            (12, 20, 10, 6), (24, 40, 16, 7)])
def test_breit_matches_the_oracle(nl, ns, nkr, seed, precision):
    p = synth.make_problem(nl, ns, nkr, seed=seed, breit=True)
    img = pyoracle.run(p, breit=True)
    got, st = run_gpu(p, precision)
    tol = TOL[precision]
    err = compare_streams(got, (img.hdr, img.idx, img.val), tol)
    print(f"n={p.n} nkr={nkr}: max |GPU - oracle| = {err:.3e} over {img.val.shape[0]} elements")
    assert err <= tol, err
    if precision == rotran.RT_PREC_FP64:
        assert list(st.nfinal) == [int(x) for x in img.nfinal]


def test_breit_ignores_the_coulomb_files_and_vice_versa():
    """A Gaunt run reads file 4 only; a Coulomb run never reads it."""
    p = synth.make_problem(4, 6, 3, seed=5, breit=True)
    cls, its, nts, v, l2, l1 = p.flat_records()
    keep = cls == 4
    off = np.concatenate([[0], np.cumsum(nts)])
    sel = np.concatenate([np.arange(off[r], off[r + 1]) for r in np.nonzero(keep)[0]])
    only4 = (cls[keep], its[keep], nts[keep], v[sel], l2[sel], l1[sel])
    with rotran.Rotran.for_problem(p, breit=True) as rt:
        rt.set_problem_coefficients(p)
        rt.add_records_bulk(*[only4[0], only4[2], only4[1], only4[3], only4[4], only4[5]])
        rt.transform()
        a = rt.result()
    b, _ = run_gpu(p, rotran.RT_PREC_FP64)
    assert compare_streams(a, b, 0.0) == 0.0
    # the Coulomb transform of the same records equals the one without file 4
    img = pyoracle.run(p)
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        got = rt.result()
    assert compare_streams(got, (img.hdr, img.idx, img.val), 1e-12) <= 1e-12


def test_breit_refused_by_batches_and_the_adjoint():
    p = synth.make_problem(4, 6, 3, seed=5, breit=True)
    rt = rotran.Rotran.for_problem(p, breit=True)
    try:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        with pytest.raises(rotran.RotranError):
            rotran.Batch([rt])
        with pytest.raises(rotran.RotranError):
            rt.adjoint(np.zeros((p.m,) * 4, dtype=np.complex128))
    finally:
        rt.close()


def test_breit_reads_srtbrei_srtbrel(tmp_path):
    """rt_read_srt_files of a Gaunt context reads SRTBREI/SRTBREL (file 4)
    alone, as SORT1 does with BREIT; the stream equals the bulk input's."""
    p = synth.make_problem(5, 7, 4, seed=9, breit=True)
    fortio.write_srt_files(p, str(tmp_path))
    with rotran.Rotran.for_problem(p, breit=True) as rt:
        rt.set_problem_coefficients(p)
        rt.read_srt_files(str(tmp_path))
        rt.transform()
        got = rt.result()
    bulk, _ = run_gpu(p, rotran.RT_PREC_FP64)
    assert compare_streams(got, bulk, 0.0) == 0.0
