"""The oracle's Gaunt (Breit) branch: structural checks of the MDBINT stream.

The restatement follows rotran's Breit path (TRANS1's Gaunt branch with
MTIMHER(-1) and MTIMHR2, TRBOUT's three masked streams, GETHTBI, UNIQUE's
sign flip, MATMUL3/MATMUL7 with QA and QB, MSUMTIM(-1), then the same
OUTPP/PPSYM record stream).  A reader rebuilds the full tensor from the
stream with the same 16-fold expansion as for MDCINT (tests/util.py) but
with the time-reversal factor of each pair of opposite sign (the Breit sign
of unique.F:34); every stored element must then imply one value per spinor
quadruple, and every quadruple must be reached."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import synth


def expand(p, img, sgn):
    m = p.m
    full = {}
    worst = 0.0

    def sp(k):
        return (p.kra[k - 1] if k > 0 else p.krb[-k - 1]) - 1

    off = 0
    for ikr, jkr, nz in img.hdr:
        i, itr, j, jtr = sp(ikr), sp(-ikr), sp(jkr), sp(-jkr)
        sij = np.sign(ikr) * np.sign(jkr) * sgn
        for z in range(nz):
            kkr, lkr = img.idx[off + z]
            v = img.val[off + z]
            k, ktr, l, ltr = sp(kkr), sp(-kkr), sp(lkr), sp(-lkr)
            skl = np.sign(kkr) * np.sign(lkr) * sgn
            c = np.conj(v)
            for q, x in (((i, j, k, l), v), ((jtr, itr, k, l), sij * v), ((i, j, ltr, ktr), skl * v),
                         ((jtr, itr, ltr, ktr), sij * skl * v), ((j, i, l, k), c), ((itr, jtr, l, k), sij * c),
                         ((j, i, ktr, ltr), skl * c), ((itr, jtr, ktr, ltr), sij * skl * c),
                         ((k, l, i, j), v), ((ltr, ktr, i, j), skl * v), ((k, l, jtr, itr), sij * v),
                         ((ltr, ktr, jtr, itr), sij * skl * v), ((l, k, j, i), c), ((ktr, ltr, j, i), skl * c),
                         ((l, k, itr, jtr), sij * c), ((ktr, ltr, itr, jtr), sij * skl * c)):
                if q in full:
                    worst = max(worst, abs(full[q] - x))
                full[q] = x
        off += nz
    return full, worst, m ** 4


@pytest.mark.parametrize("nl,ns,nkr,seed", [(3, 4, 2, 0), (4, 6, 3, 2), (5, 7, 4, 3)])
def test_breit_stream_is_consistent_under_the_breit_reader_rules(nl, ns, nkr, seed):
    p = synth.make_problem(nl, ns, nkr, seed=seed, breit=True)
    img = pyoracle.run(p, breit=True)
    scale = float(np.abs(img.val).max())
    full, worst, nq = expand(p, img, -1)
    assert len(full) == nq, "a spinor quadruple is not reachable from the stream"
    assert worst <= 1e-14 * scale, worst
    # the Coulomb reader rules (time-reversal factor without the Breit sign)
    # do not fit the Gaunt stream: the sign of unique.F:34 matters
    _, worst_c, _ = expand(p, img, +1)
    assert worst_c > 1e-3 * scale


def test_breit_reads_file4_only_with_its_sign():
    """SORT1 reads file 4 alone for the Gaunt integrals (sort1.F:55-57), and
    GETTW turns their sign (gettw.F:51-55): Coulomb records added to the
    input change nothing, and negated Gaunt records negate the stream."""
    p = synth.make_problem(4, 5, 2, seed=4, breit=True)
    a = pyoracle.run(p, breit=True)
    cls, its, nts, v, l2, l1 = p.flat_records()
    sel = cls == 4
    ends = np.cumsum(nts)
    keep = np.zeros(v.size, bool)
    for r in np.nonzero(sel)[0]:
        keep[ends[r] - nts[r]:ends[r]] = True
    only4 = (cls[sel], its[sel], nts[sel], v[keep], l2[keep], l1[keep])
    b = pyoracle.run(p, breit=True, records=only4)
    neg = (cls[sel], its[sel], nts[sel], -v[keep], l2[keep], l1[keep])
    c = pyoracle.run(p, breit=True, records=neg)
    assert np.array_equal(a.hdr, b.hdr) and np.array_equal(a.val, b.val)
    assert np.array_equal(a.hdr, c.hdr) and np.allclose(c.val, -a.val, rtol=0, atol=1e-22)
