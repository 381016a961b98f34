"""The CPU oracle against an independent dense formulation (no GPU)."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import synth
from util import permute_spinors


def dense_full(p):
    """(ij|kl) over all spinors by the textbook four-index sum (small n)."""
    n, m = p.n, p.m
    g = synth.dense_ao_tensor(p.model, p.mfil).reshape(n * n, n * n)
    d = (np.einsum("pa,qb->abpq", p.qa.conj(), p.qa)
         + np.einsum("pa,qb->abpq", p.qb.conj(), p.qb)).reshape(m * m, n * n)
    return ((d @ g) @ d.T).reshape(m, m, m, m)


def spinor_of(p, k):
    return (p.kra[k - 1] if k > 0 else p.krb[-k - 1]) - 1


def check_against_dense(p, img, tol=1e-13):
    v = dense_full(p)
    off = 0
    err = 0.0
    for a, b, nz in img.hdr:
        ia, ib = spinor_of(p, a), spinor_of(p, b)
        for z in range(nz):
            c, d = img.idx[off + z]
            err = max(err, abs(img.val[off + z] - v[ia, ib, spinor_of(p, c), spinor_of(p, d)]))
        off += nz
    assert err <= tol * max(1.0, np.abs(v).max()), err
    return err


def test_inttyp_table():
    n = 6
    for a in range(1, n + 1):
        for b in range(1, a + 1):
            for c in range(1, a + 1):
                for d in range(1, c + 1):
                    if (c, d) > (a, b):
                        continue
                    assert int(synth.inttyp(a, b, c, d)) == pyoracle.inttyp(a, b, c, d)


def test_type_factor_undoes_symmetrisation():
    p = synth.make_problem(5, 7, 3, seed=3)
    cls, its, nts, v, l2, l1 = p.flat_records()
    a, b, c, d = l2 >> 16, l2 & 0xFFFF, l1 >> 16, l1 & 0xFFFF
    coinc = (a == b).astype(int) + (c == d) + ((a == c) & (b == d))
    f = np.array([pyoracle.gettw_factor(int(t)) for t in np.repeat(its, nts)])
    assert np.all(f * 2.0 ** coinc == 1.0)


@pytest.mark.parametrize("nl,ns,nkr,mfil,seed", [
    (3, 4, 2, 3, 0), (6, 8, 4, 3, 1), (6, 8, 4, 2, 2), (7, 0, 3, 1, 3), (1, 1, 1, 3, 4),
    (5, 9, 5, 3, 5)])
def test_oracle_equals_dense(nl, ns, nkr, mfil, seed):
    p = synth.make_problem(nl, ns, nkr, seed=seed, mfil=mfil)
    img = pyoracle.run(p)
    check_against_dense(p, img)
    # one record per (IKR >= JKR) and class, classes in order 1..4
    k = nkr * (nkr + 1) // 2
    assert img.hdr.shape[0] == 4 * k
    signs = np.sign(img.hdr[:, :2])
    assert np.all(signs[:k] == [-1, -1]) and np.all(signs[k:] == [-1, 1])


def test_oracle_shuffled_spinor_order():
    p = synth.make_problem(6, 8, 4, seed=7)
    rng = np.random.default_rng(0)
    q = permute_spinors(p, rng.permutation(p.m))
    img = pyoracle.run(q)
    check_against_dense(q, img)


def test_oracle_irrep_blocks():
    p = synth.make_problem(8, 10, 4, seed=8, n_irrep=4)
    img = pyoracle.run(p)
    check_against_dense(p, img)


def test_oracle_thresholds():
    p = synth.make_problem(6, 8, 4, seed=9)
    full = pyoracle.run(p)
    cut = pyoracle.run(p, throut=1e-3)
    assert cut.idx.shape[0] < full.idx.shape[0]
    assert np.all(np.abs(cut.val) > 1e-3)
    every = pyoracle.run(p, throut=-1.0)  # PPSYM writes all NKR*NKR positions
    assert np.all(every.hdr[:, 2] == p.nkr ** 2)
    screened = pyoracle.run(p, thrgen=1e-4)
    assert screened.nhalft < full.nhalft


def test_oracle_golden_fixture():
    """The committed fixture (dense formulation values) reproduces."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_n14_k4.npz")
    g = np.load(path)
    p = synth.make_problem(6, 8, 4, seed=11)
    img = pyoracle.run(p)
    assert np.array_equal(img.hdr, g["hdr"]) and np.array_equal(img.idx, g["idx"])
    assert np.max(np.abs(img.val - g["dense_val"])) <= 1e-13
