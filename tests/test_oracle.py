"""The CPU oracle against an independent dense formulation (no GPU)."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import synth
from util import dense_full, permute_spinors


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


@pytest.mark.parametrize("nl,ns,nkr,seed,shuffle,mfil,nirr", [
    (3, 4, 2, 0, False, 3, 1), (5, 7, 3, 3, False, 3, 1), (4, 6, 3, 5, True, 3, 1),
    (5, 6, 3, 6, False, 2, 1), (6, 0, 3, 7, False, 1, 1), (6, 8, 3, 8, False, 3, 4)])
def test_oracle_stream_reconstructs_the_tensor_as_a_reader_does(nl, ns, nkr, seed, shuffle, mfil,
                                                                 nirr):
    """Structural parity of the MDCINT stream with its reader (rdtwo.F:29-83):
    expanding every element into its 16 related quadruples reproduces the
    whole dense (ij|kl), consistently (MFIL 1-3, 4-irrep blocks)."""
    from util import check_rdtwo_reconstruction
    p = synth.make_problem(nl, ns, nkr, seed=seed, mfil=mfil, n_irrep=nirr)
    if shuffle:
        p = permute_spinors(p, np.random.default_rng(seed).permutation(p.m))
    img = pyoracle.run(p)
    dense = dense_full(p)
    check_rdtwo_reconstruction(img.hdr, img.idx, img.val, p.kra, p.krb, dense,
                               tol=1e-13 * max(1.0, np.abs(dense).max()), throut=1e-16)


@pytest.mark.parametrize("mistake", ["conjugate_one", "drop_record", "flip_sign"])
def test_reconstruction_check_catches_planted_mistakes(mistake):
    from util import check_rdtwo_reconstruction
    p = synth.make_problem(3, 4, 2, seed=0)
    img = pyoracle.run(p)
    dense = dense_full(p)
    hdr, idx, val = img.hdr.copy(), img.idx.copy(), img.val.copy()
    z = int(np.argmax(np.abs(val.imag)))  # an element with an imaginary part
    if mistake == "conjugate_one":
        val[z] = np.conj(val[z])
    elif mistake == "flip_sign":
        val[z] = -val[z]
    else:  # drop the largest record's elements
        r = int(np.argmax(hdr[:, 2]))
        start = int(hdr[:r, 2].sum())
        keep = np.r_[0:start, start + hdr[r, 2]:val.size]
        idx, val = idx[keep], val[keep]
        hdr[r, 2] = 0
    with pytest.raises(AssertionError):
        check_rdtwo_reconstruction(hdr, idx, val, p.kra, p.krb, dense,
                                   tol=1e-13 * max(1.0, np.abs(dense).max()), throut=1e-16)


def test_reconstruction_property_over_random_small_problems():
    """Property form of the reader check: any small problem (sizes, MFIL,
    irreps, seed, spinor order) gives a stream that reconstructs the tensor."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from util import check_rdtwo_reconstruction

    @hyp.settings(max_examples=20, deadline=None, derandomize=True)
    @hyp.given(nl=st.integers(1, 5), ns=st.integers(0, 6), nkr=st.integers(1, 3),
               seed=st.integers(0, 10_000), mfil=st.integers(1, 3), nirr=st.sampled_from([1, 4]),
               shuffle=st.booleans())
    def prop(nl, ns, nkr, seed, mfil, nirr, shuffle):
        if mfil == 1:
            ns = 0
        if ns == 0:
            mfil = 1
        hyp.assume(nkr <= nl + ns)
        p = synth.make_problem(nl, ns, nkr, seed=seed, mfil=mfil, n_irrep=nirr)
        if shuffle:
            p = permute_spinors(p, np.random.default_rng(seed).permutation(p.m))
        img = pyoracle.run(p)
        dense = dense_full(p)
        check_rdtwo_reconstruction(img.hdr, img.idx, img.val, p.kra, p.krb, dense,
                                   tol=1e-13 * max(1.0, np.abs(dense).max()), throut=1e-16)

    prop()
