"""The skeleton Fock oracle (tmoone's MFDFOCK/FOCK and MFDBREIT/GAUNT restated
in oracle/tmoone_fock_oracle.c) against dense formulations (CPU only).

FOCK adds each unique integral (IJ|KL) of a record of type IT
(source/tmoone/fock.F) to lower-triangle Fock elements.  For one set of
densities with a real symmetric part D0 (AAR) and real antisymmetric parts
D1, D2, D3 (AAI, BAR, BAI) -- the quaternion structure of a Kramers-
restricted density -- the complete skeleton must equal, element (i,j) with
i >= j,

    F0(i,j) = sum_kl [2 (ij|kl) - (ik|jl)] D0(k,l)
    Fx(i,j) = - sum_kl (ik|jl) Dx(k,l)            x = 1, 2, 3

with (ij|kl) the full real integral tensor (eight-fold permutation
symmetry) rebuilt from the unique records."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402

from molfdir_gb300 import synth  # noqa: E402


def full_tensor(records, n, mfil=3):
    cls, its, nts, v, l2, l1 = records
    off = np.concatenate([[0], np.cumsum(nts)])
    keep = np.concatenate([np.arange(off[r], off[r + 1]) for r in range(cls.size) if 1 <= cls[r] <= mfil]
                          or [np.zeros(0, np.int64)]).astype(np.int64)
    a, b = (l2[keep] >> 16) - 1, (l2[keep] & 0xFFFF) - 1
    c, d = (l1[keep] >> 16) - 1, (l1[keep] & 0xFFFF) - 1
    g = np.zeros((n,) * 4)
    seen = np.zeros((n,) * 4, np.int32)
    for (p, q, r, s) in ((a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                         (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)):
        g[p, q, r, s] = v[keep]
    np.add.at(seen, (a, b, c, d), 1)
    assert seen.max() <= 1, "a unique integral appears twice"
    return g


def tri_pack(m):
    n = m.shape[0]
    i, j = np.tril_indices(n)
    order = np.argsort(i * (i + 1) // 2 + j)
    return m[i[order], j[order]]


def densities(n, nmat, seed):
    rng = np.random.default_rng(seed)
    out, full = [], []
    for _ in range(nmat):
        s = rng.standard_normal((n, n))
        s = s + s.T
        anti = []
        for _ in range(3):
            x = rng.standard_normal((n, n))
            anti.append(x - x.T)
        mats = [s, anti[1], anti[0], anti[2]]  # AAR, BAR, AAI, BAI
        full.append(mats)
        out.append(np.stack([tri_pack(m) for m in mats]))
    return np.stack(out), full


@pytest.mark.parametrize("nl,ns,nkr,seed,irreps", [(3, 4, 2, 0, False), (4, 6, 3, 1, False),
                                                   (5, 7, 3, 2, True), (6, 9, 4, 3, False)])
def test_fock_oracle_is_coulomb_minus_exchange(nl, ns, nkr, seed, irreps):
    kw = {"n_irrep": 4} if irreps else {}
    try:
        p = synth.make_problem(nl, ns, nkr, seed=seed, **kw)
    except TypeError:
        if irreps:
            pytest.skip("no irrep option in the generator")
        raise
    n = p.n
    recs = p.flat_records()
    g = full_tensor(recs, n, p.mfil)
    dens, full = densities(n, 2, seed)
    f = pyoracle.fock_skeleton(recs, n, dens, mfil=p.mfil)
    i, j = np.tril_indices(n)
    order = np.argsort(i * (i + 1) // 2 + j)
    i, j = i[order], j[order]
    off = i != j
    for s in range(2):
        d0, d2, d1, d3 = full[s]   # AAR, BAR, AAI, BAI
        jmat = np.einsum("ijkl,kl->ij", g, d0)
        kmat = [np.einsum("ikjl,kl->ij", g, x) for x in (d0, d2, d1, d3)]
        want = [2 * jmat - kmat[0], -kmat[1], -kmat[2], -kmat[3]]
        scale = max(np.abs(w).max() for w in want)
        assert np.allclose(f[s, 0], want[0][i, j], atol=1e-12 * scale, rtol=0)
        for x in (1, 2, 3):
            assert np.allclose(f[s, x][off], want[x][i, j][off], atol=1e-12 * scale, rtol=0), x


def test_fock_oracle_rejects_bad_labels():
    p = synth.make_problem(3, 4, 2, seed=0)
    cls, its, nts, v, l2, l1 = p.flat_records()
    l2 = l2.copy()
    l2[0] = (p.n + 1) << 16 | 1
    n = p.n
    with pytest.raises(ValueError):
        pyoracle.fock_skeleton((cls, its, nts, v, l2, l1), n, np.zeros((1, 4, n * (n + 1) // 2)))


def gaunt_tensor(records, n):
    """The full (SL|SL) tensor from the file-4 records (eight-fold permutation symmetry)."""
    cls, its, nts, v, l2, l1 = records
    off = np.concatenate([[0], np.cumsum(nts)])
    keep = np.concatenate([np.arange(off[r], off[r + 1]) for r in range(cls.size) if cls[r] == 4])
    a, b = (l2[keep] >> 16) - 1, (l2[keep] & 0xFFFF) - 1
    c, d = (l1[keep] >> 16) - 1, (l1[keep] & 0xFFFF) - 1
    g = np.zeros((n,) * 4)
    for (p, q, r, s) in ((a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                         (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)):
        g[p, q, r, s] = v[keep]
    return g


@pytest.mark.parametrize("nl,ns,nkr,seed", [(3, 4, 2, 0), (4, 6, 3, 2), (6, 9, 3, 5)])
def test_gaunt_oracle_is_three_k_and_minus_k(nl, ns, nkr, seed):
    """GAUNT (source/tmoone/gaunt.F) restated by the oracle against a dense
    formulation: for a Kramers-restricted density (AAR symmetric; BAR, AAI,
    BAI antisymmetric) the Gaunt skeleton is, element (i,j) with i >= j,
    3 K[D](i,j) for AAR and -K[D](i,j) for the others (off the diagonal),
    K[D](i,j) = sum_kl (ik|jl) D(k,l) over the (SL|SL) integrals -- the
    scalar and vector parts of sigma . sigma."""
    p = synth.make_problem(nl, ns, nkr, seed=seed, breit=True)
    recs = p.flat_records()
    n = p.n
    g = gaunt_tensor(recs, n)
    dens, full = densities(n, 2, seed)
    f = pyoracle.fock_gaunt(recs, n, dens)
    i, j = np.tril_indices(n)
    order = np.argsort(i * (i + 1) // 2 + j)
    i, j = i[order], j[order]
    off = i != j
    for s in range(2):
        mats = full[s]   # AAR, BAR, AAI, BAI
        k = [np.einsum("ikjl,kl->ij", g, x) for x in mats]
        want = [3.0 * k[0], -k[1], -k[2], -k[3]]
        scale = max(np.abs(w).max() for w in want)
        assert np.allclose(f[s, 0], want[0][i, j], atol=1e-12 * scale, rtol=0)
        for x in (1, 2, 3):
            assert np.allclose(f[s, x][off], want[x][i, j][off], atol=1e-12 * scale, rtol=0), x


def test_gaunt_oracle_reads_file_4_only_and_rejects_other_types():
    p = synth.make_problem(4, 6, 3, seed=2, breit=True)
    cls, its, nts, v, l2, l1 = p.flat_records()
    n = p.n
    dens, _ = densities(n, 1, 2)
    f = pyoracle.fock_gaunt((cls, its, nts, v, l2, l1), n, dens)
    assert np.abs(f).max() > 0
    # without the file-4 records nothing is added
    keep = cls != 4
    off = np.concatenate([[0], np.cumsum(nts)])
    sel = np.concatenate([np.arange(off[r], off[r + 1]) for r in np.nonzero(keep)[0]])
    f0 = pyoracle.fock_gaunt((cls[keep], its[keep], nts[keep], v[sel], l2[sel], l1[sel]), n, dens)
    assert not f0.any()
    # linear in the integrals: scaling them scales the sets
    f2 = pyoracle.fock_gaunt((cls, its, nts, 2.0 * v, l2, l1), n, dens)
    assert np.allclose(f2, 2.0 * f, rtol=0, atol=1e-14 * np.abs(f).max())
    its = its.copy()
    its[np.nonzero(cls == 4)[0][0]] = 12
    with pytest.raises(ValueError):
        pyoracle.fock_gaunt((cls, its, nts, v, l2, l1), n, dens)
