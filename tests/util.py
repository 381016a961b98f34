"""Helpers shared by the tests: problem variants and record-stream checks."""

from __future__ import annotations

import copy

import numpy as np


def permute_spinors(problem, perm):
    """Reorder the spinors: new spinor k is old spinor perm[k] (0-based)."""
    p = copy.copy(problem)
    perm = np.asarray(perm)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    p.qa = np.ascontiguousarray(problem.qa[:, perm])
    p.qb = np.ascontiguousarray(problem.qb[:, perm])
    old_itr = problem.itrmo[perm]
    p.itrmo = (np.sign(old_itr) * (inv[np.abs(old_itr) - 1] + 1)).astype(np.int32)
    p.kra = (inv[problem.kra - 1] + 1).astype(np.int32)
    p.krb = (inv[problem.krb - 1] + 1).astype(np.int32)
    p.ikrmo = problem.ikrmo[perm].astype(np.int32)
    return p


def compare_streams(got, ref, tol, presence_tol=None):
    """Same records in the same order, same element labels, values within tol.

    got/ref: (hdr, idx, val).  Returns the max |difference| over elements
    present in both.  An element present in only one stream is accepted when
    both its values are at most ``presence_tol`` (default ``tol``): a value
    within rounding of THROUT, or, for a large THROUT, an integral whose
    canonical and particle-interchanged halves the reference filters
    separately (outpp1.F:34, outpp2.F:40) while the GPU filters the sum.
    """
    presence_tol = tol if presence_tol is None else presence_tol
    gh, gi, gv = got
    rh, ri, rv = ref
    assert gh.shape[0] == rh.shape[0], f"record count {gh.shape[0]} != {rh.shape[0]}"
    assert np.array_equal(gh[:, :2], rh[:, :2]), "record labels / order differ"
    if np.array_equal(gh[:, 2], rh[:, 2]) and np.array_equal(gi, ri):
        return float(np.max(np.abs(gv - rv))) if gv.size else 0.0
    err = 0.0
    go = np.concatenate([[0], np.cumsum(gh[:, 2])])
    ro = np.concatenate([[0], np.cumsum(rh[:, 2])])
    for r in range(gh.shape[0]):
        a = {tuple(gi[z]): gv[z] for z in range(go[r], go[r + 1])}
        b = {tuple(ri[z]): rv[z] for z in range(ro[r], ro[r + 1])}
        for k in set(a) | set(b):
            va, vb = a.get(k, 0.0), b.get(k, 0.0)
            if (k in a) != (k in b):
                assert abs(va) <= presence_tol and abs(vb) <= presence_tol, \
                    f"record {r} element {k}: {va} vs {vb}"
                continue
            err = max(err, abs(va - vb))
        ka = [k for k in gi[go[r]:go[r + 1]].tolist() if tuple(k) in b]
        kb = [k for k in ri[ro[r]:ro[r + 1]].tolist() if tuple(k) in a]
        assert ka == kb, f"record {r}: element order differs"
    return err


def rdtwo_expand(hdr, idx, val, kra, krb, m):
    """The spinor integral tensor a MDCINT reader reconstructs: goscip's RDTWO
    (source/goscip/rdtwo.F:29-83) stores each element (ij|kl) under 16
    quadruples -- itself, its complex conjugate (ji|lk)*, the particle
    interchange (kl|ij) and (lk|ji)*, each with the time-reversed partners of
    the pairs, signed by SignIJ = sign(IKR) sign(JKR) and SignKL.  Returns
    (full, hits): the implied values (later assignments win, as in RDTWO)
    and, per quadruple, the list of all implied values, for consistency
    checks.  Kramers index k > 0 is spinor kra[k-1], k < 0 is krb[-k-1]."""
    full = np.zeros((m, m, m, m), np.complex128)
    hits = {}

    def sp(k):
        return (kra[k - 1] if k > 0 else krb[-k - 1]) - 1

    off = 0
    for ikr, jkr, nz in hdr:
        i, itr, j, jtr = sp(ikr), sp(-ikr), sp(jkr), sp(-jkr)
        sij = np.sign(ikr) * np.sign(jkr)
        for z in range(nz):
            kkr, lkr = idx[off + z]
            v = val[off + z]
            k, ktr, l, ltr = sp(kkr), sp(-kkr), sp(lkr), sp(-lkr)
            skl = np.sign(kkr) * np.sign(lkr)
            c = np.conj(v)
            for q, x in (((i, j, k, l), v), ((jtr, itr, k, l), sij * v),
                         ((i, j, ltr, ktr), skl * v), ((jtr, itr, ltr, ktr), sij * skl * v),
                         ((j, i, l, k), c), ((itr, jtr, l, k), sij * c),
                         ((j, i, ktr, ltr), skl * c), ((itr, jtr, ktr, ltr), sij * skl * c),
                         ((k, l, i, j), v), ((ltr, ktr, i, j), skl * v),
                         ((k, l, jtr, itr), sij * v), ((ltr, ktr, jtr, itr), sij * skl * v),
                         ((l, k, j, i), c), ((ktr, ltr, j, i), skl * c),
                         ((l, k, itr, jtr), sij * c), ((ktr, ltr, itr, jtr), sij * skl * c)):
                full[q] = x
                hits.setdefault(q, []).append(x)
        off += nz
    return full, hits


def check_rdtwo_reconstruction(hdr, idx, val, kra, krb, dense, tol, throut=0.0):
    """Every quadruple a reader reconstructs equals the dense tensor, every
    implied value agrees, and every quadruple the stream leaves out is at
    most THROUT (plus tol) in the dense tensor.  Returns the max error."""
    m = dense.shape[0]
    full, hits = rdtwo_expand(hdr, idx, val, kra, krb, m)
    err = 0.0
    for q, xs in hits.items():
        for x in xs:
            err = max(err, abs(x - dense[q]))
    mask = np.zeros(dense.shape, bool)
    if hits:
        mask[tuple(np.array(list(hits)).T)] = True
    missing = float(np.abs(dense[~mask]).max()) if (~mask).any() else 0.0
    assert missing <= throut + tol, f"an integral of size {missing:.3e} is not reachable"
    assert err <= tol, f"reconstructed value off by {err:.3e}"
    return err


def dense_full(p):
    """(ij|kl) over all spinors by the textbook four-index sum (small n)."""
    from molfdir_gb300 import synth
    n, m = p.n, p.m
    g = synth.dense_ao_tensor(p.model, p.mfil).reshape(n * n, n * n)
    d = (np.einsum("pa,qb->abpq", p.qa.conj(), p.qa)
         + np.einsum("pa,qb->abpq", p.qb.conj(), p.qb)).reshape(m * m, n * n)
    return ((d @ g) @ d.T).reshape(m, m, m, m)
