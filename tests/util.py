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
    separately (outpp1.F:76, outpp2.F:156) while the GPU filters the sum.
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
