"""Seeded synthetic inputs for the rotran four-index transformation.

The model follows the workload definitions used to benchmark this package:

* ``n_L`` large- and ``n_S`` small-component real scalar AO functions with
  centres uniform in a 10-bohr box and exponents log-uniform in [0.1, 50]
  (the exponents are recorded for completeness; the integral model below
  only uses the centres).
* AO integrals ``(ij|kl) = sum_Q B[ij,Q] B[kl,Q]`` with ``Q = 3n`` and
  ``B[ij,Q] = exp(-|x_i-x_j|^2 / 2 sigma^2) N(0,1) / sqrt(Q)``, ``sigma = 2``,
  which gives exact 8-fold permutational symmetry and a positive
  semidefinite supermatrix.  Small-component pairs are scaled by
  ``1/(4c^2)`` with ``c = 137.036``.
* Only the pair classes the Coulomb path of rotran transforms exist:
  (LL|LL), (SS|LL) and (SS|SS) (mixed SL pairs are excluded, as in
  ``source/rotran/makind.F:75-77``).
* Optionally the AOs are partitioned into the four irreps of an abelian
  group of order 4 (C2v-like, product = xor of 2-bit labels) and the
  integrals are exactly zero unless ``irr(i)^irr(j) == irr(k)^irr(l)``.
* Spinor coefficients: Kramers pairs of 2n-component vectors with the
  time-reversal (quaternion) structure
  ``QA(jbar) = -conj(QB(j))``, ``QB(jbar) = conj(QA(j))``
  (``source/rotran/kramers.F:134-150``), orthonormalised by the polar
  factor, which keeps that structure.

Integral records follow reltwel's record layout
(``source/reltwel/mfdtwoe.F:520-545``, ``source/reltwel/wrbuf.F:35-46``):
one record holds integrals of a single index-coincidence type ``IT``
(``source/rotran/inttyp.F``), at most ``N2 = 12288`` of them, with labels
``LABEL = I<<16|K`` (first, larger pair) and ``LABEL1 = L<<16|N``;
every file ends with a type-14 record flagged ``FINISH``.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

C_LIGHT = 137.036
RECORD_MAX = 12288  # N2 of reltwel (reltwel/paracom.inc)


# ---------------------------------------------------------------------------
# integral-type table (source/rotran/inttyp.F) and GETTW scale factors
# ---------------------------------------------------------------------------

def inttyp(i, j, k, l):
    """Vectorised INTTYP(IMM,JMM,KMM,LMM) of ``source/rotran/inttyp.F:1-79``.

    Arguments are the four labels of a canonically ordered integral
    ``(i j | k l)``; returns the coincidence type 1..14 as ``int8``.
    """
    i, j, k, l = (np.asarray(x, dtype=np.int64) for x in (i, j, k, l))
    out = np.zeros(np.broadcast(i, j, k, l).shape, dtype=np.int8)
    kgj = k > j
    # K > J branch (inttyp.F:9-36)
    a = kgj & (j > l)
    out = np.where(a & (i != k), 13, out)
    out = np.where(a & (i == k), 10, out)
    b = kgj & ~(j > l)
    out = np.where(b & (j != l) & (k != l), 14, out)
    out = np.where(b & (j != l) & (k == l), 8, out)
    out = np.where(b & (j == l) & (i != k), 11, out)
    out = np.where(b & (j == l) & (i == k), 2, out)
    # K <= J branch (inttyp.F:37-75)
    c = ~kgj & (k != l)
    out = np.where(c & (i != j) & (j != k), 12, out)
    out = np.where(c & (i != j) & (j == k), 9, out)
    out = np.where(c & (i == j) & (j != k), 5, out)
    out = np.where(c & (i == j) & (j == k), 4, out)
    d = ~kgj & (k == l)
    out = np.where(d & (j != k) & (i != j), 7, out)
    out = np.where(d & (j != k) & (i == j), 3, out)
    out = np.where(d & (j == k) & (i != j), 6, out)
    out = np.where(d & (j == k) & (i == j), 1, out)
    return out.astype(np.int8)


def gettw_factor(it):
    """Scale factor GETTW applies to a record of type ``it`` (gettw.F:33-45)."""
    it = np.asarray(it)
    f = np.ones(it.shape, dtype=np.float64)
    f = np.where(it == 1, 0.125, f)
    f = np.where(it == 3, 0.25, f)
    f = np.where((it == 2) | ((it >= 4) & (it <= 8)), 0.5, f)
    return f


# ---------------------------------------------------------------------------
# spinors
# ---------------------------------------------------------------------------

def make_spinors(n: int, nkr: int, rng: np.random.Generator):
    """Kramers-paired orthonormal spinor coefficients.

    Returns ``qa, qb`` (``n x 2*nkr`` complex, Fortran order semantics:
    column ``j`` is spinor ``j+1``) and the 1-based index tables of
    ``source/rotran/getmos.F:166-199``: ``itrmo`` (partner, + for the
    unbarred member), ``kra``/``krb`` (spinor of the unbarred / barred member
    of each pair) and ``ikrmo`` (+/- pair index).  Spinor ``2k-1`` is the
    unbarred and ``2k`` the barred member of pair ``k``.
    """
    m = 2 * nkr
    if nkr > n:
        raise ValueError("need nkr <= n for orthonormal spinors")
    a = rng.standard_normal((n, nkr)) + 1j * rng.standard_normal((n, nkr))
    b = rng.standard_normal((n, nkr)) + 1j * rng.standard_normal((n, nkr))
    # quaternion-structured 2n x 2nkr matrix: [A, -conj(B); B, conj(A)]
    big = np.zeros((2 * n, m), dtype=np.complex128)
    big[:n, 0::2] = a
    big[n:, 0::2] = b
    big[:n, 1::2] = -np.conj(b)
    big[n:, 1::2] = np.conj(a)
    # polar factor U = M (M^H M)^(-1/2) keeps the quaternion structure
    w, v = np.linalg.eigh(big.conj().T @ big)
    u = big @ (v * (1.0 / np.sqrt(w))) @ v.conj().T
    qa = np.ascontiguousarray(u[:n, :])
    qb = np.ascontiguousarray(u[n:, :])
    # impose the structure exactly, as KRAMERS does for barred spinors
    qa[:, 1::2] = -np.conj(qb[:, 0::2])
    qb[:, 1::2] = np.conj(qa[:, 0::2])
    itrmo = np.zeros(m, dtype=np.int32)
    ikrmo = np.zeros(m, dtype=np.int32)
    kra = np.arange(1, m + 1, 2, dtype=np.int32)
    krb = np.arange(2, m + 1, 2, dtype=np.int32)
    itrmo[0::2] = krb
    itrmo[1::2] = -kra
    ikrmo[0::2] = np.arange(1, nkr + 1)
    ikrmo[1::2] = -np.arange(1, nkr + 1)
    return qa, qb, itrmo, kra, krb, ikrmo


# ---------------------------------------------------------------------------
# AO model
# ---------------------------------------------------------------------------

def pair_list(lo: int, hi: int):
    """All pairs (p, q), hi >= p >= q >= lo (1-based), in pair-index order."""
    ps, qs = [], []
    for p in range(lo, hi + 1):
        ps.append(np.full(p - lo + 1, p, dtype=np.int32))
        qs.append(np.arange(lo, p + 1, dtype=np.int32))
    if not ps:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    return np.concatenate(ps), np.concatenate(qs)


@dataclasses.dataclass
class AOModel:
    n_l: int
    n_s: int
    centres: np.ndarray
    exponents: np.ndarray
    irrep: np.ndarray          # per AO, 0..3 (all 0 without block symmetry)
    n_irrep: int
    pl: np.ndarray             # LL pairs (p), 1-based
    ql: np.ndarray
    ps: np.ndarray             # SS pairs (p), 1-based
    qs: np.ndarray
    bl: np.ndarray             # B rows of the LL pairs
    bs: np.ndarray             # B rows of the SS pairs (scaled by 1/(4c^2))

    @property
    def n(self):
        return self.n_l + self.n_s


def make_ao_model(n_l: int, n_s: int, rng: np.random.Generator,
                  sigma: float = 2.0, n_irrep: int = 1) -> AOModel:
    n = n_l + n_s
    centres = rng.uniform(0.0, 10.0, size=(n, 3))
    exponents = np.exp(rng.uniform(math.log(0.1), math.log(50.0), size=n))
    if n_irrep == 1:
        irrep = np.zeros(n, dtype=np.int32)
    elif n_irrep == 4:
        irrep = rng.integers(0, 4, size=n).astype(np.int32)
    else:
        raise ValueError("n_irrep must be 1 or 4")
    nq = 3 * n
    pl, ql = pair_list(1, n_l)
    ps, qs = pair_list(n_l + 1, n)

    def brows(p, q):
        d2 = np.sum((centres[p - 1] - centres[q - 1]) ** 2, axis=1)
        env = np.exp(-d2 / (2.0 * sigma * sigma))
        return env[:, None] * rng.standard_normal((p.size, nq)) / math.sqrt(nq)

    bl = brows(pl, ql)
    bs = brows(ps, qs) / (4.0 * C_LIGHT * C_LIGHT)
    return AOModel(n_l, n_s, centres, exponents, irrep, n_irrep,
                   pl, ql, ps, qs, bl, bs)


def breit_pairs(model: AOModel):
    """The SL pairs (p small, q large component; 1-based, p > q) of the Gaunt
    integrals and their B rows: (pq|rs) = sum_Q B[pq,Q] B[rs,Q] with the
    same Gaussian-envelope model as the Coulomb classes, each SL pair scaled
    by 1/(2c).  The rows come from their own seeded generator (the AO
    model's centres fix it), so adding the Gaunt file leaves the Coulomb
    integrals and spinors of a problem unchanged."""
    if getattr(model, "_breit", None) is None:
        n_l, n = model.n_l, model.n
        p = np.repeat(np.arange(n_l + 1, n + 1, dtype=np.int32), n_l)
        q = np.tile(np.arange(1, n_l + 1, dtype=np.int32), model.n_s)
        seed = int(np.abs(model.centres).sum() * 1e6) % (2 ** 31)
        rng = np.random.default_rng(seed)
        nq = 3 * n
        d2 = np.sum((model.centres[p - 1] - model.centres[q - 1]) ** 2, axis=1)
        env = np.exp(-d2 / (2.0 * 2.0 * 2.0))
        b = env[:, None] * rng.standard_normal((p.size, nq)) / math.sqrt(nq) / (2.0 * C_LIGHT)
        model._breit = (p, q, b)
    return model._breit


def _file_integrals(model: AOModel, which: str, chunk: int = 2048):
    """Unique canonical integrals of one SRT file as flat arrays.

    ``which`` is ``"LL"`` ((LL|LL)), ``"SL"`` ((SS|LL), first pair SS),
    ``"SS"``, or ``"BR"`` (the Gaunt (SL|SL) integrals of the Breit file).  Returns ``(value, label2, label1, it)``: ``label2`` packs
    the first (larger) pair ``I<<16|K``, ``label1`` the second ``L<<16|N``.
    """
    if which == "LL":
        pa, qa_, ba, pc, qc, bc, tri = model.pl, model.ql, model.bl, model.pl, model.ql, model.bl, True
    elif which == "SL":
        pa, qa_, ba, pc, qc, bc, tri = model.ps, model.qs, model.bs, model.pl, model.ql, model.bl, False
    elif which == "SS":
        pa, qa_, ba, pc, qc, bc, tri = model.ps, model.qs, model.bs, model.ps, model.qs, model.bs, True
    elif which == "BR":
        pb, qb_, bb = breit_pairs(model)
        pa, qa_, ba, pc, qc, bc, tri = pb, qb_, bb, pb, qb_, bb, True
    else:
        raise ValueError(which)
    irr = model.irrep
    ga = irr[pa - 1] ^ irr[qa_ - 1]
    gc = irr[pc - 1] ^ irr[qc - 1]
    vals, l2s, l1s, its = [], [], [], []
    for s0 in range(0, pa.size, chunk):
        s1 = min(pa.size, s0 + chunk)
        ncd = s1 if tri else pc.size
        g = ba[s0:s1] @ bc[:ncd].T
        rows = np.arange(s0, s1)[:, None]
        cols = np.arange(ncd)[None, :]
        mask = np.ones(g.shape, dtype=bool)
        if tri:
            mask &= cols <= rows
        if model.n_irrep > 1:
            mask &= ga[s0:s1, None] == gc[None, :ncd]
        ri, ci = np.nonzero(mask)
        a = pa[s0 + ri]
        b = qa_[s0 + ri]
        c = pc[ci]
        d = qc[ci]
        vals.append(g[ri, ci])
        l2s.append(((a.astype(np.int64) << 16) | b).astype(np.int32))
        l1s.append(((c.astype(np.int64) << 16) | d).astype(np.int32))
        its.append(inttyp(a, b, c, d))
    if not vals:
        z = np.zeros(0)
        return z, z.astype(np.int32), z.astype(np.int32), z.astype(np.int8)
    return (np.concatenate(vals), np.concatenate(l2s), np.concatenate(l1s),
            np.concatenate(its))


@dataclasses.dataclass
class SrtRecord:
    """One SRTTW/SRTLB record pair (gettw.F:15-29)."""
    it: int
    finish: bool
    rint: np.ndarray     # float64, unscaled integral values
    label2: np.ndarray   # int32, I<<16|K of the first pair
    label1: np.ndarray   # int32, L<<16|N of the second pair


def file_records(model: AOModel, which: str, record_max: int = RECORD_MAX):
    """Split a file's integrals into reltwel-style records (wrbuf.F)."""
    v, l2, l1, it = _file_integrals(model, which)
    recs = []
    for t in range(1, 15):
        sel = np.nonzero(it == t)[0]
        chunks = [sel[s0:s0 + record_max] for s0 in range(0, sel.size, record_max)]
        if t == 14:
            # the closing WRBUF call always writes a type-14 record, possibly
            # empty, with FINISH set (wrbuf.F:27-38)
            last = chunks.pop() if chunks else sel[:0]
        for idx in chunks:
            recs.append(SrtRecord(t, False, v[idx], l2[idx], l1[idx]))
        if t == 14:
            recs.append(SrtRecord(14, True, v[last], l2[last], l1[last]))
    return recs


# ---------------------------------------------------------------------------
# full problem
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Problem:
    model: AOModel
    nkr: int
    qa: np.ndarray
    qb: np.ndarray
    itrmo: np.ndarray
    kra: np.ndarray
    krb: np.ndarray
    ikrmo: np.ndarray
    mfil: int
    files: dict            # "LL"/"SL"/"SS" -> list[SrtRecord]

    @property
    def n(self):
        return self.model.n

    @property
    def nsc1(self):
        return self.model.n_l

    @property
    def m(self):
        return 2 * self.nkr

    def all_records(self):
        """(file_class, record) in the order SORT1 reads them (sort1.F:60);
        the Gaunt file (class 4, SRTBREI) follows when the problem has one."""
        order = [("LL", 1), ("SL", 2), ("SS", 3)][: self.mfil] + [("BR", 4)]
        for key, cls in order:
            for r in self.files.get(key, []):
                yield cls, r

    def flat_records(self):
        """Concatenated arrays + per-record table, for bulk submission."""
        cls, its, nts, vs, l2s, l1s = [], [], [], [], [], []
        for c, r in self.all_records():
            cls.append(c)
            its.append(r.it)
            nts.append(r.rint.size)
            vs.append(r.rint)
            l2s.append(r.label2)
            l1s.append(r.label1)
        cat = (lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt))
        return (np.asarray(cls, np.int32), np.asarray(its, np.int32),
                np.asarray(nts, np.int64), cat(vs, np.float64),
                cat(l2s, np.int32), cat(l1s, np.int32))

    def imoras_pairs(self):
        """MDCINT header orbital pairs (inittwoe.F:21-23) for one C1 irrep."""
        out = np.empty(2 * self.nkr, dtype=np.int32)
        out[0::2] = self.kra
        out[1::2] = self.krb
        return out


def make_problem(n_l: int, n_s: int, nkr: int, seed: int = 0,
                 n_irrep: int = 1, mfil: int = 3, breit: bool = False) -> Problem:
    """Build one seeded transform instance (AO records + spinors); with
    ``breit`` also the Gaunt (SL|SL) file (class 4)."""
    rng = np.random.default_rng(seed)
    model = make_ao_model(n_l, n_s, rng, n_irrep=n_irrep)
    qa, qb, itrmo, kra, krb, ikrmo = make_spinors(model.n, nkr, rng)
    files = {"LL": file_records(model, "LL")}
    if mfil >= 2 and n_s > 0:
        files["SL"] = file_records(model, "SL")
    if mfil >= 3 and n_s > 0:
        files["SS"] = file_records(model, "SS")
    if breit and n_s > 0 and n_l > 0:
        files["BR"] = file_records(model, "BR")
    return Problem(model, nkr, qa, qb, itrmo, kra, krb, ikrmo, mfil, files)


# named workloads -----------------------------------------------------------

CONFIGS = {
    # (n_L, n_S, nkr, n_irrep)
    "c1_fp64_n64": (24, 40, 32, 1),
    "c2_precision_n400": (160, 240, 120, 1),
    "c4_adjoint_n256": (100, 156, 64, 1),
    "c5_large_n480": (192, 288, 200, 4),
}


def batched_instances(count: int = 48, seed0: int = 0):
    """Sizes of the 48-instance batched workload (seeds 0..47).

    n_AO ~ U[40, 200] with a 60% small-component share and nkr ~ U[16, 80]
    (nkr is capped at n so that the spinors stay orthonormal).
    """
    out = []
    for s in range(seed0, seed0 + count):
        rng = np.random.default_rng(10_000 + s)
        n = int(rng.integers(40, 201))
        n_s = int(round(0.6 * n))
        nkr = int(min(rng.integers(16, 81), n // 2))
        out.append((n - n_s, n_s, nkr, s))
    return out


def dense_ao_tensor(model: AOModel, mfil: int = 3) -> np.ndarray:
    """Full (pq|rs) over all n AOs (small n only; test helper)."""
    n = model.n
    g = np.zeros((n, n, n, n))
    blocks = [(model.pl, model.ql, model.bl, "L"), (model.ps, model.qs, model.bs, "S")]
    irr = model.irrep
    for pa, qa_, ba, ca in blocks:
        for pc, qc, bc, cc in blocks:
            if ca == "S" and cc == "S" and mfil < 3:
                continue
            if (ca != cc) and mfil < 2:
                continue
            if pa.size == 0 or pc.size == 0:
                continue
            v = ba @ bc.T
            if model.n_irrep > 1:
                allowed = (irr[pa - 1] ^ irr[qa_ - 1])[:, None] == (irr[pc - 1] ^ irr[qc - 1])[None, :]
                v = np.where(allowed, v, 0.0)
            a, b, c, d = pa - 1, qa_ - 1, pc - 1, qc - 1
            for (x, y) in ((a, b), (b, a)):
                for (z, w) in ((c, d), (d, c)):
                    g[x[:, None], y[:, None], z[None, :], w[None, :]] = v
    return g


# ---------------------------------------------------------------------------
# device-side record generation for the large workloads (torch, same model)
# ---------------------------------------------------------------------------

def _inttyp_torch(i, j, k, l):
    import torch
    out = torch.zeros_like(i, dtype=torch.int8)
    kgj = k > j
    w = torch.where
    a = kgj & (j > l)
    out = w(a & (i != k), 13, out); out = w(a & (i == k), 10, out)
    b = kgj & ~(j > l)
    out = w(b & (j != l) & (k != l), 14, out); out = w(b & (j != l) & (k == l), 8, out)
    out = w(b & (j == l) & (i != k), 11, out); out = w(b & (j == l) & (i == k), 2, out)
    c = ~kgj & (k != l)
    out = w(c & (i != j) & (j != k), 12, out); out = w(c & (i != j) & (j == k), 9, out)
    out = w(c & (i == j) & (j != k), 5, out); out = w(c & (i == j) & (j == k), 4, out)
    d = ~kgj & (k == l)
    out = w(d & (j != k) & (i != j), 7, out); out = w(d & (j != k) & (i == j), 3, out)
    out = w(d & (j == k) & (i != j), 6, out); out = w(d & (j == k) & (i == j), 1, out)
    return out.to(torch.int8)


def device_records(problem_or_model, mfil: int = 3, device="cuda", chunk: int = 4096):
    """All integral records of a problem generated on a CUDA device.

    Returns ``(file_class, itype, nt)`` host arrays (one record per file and
    integral type) and device tensors ``(rint, label2, label1)`` holding the
    records concatenated in that order.  Values equal ``_file_integrals`` up
    to the summation order of the B B^T products.
    """
    import torch
    model = problem_or_model.model if hasattr(problem_or_model, "model") else problem_or_model
    irr = torch.as_tensor(model.irrep, device=device, dtype=torch.int32)
    files = [("LL", 1)]
    if mfil >= 2 and model.n_s > 0:
        files.append(("SL", 2))
    if mfil >= 3 and model.n_s > 0:
        files.append(("SS", 3))
    tl = (torch.as_tensor(model.pl, device=device).long(), torch.as_tensor(model.ql, device=device).long(),
          torch.as_tensor(model.bl, device=device))
    ts = (torch.as_tensor(model.ps, device=device).long(), torch.as_tensor(model.qs, device=device).long(),
          torch.as_tensor(model.bs, device=device))
    cls_l, it_l, nt_l, vs, l2s, l1s = [], [], [], [], [], []
    for key, fc in files:
        (pa, qa_, ba), (pc, qc, bc), tri = {
            "LL": (tl, tl, True), "SL": (ts, tl, False), "SS": (ts, ts, True)}[key]
        ga = irr[pa - 1] ^ irr[qa_ - 1]
        gc = irr[pc - 1] ^ irr[qc - 1]
        fv, f2, f1, ft = [], [], [], []
        for s0 in range(0, pa.numel(), chunk):
            s1 = min(pa.numel(), s0 + chunk)
            ncd = s1 if tri else pc.numel()
            g = ba[s0:s1] @ bc[:ncd].T
            mask = torch.ones_like(g, dtype=torch.bool)
            if tri:
                rows = torch.arange(s0, s1, device=device)[:, None]
                cols = torch.arange(ncd, device=device)[None, :]
                mask &= cols <= rows
            if model.n_irrep > 1:
                mask &= ga[s0:s1, None] == gc[None, :ncd]
            ri, ci = torch.nonzero(mask, as_tuple=True)
            a, b, c, d = pa[s0 + ri], qa_[s0 + ri], pc[ci], qc[ci]
            fv.append(g[ri, ci])
            f2.append(((a << 16) | b).to(torch.int32))
            f1.append(((c << 16) | d).to(torch.int32))
            ft.append(_inttyp_torch(a, b, c, d))
            del g, mask, ri, ci
        v, l2, l1, it = (torch.cat(x) for x in (fv, f2, f1, ft))
        order = torch.argsort(it, stable=True)
        v, l2, l1, it = v[order], l2[order], l1[order], it[order]
        counts = torch.bincount(it.long(), minlength=15).cpu().numpy()
        for t in range(1, 15):
            if counts[t]:
                cls_l.append(fc); it_l.append(t); nt_l.append(int(counts[t]))
        vs.append(v); l2s.append(l2); l1s.append(l1)
        del order, it
    return (np.asarray(cls_l, np.int32), np.asarray(it_l, np.int32), np.asarray(nt_l, np.int64),
            torch.cat(vs), torch.cat(l2s), torch.cat(l1s))


def make_spinor_problem(n_l: int, n_s: int, nkr: int, seed: int = 0, n_irrep: int = 1,
                        mfil: int = 3) -> Problem:
    """Model and spinors of a workload without host-side integral records
    (for the device-side record generation of large workloads)."""
    rng = np.random.default_rng(seed)
    model = make_ao_model(n_l, n_s, rng, n_irrep=n_irrep)
    qa, qb, itrmo, kra, krb, ikrmo = make_spinors(model.n, nkr, rng)
    return Problem(model, nkr, qa, qb, itrmo, kra, krb, ikrmo, mfil, {})


def bucket_records(model: AOModel, pq_pairs, mfil: int = 3):
    """The integral records rotran sorts into the given pq buckets.

    Bucket pq (label1) holds (rs|pq) with rs >= pq of the same class
    ((LL|LL) or (SS|SS)) and, for an LL pair, every (SS|LL) integral
    (sort1.F:78-142).  Returns flat record arrays like
    ``Problem.flat_records`` (one record per file and type).
    """
    nl = model.n_l
    lidx = {(int(p), int(q)): i for i, (p, q) in enumerate(zip(model.pl, model.ql))}
    sidx = {(int(p), int(q)): i for i, (p, q) in enumerate(zip(model.ps, model.qs))}
    irr = model.irrep
    out = {}
    for (p, q) in pq_pairs:
        cls_pq = "L" if p <= nl else "S"
        if cls_pq == "L":
            t = lidx[(p, q)]
            parts = [(1, model.pl[t:], model.ql[t:], model.bl[t:], model.bl[t])]
            if mfil >= 2 and model.n_s:
                parts.append((2, model.ps, model.qs, model.bs, model.bl[t]))
        else:
            if mfil < 3:
                continue
            t = sidx[(p, q)]
            parts = [(3, model.ps[t:], model.qs[t:], model.bs[t:], model.bs[t])]
        for fc, a, b, brs, bpq in parts:
            v = brs @ bpq
            keep = np.ones(v.size, dtype=bool)
            if model.n_irrep > 1:
                keep = (irr[a - 1] ^ irr[b - 1]) == (irr[p - 1] ^ irr[q - 1])
            a, b, v = a[keep], b[keep], v[keep]
            c = np.full(a.size, p, np.int64)
            d = np.full(a.size, q, np.int64)
            it = inttyp(a, b, c, d)
            l2 = ((a.astype(np.int64) << 16) | b).astype(np.int32)
            l1 = ((c << 16) | d).astype(np.int32)
            for ty in np.unique(it):
                m_ = it == ty
                out.setdefault((fc, int(ty)), []).append((v[m_], l2[m_], l1[m_]))
    keys = sorted(out)
    cls = np.asarray([k[0] for k in keys], np.int32)
    its = np.asarray([k[1] for k in keys], np.int32)
    nts = np.asarray([sum(x[0].size for x in out[k]) for k in keys], np.int64)
    cat = lambda j, dt: (np.concatenate([x[j] for k in keys for x in out[k]]).astype(dt)
                         if keys else np.zeros(0, dt))
    return cls, its, nts, cat(0, np.float64), cat(1, np.int32), cat(2, np.int32)
