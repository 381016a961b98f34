"""ctypes binding of the CPU oracle (test infrastructure only).

Imported by the tests, by the smoke check and by bench.py's CPU-baseline
leg; never by the product package.  ``build()`` compiles
``oracle/rotran_oracle.c`` (rotran) and ``oracle/tmoone_fock_oracle.c``
(tmoone's skeleton Fock build) into ``oracle/_build/liborotran.so``.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborotran.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("rotran_oracle.c", "tmoone_fock_oracle.c", "rotran_oracle.h")]
    if force or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(f) for f in srcs):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-std=c11", "-shared",
                               "-o", LIB, srcs[0], srcs[1], "-lm"], cwd=HERE)
    return LIB


class _Params(C.Structure):
    _fields_ = [("nsc", C.c_int), ("nsc1", C.c_int), ("nsp", C.c_int), ("nkr", C.c_int),
                ("mfil", C.c_int), ("quater", C.c_int), ("thrgen", C.c_double),
                ("throut", C.c_double), ("nthreads", C.c_int), ("limit_pq", C.c_long),
                ("limit_ij", C.c_long), ("pq_select", C.POINTER(C.c_long)),
                ("n_pq_select", C.c_long), ("fake_list_len", C.c_long), ("breit", C.c_int)]


class _Result(C.Structure):
    _fields_ = [("nrec", C.c_long), ("hdr", C.POINTER(C.c_int)), ("nz_total", C.c_long),
                ("idx", C.POINTER(C.c_int)), ("val", C.POINTER(C.c_double)),
                ("nhalft", C.c_long), ("nskel", C.c_long), ("nfinal", C.c_long * 4),
                ("npq_done", C.c_long), ("nij_done", C.c_long), ("nij_total", C.c_long),
                ("t_first", C.c_double), ("t_second", C.c_double), ("t_pp", C.c_double),
                ("nijsiz", C.c_int), ("nc2", C.c_int)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_run.restype = C.c_int
        _lib.orc_inttyp.restype = C.c_int
        _lib.orc_gettw_factor.restype = C.c_double
        _lib.orc_gettw_factor.argtypes = [C.c_int]
    return _lib


@dataclasses.dataclass
class MdcintImage:
    """MDCINT contents: per record (IKR*IS, JKR*JS, NZ) + entries."""
    hdr: np.ndarray      # (nrec, 3) int32
    idx: np.ndarray      # (nz, 2) int32
    val: np.ndarray      # (nz,) complex128
    nhalft: int = 0
    nskel: int = 0
    nfinal: tuple = ()
    times: tuple = ()
    npq_done: int = 0
    nij_done: int = 0
    nij_total: int = 0


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def run(problem, thrgen=1e-16, throut=1e-16, nthreads=0, limit_pq=0, limit_ij=0,
        quater=True, records=None, pq_select=None, fake_list_len=0, breit=False) -> MdcintImage:
    """The oracle's MDCINT (or, with breit, MDBINT) stream of a problem."""
    lib = _load()
    cls, its, nts, v, l2, l1 = problem.flat_records() if records is None else records
    qa = np.asfortranarray(problem.qa).astype(np.complex128)
    qa_flat = np.ascontiguousarray(qa.T).reshape(-1)  # column-major QA(p,i)
    sel = None if pq_select is None else np.ascontiguousarray(pq_select, np.int64)
    prm = _Params(problem.n, problem.nsc1, problem.m, problem.nkr, problem.mfil,
                  1 if quater else 0, thrgen, throut, nthreads, limit_pq, limit_ij,
                  None if sel is None else _ptr(sel, C.c_long),
                  0 if sel is None else sel.size, fake_list_len, 1 if breit else 0)
    res = _Result()
    itrmo = np.ascontiguousarray(problem.itrmo, np.int32)
    kra = np.ascontiguousarray(problem.kra, np.int32)
    krb = np.ascontiguousarray(problem.krb, np.int32)
    ikrmo = np.ascontiguousarray(problem.ikrmo, np.int32)
    rc = lib.orc_run(C.byref(prm), qa_flat.ctypes.data_as(C.POINTER(C.c_double)),
                     _ptr(itrmo, C.c_int), _ptr(kra, C.c_int), _ptr(krb, C.c_int),
                     _ptr(ikrmo, C.c_int), C.c_long(cls.size), _ptr(cls, C.c_int),
                     _ptr(its, C.c_int), _ptr(nts, C.c_long), _ptr(v, C.c_double),
                     _ptr(l2, C.c_int), _ptr(l1, C.c_int), C.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle failed with status {rc}")
    try:
        hdr = np.ctypeslib.as_array(res.hdr, shape=(res.nrec * 3,)).reshape(-1, 3).copy() \
            if res.nrec else np.zeros((0, 3), np.int32)
        if res.nz_total:
            idx = np.ctypeslib.as_array(res.idx, shape=(res.nz_total * 2,)).reshape(-1, 2).copy()
            vv = np.ctypeslib.as_array(res.val, shape=(res.nz_total * 2,)).copy()
        else:
            idx = np.zeros((0, 2), np.int32)
            vv = np.zeros(0)
        img = MdcintImage(hdr, idx, vv[0::2] + 1j * vv[1::2], res.nhalft, res.nskel,
                          tuple(res.nfinal), (res.t_first, res.t_second, res.t_pp),
                          res.npq_done, res.nij_done, res.nij_total)
    finally:
        lib.orc_free(C.byref(res))
    return img


def fock_skeleton(records, nsc, dens, mfil=3):
    """tmoone's skeleton Fock sets (MFDFOCK/FOCK) of flat records
    ``(cls, its, nts, v, l2, l1)``; ``dens`` is (nmat, 4, nsc(nsc+1)/2) in the
    order AAR, BAR, AAI, BAI.  Returns the Fock sets in the same shape."""
    lib = _load()
    cls, its, l2, l1 = (np.ascontiguousarray(x, np.int32) for x in
                        (records[0], records[1], records[4], records[5]))
    nts = np.ascontiguousarray(records[2], np.int64)
    v = np.ascontiguousarray(records[3], np.float64)
    d = np.ascontiguousarray(dens, np.float64)
    assert d.ndim == 3 and d.shape[1] == 4 and d.shape[2] == nsc * (nsc + 1) // 2
    f = np.empty_like(d)
    rc = lib.orc_fock_skeleton(C.c_long(cls.size), _ptr(cls, C.c_int), _ptr(its, C.c_int),
                               _ptr(nts, C.c_long), _ptr(v, C.c_double), _ptr(l2, C.c_int),
                               _ptr(l1, C.c_int), mfil, nsc, d.shape[0], _ptr(d, C.c_double),
                               _ptr(f, C.c_double))
    if rc != 0:
        raise ValueError("integral label outside 1..NSC")
    return f


def fock_gaunt(records, nsc, dens, fock=None):
    """tmoone's Gaunt contributions (MFDBREIT/GAUNT) of the file-4 records,
    added to ``fock`` (a copy; zero when None) as MFDBREIT does after MFDFOCK."""
    lib = _load()
    cls, its, l2, l1 = (np.ascontiguousarray(x, np.int32) for x in
                        (records[0], records[1], records[4], records[5]))
    nts = np.ascontiguousarray(records[2], np.int64)
    v = np.ascontiguousarray(records[3], np.float64)
    d = np.ascontiguousarray(dens, np.float64)
    assert d.ndim == 3 and d.shape[1] == 4 and d.shape[2] == nsc * (nsc + 1) // 2
    f = np.zeros_like(d) if fock is None else np.array(fock, np.float64, copy=True, order="C")
    rc = lib.orc_fock_gaunt(C.c_long(cls.size), _ptr(cls, C.c_int), _ptr(its, C.c_int),
                            _ptr(nts, C.c_long), _ptr(v, C.c_double), _ptr(l2, C.c_int),
                            _ptr(l1, C.c_int), nsc, d.shape[0], 0 if fock is None else 1,
                            _ptr(d, C.c_double), _ptr(f, C.c_double))
    if rc == 1:
        raise ValueError("integral label outside 1..NSC")
    if rc == 2:
        raise ValueError("invalid integral type for GAUNT")
    return f


def inttyp(a, b, c, d):
    return _load().orc_inttyp(a, b, c, d)


def gettw_factor(it):
    return _load().orc_gettw_factor(it)


def time_sample(problem, seconds=15.0, nthreads=0, steps=1, warmup=0):
    """Time the restatement on a bounded sample of a (large) workload.

    TRANS1 runs over pq blocks spread evenly over the transformed blocks
    (their integral buckets generated on the host), TRANS2 over the first
    items with half-transformed lists of the full length (one entry per
    transformed pq block).  The two halves are timed separately and each is
    scaled by its own share of the full transform,

        T = t1 * P / n_pq + t2 * K(K+1) / n_items,

    so the estimate does not depend on how the sample mixes the two.  The
    sample is sized to take about ``seconds``.  Returns the algorithmic
    TFLOP/s of the full transform (same per-block and per-item FLOP counts as
    the GPU library) over T, and a description.
    """
    from molfdir_gb300 import synth
    model = problem.model
    nl, ns, n, m, k = model.n_l, model.n_s, problem.n, problem.m, problem.nkr
    pairs = [(p, q) for p in range(1, n + 1) for q in range(1, p + 1)
             if (p <= nl) == (q <= nl) and (p <= nl or problem.mfil >= 3)]
    P = len(pairs)
    items = k * (k + 1)
    blk = nl * nl + ns * ns
    f_pq = 4.0 * blk * m + 8.0 * n * m * m
    f_it = 8.0 * blk * m + 8.0 * n * m * m
    flops_full = P * f_pq + items * f_it

    def sample_run(npq, nit):
        idx = np.linspace(0, P - 1, npq).round().astype(int)
        sel_pairs = [pairs[i] for i in idx]
        recs = synth.bucket_records(model, sel_pairs, problem.mfil)
        sel = [p * (p - 1) // 2 + q for p, q in sel_pairs]
        return recs, sel

    # calibration: grow each half to about a third of the budget
    npq, nit = 8, 4
    for attempt in range(3):
        recs, sel = sample_run(npq, nit)
        img = run(problem, nthreads=nthreads, records=recs, pq_select=sel, limit_ij=nit,
                  fake_list_len=P)
        t1, t2 = img.times[0], img.times[1]
        if attempt == 2 or (t1 > 0.25 * seconds and t2 > 0.25 * seconds):
            break
        npq = min(P, max(npq, int(npq * seconds / 3 / max(t1, 1e-3))))
        nit = min(items, max(nit, int(nit * seconds / 3 / max(t2, 1e-3))))
    t1s, t2s = [], []
    for s_ in range(warmup + steps):
        img = run(problem, nthreads=nthreads, records=recs, pq_select=sel, limit_ij=nit,
                  fake_list_len=P)
        if s_ >= warmup:
            t1s.append(img.times[0])
            t2s.append(img.times[1])
    t1, t2 = float(np.mean(t1s)), float(np.mean(t2s))
    T = t1 * P / img.npq_done + t2 * items / img.nij_done
    return {"tflops": flops_full / T / 1e12, "ms_per_step": T * 1e3,
            "seconds_first_half": t1 * P / img.npq_done,
            "seconds_second_half": t2 * items / img.nij_done,
            "sample": (f"TRANS1 over {img.npq_done} of {P} pq blocks (evenly spaced) in {t1:.2f} s "
                       f"and TRANS2 over {img.nij_done} of {items} Kramers pairs with full-length "
                       f"half-transformed lists in {t2:.2f} s, each half scaled by its own "
                       f"fraction; full-transform algorithmic FLOPs {flops_full:.3e}")}
