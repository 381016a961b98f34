"""ctypes binding of the CPU oracle (test infrastructure only).

Imported by the tests, by the smoke check and by bench.py's CPU-baseline
leg; never by the product package.  ``build()`` compiles
``oracle/rotran_oracle.c`` into ``oracle/_build/liborotran.so``.
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
    src = os.path.join(HERE, "rotran_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-std=c11", "-shared",
                               "-o", LIB, src, "-lm"], cwd=HERE)
    return LIB


class _Params(C.Structure):
    _fields_ = [("nsc", C.c_int), ("nsc1", C.c_int), ("nsp", C.c_int), ("nkr", C.c_int),
                ("mfil", C.c_int), ("quater", C.c_int), ("thrgen", C.c_double),
                ("throut", C.c_double), ("nthreads", C.c_int), ("limit_pq", C.c_long),
                ("limit_ij", C.c_long)]


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
        quater=True) -> MdcintImage:
    lib = _load()
    cls, its, nts, v, l2, l1 = problem.flat_records()
    qa = np.asfortranarray(problem.qa).astype(np.complex128)
    qa_flat = np.ascontiguousarray(qa.T).reshape(-1)  # column-major QA(p,i)
    prm = _Params(problem.n, problem.nsc1, problem.m, problem.nkr, problem.mfil,
                  1 if quater else 0, thrgen, throut, nthreads, limit_pq, limit_ij)
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


def inttyp(a, b, c, d):
    return _load().orc_inttyp(a, b, c, d)


def gettw_factor(it):
    return _load().orc_gettw_factor(it)
