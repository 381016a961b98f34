"""Python mirror of the rotran drop-in C-ABI (``include/rotran_gb300.h``).

``Rotran`` wraps one library context: the calls a rotran driver makes in
place of SR2INI/SORT1/TRANS1/SR2FLSH/TRANS2/INITTWOE/PPSYM/EXITTWOE
(``source/rotran/rotran.F:236-333``).  Errors are raised as ``RotranError``
carrying the Q2JOB class of the failure (``source/general/q2job.F:8-23``).
The library has no CPU path: loading it or creating a context without a
usable sm_103a device raises.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

RT_PREC_FP64 = 0
RT_PREC_SPLIT_BF16 = 1
RT_ERR_EOF, RT_ERR_USER, RT_ERR_DIM = 1, 2, 3
RT_ERR_PROGRAM = 6

ERROR_CLASSES = {
    1: "end of file / missing data",
    2: "user error (inconsistent input)",
    3: "dimension bound exceeded",
    4: "internal dimension error",
    5: "non-matching parameters",
    6: "program error",
}


class RotranError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[Q2JOB class {code}: {ERROR_CLASSES.get(code, '?')}] {msg}")
        self.code = code


class RtBatchStats(C.Structure):
    _fields_ = [("instances", C.c_int), ("grouped_launches", C.c_int),
                ("kernel_launches", C.c_int), ("graph_nodes", C.c_int), ("tile128", C.c_int),
                ("tile64", C.c_int), ("ms_last", C.c_double), ("ms_tune", C.c_double),
                ("flops_algorithmic", C.c_double), ("flops_gemm_executed", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class RtConfig(C.Structure):
    _fields_ = [("nsc", C.c_int), ("nsc1", C.c_int), ("nsp", C.c_int), ("nkr", C.c_int),
                ("mfil", C.c_int), ("breit", C.c_int), ("thrgen", C.c_double),
                ("throut", C.c_double), ("precision", C.c_int), ("slices", C.c_int),
                ("n_irrep", C.c_int), ("ao_irrep", C.POINTER(C.c_int)),
                ("mem_budget", C.c_longlong), ("half_buckets", C.c_int)]


class RtStats(C.Structure):
    _fields_ = [("nhalft", C.c_longlong), ("nfinal", C.c_longlong * 4),
                ("nrec", C.c_longlong * 4), ("ms_upload", C.c_double),
                ("ms_scatter", C.c_double), ("ms_first", C.c_double),
                ("ms_second", C.c_double), ("ms_output", C.c_double),
                ("ms_total", C.c_double), ("flops_algorithmic", C.c_double),
                ("device_bytes", C.c_longlong), ("gpu_launches", C.c_int),
                ("gemm_launches", C.c_int), ("ms_gemm", C.c_double),
                ("flops_gemm_executed", C.c_double), ("flops_gemm_algorithmic", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["nfinal"] = list(self.nfinal)
        d["nrec"] = list(self.nrec)
        return d


class RtPlanInfo(C.Structure):
    _fields_ = [("npairs", C.c_longlong), ("nitems", C.c_longlong),
                ("expand_bytes_per_pair", C.c_longlong), ("hp_bytes", C.c_longlong),
                ("nrec", C.c_longlong * 4), ("elem_cap", C.c_longlong * 4),
                ("flops_algorithmic", C.c_double)]


EXPORTS = ["rt_plan", "rt_create", "rt_set_coefficients", "rt_add_ao_records",
           "rt_add_ao_records_bulk", "rt_read_srt_files", "rt_clear_ao_records",
           "rt_transform", "rt_result_sizes", "rt_copy_result", "rt_write_mdcint",
           "rt_get_stats", "rt_last_error", "rt_destroy", "rt_kramers_check", "rt_split_dgemm",
           "rt_split_dgemm_noalloc", "rt_adjoint", "rt_batch_create", "rt_batch_run",
           "rt_batch_get_stats", "rt_batch_last_error", "rt_batch_destroy", "rt_srtpq_scan",
           "rt_read_srtpq_files", "rt_set_result_host", "rt_fock_skeleton", "rt_fock_gaunt",
           "rt_queue_ao_records_bulk", "rt_set_result_host_deferred", "rt_result_host_wait"]

_lib = None


def load(build: bool = True):
    """Load (building first if needed) the in-tree shared library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the sm_103a library first")
    lib = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    lib.rt_plan.argtypes = [P(RtConfig), P(RtPlanInfo)]
    lib.rt_create.argtypes = [P(vp), P(RtConfig)]
    lib.rt_set_coefficients.argtypes = [vp, P(C.c_double), C.c_int, P(C.c_int), P(C.c_int),
                                        P(C.c_int), P(C.c_int), P(C.c_int)]
    lib.rt_add_ao_records.argtypes = [vp, C.c_int, C.c_int, C.c_int, P(C.c_double),
                                      P(C.c_int), P(C.c_int)]
    lib.rt_add_ao_records_bulk.argtypes = [vp, C.c_longlong, P(C.c_int), P(C.c_longlong),
                                           P(C.c_int), P(C.c_double), P(C.c_int), P(C.c_int)]
    lib.rt_read_srt_files.argtypes = [vp, C.c_char_p]
    lib.rt_clear_ao_records.argtypes = [vp]
    lib.rt_transform.argtypes = [vp]
    lib.rt_result_sizes.argtypes = [vp, P(C.c_longlong), P(C.c_longlong)]
    lib.rt_copy_result.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_double)]
    lib.rt_write_mdcint.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p]
    lib.rt_get_stats.argtypes = [vp, P(RtStats)]
    lib.rt_last_error.argtypes = [vp]
    lib.rt_last_error.restype = C.c_char_p
    lib.rt_destroy.argtypes = [vp]
    lib.rt_destroy.restype = None
    lib.rt_kramers_check.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_double), C.c_int,
                                     P(C.c_int), P(C.c_double)]
    lib.rt_split_dgemm.argtypes = [C.c_int, C.c_int, C.c_int, P(C.c_double), P(C.c_double),
                                   P(C.c_double), C.c_int, C.c_int]
    lib.rt_split_dgemm_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int, vp]
    lib.rt_adjoint.argtypes = [vp, vp, vp, P(C.c_double)]
    lib.rt_batch_create.argtypes = [P(vp), P(vp), C.c_int]
    lib.rt_batch_run.argtypes = [vp]
    lib.rt_batch_get_stats.argtypes = [vp, P(RtBatchStats)]
    lib.rt_batch_last_error.argtypes = [vp]
    lib.rt_batch_last_error.restype = C.c_char_p
    lib.rt_batch_destroy.argtypes = [vp]
    lib.rt_batch_destroy.restype = None
    lib.rt_srtpq_scan.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_longlong,
                                  P(C.c_longlong), P(C.c_longlong), P(C.c_int), P(C.c_int),
                                  P(C.c_longlong), P(C.c_double), P(C.c_int), P(C.c_int)]
    lib.rt_read_srtpq_files.argtypes = [vp, C.c_char_p, C.c_int]
    lib.rt_set_result_host.argtypes = [vp, P(P(C.c_int)), P(P(C.c_double)), P(C.c_longlong)]
    lib.rt_fock_skeleton.argtypes = [vp, C.c_int, vp, vp, P(C.c_double)]
    lib.rt_fock_gaunt.argtypes = [vp, C.c_int, vp, vp, C.c_int, P(C.c_double)]
    lib.rt_queue_ao_records_bulk.argtypes = lib.rt_add_ao_records_bulk.argtypes
    lib.rt_set_result_host_deferred.argtypes = [vp, C.c_int]
    lib.rt_result_host_wait.argtypes = [vp]
    for name in EXPORTS:
        f = getattr(lib, name)
        if name not in ("rt_last_error", "rt_destroy", "rt_batch_last_error", "rt_batch_destroy"):
            f.restype = C.c_int
    _lib = lib
    return lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def make_config(nsc, nsc1, nkr, mfil=3, thrgen=1e-16, throut=1e-16,
                precision=RT_PREC_FP64, slices=0, ao_irrep=None, mem_budget=0, breit=False,
                half_buckets=False):
    """``breit``: the Gaunt transform of file 4 into MDBINT (BREIT in rotran's
    namelist) instead of the Coulomb transform of files 1..MFIL.
    ``half_buckets``: rotran's own half-transformed intermediate (each
    integral under its LABEL1 pair; THRGEN and NHALFT exactly rotran's)."""
    cfg = RtConfig(nsc, nsc1, 2 * nkr, nkr, mfil, 1 if breit else 0, thrgen, throut, precision,
                   slices, 1, None, mem_budget, 1 if half_buckets else 0)
    keep = None
    if ao_irrep is not None and int(np.max(ao_irrep)) > 0:
        keep = np.ascontiguousarray(ao_irrep, dtype=np.int32)
        cfg.n_irrep = 4
        cfg.ao_irrep = _p(keep, C.c_int)
    return cfg, keep


def plan(cfg: RtConfig) -> RtPlanInfo:
    lib = load()
    out = RtPlanInfo()
    rc = lib.rt_plan(C.byref(cfg), C.byref(out))
    if rc:
        raise RotranError(rc, lib.rt_last_error(None).decode())
    return out


def kramers_check(qa: np.ndarray, qb: np.ndarray):
    """KRAMERS pairing (kramers.F:26-131): returns (ITRMO, max deviation)."""
    lib = load()
    n, m = qa.shape
    a = np.asfortranarray(qa, dtype=np.complex128)
    b = np.asfortranarray(qb, dtype=np.complex128)
    itrmo = np.zeros(m, dtype=np.int32)
    dif = C.c_double(0.0)
    rc = lib.rt_kramers_check(n, m, a.ctypes.data_as(C.POINTER(C.c_double)),
                              b.ctypes.data_as(C.POINTER(C.c_double)), n,
                              _p(itrmo, C.c_int), C.byref(dif))
    if rc:
        raise RotranError(rc, "VECTORS SHOULD BE TRUE KRAMERS PAIRS / MOS WITHOUT KRAMERS PARTNER")
    return itrmo, dif.value


class Rotran:
    """One transformation context on the current CUDA device."""

    def __init__(self, cfg: RtConfig, _keep=None):
        self.lib = load()
        self._keep = _keep
        self.cfg = cfg
        h = C.c_void_p()
        rc = self.lib.rt_create(C.byref(h), C.byref(cfg))
        if rc:
            raise RotranError(rc, self.lib.rt_last_error(None).decode())
        self.h = h

    @classmethod
    def for_problem(cls, problem, **kw):
        """A context for a synthetic problem; ``breit=True`` transforms its
        Gaunt file instead of the Coulomb files."""
        cfg, keep = make_config(problem.n, problem.nsc1, problem.nkr, mfil=problem.mfil,
                                ao_irrep=problem.model.irrep if problem.model.n_irrep > 1 else None,
                                **kw)
        return cls(cfg, keep)

    def _check(self, rc):
        if rc:
            raise RotranError(rc, self.lib.rt_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.rt_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- inputs ---------------------------------------------------------------
    def set_coefficients(self, qa, itrmo, kra, krb, ikrmo, imoras_pairs=None):
        a = np.asfortranarray(qa, dtype=np.complex128)
        it = np.ascontiguousarray(itrmo, np.int32)
        ka = np.ascontiguousarray(kra, np.int32)
        kb = np.ascontiguousarray(krb, np.int32)
        ik = np.ascontiguousarray(ikrmo, np.int32)
        im = None if imoras_pairs is None else np.ascontiguousarray(imoras_pairs, np.int32)
        self._check(self.lib.rt_set_coefficients(
            self.h, a.ctypes.data_as(C.POINTER(C.c_double)), a.shape[0], _p(it, C.c_int),
            _p(ka, C.c_int), _p(kb, C.c_int), _p(ik, C.c_int),
            None if im is None else _p(im, C.c_int)))

    def set_problem_coefficients(self, problem):
        self.set_coefficients(problem.qa, problem.itrmo, problem.kra, problem.krb,
                              problem.ikrmo, problem.imoras_pairs())

    def add_record(self, file_class, itype, rint, label2, label1):
        v = np.ascontiguousarray(rint, np.float64)
        a = np.ascontiguousarray(label2, np.int32)
        b = np.ascontiguousarray(label1, np.int32)
        self._check(self.lib.rt_add_ao_records(self.h, int(file_class), int(v.size), int(itype),
                                               _p(v, C.c_double), _p(a, C.c_int), _p(b, C.c_int)))

    def add_records_bulk(self, file_class, nt, itype, rint, label2, label1):
        fc = np.ascontiguousarray(file_class, np.int32)
        n = np.ascontiguousarray(nt, np.int64)
        it = np.ascontiguousarray(itype, np.int32)
        v = np.ascontiguousarray(rint, np.float64)
        a = np.ascontiguousarray(label2, np.int32)
        b = np.ascontiguousarray(label1, np.int32)
        self._check(self.lib.rt_add_ao_records_bulk(
            self.h, int(fc.size), _p(fc, C.c_int), _p(n, C.c_longlong), _p(it, C.c_int),
            _p(v, C.c_double), _p(a, C.c_int), _p(b, C.c_int)))

    def add_records_bulk_ptr(self, file_class, nt, itype, p_rint, p_label2, p_label1):
        """Bulk records from raw host or device pointers (cudaMemcpyDefault)."""
        fc = np.ascontiguousarray(file_class, np.int32)
        n = np.ascontiguousarray(nt, np.int64)
        it = np.ascontiguousarray(itype, np.int32)
        self._check(self.lib.rt_add_ao_records_bulk(
            self.h, int(fc.size), _p(fc, C.c_int), _p(n, C.c_longlong), _p(it, C.c_int),
            C.cast(C.c_void_p(p_rint), C.POINTER(C.c_double)),
            C.cast(C.c_void_p(p_label2), C.POINTER(C.c_int)),
            C.cast(C.c_void_p(p_label1), C.POINTER(C.c_int))))

    def queue_records_bulk_ptr(self, file_class, nt, itype, p_rint, p_label2, p_label1):
        """Queue the next record set (``rt_queue_ao_records_bulk``): its copies
        overlap the next ``transform()``, after which it is the context's
        records.  The arrays behind the pointers must stay alive until then."""
        fc = np.ascontiguousarray(file_class, np.int32)
        n = np.ascontiguousarray(nt, np.int64)
        it = np.ascontiguousarray(itype, np.int32)
        self._check(self.lib.rt_queue_ao_records_bulk(
            self.h, int(fc.size), _p(fc, C.c_int), _p(n, C.c_longlong), _p(it, C.c_int),
            C.cast(C.c_void_p(p_rint), C.POINTER(C.c_double)),
            C.cast(C.c_void_p(p_label2), C.POINTER(C.c_int)),
            C.cast(C.c_void_p(p_label1), C.POINTER(C.c_int))))

    def add_records_bulk_device(self, file_class, nt, itype, rint, label2, label1):
        """Bulk records held in torch tensors (device or host)."""
        self.add_records_bulk_ptr(file_class, nt, itype, rint.data_ptr(), label2.data_ptr(),
                                  label1.data_ptr())

    def add_problem_records(self, problem, bulk=True):
        if bulk:
            cls, its, nts, v, l2, l1 = problem.flat_records()
            self.add_records_bulk(cls, nts, its, v, l2, l1)
        else:
            for cls, r in problem.all_records():
                self.add_record(cls, r.it, r.rint, r.label2, r.label1)

    def read_srt_files(self, directory):
        self._check(self.lib.rt_read_srt_files(self.h, os.fsencode(directory)))

    def read_srtpq_files(self, directory, nranks=1):
        """The MPI version's pq-sorted files SRTPQIL[.r]/SRTPQLN[.r], r < nranks."""
        self._check(self.lib.rt_read_srtpq_files(self.h, os.fsencode(directory), nranks))

    def clear_records(self):
        self._check(self.lib.rt_clear_ao_records(self.h))

    # -- run ------------------------------------------------------------------
    def transform(self):
        self._check(self.lib.rt_transform(self.h))

    def result_sizes(self):
        nr, nz = C.c_longlong(), C.c_longlong()
        self._check(self.lib.rt_result_sizes(self.h, C.byref(nr), C.byref(nz)))
        return nr.value, nz.value

    def result(self, hdr=None, idx=None, val=None):
        """MDCINT record stream: (hdr (nrec,3), idx (nz,2), val (nz,) complex)."""
        nr, nz = self.result_sizes()
        hdr = np.empty((nr, 3), np.int32) if hdr is None else hdr
        idx = np.empty((nz, 2), np.int32) if idx is None else idx
        val = np.empty(nz, np.complex128) if val is None else val
        self._check(self.lib.rt_copy_result(self.h, _p(hdr, C.c_int), _p(idx, C.c_int),
                                            val.ctypes.data_as(C.POINTER(C.c_double))))
        return hdr, idx, val

    def fock_skeleton(self, dens, out=None):
        """tmoone's skeleton Fock sets from the context's records (``rt_fock_skeleton``).

        ``dens``: float64 array (nmat, 4, NSC(NSC+1)/2), sets of DAAR, DBAR, DAAI,
        DBAI (numpy, or a torch tensor on the host or the device).  Returns the
        Fock sets in the same shape and kind (``out`` if given) and the kernel's
        device milliseconds."""
        nmat = dens.shape[0]
        if out is None:
            out = dens.new_empty(dens.shape) if hasattr(dens, "data_ptr") else np.empty_like(dens)
        pd = dens.data_ptr() if hasattr(dens, "data_ptr") else dens.ctypes.data
        pf = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        ms = C.c_double()
        self._check(self.lib.rt_fock_skeleton(self.h, nmat, C.c_void_p(pd), C.c_void_p(pf), C.byref(ms)))
        return out, ms.value

    def fock_gaunt(self, dens, fock=None):
        """tmoone's Gaunt contributions from the context's file-4 records
        (``rt_fock_gaunt``), added to ``fock`` (modified in place; as MFDBREIT
        after MFDFOCK) or, with ``fock`` None, into new zeroed sets.  Returns
        the sets and the kernel's device milliseconds."""
        acc = fock is not None
        if fock is None:
            fock = dens.new_empty(dens.shape) if hasattr(dens, "data_ptr") else np.empty_like(dens)
        pd = dens.data_ptr() if hasattr(dens, "data_ptr") else dens.ctypes.data
        pf = fock.data_ptr() if hasattr(fock, "data_ptr") else fock.ctypes.data
        ms = C.c_double()
        self._check(self.lib.rt_fock_gaunt(self.h, dens.shape[0], C.c_void_p(pd), C.c_void_p(pf),
                                           1 if acc else 0, C.byref(ms)))
        return fock, ms.value

    def headers(self):
        """The MDCINT record headers (nrec, 3) alone (``rt_copy_result`` with no element buffers)."""
        nr, _ = self.result_sizes()
        hdr = np.empty((nr, 3), np.int32)
        self._check(self.lib.rt_copy_result(self.h, _p(hdr, C.c_int), None, None))
        return hdr

    def set_result_host(self, idx=None, val=None):
        """Stream the following transforms' elements into host arrays (``rt_set_result_host``).

        ``idx[c]``: int32 array of shape (cap_c, 2), ``val[c]``: complex128 array of
        shape (cap_c,) for record class c = 0..3, C-contiguous; pinned memory (for
        instance numpy views of pinned torch tensors) lets the copies overlap the
        transform.  Class c's elements land in ``idx[c][:n_c]``, ``val[c][:n_c]``
        with n_c = ``stats().nfinal[c]``.  No arguments unregisters.  The arrays
        must stay alive while registered."""
        if idx is None or val is None:
            self._host = None
            self._check(self.lib.rt_set_result_host(self.h, None, None, None))
            return
        assert len(idx) == 4 and len(val) == 4
        caps = []
        for a, v in zip(idx, val):
            assert a.dtype == np.int32 and a.ndim == 2 and a.shape[1] == 2 and a.flags.c_contiguous
            assert v.dtype == np.complex128 and v.ndim == 1 and v.flags.c_contiguous
            caps.append(min(a.shape[0], v.shape[0]))
        ip = (C.POINTER(C.c_int) * 4)(*[_p(a, C.c_int) for a in idx])
        dp = (C.POINTER(C.c_double) * 4)(*[v.ctypes.data_as(C.POINTER(C.c_double)) for v in val])
        cp = (C.c_longlong * 4)(*caps)
        self._host = (list(idx), list(val))
        self._check(self.lib.rt_set_result_host(self.h, ip, dp, cp))

    def set_result_host_deferred(self, deferred=True):
        """``rt_set_result_host_deferred``: transform() returns before its last
        host copies land; ``result_host_wait()`` (or any result read) completes them."""
        self._check(self.lib.rt_set_result_host_deferred(self.h, 1 if deferred else 0))

    def result_host_wait(self):
        self._check(self.lib.rt_result_host_wait(self.h))

    def write_mdcint(self, path, datex="", timex=""):
        self._check(self.lib.rt_write_mdcint(self.h, os.fsencode(path), datex.encode()[:10],
                                             timex.encode()[:8]))

    def adjoint(self, gamma):
        """dE/dC and E for E = sum gamma[i,j,k,l] (ij|kl) (``rt_adjoint``).

        ``gamma``: complex (m, m, m, m) numpy array indexed [i, j, k, l], or
        the device address of an NSP^4 COMPLEX*16 array in Fortran order.
        Returns (dEdC as a complex (n, m) array, E)."""
        n, m = self.cfg.nsc, self.cfg.nsp
        if isinstance(gamma, np.ndarray):
            g = np.asfortranarray(gamma, dtype=np.complex128)
            assert g.shape == (m, m, m, m)
            gp = g.ctypes.data
        else:
            g, gp = None, int(gamma)
        out = np.empty((m, n), dtype=np.complex128)  # Fortran (n, m)
        e = C.c_double()
        self._check(self.lib.rt_adjoint(self.h, C.c_void_p(gp), C.c_void_p(out.ctypes.data),
                                         C.byref(e)))
        return out.T.copy(), e.value

    def stats(self):
        s = RtStats()
        self._check(self.lib.rt_get_stats(self.h, C.byref(s)))
        return s


def srtpq_scan(directory, nranks: int, nsc: int, nsc1: int):
    """Parse SRTPQIL[.r]/SRTPQLN[.r] (r < nranks) without a context or GPU.

    Returns ``(file_class, itype, nt, rint, label2, label1)``: one record
    per (file class, integral type), the integrals as ``rt_add_ao_records``
    takes them (label1 = the stream's pq pair, label2 = the entry's label).
    """
    lib = load()
    nrec, nint = C.c_longlong(), C.c_longlong()
    d = os.fsencode(directory)
    rc = lib.rt_srtpq_scan(d, nranks, nsc, nsc1, 0, C.byref(nrec), C.byref(nint),
                           None, None, None, None, None, None)
    if rc == 0 and nint.value == 0:
        z = np.zeros(0)
        return (z.astype(np.int32), z.astype(np.int32), z.astype(np.int64), z,
                z.astype(np.int32), z.astype(np.int32))
    if rc not in (0, RT_ERR_DIM):
        raise RotranError(rc, lib.rt_last_error(None).decode(errors="replace"))
    nr, ni = nrec.value, nint.value
    cls = np.empty(nr, np.int32)
    its = np.empty(nr, np.int32)
    nts = np.empty(nr, np.int64)
    v = np.empty(ni, np.float64)
    l2 = np.empty(ni, np.int32)
    l1 = np.empty(ni, np.int32)
    rc = lib.rt_srtpq_scan(d, nranks, nsc, nsc1, ni, C.byref(nrec), C.byref(nint),
                           _p(cls, C.c_int), _p(its, C.c_int), _p(nts, C.c_longlong),
                           _p(v, C.c_double), _p(l2, C.c_int), _p(l1, C.c_int))
    if rc:
        raise RotranError(rc, lib.rt_last_error(None).decode(errors="replace"))
    return cls, its, nts, v, l2, l1


def split_dgemm(a: np.ndarray, b: np.ndarray, slices: int = 5, mode: int = 0) -> np.ndarray:
    """C = A B through the split-precision tensor-core engine (``rt_split_dgemm``)."""
    lib = load()
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    m, k = a.shape
    k2, n = b.shape
    assert k == k2
    c = np.empty((m, n), np.float64)
    rc = lib.rt_split_dgemm(m, n, k, _p(a, C.c_double), _p(b, C.c_double), _p(c, C.c_double),
                            slices, mode)
    if rc:
        raise RotranError(rc, "rt_split_dgemm failed")
    return c


def split_dgemm_noalloc(m: int, n: int, k: int, a_ptr: int, b_ptr: int, c_ptr: int,
                        slices: int = 6, stream: int = 0) -> None:
    """C = A B on device-resident row-major FP64 matrices through
    ``rt_split_dgemm_noalloc`` (no device allocation; fixed scratch array).
    Pointers and the stream are raw addresses (e.g. ``tensor.data_ptr()``,
    ``torch.cuda.current_stream().cuda_stream``)."""
    lib = load()
    rc = lib.rt_split_dgemm_noalloc(m, n, k, C.c_void_p(a_ptr), C.c_void_p(b_ptr),
                                    C.c_void_p(c_ptr), slices, C.c_void_p(stream or None))
    if rc:
        raise RotranError(rc, lib.rt_last_error(None).decode())


class Batch:
    """Batched transforms of several split-precision contexts (``rt_batch_*``):
    one grouped GEMM launch per stage, captured as a CUDA graph on the first
    ``run()`` (after tuning the tile width per stage) and replayed after.
    Close the batch before closing any of its contexts."""

    def __init__(self, rts):
        self.lib = load()
        self.rts = list(rts)  # keep the contexts alive
        arr = (C.c_void_p * len(self.rts))(*[r.h for r in self.rts])
        h = C.c_void_p()
        rc = self.lib.rt_batch_create(C.byref(h), arr, len(self.rts))
        if rc:
            raise RotranError(rc, self.lib.rt_last_error(None).decode())
        self.h = h

    def run(self):
        rc = self.lib.rt_batch_run(self.h)
        if rc:
            raise RotranError(rc, self.lib.rt_batch_last_error(self.h).decode())

    def stats(self) -> RtBatchStats:
        s = RtBatchStats()
        rc = self.lib.rt_batch_get_stats(self.h, C.byref(s))
        if rc:
            raise RotranError(rc, "rt_batch_get_stats failed")
        return s

    def close(self):
        if getattr(self, "h", None):
            self.lib.rt_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
