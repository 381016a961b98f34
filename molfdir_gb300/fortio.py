"""gfortran sequential unformatted files of the rotran interface.

Records are framed by 4-byte little-endian length markers (negative
markers continue a record in sub-records).  Layouts follow the reference:

* SRTTW record: ``NT, IT, FINISH, RINT(NT)`` (``source/reltwel/wrbuf.F:38-39``)
* SRTLB record (32-bit labels): ``NT, IT, FINISH, LABEL(NT), LABEL1(NT)``
  (``source/reltwel/wrbuf.F:44-45``)
* MDCINT: header ``DATEX(c10), TIMEX(c8), NKR, (KR(i), KR(-i)) * NKR``
  (``source/rotran/inittwoe.F:139-141``), records
  ``IKR, JKR, NZ, (INDK, INDL) * NZ, (complex) * NZ``
  (``source/rotran/ppsym.F:89-91``), terminator ``0, 0, 0``
  (``source/rotran/exittwoe.F:149``), read as in
  ``source/goscip/rdtwo.F:17-28``.
"""

from __future__ import annotations

import os
import struct

import numpy as np

SRT_NAMES = {1: ("SRTTWLL", "SRTLBLL"), 2: ("SRTTWSL", "SRTLBSL"), 3: ("SRTTWSS", "SRTLBSS")}


def write_record(f, payload: bytes):
    n = len(payload)
    if n > 0x7FFFFFFF:
        raise ValueError("record too long for a single marker")
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def read_record(f):
    """Return the payload of the next record, or None at end of file."""
    out = bytearray()
    while True:
        head = f.read(4)
        if not head:
            if out:
                raise EOFError("truncated record")
            return None
        if len(head) < 4:
            raise EOFError("truncated record marker")
        (n,) = struct.unpack("<i", head)
        more = n < 0
        n = abs(n)
        data = f.read(n)
        if len(data) < n:
            raise EOFError("truncated record")
        out += data
        tail = f.read(4)
        if len(tail) < 4:
            raise EOFError("truncated record marker")
        if not more:
            return bytes(out)


def write_srt_files(problem, directory: str):
    """Write SRTTW*/SRTLB* files of a synthetic problem (files 1..MFIL)."""
    os.makedirs(directory, exist_ok=True)
    keys = {1: "LL", 2: "SL", 3: "SS"}
    for cls in range(1, problem.mfil + 1):
        tw, lb = SRT_NAMES[cls]
        recs = problem.files.get(keys[cls], [])
        with open(os.path.join(directory, tw), "wb") as fa, open(os.path.join(directory, lb), "wb") as fb:
            for r in recs:
                nt = r.rint.size
                head = struct.pack("<iii", nt, r.it, 1 if r.finish else 0)
                write_record(fa, head + np.asarray(r.rint, "<f8").tobytes())
                write_record(fb, head + np.asarray(r.label2, "<i4").tobytes()
                             + np.asarray(r.label1, "<i4").tobytes())


def read_mdcint(path: str):
    """Read an MDCINT file: (datex, timex, nkr, header pairs, hdr, idx, val)."""
    hdrs, idxs, vals = [], [], []
    with open(path, "rb") as f:
        h = read_record(f)
        datex = h[:10].decode("latin-1")
        timex = h[10:18].decode("latin-1")
        (nkr,) = struct.unpack_from("<i", h, 18)
        pairs = np.frombuffer(h, "<i4", 2 * nkr, 22).copy()
        while True:
            r = read_record(f)
            if r is None:
                raise EOFError("MDCINT without terminator")
            ikr, jkr, nz = struct.unpack_from("<iii", r, 0)
            if ikr == 0:
                break
            if len(r) != 12 + 24 * nz:
                raise ValueError("malformed MDCINT record")
            hdrs.append((ikr, jkr, nz))
            idxs.append(np.frombuffer(r, "<i4", 2 * nz, 12).reshape(nz, 2))
            v = np.frombuffer(r, "<f8", 2 * nz, 12 + 8 * nz)
            vals.append(v[0::2] + 1j * v[1::2])
    hdr = np.asarray(hdrs, np.int32).reshape(-1, 3)
    idx = np.concatenate(idxs) if idxs else np.zeros((0, 2), np.int32)
    val = np.concatenate(vals) if vals else np.zeros(0, np.complex128)
    return datex, timex, nkr, pairs, hdr, idx, val
