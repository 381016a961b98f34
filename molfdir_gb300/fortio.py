"""gfortran files of the rotran interface.

Sequential unformatted records are framed by 4-byte little-endian length
markers (negative markers continue a record in sub-records); direct-access
records have a fixed length and no markers.  Layouts follow the reference:

* SRTTW record: ``NT, IT, FINISH, RINT(NT)`` (``source/reltwel/wrbuf.F:38-39``)
* SRTLB record (32-bit labels): ``NT, IT, FINISH, LABEL(NT), LABEL1(NT)``
  (``source/reltwel/wrbuf.F:44-45``)
* MDCINT: header ``DATEX(c10), TIMEX(c8), NKR, (KR(i), KR(-i)) * NKR``
  (``source/rotran/inittwoe.F:21-23``), records
  ``IKR, JKR, NZ, (INDK, INDL) * NZ, (complex) * NZ``
  (``source/rotran/ppsym.F:89-91``), terminator ``0, 0, 0``
  (``source/rotran/exittwoe.F:6``), read as in
  ``source/goscip/rdtwo.F:17-28``.
* SRTPQIL[.r] (direct access) and SRTPQLN[.r] (sequential) of the MPI
  integral program, read by the MPI rotran's GETPQ
  (``source/reltwel/mfdtwoe.par.F:344-352,919-926,1031-1033``,
  ``source/rotran/getpq.F:57-60``).
"""

from __future__ import annotations

import os
import struct

import numpy as np

SRT_NAMES = {1: ("SRTTWLL", "SRTLBLL"), 2: ("SRTTWSL", "SRTLBSL"), 3: ("SRTTWSS", "SRTLBSS"),
             4: ("SRTBREI", "SRTBREL")}  # reltwel/mfdata3.F:41-42


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
    """Write SRTTW*/SRTLB* files of a synthetic problem (files 1..MFIL), and
    SRTBREI/SRTBREL when it has Gaunt integrals."""
    os.makedirs(directory, exist_ok=True)
    keys = {1: "LL", 2: "SL", 3: "SS", 4: "BR"}
    classes = list(range(1, problem.mfil + 1)) + ([4] if "BR" in problem.files else [])
    for cls in classes:
        tw, lb = SRT_NAMES[cls]
        recs = problem.files.get(keys[cls], [])
        with open(os.path.join(directory, tw), "wb") as fa, open(os.path.join(directory, lb), "wb") as fb:
            for r in recs:
                nt = r.rint.size
                head = struct.pack("<iii", nt, r.it, 1 if r.finish else 0)
                write_record(fa, head + np.asarray(r.rint, "<f8").tobytes())
                write_record(fb, head + np.asarray(r.label2, "<i4").tobytes()
                             + np.asarray(r.label1, "<i4").tobytes())


def srtpq_name(base: str, rank: int) -> str:
    """File name of a rank (``source/reltwel/mfdtwoe.par.F:332-342``)."""
    return base if rank == 0 else f"{base}.{rank}"


def write_srtpq_files(problem, directory: str, nranks: int = 1, nbuf: int = 256,
                      split_every: int = 0, breit_pairs: int = 0, seed: int = 0):
    """Write a problem's integrals in the MPI format SRTPQIL[.r]/SRTPQLN[.r].

    Layout of ``source/reltwel/mfdtwoe.par.F`` (32-bit labels): every
    integral goes to the stream of its second pair (label1, the pq pair
    ``IPQL``) with ``LBUF = I<<16|K`` of its first pair; a stream's bucket
    is written as a direct-access record of ``IRECL = 12 + 12*nbuf`` bytes
    (``IPQL, NT, INXT, RBUF(NT), LBUF(NT)``, zero-padded) when it holds
    ``nbuf`` entries, ``INXT`` linking to the stream's previous record
    (:919-926), and the part-filled buckets are flushed in stream order at
    the end (:976-994).  The full records of different streams interleave
    in a seeded random order; streams are dealt to ranks round robin.

    ``split_every = k > 0`` writes every k-th integral as two entries of
    half the value (the generator's repeated entries, which GETPQ's reader
    sums); ``breit_pairs`` adds that many streams of SL pq pairs with random
    values, which a Coulomb reader must skip.
    """
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(seed)
    n, nl = problem.model.n, problem.model.n_l
    _, _, _, v, l2, l1 = problem.flat_records()
    if split_every > 0:
        sel = np.arange(0, v.size, split_every)
        v = v.copy()
        v[sel] *= 0.5
        v = np.concatenate([v, v[sel]])
        l2 = np.concatenate([l2, l2[sel]])
        l1 = np.concatenate([l1, l1[sel]])
    if breit_pairs and nl < n:
        bv, b2, b1 = [v], [l2], [l1]
        for _ in range(breit_pairs):
            p, q = int(rng.integers(nl + 1, n + 1)), int(rng.integers(1, nl + 1))
            k = int(rng.integers(1, 2 * nbuf + 2))
            r = rng.integers(nl + 1, n + 1, k)
            t = rng.integers(1, nl + 1, k)
            bv.append(rng.standard_normal(k))
            b2.append(((r << 16) | t).astype(np.int32))
            b1.append(np.full(k, (p << 16) | q, np.int32))
        v, l2, l1 = np.concatenate(bv), np.concatenate(b2), np.concatenate(b1)
    pqi = (l1 >> 16).astype(np.int64)
    pqi = pqi * (pqi - 1) // 2 + (l1 & 0xFFFF)
    order = np.argsort(pqi, kind="stable")
    v, l2, pqi = v[order], l2[order], pqi[order]
    streams, first, count = np.unique(pqi, return_index=True, return_counts=True)
    irecl = 12 + 12 * nbuf
    for rank in range(nranks):
        mine = np.arange(rank, streams.size, nranks)
        # records per stream: full ones, then the part-filled flush
        nfull = count[mine] // nbuf
        part = count[mine] % nbuf
        rs = np.repeat(mine, nfull)
        rc = np.concatenate([np.arange(c) for c in nfull]) if rs.size else np.zeros(0, np.int64)
        key = rc + rng.random(rs.size)  # increasing within a stream, interleaved across
        o = np.argsort(key, kind="stable")
        rs, rc = rs[o], rc[o]
        fl = mine[part > 0]
        rec_stream = np.concatenate([rs, fl]).astype(np.int64)
        rec_start = np.concatenate([first[rs] + rc * nbuf, first[fl] + nfull[part > 0] * nbuf])
        rec_len = np.concatenate([np.full(rs.size, nbuf), part[part > 0]]).astype(np.int64)
        nrec = rec_stream.size
        link = np.zeros(nrec, np.int64)
        prev = {}
        for r, st in enumerate(rec_stream.tolist()):
            link[r] = prev.get(st, 0)
            prev[st] = r + 1
        buf = np.zeros((nrec, irecl), np.uint8)
        head = np.stack([streams[rec_stream], rec_len, link], axis=1).astype("<i4")
        buf[:, :12] = head.view(np.uint8).reshape(nrec, 12)
        for r in range(nrec):
            a, m = int(rec_start[r]), int(rec_len[r])
            buf[r, 12:12 + 8 * m] = np.asarray(v[a:a + m], "<f8").view(np.uint8)
            buf[r, 12 + 8 * m:12 + 12 * m] = np.asarray(l2[a:a + m], "<i4").view(np.uint8)
        with open(os.path.join(directory, srtpq_name("SRTPQIL", rank)), "wb") as f:
            f.write(buf.tobytes())
        with open(os.path.join(directory, srtpq_name("SRTPQLN", rank)), "wb") as f:
            write_record(f, struct.pack("<6i", nrec, irecl, 1, nl, nl + 1, n))


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
