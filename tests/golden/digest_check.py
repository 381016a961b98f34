"""Check an MDCINT record stream against an oracle digest fixture.

The fixtures (``oracle_digest_*.npz``, made by ``make_oracle_digest.py``)
hold per record (IKR*IS, JKR*JS, NZ), the sum of |value|, the number of
elements within rounding of THROUT, NHALFT/NFINAL, and a seeded sample of
elements.  ``check_stream`` compares a stream (hdr, idx, val) with them:

* records: same labels in the same order;
* NZ per record: equal, or different by at most the record's count of
  near-threshold elements (values at most ``near`` can fall on either side
  of THROUT under rounding-level differences of the inputs);
* every sampled element: present with a value within ``tol`` (or, if absent,
  of magnitude at most ``near``);
* sum of |value| per record: within ``tol`` times the record's NZ (plus the
  near-threshold allowance).

Used by the GPU tests and by ``bench.py`` (read-only data; no oracle code).
"""

from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PRECISION = os.path.join(HERE, "oracle_digest_n400_k120.npz")
BATCHED = os.path.join(HERE, "oracle_digest_batched48.npz")


def load(path):
    if not os.path.exists(path):
        return None
    z = np.load(path, allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def record_sums(nz, x):
    """Per-record sums of x over records of nz elements each (0 for empty)."""
    nz = np.asarray(nz, np.int64)
    out = np.zeros(nz.size, x.dtype if x.size else np.float64)
    ne = np.nonzero(nz > 0)[0]
    if ne.size:
        off = np.concatenate([[0], np.cumsum(nz)])
        out[ne] = np.add.reduceat(x, off[ne])
    return out


def _lookup(hdr, idx, val, recs, ks, ls):
    """Values of elements (record, INDK, INDL) in a stream; NaN if absent."""
    off = np.concatenate([[0], np.cumsum(hdr[:, 2].astype(np.int64))])
    out = np.full(recs.size, np.nan + 0j)
    want = (ks.astype(np.int64) + 32768) << 16 | (ls.astype(np.int64) + 32768)
    order = np.argsort(recs, kind="stable")
    bounds = np.concatenate([[0], np.nonzero(np.diff(recs[order]))[0] + 1, [recs.size]])
    for g in range(bounds.size - 1):
        sel = order[bounds[g]:bounds[g + 1]]
        r = int(recs[sel[0]])
        a, b = off[r], off[r + 1]
        if a == b:
            continue
        keys = (idx[a:b, 0].astype(np.int64) + 32768) << 16 | (idx[a:b, 1].astype(np.int64) + 32768)
        srt = np.argsort(keys, kind="stable")
        pos = np.searchsorted(keys[srt], want[sel])
        pos = np.minimum(pos, keys.size - 1)
        hit = keys[srt][pos] == want[sel]
        out[sel[hit]] = val[a + srt[pos[hit]]]
    return out


def check_stream(dg, hdr, idx, val, tol, sample_keys=("sample_rec", "sample_k", "sample_l", "sample_val")):
    """Compare a full stream with the precision-study digest; returns a dict
    of findings with ``ok`` set when every check passes."""
    near = float(dg["meta"]["near"])
    res = {"tol": tol}
    rh = dg["hdr"]
    res["records_identical"] = bool(hdr.shape[0] == rh.shape[0] and np.array_equal(hdr[:, :2], rh[:, :2]))
    if not res["records_identical"]:
        res["ok"] = False
        return res
    dnz = np.abs(hdr[:, 2].astype(np.int64) - rh[:, 2].astype(np.int64))
    res["nz_identical"] = bool(not dnz.any())
    res["nz_within_near"] = bool(np.all(dnz <= dg["nnear"]))
    res["elements"] = int(hdr[:, 2].sum())
    absum = record_sums(hdr[:, 2], np.abs(val))
    allow = tol * np.maximum(hdr[:, 2], rh[:, 2]) + near * dg["nnear"] + 1e-300
    res["absum_max_excess"] = float(np.max(np.abs(absum - dg["absum"]) / allow)) if absum.size else 0.0
    sr, sk, sl, sv = (dg[k] for k in sample_keys)
    got = _lookup(hdr, idx, val, sr, sk.astype(np.int32), sl.astype(np.int32))
    miss = np.isnan(got.real)
    res["sample_size"] = int(sr.size)
    res["sample_missing"] = int(miss.sum())
    res["sample_missing_ok"] = bool(np.all(np.abs(sv[miss]) <= near))
    err = np.abs(got[~miss] - sv[~miss])
    res["sample_max_abs_err"] = float(err.max()) if err.size else 0.0
    res["sample_rms_err"] = float(np.sqrt(np.mean(err ** 2))) if err.size else 0.0
    res["ok"] = bool(res["nz_within_near"] and res["absum_max_excess"] <= 1.0 and res["sample_missing_ok"]
                     and res["sample_max_abs_err"] <= tol)
    return res


def batched_instance(dg, i):
    """The digest of instance i of the batched fixture."""
    nrec = dg["inst_nrec"].astype(np.int64)
    r0 = int(nrec[:i].sum())
    sel = dg["s_inst"] == i
    return {"nz": dg["nz"][r0:r0 + nrec[i]], "nnear": dg["nnear"][r0:r0 + nrec[i]],
            "absum": float(dg["absum"][i]), "wsum": float(dg["wsum"][i]), "counts": dg["counts"][i],
            "s_rec": dg["s_rec"][sel], "s_k": dg["s_k"][sel], "s_l": dg["s_l"][sel],
            "s_val": dg["s_val"][sel], "near": float(dg["meta"]["near"]),
            "size": dg["meta"]["sizes"][i]}


def checksum_weights(seed, nrec):
    """Per-record weights of an instance's checksum (as the fixture script)."""
    return np.random.default_rng(seed).uniform(0.5, 1.5, size=nrec)


def check_batched_instance(inst, hdr, idx, val, tol):
    near = inst["near"]
    res = {}
    nz = hdr[:, 2].astype(np.int64)
    res["records"] = int(hdr.shape[0]) == int(inst["nz"].size)
    if not res["records"]:
        res["ok"] = False
        return res
    dnz = np.abs(nz - inst["nz"])
    res["nz_within_near"] = bool(np.all(dnz <= inst["nnear"]))
    absum = record_sums(nz, np.abs(val))
    w = checksum_weights(inst["size"][3], nz.size)
    allow = tol * max(int(nz.sum()), 1) + near * int(inst["nnear"].sum())
    res["absum_err"] = float(abs(absum.sum() - inst["absum"]))
    res["wsum_err"] = float(abs(np.dot(w, absum) - inst["wsum"]))
    got = _lookup(hdr, idx, val, inst["s_rec"], inst["s_k"].astype(np.int32), inst["s_l"].astype(np.int32))
    miss = np.isnan(got.real)
    res["sample_missing_ok"] = bool(np.all(np.abs(inst["s_val"][miss]) <= near))
    err = np.abs(got[~miss] - inst["s_val"][~miss])
    res["sample_max_abs_err"] = float(err.max()) if err.size else 0.0
    res["ok"] = bool(res["nz_within_near"] and res["absum_err"] <= allow and res["wsum_err"] <= 1.5 * allow
                     and res["sample_missing_ok"] and res["sample_max_abs_err"] <= tol)
    return res
