"""Digest fixtures of the CPU oracle on the benchmarked workloads.

The full MDCINT stream of a large workload is too big to commit (4.9 GB at
n = 400 with 120 Kramers pairs), so this script runs the oracle
(``oracle/rotran_oracle.c``, the restatement of rotran) once on the full
workload and keeps a digest the GPU tests can check a transform against:

* ``hdr``: every record's (IKR*IS, JKR*JS, NZ), in file order;
* ``absum``: per record the sum of |value| over its elements;
* ``nnear``: per record the number of elements with |value| <= NEAR (those
  can fall on either side of THROUT under rounding-level differences);
* a seeded uniform sample of elements (record, INDK, INDL, value);
* NHALFT, NSKEL and NFINAL1..4.

Workloads (seeded, the generator of ``molfdir_gb300/synth.py``):

* ``precision``: 160 L + 240 S functions, 120 Kramers pairs, seed 0, the
  precision-study transform (about 8.7e8 integrals);
* ``batched``: the 48 instances of the batched workload
  (``synth.batched_instances()``), a smaller digest per instance
  (NZ and near-threshold counts per record, the sum of |value| and a
  weighted checksum of the per-record sums, a sample).

The integral records are generated on the host in the order the GPU tests
and ``bench.py`` generate them on the device (one record per file and
integral type, file order LL, SL, SS, stable in the generator's order); the
two differ only in the summation order of the B B^T products.  Large record
arrays are written to memory-mapped files under ``--scratch`` and deleted at
the end.  Usage::

    python tests/golden/make_oracle_digest.py precision --scratch DIR
    python tests/golden/make_oracle_digest.py batched
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), HERE]

import pyoracle  # noqa: E402
from digest_check import checksum_weights, record_sums  # noqa: E402
from molfdir_gb300 import synth  # noqa: E402

NEAR = 1e-13       # |value| at or below which an element may flip presence
SAMPLE_SEED = 20261204


def host_records(model, mfil=3, scratch=None, tag="r", reuse=False):
    """Records (file_class, itype, nt, rint, label2, label1) of a problem:
    one record per file and integral type, integrals of a file ordered by
    type (stable), the layout of ``synth.device_records``.  With ``scratch``
    the three arrays are memory-mapped files there (with ``reuse``, files of
    the right size left there by an earlier run are taken as they are)."""
    files = [("LL", 1)]
    if mfil >= 2 and model.n_s > 0:
        files.append(("SL", 2))
    if mfil >= 3 and model.n_s > 0:
        files.append(("SS", 3))
    parts, cls, its, nts = [], [], [], []
    total = 0
    for key, fc in files:
        v, l2, l1, it = synth._file_integrals(model, key)
        order = np.argsort(it, kind="stable")
        counts = np.bincount(it.astype(np.int64), minlength=15)
        for t in range(1, 15):
            if counts[t]:
                cls.append(fc)
                its.append(t)
                nts.append(int(counts[t]))
        parts.append((v[order], l2[order], l1[order]))
        total += v.size
        del v, l2, l1, it, order
    if scratch is not None and reuse and os.path.exists(os.path.join(scratch, f"{tag}_l1.npy")):
        paths = [os.path.join(scratch, f"{tag}_{x}.npy") for x in ("rint", "l2", "l1")]
        arrs = [np.load(q, mmap_mode="r") for q in paths]
        if all(a.size == total for a in arrs):
            del parts
            return (np.asarray(cls, np.int32), np.asarray(its, np.int32), np.asarray(nts, np.int64),
                    *arrs)
    if scratch is None:
        rint = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0)
        lab2 = np.concatenate([p[1] for p in parts]).astype(np.int32)
        lab1 = np.concatenate([p[2] for p in parts]).astype(np.int32)
    else:
        rint = np.lib.format.open_memmap(os.path.join(scratch, f"{tag}_rint.npy"), "w+", np.float64, (total,))
        lab2 = np.lib.format.open_memmap(os.path.join(scratch, f"{tag}_l2.npy"), "w+", np.int32, (total,))
        lab1 = np.lib.format.open_memmap(os.path.join(scratch, f"{tag}_l1.npy"), "w+", np.int32, (total,))
        o = 0
        for v, l2, l1 in parts:
            rint[o:o + v.size] = v
            lab2[o:o + v.size] = l2
            lab1[o:o + v.size] = l1
            o += v.size
        rint.flush(); lab2.flush(); lab1.flush()
    del parts
    return (np.asarray(cls, np.int32), np.asarray(its, np.int32), np.asarray(nts, np.int64),
            rint, lab2, lab1)


def record_digest(img):
    """Per record NZ, sum |v| and near-threshold counts of an oracle image."""
    nz = img.hdr[:, 2].astype(np.int64)
    off = np.concatenate([[0], np.cumsum(nz)])
    a = np.abs(img.val)
    return off, record_sums(nz, a), record_sums(nz, (a <= NEAR).astype(np.int64)).astype(np.int32)


def sample(img, off, count, rng):
    nzt = img.val.size
    pos = np.sort(rng.choice(nzt, size=min(count, nzt), replace=False)) if nzt else np.zeros(0, np.int64)
    rec = np.searchsorted(off, pos, side="right") - 1
    return (rec.astype(np.int32), img.idx[pos, 0].astype(np.int16), img.idx[pos, 1].astype(np.int16),
            img.val[pos].astype(np.complex128))


def run_precision(args):
    nl, ns, nkr, seed = 160, 240, 120, 0
    os.makedirs(args.scratch, exist_ok=True)
    prob = synth.make_spinor_problem(nl, ns, nkr, seed=seed)
    t0 = time.time()
    recs = host_records(prob.model, 3, scratch=args.scratch, tag="precision", reuse=args.reuse)
    t1 = time.time()
    print(f"records: {recs[3].size} integrals in {t1 - t0:.0f} s", flush=True)
    img = pyoracle.run(prob, nthreads=args.threads, records=recs)
    t2 = time.time()
    print(f"oracle: {t2 - t1:.0f} s (first {img.times[0]:.0f}, second {img.times[1]:.0f}, "
          f"pp {img.times[2]:.0f}); {img.hdr.shape[0]} records, {img.val.size} elements", flush=True)
    del recs
    if args.keep_stream:
        for name, arr in (("hdr", img.hdr), ("idx", img.idx), ("val", img.val)):
            np.save(os.path.join(args.scratch, f"precision_stream_{name}.npy"), arr)
    off, absum, nnear = record_digest(img)
    srec, sk, sl, sv = sample(img, off, args.samples, np.random.default_rng(SAMPLE_SEED))
    meta = dict(workload="precision_study_n400_k120", n_l=nl, n_s=ns, nkr=nkr, seed=seed,
                thrgen=1e-16, throut=1e-16, near=NEAR, elements=int(img.val.size),
                oracle_seconds=t2 - t1, threads=args.threads,
                max_abs_value=float(np.abs(img.val).max()) if img.val.size else 0.0)
    out = os.path.join(HERE, "oracle_digest_n400_k120.npz")
    np.savez_compressed(out, hdr=img.hdr.astype(np.int32), absum=absum, nnear=nnear,
                        sample_rec=srec, sample_k=sk, sample_l=sl, sample_val=sv,
                        counts=np.array([img.nhalft, img.nskel, *img.nfinal], np.int64),
                        meta=json.dumps(meta))
    print("wrote", out, os.path.getsize(out), "bytes")
    if not args.keep_stream:
        shutil.rmtree(args.scratch, ignore_errors=True)


def run_batched(args):
    sizes = synth.batched_instances()
    rng = np.random.default_rng(SAMPLE_SEED)
    cols = {k: [] for k in ("inst_nrec", "nz", "nnear", "absum", "wsum", "counts",
                            "s_inst", "s_rec", "s_k", "s_l", "s_val")}
    t0 = time.time()
    for i, (nl, ns, nkr, seed) in enumerate(sizes):
        prob = synth.make_spinor_problem(nl, ns, nkr, seed=seed)
        recs = host_records(prob.model, 3)
        img = pyoracle.run(prob, nthreads=args.threads, records=recs)
        off, absum, nnear = record_digest(img)
        w = checksum_weights(seed, img.hdr.shape[0])
        cols["inst_nrec"].append(img.hdr.shape[0])
        cols["nz"].append(img.hdr[:, 2].astype(np.int32))
        cols["nnear"].append(nnear)
        cols["absum"].append(float(absum.sum()))
        cols["wsum"].append(float(np.dot(w, absum)))
        cols["counts"].append([img.nhalft, img.nskel, *img.nfinal])
        srec, sk, sl, sv = sample(img, off, args.samples_per_instance, rng)
        cols["s_inst"].append(np.full(srec.size, i, np.int16))
        cols["s_rec"].append(srec)
        cols["s_k"].append(sk)
        cols["s_l"].append(sl)
        cols["s_val"].append(sv)
        print(f"instance {i}: n={nl + ns} K={nkr} records {img.hdr.shape[0]} elements {img.val.size}",
              flush=True)
    meta = dict(workload="batched_48", sizes=[list(map(int, s)) for s in sizes], thrgen=1e-16,
                throut=1e-16, near=NEAR, oracle_seconds=time.time() - t0, threads=args.threads)
    out = os.path.join(HERE, "oracle_digest_batched48.npz")
    np.savez_compressed(out, inst_nrec=np.array(cols["inst_nrec"], np.int32),
                        nz=np.concatenate(cols["nz"]), nnear=np.concatenate(cols["nnear"]),
                        absum=np.array(cols["absum"]), wsum=np.array(cols["wsum"]),
                        counts=np.array(cols["counts"], np.int64),
                        s_inst=np.concatenate(cols["s_inst"]), s_rec=np.concatenate(cols["s_rec"]),
                        s_k=np.concatenate(cols["s_k"]), s_l=np.concatenate(cols["s_l"]),
                        s_val=np.concatenate(cols["s_val"]), meta=json.dumps(meta))
    print("wrote", out, os.path.getsize(out), "bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["precision", "batched"])
    ap.add_argument("--scratch", default=os.path.join(ROOT, "_work", "big"))
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--samples", type=int, default=1 << 15)
    ap.add_argument("--samples-per-instance", type=int, default=768)
    ap.add_argument("--reuse", action="store_true", help="take record files left in --scratch")
    ap.add_argument("--keep-stream", action="store_true",
                    help="also save the oracle's full stream in --scratch and keep the directory")
    args = ap.parse_args()
    (run_precision if args.workload == "precision" else run_batched)(args)


if __name__ == "__main__":
    main()
