"""The benchmarked workloads against the oracle, at full size (needs a GB300).

The oracle (oracle/rotran_oracle.c) was run once on the full workloads and
its streams reduced to digests (tests/golden/make_oracle_digest.py): every
record's labels and NZ, per-record sums of |value|, near-threshold counts,
NHALFT/NFINAL and a seeded sample of elements.  Here the GPU transforms the
same seeded inputs (records generated on the device; they differ from the
oracle's host-generated ones only in the summation order of the B B^T
products) and every digest item is checked:

* precision study (160 L + 240 S functions, 120 Kramers pairs, 8.7e8
  integrals): FP64 path within 1e-12, split path within 1e-10, identical
  record labels and order, NZ per record equal up to elements within
  rounding of THROUT;
* the 48 batched instances through the batch API (split) and one by one in
  FP64: per instance the record count, NZ per record, two checksums and the
  sampled elements.
"""

import os
import sys

import numpy as np
import pytest

from molfdir_gb300 import rotran, synth

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import digest_check  # noqa: E402

pytestmark = pytest.mark.gpu


def _ctx(p, prec, recs):
    rt = rotran.Rotran.for_problem(p, precision=prec)
    rt.set_problem_coefficients(p)
    cls, its, nts, dv, dl2, dl1 = recs
    rt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
    return rt


@pytest.mark.parametrize("precision,tol", [(rotran.RT_PREC_FP64, 1e-12), (rotran.RT_PREC_SPLIT_BF16, 1e-10)],
                         ids=["fp64", "split"])
def test_precision_study_matches_the_oracle_digest(precision, tol):
    import torch
    dg = digest_check.load(digest_check.PRECISION)
    assert dg is not None, "oracle digest fixture missing"
    m = dg["meta"]
    p = synth.make_spinor_problem(m["n_l"], m["n_s"], m["nkr"], seed=m["seed"])
    recs = synth.device_records(p, 3, device="cuda")
    rt = _ctx(p, precision, recs)
    try:
        rt.transform()
        hdr, idx, val = rt.result()
    finally:
        rt.close()
        del recs
        torch.cuda.empty_cache()
    res = digest_check.check_stream(dg, hdr, idx, val, tol)
    print(res)
    assert res["records_identical"]
    assert res["nz_within_near"]
    assert res["sample_missing_ok"] and res["sample_max_abs_err"] <= tol
    assert res["absum_max_excess"] <= 1.0
    assert res["ok"]


def test_batched_instances_match_the_oracle_digest():
    import torch
    dg = digest_check.load(digest_check.BATCHED)
    assert dg is not None, "oracle digest fixture missing"
    sizes = dg["meta"]["sizes"]
    probs, recs = [], []
    for nl, ns, nkr, seed in sizes:
        p = synth.make_spinor_problem(nl, ns, nkr, seed=seed)
        probs.append(p)
        recs.append(synth.device_records(p, 3, device="cuda"))
    rts = [_ctx(p, rotran.RT_PREC_SPLIT_BF16, r) for p, r in zip(probs, recs)]
    batch = rotran.Batch(rts)
    try:
        batch.run()
        batch.run()  # the replayed graph
        split = [rt.result() for rt in rts]
    finally:
        batch.close()
        for rt in rts:
            rt.close()
    worst = {"split": 0.0, "fp64": 0.0}
    for i, (p, r) in enumerate(zip(probs, recs)):
        inst = digest_check.batched_instance(dg, i)
        res = digest_check.check_batched_instance(inst, *split[i], 1e-10)
        assert res["ok"], (i, sizes[i], res)
        worst["split"] = max(worst["split"], res["sample_max_abs_err"])
        rt = _ctx(p, rotran.RT_PREC_FP64, r)
        try:
            rt.transform()
            got = rt.result()
        finally:
            rt.close()
        res = digest_check.check_batched_instance(inst, *got, 1e-12)
        assert res["ok"], (i, sizes[i], res)
        worst["fp64"] = max(worst["fp64"], res["sample_max_abs_err"])
    print("worst sampled |GPU - oracle|:", worst)
    del recs
    torch.cuda.empty_cache()
