"""The split path beyond 512 scalar functions (needs a GB300).

GEMM2 and GEMM4 contract over K = 2 NSC (both planes of the AO index).  At
NSC = 600 that is K = 1200, beyond the 819 up to which the narrow slicing
(leading digit in [-128, 128]) keeps the three exact FP32 accumulators
exact; such operands are sliced wide (every digit in [-64, 64]), exact to
K = 1365.  The records are those of a subset of pq buckets (an integral set
of realistic density would hold about 4e9 integrals at this size); both
paths transform the same records."""

import numpy as np
import pytest

from molfdir_gb300 import rotran, synth
from util import compare_streams

pytestmark = pytest.mark.gpu


def _run(p, recs, precision):
    with rotran.Rotran.for_problem(p, precision=precision) as rt:
        rt.set_problem_coefficients(p)
        rt.add_records_bulk(*recs)
        rt.transform()
        return rt.result()


def test_split_matches_fp64_at_nsc_600():
    p = synth.make_spinor_problem(240, 360, 16, seed=21)
    rng = np.random.default_rng(3)
    model = p.model
    ll = [(int(a), int(b)) for a, b in zip(model.pl, model.ql)]
    ss = [(int(a), int(b)) for a, b in zip(model.ps, model.qs)]
    pick = [ll[i] for i in rng.choice(len(ll), 120, replace=False)] + \
           [ss[i] for i in rng.choice(len(ss), 120, replace=False)]
    cls, its, nts, v, l2, l1 = synth.bucket_records(model, sorted(pick))
    recs = (cls, nts, its, v, l2, l1)
    split = _run(p, recs, rotran.RT_PREC_SPLIT_BF16)
    fp64 = _run(p, recs, rotran.RT_PREC_FP64)
    err = compare_streams(split, fp64, 1e-10)
    scale = float(np.abs(fp64[2]).max())
    print(f"K = 2 NSC = 1200: max |split - FP64| = {err:.3e}, max |value| = {scale:.3e}, "
          f"{fp64[2].shape[0]} elements")
    assert err <= 1e-10
    assert fp64[2].shape[0] > 50000

