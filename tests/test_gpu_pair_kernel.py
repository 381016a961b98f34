"""The CTA-pair split GEMM (tcgen05 cta_group::2, selected with
RT_GEMM_KERNEL=pair) against the oracle (needs a GB300).

The single-CTA kernel is the default; the pair kernel computes the same
digit products with the same accumulation.  The choice is read once per
context's split state, so the transform runs in a child process with the
variable set.  The child also runs the pair kernel's abort path (both CTAs
stop, drain, meet at the cluster barrier and free TMEM): with no tensor
copies issued its waits run out, the call returns class 6, and the same
context then transforms correctly."""

import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
sys.path[:0] = [{tests!r}, {oracle!r}, {root!r}]
import pyoracle
from molfdir_gb300 import rotran, synth
from util import compare_streams
out = {{}}
for prec, tol in ((rotran.RT_PREC_SPLIT_BF16, 1e-10), (rotran.RT_PREC_FP64, 1e-12)):
    p = synth.make_problem(24, 40, 40, seed=3)
    img = pyoracle.run(p)
    with rotran.Rotran.for_problem(p, precision=prec) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        got = rt.result()
    out[str(prec)] = compare_streams(got, (img.hdr, img.idx, img.val), tol)
# the pair kernel's abort path: no copies, 50 ms waits, class 6, then correct
import os
import numpy as np
p = synth.make_problem(24, 40, 40, seed=3)
with rotran.Rotran.for_problem(p, precision=rotran.RT_PREC_SPLIT_BF16) as rt:
    rt.set_problem_coefficients(p)
    rt.add_problem_records(p)
    rt.transform()
    good = rt.result()
    os.environ["RT_TEST_GEMM_NO_COPIES"] = "1"
    try:
        rt.transform()
        out["abort"] = "no error"
    except rotran.RotranError as e:
        out["abort"] = [e.code, str(e)]
    del os.environ["RT_TEST_GEMM_NO_COPIES"]
    rt.transform()
    again = rt.result()
out["recovered"] = all(np.array_equal(a, b) for a, b in zip(good, again))
print(json.dumps(out))
"""


def test_pair_kernel_transform_matches_the_oracle():
    env = dict(os.environ, RT_GEMM_KERNEL="pair", RT_TRACE="1")
    code = CHILD.format(tests=HERE, oracle=os.path.join(ROOT, "oracle"), root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "CTA-pair kernel" in r.stderr
    err = json.loads(r.stdout.strip().splitlines()[-1])
    print(err)
    assert err["1"] <= 1e-10
    assert err["0"] <= 1e-12
    code, msg = err["abort"]
    assert code == 6 and "gave up" in msg and "could not confirm" not in msg
    assert err["recovered"]
