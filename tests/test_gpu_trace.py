"""RT_TRACE: per-phase timing lines of rt_transform and rt_adjoint on stderr
(needs a GB300).  The switch is read at rt_create, so each case runs in a
child process with the variable set."""

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, {root!r})
from molfdir_gb300 import rotran, synth
prob = synth.make_problem(6, 8, 4, seed=1)
for prec in (rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16):
    with rotran.Rotran.for_problem(prob, precision=prec) as rt:
        rt.set_problem_coefficients(prob)
        rt.add_problem_records(prob)
        rt.transform()
        rt.transform()
print("child ok")
"""

PHASES = ["staged records", "tables and work arena", "bucketing kernels", "bucketing status check",
          "A: expand G_pq(r,s)", "A: GEMM1", "A: slice HA + GEMM2", "A: Kramers selection",
          "B: expand M_ij(p,q)", "B: GEMM3", "B: slice RK + GEMM4", "B: MDCINT selection",
          "counts read back"]


def run_child(trace):
    env = dict(os.environ)
    env.pop("RT_TRACE", None)
    if trace is not None:
        env["RT_TRACE"] = trace
    return subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                          capture_output=True, text=True, timeout=600)


def test_trace_lines():
    r = run_child("1")
    assert r.returncode == 0, r.stderr[-2000:]
    assert "child ok" in r.stdout
    blocks = r.stderr.split("rotran-gb300 rt_transform trace")
    assert len(blocks) == 5  # text before the first block + 4 transforms
    for b in blocks[1:]:
        # phase lines only ("[rt] ..." lines report the split GEMM set-up)
        lines = [ln.strip() for ln in b.strip().splitlines()[1:] if not ln.startswith("[rt]")]
        names = [ln.rsplit(None, 2)[0] for ln in lines if ln]
        for ph in PHASES:
            assert ph in names, (ph, names)
        # every line: name, device ms >= 0, host ms non-decreasing
        host = [float(ln.rsplit(None, 2)[2]) for ln in lines if ln]
        dev = [float(ln.rsplit(None, 2)[1]) for ln in lines if ln]
        assert all(d >= 0.0 for d in dev)
        assert host == sorted(host)


@pytest.mark.parametrize("value", [None, "0"])
def test_trace_off(value):
    r = run_child(value)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "trace" not in r.stderr
