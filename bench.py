"""Throughput of the GB300 rotran four-index transformation.

One step = one complete transformation (record scatter, both
half-transformations, MDCINT selection) of the precision-study workload:
160 large + 240 small component functions (n = 400), 120 Kramers pairs,
seeded synthetic integrals (about 8.7e8 unique (LL|LL), (SS|LL) and (SS|SS)
integrals, 14 GB of records, larger than L2).  ``value`` is the algorithmic
FLOP rate with the integral records already resident in device memory;
``e2e`` repeats the step through the public API from pinned host memory,
host->device copy of the records and device->host copy of the MDCINT
stream included: each item chunk's elements are copied to pinned host
buffers while the next chunks run, and each step's records are queued
during the step before (the first step's are copied inside the timed region
too); ``e2e.sequential`` copies each step's records before it, and
``e2e.copied_after`` also copies the whole stream after the transform.  ``--impl reference`` times the CPU restatement of rotran
(the reference is Fortran 77 and cannot be built here) on a bounded sample of
the same workload with all host cores.

The line also carries ``fock``: tmoone's skeleton Fock build over the same
resident records (``--workload fock`` measures it with oracle checks).

Multi-GPU: every rank runs an independent replica of the workload (no
collective on the data path); value = all ranks' work / max rank time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="precision_study_n400_k120", n_l=160, n_s=240, nkr=120, seed=0)
SMALL = dict(name="c1_n64_k32", n_l=24, n_s=40, nkr=32, seed=0)
# a profiling case: the same kernels at a size whose device footprint stays
# near 1 GB (inputs still larger than L2)
PROFILE = dict(name="profile_n128_k32", n_l=48, n_s=80, nkr=32, seed=0)
# a second profiling case whose GEMM2/GEMM4 (M = 2m = 240) run as CTA pairs
PROFILE2 = dict(name="profile_n200_k60", n_l=80, n_s=120, nkr=60, seed=0)
# the large single transform: 192 L + 288 S AOs, 200 Kramers pairs, AOs in 4
# irreps with the integrals zero outside the symmetry-allowed blocks
LARGE = dict(name="large_c2v_n480_k200", n_l=192, n_s=288, nkr=200, seed=0, n_irrep=4)
# DRAM bytes per k_split_gemm launch from an ncu launch-list capture of the
# same transform (dram__bytes_read.sum + dram__bytes_write.sum averaged over
# its GEMM launches; summary in profiles/launches_split_n400_k120.md).  It is
# not measured by the run that prints it: the line labels it so.
TRAFFIC = {"precision_study_n400_k120": 34310516753}
TRAFFIC_SOURCE = "ncu launch list of this workload (profiles/launches_split_n400_k120.md), not this run"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    except OSError:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dense_equivalent_flops(n, nkr):
    """The dense count of the reference algorithm over all n(n+1)/2 AO pairs:
    F1 = P (4 n^2 m + 8 n m^2) (MATMUL1 as a dense real x complex product,
    then the m x m x n ZGEMM) and F2 = K(K+1) (8 n^2 m + 8 n m^2) (the
    symmetric expansion as a dense complex product, then the ZGEMM), m = 2K.
    It includes the SL pairs Coulomb rotran never transforms and the zero
    L/S blocks of each pair, so it is about 2x the work done; the bench's
    value uses the count of nonzero blocks instead (flops_algorithmic)."""
    m, P = 2 * nkr, n * (n + 1) // 2
    return P * (4.0 * n * n * m + 8.0 * n * m * m) + nkr * (nkr + 1) * (8.0 * n * n * m + 8.0 * n * m * m)


def workload_counts(prob):
    """Integral count and algorithmic FLOPs of a workload, from the generator
    alone (no device): the dense-block count of the reference algorithm
    over the transformed pq blocks, GEMM1 over the symmetry-allowed AO
    blocks (the library's rt_stats.flops_algorithmic)."""
    mdl = prob.model
    nl, ns = mdl.n_l, mdl.n_s
    n, m, k = nl + ns, prob.m, prob.nkr
    irr, ng = mdl.irrep, mdl.n_irrep
    comp = [np.arange(nl), np.arange(nl, n)]
    nb = [[int(np.sum(irr[c] == g)) for g in range(ng)] for c in comp]
    npair = np.zeros((2, ng), np.int64)
    for ci, c in enumerate(comp):
        ir = irr[c]
        x = ir[:, None] ^ ir[None, :]
        tri = np.tril(np.ones((c.size, c.size), bool))
        npair[ci] = np.bincount(x[tri], minlength=ng)[:ng]
    P = int(npair.sum()) if prob.mfil >= 3 else int(npair[0].sum())
    f1 = 8.0 * n * m * m * P
    for ci in range(2 if prob.mfil >= 3 else 1):
        for gam in range(ng):
            f1 += npair[ci, gam] * sum(4.0 * nb[cr][g] * nb[cr][g ^ gam] * m
                                       for cr in range(2) for g in range(ng))
    f2 = k * (k + 1) * (8.0 * nl * nl * m + 8.0 * ns * ns * m + 8.0 * n * m * m)
    L, S = npair[0], npair[1]
    nint = int(sum(L[g] * (L[g] + 1) // 2 + S[g] * L[g] + S[g] * (S[g] + 1) // 2 for g in range(ng)))
    return nint, float(f1 + f2)


def workload_config(work, prob, world):
    """The `config` object of both arms: the workload only."""
    nint, flops = workload_counts(prob)
    return {"workload": work["name"], "n": prob.n, "n_large": work["n_l"], "n_small": work["n_s"],
            "nkr": work["nkr"], "seed": work["seed"], "n_irrep": work.get("n_irrep", 1),
            "integrals": nint, "flops_algorithmic": flops,
            "flops_dense_equivalent": dense_equivalent_flops(prob.n, work["nkr"]),
            "l2": "inputs larger than L2 (integral records 16 B each)",
            "parallelism": f"replicas x{world}"}


def oracle_check(result, tol):
    """The MDCINT stream against the oracle's digest of the full
    precision-study transform (tests/golden), or None without the fixture."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import digest_check
    dg = digest_check.load(digest_check.PRECISION)
    if dg is None:
        return None
    hdr, idx, val = result
    res = digest_check.check_stream(dg, hdr, idx, val, tol)
    res["nhalft_oracle"] = int(dg["counts"][0])
    res["nfinal_oracle"] = [int(x) for x in dg["counts"][2:6]]
    return res


def cpu_sample(work, steps=1, warmup=0, seconds=15.0):
    """CPU restatement of rotran on a bounded sample of the workload:
    TRANS1 over the first pq blocks and TRANS2 over the first items with
    full-length half-transformed lists; returns (GFLOP/s, cores, sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from molfdir_gb300 import synth
    cores = os.cpu_count() or 1
    p = synth.make_spinor_problem(work["n_l"], work["n_s"], work["nkr"], seed=work["seed"],
                                  n_irrep=work.get("n_irrep", 1))
    res = pyoracle.time_sample(p, seconds=seconds, nthreads=cores, steps=steps, warmup=warmup)
    return res, cores


def run_gemm_case(args, rank):
    """One split GEMM of the shape of the second and fourth quarter steps, for
    kernel profiling (float-float operands sliced on the device): by default
    n = 400, 120 Kramers pairs (M = 2m = 480, K = 2n = 800), N = 32768;
    ``--gemm-shape 800,960,32768`` gives the n = 480, 200 Kramers pair shape."""
    from molfdir_gb300 import rotran
    rng = np.random.default_rng(0)
    m_, k_, n_ = (int(x) for x in args.gemm_shape.split(","))
    a = rng.standard_normal((m_, k_))
    b = rng.standard_normal((k_, n_))
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        rotran.split_dgemm(a, b, slices=args.slices, mode=1)
        dt = time.perf_counter() - t0
    if rank == 0:
        print(json.dumps({"workload": f"gemm_m{m_}_k{k_}_n{n_}", "slices": args.slices,
                          "seconds_per_call_with_host_work": dt}))


def run_breit_case(args, rank):
    """The Gaunt transform (BREIT, (SL|SL) integrals to MDBINT) at n = 200
    (80 L + 120 S AOs), 60 Kramers pairs, seed 0: 4.6e7 Gaunt integrals
    (host-generated), the split path timed over the steps after the warm-ups
    and one FP64 transform as the accuracy and speed reference."""
    import torch
    from molfdir_gb300 import rotran, synth
    if rank != 0:
        return
    prob = synth.make_problem(80, 120, 60, seed=0, breit=True, mfil=1)
    recs = prob.flat_records()
    keep = recs[0] == 4
    off = np.concatenate([[0], np.cumsum(recs[2])])
    sel = np.concatenate([np.arange(off[r], off[r + 1]) for r in np.nonzero(keep)[0]])
    cls, its, nts = recs[0][keep], recs[1][keep], recs[2][keep]
    v, l2, l1 = recs[3][sel], recs[4][sel], recs[5][sel]
    out = {"workload": "breit_n200_k60", "n": prob.n, "n_large": prob.nsc1, "nkr": prob.nkr,
           "integrals": int(v.size), "steps": args.steps, "warmup": args.warmup}
    legs = {}
    for name, prec, steps, warm in (("split", rotran.RT_PREC_SPLIT_BF16, args.steps, args.warmup),
                                    ("fp64", rotran.RT_PREC_FP64, 1, 0)):
        with rotran.Rotran.for_problem(prob, precision=prec, breit=True) as rt:
            rt.set_problem_coefficients(prob)
            rt.add_records_bulk(cls, nts, its, v, l2, l1)
            for _ in range(warm):
                rt.transform()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ms = []
            for _ in range(max(1, steps)):
                rt.transform()
                ms.append(rt.stats().ms_total)
            sec = max((time.perf_counter() - t0) / max(1, steps), statistics.mean(ms) / 1e3)
            st = rt.stats()
            legs[name] = {"sec": sec, "flops": st.flops_algorithmic, "result": rt.result(),
                          "ms_gemm": st.ms_gemm, "nfinal": list(st.nfinal)}
    sh, si, sv = legs["split"]["result"]
    fh, fi, fv = legs["fp64"]["result"]
    same = np.array_equal(sh, fh) and np.array_equal(si, fi)
    out.update({
        "value": legs["split"]["flops"] / legs["split"]["sec"] / 1e12, "unit": "TFLOP/s",
        "ms_per_step": legs["split"]["sec"] * 1e3, "ms_gemm": legs["split"]["ms_gemm"],
        "flops_algorithmic": legs["split"]["flops"],
        "fp64": {"value": legs["fp64"]["flops"] / legs["fp64"]["sec"] / 1e12,
                 "ms_per_step": legs["fp64"]["sec"] * 1e3,
                 "split_speedup": legs["fp64"]["sec"] / legs["split"]["sec"]},
        "split_vs_fp64": {"same_elements": bool(same),
                          "max_abs_err": float(np.abs(sv - fv).max()) if same and sv.size else None,
                          "max_abs_value": float(np.abs(fv).max()) if fv.size else 0.0},
        "mdbint": {"records": int(fh.shape[0]), "elements": int(fv.size), "nfinal": legs["fp64"]["nfinal"]}})
    print(json.dumps(out))


def run_fock_case(args, rank, hbm_peak, peak_kind):
    """tmoone's skeleton Fock build (MFDFOCK/FOCK, rt_fock_skeleton) over the
    precision-study workload's 8.7e8 resident integral records (n = 400,
    14 GB, larger than L2; ``fock_small``: the n = 200 profiling case, 5.5e7
    integrals, 0.9 GB): closed shell (one density set) and closed plus
    open shell (two), kernel time by CUDA events over the steps after the
    warm-ups.  Checks: GPU vs the oracle on the first records (about 3e7
    integrals, 1e-12 of max|F|), linearity F(D1 + D2) = F(D1) + F(D2) at full
    size, and the two-set call equal to two one-set calls.  The CPU baseline
    is the oracle (one thread, as FOCK runs) on the same sample."""
    import torch
    from molfdir_gb300 import rotran, synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    if rank != 0:
        return
    work = PROFILE2 if args.workload == "fock_small" else WORKLOAD
    prob = synth.make_spinor_problem(work["n_l"], work["n_s"], work["nkr"], seed=work["seed"])
    cls, its, nts, dv, dl2, dl1 = synth.device_records(prob, 3, device="cuda")
    torch.cuda.synchronize()
    nint = int(nts.sum())
    n = prob.n
    ntri = n * (n + 1) // 2
    g = torch.Generator(device="cuda").manual_seed(0)
    d1 = torch.randn((1, 4, ntri), device="cuda", dtype=torch.float64, generator=g)
    d2 = torch.randn((1, 4, ntri), device="cuda", dtype=torch.float64, generator=g)
    out = {"workload": f"fock_skeleton_n{n}", "n": n, "integrals": nint, "records": int(cls.size),
           "steps": args.steps, "warmup": args.warmup}
    with rotran.Rotran.for_problem(prob) as rt:
        rt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
        legs = {}
        for name, dens in (("closed", d1), ("closed_open", torch.cat([d1, d2]))):
            for _ in range(args.warmup):
                rt.fock_skeleton(dens)
            ms = []
            t0 = time.perf_counter()
            for _ in range(max(1, args.steps)):
                f, k = rt.fock_skeleton(dens)
                ms.append(k)
            wall = (time.perf_counter() - t0) / max(1, args.steps)
            legs[name] = {"ms_kernel": statistics.mean(ms), "ms_call": wall * 1e3, "fock": f}
        f1 = legs["closed"]["fock"]
        f2, _ = rt.fock_skeleton(d2)
        f12, _ = rt.fock_skeleton(d1 + d2)
        scale = float(f12.abs().max())
        lin = float((f12 - f1 - f2).abs().max()) / scale
        pair = legs["closed_open"]["fock"]
        two = float(max((pair[0] - f1[0]).abs().max(), (pair[1] - f2[0]).abs().max())) / scale
    # the first records on the host: oracle vs GPU
    nts_h = np.asarray(nts)
    cum = np.cumsum(nts_h)
    nr = int(np.searchsorted(cum, 30_000_000)) + 1
    ns = int(cum[nr - 1])
    sample = (np.asarray(cls)[:nr], np.asarray(its)[:nr], nts_h[:nr], dv[:ns].cpu().numpy(),
              dl2[:ns].cpu().numpy(), dl1[:ns].cpu().numpy())
    dh = d1.cpu().numpy()
    t0 = time.perf_counter()
    want = pyoracle.fock_skeleton(sample, n, dh, mfil=3)
    cpu_sec = time.perf_counter() - t0
    with rotran.Rotran.for_problem(prob) as rt:
        rt.add_records_bulk(*(sample[0], sample[2], sample[1], sample[3], sample[4], sample[5]))
        got, _ = rt.fock_skeleton(dh)
    err = float(np.abs(got - want).max() / np.abs(want).max())
    gaunt = None
    if args.workload == "fock":
        # tmoone's Gaunt contributions (MFDBREIT/GAUNT) over the Gaunt file of
        # the n = 200, 60 Kramers pair case (4.6e7 (SL|SL) integrals)
        bp = synth.make_problem(80, 120, 60, seed=0, breit=True, mfil=1)
        brecs = bp.flat_records()
        keep = brecs[0] == 4
        boff = np.concatenate([[0], np.cumsum(brecs[2])])
        bsel = np.concatenate([np.arange(boff[r], boff[r + 1]) for r in np.nonzero(keep)[0]])
        b6 = (brecs[0][keep], brecs[1][keep], brecs[2][keep], brecs[3][bsel], brecs[4][bsel], brecs[5][bsel])
        bn = bp.n
        bd = np.random.default_rng(1).standard_normal((1, 4, bn * (bn + 1) // 2))
        bcfg, bkeep = rotran.make_config(bn, bp.nsc1, bp.nkr, mfil=3)
        with rotran.Rotran(bcfg, bkeep) as rt:
            rt.add_records_bulk(b6[0], b6[2], b6[1], b6[3], b6[4], b6[5])
            for _ in range(args.warmup):
                rt.fock_gaunt(bd)
            gms = []
            for _ in range(max(1, args.steps)):
                gf, k = rt.fock_gaunt(bd)
                gms.append(k)
        t0 = time.perf_counter()
        gw = pyoracle.fock_gaunt(b6, bn, bd)
        gcpu = time.perf_counter() - t0
        gint = int(b6[3].size)
        gaunt = {"integrals": gint, "ms_kernel": statistics.mean(gms),
                 "value": gint / (statistics.mean(gms) / 1e3), "unit": "integrals/s",
                 "oracle_max_rel_err": float(np.abs(gf - gw).max() / np.abs(gw).max()),
                 "max_abs_element": float(np.abs(gw).max()),
                 "cpu_baseline": {"value": gint / gcpu, "unit": "integrals/s", "cores": 1, "kind": "port",
                                  "sample": "all Gaunt integrals of the case"}}
    ms = legs["closed"]["ms_kernel"]
    achieved = 16.0 * nint / (ms / 1e3) / 1e9
    out.update({
        "metric": "skeleton Fock integrals/s", "value": nint / (ms / 1e3), "unit": "integrals/s",
        "ms_kernel": ms, "ms_call": legs["closed"]["ms_call"],
        "closed_open": {"ms_kernel": legs["closed_open"]["ms_kernel"],
                        "value": nint / (legs["closed_open"]["ms_kernel"] / 1e3)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "bytes_per_integral": 16,
                     "traffic": 16.09 * nint,
                     "traffic_source": "ncu capture of the n = 200 case (profiles/k_fock_skeleton_n200.md): "
                                       "16.09 DRAM bytes per integral, scaled by the integrals",
                     "peak_source": f"hbm_gbs of {peak_kind}",
                     "limiter": "work per integral (18 atomics and gathers for the generic types), "
                                "not HBM"},
        "checks": {"oracle_sample_integrals": ns, "oracle_max_rel_err": err,
                   "linearity_rel_err": lin, "two_sets_vs_one_rel_err": two},
        "cpu_baseline": {"value": ns / cpu_sec, "unit": "integrals/s", "cores": 1, "kind": "port",
                         "sample": f"first {nr} records ({ns} integrals), one density set"},
        "gaunt": gaunt,
    })
    print(json.dumps(out))


def run_files_case(args, rank):
    """Integral input from files at n = 160 (64 L + 96 S AOs), 40 Kramers
    pairs, 2.27e7 integrals: the serial SRTTW/SRTLB files (SORT1's input)
    and the MPI version's pq-sorted SRTPQIL files of 4 ranks (GETPQ's
    input), each read into a context (host parse + upload) and transformed
    on the split path; the two MDCINT streams must agree."""
    import tempfile
    from molfdir_gb300 import fortio, rotran, synth
    if rank != 0:
        return
    prob = synth.make_problem(64, 96, 40, seed=0)
    nint = int(prob.flat_records()[3].size)
    out = {"workload": "files_n160_k40", "integrals": nint, "steps": args.steps,
           "warmup": args.warmup}
    results = {}
    with tempfile.TemporaryDirectory() as d:
        fortio.write_srt_files(prob, d)
        fortio.write_srtpq_files(prob, d, nranks=4)
        names = sorted(os.listdir(d))
        for fmt, files in (("srt", [f for f in names if f.startswith("SRTTW") or f.startswith("SRTLB")]),
                           ("srtpq", [f for f in names if f.startswith("SRTPQ")])):
            nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in files)
            rd, tr = [], []
            for step in range(args.warmup + args.steps):
                rt = rotran.Rotran.for_problem(prob, precision=rotran.RT_PREC_SPLIT_BF16,
                                               slices=args.slices)
                rt.set_problem_coefficients(prob)
                t0 = time.perf_counter()
                if fmt == "srt":
                    rt.read_srt_files(d)
                else:
                    rt.read_srtpq_files(d, nranks=4)
                t1 = time.perf_counter()
                rt.transform()
                t2 = time.perf_counter()
                if step >= args.warmup:
                    rd.append(t1 - t0)
                    tr.append(t2 - t1)
                results[fmt] = rt.result()
                rt.close()
            r = statistics.median(rd)
            out[fmt] = {"file_bytes": nbytes, "read_s": r, "read_GBps": nbytes / r / 1e9,
                        "read_Mintegrals_per_s": nint / r / 1e6,
                        "transform_s_incl_staged_upload": statistics.median(tr)}
    a, b = results["srt"], results["srtpq"]
    same = np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    out["same_records_and_elements"] = bool(same)
    out["max_abs_diff"] = float(np.max(np.abs(a[2] - b[2]))) if same and a[2].size else None
    print(json.dumps(out))


def batched_leg(args, world, local, steps, warmup, with_fp64=True, oracle=True):
    """48 independent transforms of uneven size (n_AO ~ U[40,200], 60% small
    component, 16..80 Kramers pairs, seeds 0..47): split precision as one
    batch (grouped GEMM launches in a captured CUDA graph, tile widths tuned),
    against the same 48 transforms run one after another in FP64, and the
    batch's streams against the oracle's digest of the 48 instances."""
    import torch
    from molfdir_gb300 import rotran, synth
    sizes = synth.batched_instances()
    probs, recs = [], []
    for nl, ns, nkr, seed in sizes:
        p = synth.make_spinor_problem(nl, ns, nkr, seed=seed)
        probs.append(p)
        recs.append(synth.device_records(p, 3, device="cuda"))
    torch.cuda.synchronize()

    def ctx(p, r, prec):
        rt = rotran.Rotran.for_problem(p, precision=prec, slices=args.slices if prec else 0)
        rt.set_problem_coefficients(p)
        cls, its, nts, dv, dl2, dl1 = r
        rt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
        return rt

    rts = [ctx(p, r, rotran.RT_PREC_SPLIT_BF16) for p, r in zip(probs, recs)]
    batch = rotran.Batch(rts)
    t0 = time.perf_counter()
    batch.run()  # tuning + capture + first replay
    t_first = time.perf_counter() - t0
    for _ in range(warmup):
        batch.run()
    dev_ms = []
    sampler = ClockSampler(local)
    sampler.__enter__()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.run()
        dev_ms.append(batch.stats().ms_last)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sampler.__exit__(None, None, None)
    bst = batch.stats()
    sec = barrier_max(max((t1 - t0) / steps, statistics.mean(dev_ms) / 1e3), world)
    flops = bst.flops_algorithmic
    results = [rt.result() for rt in rts]
    batch.close()
    for rt in rts:
        rt.close()
    ocheck = None
    if oracle:
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        import digest_check
        dg = digest_check.load(digest_check.BATCHED)
        if dg is not None:
            bad, worst = [], 0.0
            for i, (h, ix, v) in enumerate(results):
                res = digest_check.check_batched_instance(digest_check.batched_instance(dg, i), h, ix, v, 1e-10)
                worst = max(worst, res.get("sample_max_abs_err", 0.0))
                if not res["ok"]:
                    bad.append(i)
            ocheck = {"instances": len(results), "failed": bad, "tol": 1e-10,
                      "sample_max_abs_err": worst, "ok": not bad}
    fp64 = None
    if with_fp64:
        t_fp = 0.0
        mx = ss = 0.0
        nel = 0
        same = True
        for p, r, (h, i, v) in zip(probs, recs, results):
            rt = ctx(p, r, rotran.RT_PREC_FP64)
            torch.cuda.synchronize()
            a = time.perf_counter()
            rt.transform()
            torch.cuda.synchronize()
            t_fp += time.perf_counter() - a
            rh, ri, rv = rt.result()
            rt.close()
            if np.array_equal(rh, h) and np.array_equal(ri, i):
                d = np.abs(v - rv)
                mx = max(mx, float(d.max()) if d.size else 0.0)
                ss += float(np.dot(d, d))
                nel += d.size
            else:
                same = False
        fp64 = {"value": flops / t_fp / 1e12, "unit": "TFLOP/s", "ms_per_step": t_fp * 1e3,
                "mode": "48 sequential FP64 transforms", "split_speedup": t_fp / sec,
                "split_vs_fp64": {"max_abs_err": mx, "rms_err": float(np.sqrt(ss / max(1, nel))),
                                  "same_elements": same, "elements": nel}}
    del recs
    torch.cuda.empty_cache()
    return {"value": flops * world / sec / 1e12, "unit": "TFLOP/s", "sec": sec, "flops": flops,
            "sizes": sizes, "bst": bst, "fp64": fp64, "oracle_check": ocheck, "clocks": sampler.summary(),
            "first_run_s": t_first}


def run_batched(args, rank, world, local, bf16_peak, peak_kind):
    """The batched workload on its own line (``--workload batched``)."""
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    b = batched_leg(args, world, local, args.steps, args.warmup, with_fp64=not args.no_fp64)
    bst, sec, sizes = b["bst"], b["sec"], b["sizes"]
    if rank == 0:
        achieved = bst.flops_gemm_executed / sec / 1e12
        line = {
            "metric": "4-index transform TFLOP/s", "value": b["value"], "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16-slices/f32-acc (split)", "data": "synthetic",
            "config": {"workload": "batched_48", "instances": len(sizes),
                       "sizes": [[nl + ns, nkr] for nl, ns, nkr, _ in sizes],
                       "slices": args.slices, "flops_algorithmic": b["flops"],
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak,
                         "unit": "TFLOP/s", "frac": achieved / bf16_peak, "traffic": None,
                         "kernel": "whole batch: grouped tcgen05 GEMM tensor FLOPs per batch time",
                         "peak_source": f"bf16_tflops of {peak_kind}"},
            "cpu_baseline": None, "e2e": None, "fp64": b["fp64"], "oracle_check": b["oracle_check"],
            "gpu_launches": bst.kernel_launches * args.steps,
            "clocks": b["clocks"], "batch": bst.as_dict(),
            "first_run_s": b["first_run_s"],
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--slices", type=int, default=5)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", default="precision",
                    choices=["precision", "c1", "profile", "profile2", "large", "batched", "gemm", "files",
                             "breit", "fock", "fock_small"])
    ap.add_argument("--gemm-shape", default="480,800,32768",
                    help="M,K,N of --workload gemm")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fock", action="store_true",
                    help="leave out the skeleton Fock build of the default line")
    ap.add_argument("--no-batched", action="store_true",
                    help="leave out the 48-instance batched leg of the default line")
    ap.add_argument("--half-buckets", action="store_true",
                    help="rotran's own half-transformed intermediate (rt_config.half_buckets = 1)")
    ap.add_argument("--per-class", action="store_true",
                    help="also split vs FP64 per AO integral class (3 + 3 extra transforms)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    hbm_peak, bf16_peak, peak_kind = peaks()
    if args.workload == "batched":
        return run_batched(args, rank, world, local, bf16_peak, peak_kind)
    if args.workload == "gemm":
        return run_gemm_case(args, rank)
    if args.workload == "files":
        return run_files_case(args, rank)
    if args.workload == "breit":
        return run_breit_case(args, rank)
    if args.workload in ("fock", "fock_small"):
        return run_fock_case(args, rank, hbm_peak, peak_kind)
    work = {"precision": WORKLOAD, "c1": SMALL, "profile": PROFILE, "profile2": PROFILE2,
            "large": LARGE}[args.workload]

    if args.impl == "reference":
        if rank != 0:
            return
        from molfdir_gb300 import synth
        rprob = synth.make_spinor_problem(work["n_l"], work["n_s"], work["nkr"], seed=work["seed"],
                                          n_irrep=work.get("n_irrep", 1))
        config = workload_config(work, rprob, args.gpus)
        del rprob
        res, cores = cpu_sample(work, steps=args.steps, warmup=args.warmup)
        line = {"metric": "4-index transform TFLOP/s", "impl": "reference",
                "value": res["tflops"], "unit": "TFLOP/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": res["tflops"], "unit": "TFLOP/s", "cores": cores,
                                 "kind": "port", "sample": res["sample"],
                                 "seconds_first_half": res["seconds_first_half"],
                                 "seconds_second_half": res["seconds_second_half"]},
                "e2e": {"value": res["tflops"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from molfdir_gb300 import rotran, synth

    prec_name = "fp64" if args.precision == "fp64" else "split"
    prec = rotran.RT_PREC_SPLIT_BF16 if prec_name == "split" else rotran.RT_PREC_FP64
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)

    prob = synth.make_spinor_problem(work["n_l"], work["n_s"], work["nkr"], seed=work["seed"],
                                     n_irrep=work.get("n_irrep", 1))
    config = workload_config(work, prob, world)
    cls, its, nts, dv, dl2, dl1 = synth.device_records(prob, 3, device="cuda")
    torch.cuda.synchronize()
    nint = int(nts.sum())
    assert nint == config["integrals"], "generator and workload count disagree"

    def make_ctx(p, slices):
        rt = rotran.Rotran.for_problem(prob, precision=p, slices=slices, half_buckets=args.half_buckets)
        rt.set_problem_coefficients(prob)
        return rt

    def run_leg(p, slices, warmup, steps, clocks=False):
        rt = make_ctx(p, slices)
        rt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
        for _ in range(warmup):
            rt.transform()
        barrier()
        torch.cuda.synchronize()
        gemm_ms, dev_ms = [], []
        sampler = ClockSampler(local) if clocks else None
        if sampler:
            sampler.__enter__()
        t0 = time.perf_counter()
        for _ in range(steps):
            rt.transform()
            st = rt.stats()
            gemm_ms.append(st.ms_gemm)
            dev_ms.append(st.ms_total)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if sampler:
            sampler.__exit__(None, None, None)
        barrier()
        sec = barrier_max(max((t1 - t0) / steps, statistics.mean(dev_ms) / 1e3), world)
        res = rt.result()
        out = dict(sec=sec, stats=st, gemm_ms=statistics.mean(gemm_ms),
                   clocks=sampler.summary() if sampler else None, result=res)
        rt.close()
        return out

    # ---- value: records resident in HBM ----
    main = run_leg(prec, args.slices, args.warmup, args.steps, clocks=True)
    st = main["stats"]
    flops = st.flops_algorithmic
    value = flops * world / main["sec"] / 1e12
    hdr, idx, val = main["result"]
    nrec, nz = hdr.shape[0], idx.shape[0]

    # ---- e2e through the public API with host buffers ----
    e2e = None
    if not args.no_e2e:
        hv, h2, h1 = (x.cpu().pin_memory() for x in (dv, dl2, dl1))
        rt = make_ctx(prec, args.slices)
        ehdr = np.empty((nrec, 3), np.int32)
        eidx = torch.empty((nz, 2), dtype=torch.int32).pin_memory()
        evalt = torch.empty((nz, 2), dtype=torch.float64).pin_memory()
        eidx_np, eval_np = eidx.numpy(), evalt.numpy().view(np.complex128).reshape(-1)

        # per-class views of the pinned element buffers, in rt_copy_result's order
        sizes = [int(x) for x in st.nfinal]
        z = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        cidx = [eidx_np[z[c]:z[c + 1]] for c in range(4)]
        cval = [eval_np[z[c]:z[c + 1]] for c in range(4)]
        phase = [0.0, 0.0, 0.0]

        def e2e_step(stream):
            a = time.perf_counter()
            rt.clear_records()
            rt.add_records_bulk_ptr(cls, nts, its, hv.data_ptr(), h2.data_ptr(), h1.data_ptr())
            b = time.perf_counter()
            rt.transform()
            c = time.perf_counter()
            if stream:   # the elements are already on the host
                ehdr[:] = rt.headers()
            else:
                rt.result(ehdr, eidx_np, eval_np)
            d = time.perf_counter()
            for i, v in enumerate((b - a, c - b, d - c)):
                phase[i] += v

        def e2e_leg(stream):
            rt.set_result_host(cidx, cval) if stream else rt.set_result_host()
            e2e_step(stream)
            barrier()
            ne = max(1, min(args.steps, 3))
            phase[:] = [0.0, 0.0, 0.0]
            t0 = time.perf_counter()
            for _ in range(ne):
                e2e_step(stream)
            t1 = time.perf_counter()
            esec = barrier_max((t1 - t0) / ne, world)
            return esec, [x * 1e3 / ne for x in phase]

        def e2e_pipelined(ne):
            # step 0's records copied first, inside the timed region; step k+1's
            # queued before step k so that they copy while step k runs; each
            # step's last element copies finish during the next step's first
            # half, the final step's inside the timed region
            rt.set_result_host(cidx, cval)
            rt.set_result_host_deferred(True)
            t0 = time.perf_counter()
            rt.clear_records()
            rt.add_records_bulk_ptr(cls, nts, its, hv.data_ptr(), h2.data_ptr(), h1.data_ptr())
            for k in range(ne):
                if k + 1 < ne:
                    rt.queue_records_bulk_ptr(cls, nts, its, hv.data_ptr(), h2.data_ptr(), h1.data_ptr())
                rt.transform()
            rt.result_host_wait()
            ehdr[:] = rt.headers()
            t1 = time.perf_counter()
            rt.set_result_host_deferred(False)
            return t1 - t0

        ssec, ph = e2e_leg(True)
        ne = max(1, min(args.steps, 3))
        e2e_pipelined(2)   # warm-up of the queue path
        barrier()
        esec = barrier_max(e2e_pipelined(ne) / ne, world)
        ok = np.array_equal(ehdr, hdr) and np.array_equal(eidx_np, idx) and \
            np.array_equal(eval_np.view(np.float64), val.view(np.float64))
        usec, uph = e2e_leg(False)
        e2e = {"value": flops * world / esec / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": nint * 16, "d2h_bytes_per_step": nz * 24 + nrec * 12,
               "ms_per_step": esec * 1e3, "steps": ne,
               "h2d": "step k+1's records queued during step k (rt_queue_ao_records_bulk); "
                      "step 0's copied first, inside the timed region",
               "d2h": "per item chunk, overlapping the transform (rt_set_result_host); the last "
                      "chunk's copies overlap the next step (rt_set_result_host_deferred)",
               "streamed_equals_resident_result": bool(ok),
               "h2d_GBps": nint * 16 / (ph[0] / 1e3) / 1e9,
               "sequential": {"value": flops * world / ssec / 1e12, "ms_per_step": ssec * 1e3,
                              "ms_records_in": ph[0], "ms_transform_and_results": ph[1],
                              "ms_headers": ph[2]},
               "copied_after": {"value": flops * world / usec / 1e12, "ms_per_step": usec * 1e3,
                                "ms_transform": uph[1], "ms_results_out": uph[2],
                                "d2h_GBps": (nz * 24 + nrec * 12) / (uph[2] / 1e3) / 1e9}}
        rt.close()
        del hv, h2, h1, eidx, evalt

    # ---- plain FP64 GPU transform: the comparison leg and accuracy reference ----
    fp64 = None
    ref_result = None
    if prec_name == "split" and not args.no_fp64:
        ref = run_leg(rotran.RT_PREC_FP64, 0, 0, 1)
        ref_result = ref["result"]
        rh, ri, rv = ref["result"]
        acc = {}
        if np.array_equal(rh, hdr) and np.array_equal(ri, idx):
            # chunked: the large workload holds ~1.6e9 elements per leg
            mx = ss = mv = 0.0
            for a in range(0, val.size, 1 << 26):
                d = np.abs(val[a:a + (1 << 26)] - rv[a:a + (1 << 26)])
                mx = max(mx, float(d.max()))
                ss += float(np.dot(d, d))
                mv = max(mv, float(np.abs(rv[a:a + (1 << 26)]).max()))
            acc = {"max_abs_err": mx, "rms_err": float(np.sqrt(ss / max(1, val.size))),
                   "max_abs_value": mv, "same_elements": True}
        else:
            acc = {"same_elements": False}
        fp64 = {"value": flops * world / ref["sec"] / 1e12, "unit": "TFLOP/s",
                "ms_per_step": ref["sec"] * 1e3, "steps": 1, "warmup": 0,
                "split_speedup": ref["sec"] / main["sec"], "split_vs_fp64": acc}

    # ---- split vs FP64 per AO integral class, each class transformed alone ----
    per_class = None
    if args.per_class and prec_name == "split" and rank == 0:
        per_class = {}
        ends = np.cumsum(nts)
        starts = ends - nts
        for c, name in ((1, "(LL|LL)"), (2, "(SS|LL)"), (3, "(SS|SS)")):
            sel = np.nonzero(cls == c)[0]
            if sel.size == 0:
                continue
            a, b = int(starts[sel[0]]), int(ends[sel[-1]])  # a class's records are contiguous
            outs = []
            for p_, s_ in ((prec, args.slices), (rotran.RT_PREC_FP64, 0)):
                rt = make_ctx(p_, s_)
                rt.add_records_bulk_ptr(cls[sel], nts[sel], its[sel], dv[a:].data_ptr(),
                                        dl2[a:].data_ptr(), dl1[a:].data_ptr())
                rt.transform()
                outs.append(rt.result())
                rt.close()
            (h1, i1, v1), (h2, i2, v2) = outs
            if np.array_equal(h1, h2) and np.array_equal(i1, i2):
                mx = ss = mv = 0.0
                for q in range(0, v1.size, 1 << 26):
                    d = np.abs(v1[q:q + (1 << 26)] - v2[q:q + (1 << 26)])
                    mx = max(mx, float(d.max()))
                    ss += float(np.dot(d, d))
                    mv = max(mv, float(np.abs(v2[q:q + (1 << 26)]).max()))
                per_class[name] = {"integrals": int(b - a), "max_abs_err": mx,
                                   "rms_err": float(np.sqrt(ss / max(1, v1.size))),
                                   "max_abs_value": mv, "same_elements": True}
            else:
                per_class[name] = {"integrals": int(b - a), "same_elements": False}
        if fp64 is not None:
            fp64["split_vs_fp64_per_class"] = per_class
            per_class = None  # reported inside the fp64 object

    # ---- CPU baseline (rank 0, N = 1) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        res, cores = cpu_sample(work)
        cpu = {"value": res["tflops"], "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": res["sample"]}

    # ---- tmoone's skeleton Fock build over the same resident records ----
    fock = None
    if work["name"] == WORKLOAD["name"] and not args.no_fock:
        ntri = prob.n * (prob.n + 1) // 2
        gen = torch.Generator(device="cuda").manual_seed(0)
        d1 = torch.randn((1, 4, ntri), device="cuda", dtype=torch.float64, generator=gen)
        d2 = torch.randn((1, 4, ntri), device="cuda", dtype=torch.float64, generator=gen)
        with rotran.Rotran.for_problem(prob) as frt:
            frt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
            for _ in range(2):
                frt.fock_skeleton(d1)
            fms = []
            for _ in range(3):
                f1, k = frt.fock_skeleton(d1)
                fms.append(k)
            f2, _ = frt.fock_skeleton(d2)
            f12, _ = frt.fock_skeleton(d1 + d2)
            lin = float((f12 - f1 - f2).abs().max() / f12.abs().max())
        fmean = statistics.mean(fms)
        fock = {"workload": "skeleton Fock build (MFDFOCK/FOCK) over these records, one density set",
                "value": nint / (fmean / 1e3), "unit": "integrals/s", "ms_kernel": fmean,
                "steps": 3, "warmup": 2, "linearity_rel_err": lin,
                "hbm_frac": 16.0 * nint / (fmean / 1e3) / 1e9 / hbm_peak}

    # ---- the batched workload (48 instances, one CUDA graph) beside it ----
    batched = None
    if work["name"] == WORKLOAD["name"] and not args.no_batched and prec_name == "split":
        b = batched_leg(args, world, local, steps=3, warmup=2, with_fp64=not args.no_fp64,
                        oracle=rank == 0)
        batched = {"workload": "batched_48 (48 instances, n_AO 40..200, 16..80 Kramers pairs, seeds 0..47)",
                   "value": b["value"], "unit": "TFLOP/s", "ms_per_step": b["sec"] * 1e3, "steps": 3,
                   "warmup": 2, "flops_algorithmic": b["flops"], "fp64": b["fp64"],
                   "oracle_check": b["oracle_check"], "clocks": b["clocks"],
                   "graph": {k: v for k, v in b["bst"].as_dict().items()
                             if k in ("grouped_launches", "kernel_launches", "graph_nodes", "tile128", "tile64")}}

    # ---- the streams against the oracle's digest of this workload ----
    ocheck = None
    if rank == 0 and work["name"] == WORKLOAD["name"]:
        tol = 1e-10 if prec_name == "split" else 1e-12
        ocheck = {prec_name: oracle_check(main["result"], tol)}
        if ref_result is not None:
            ocheck["fp64"] = oracle_check(ref_result, 1e-12)
        if ocheck[prec_name] is None:
            ocheck = {"unavailable": "tests/golden/oracle_digest_n400_k120.npz missing"}
        else:
            ocheck[prec_name]["nhalft"] = int(st.nhalft)

    if rank == 0:
        gsec = main["gemm_ms"] / 1e3
        if prec_name == "split":
            # algorithmic FLOPs (each product counted once) against the BF16
            # peak divided by the digit products one algorithmic product costs
            prods = args.slices * (args.slices + 1) // 2
            achieved = st.flops_gemm_algorithmic / gsec / 1e12
            executed = st.flops_gemm_executed / gsec / 1e12
            roof = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak / prods,
                    "unit": "TFLOP/s", "frac": achieved / (bf16_peak / prods),
                    "traffic": TRAFFIC.get(work["name"]),
                    "traffic_source": TRAFFIC_SOURCE if work["name"] in TRAFFIC else None,
                    "kernel": "k_split_gemm (tcgen05 BF16 digit products)",
                    "peak_source": f"bf16_tflops of {peak_kind} / {prods} digit products",
                    "executed_tflops": executed, "executed_frac": executed / bf16_peak,
                    "gemm_launches": st.gemm_launches,
                    "traffic_unit": "DRAM bytes per launch (ncu)"}
        else:
            achieved = st.flops_gemm_algorithmic / gsec / 1e12 if gsec > 0 else None
            roof = {"bound": "fp64", "achieved": achieved, "peak": None, "unit": "TFLOP/s",
                    "frac": None, "traffic": None, "kernel": "k_gemm_f64"}
        line = {
            "metric": "4-index transform TFLOP/s", "value": value, "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": main["sec"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16-slices/f32-acc (split)" if prec_name == "split" else "f64",
            "data": "synthetic",
            "config": config,
            "precision": {"path": prec_name, "slices": args.slices if prec_name == "split" else None,
                          "half_buckets": bool(args.half_buckets)},
            "tflops_dense_equivalent": config["flops_dense_equivalent"] * world / main["sec"] / 1e12,
            "oracle_check": ocheck,
            "batched": batched, "fock": fock,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "fp64": fp64,
            "gpu_launches": st.gpu_launches * args.steps, "clocks": main["clocks"],
            "stats": st.as_dict(), "mdcint": {"records": nrec, "elements": nz},
        }
        if per_class is not None:
            line["split_vs_fp64_per_class"] = per_class
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
