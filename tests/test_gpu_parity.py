"""GPU transformation vs the CPU oracle, through the C-ABI (needs a GB300)."""

import numpy as np
import pytest

import pyoracle
from molfdir_gb300 import fortio, rotran, synth
from util import check_rdtwo_reconstruction, compare_streams, dense_full, permute_spinors

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def run_gpu(p, precision=rotran.RT_PREC_FP64, bulk=True, **kw):
    with rotran.Rotran.for_problem(p, precision=precision, **kw) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p, bulk=bulk)
        rt.transform()
        out = rt.result()
        st = rt.stats()
    return out, st


def ref_stream(p, **kw):
    img = pyoracle.run(p, **kw)
    return img, (img.hdr, img.idx, img.val)


@pytest.mark.parametrize("nl,ns,nkr,mfil,seed", [
    (3, 4, 2, 3, 0), (6, 8, 4, 3, 1), (6, 8, 4, 2, 2), (7, 0, 3, 1, 3), (1, 1, 1, 3, 4),
    (5, 9, 5, 3, 5), (12, 20, 10, 3, 6)])
def test_fp64_small(nl, ns, nkr, mfil, seed):
    p = synth.make_problem(nl, ns, nkr, seed=seed, mfil=mfil)
    img, ref = ref_stream(p)
    got, st = run_gpu(p)
    err = compare_streams(got, ref, TOL_FP64)
    assert err <= TOL_FP64, err
    assert list(st.nfinal) == [int(x) for x in img.nfinal]


def test_fp64_config1_n64_k32():
    """The CPU-sized case: 24 L + 40 S functions, 32 Kramers pairs, seed 0."""
    p = synth.make_problem(24, 40, 32, seed=0)
    img, ref = ref_stream(p)
    got, st = run_gpu(p)
    err = compare_streams(got, ref, TOL_FP64)
    assert err <= TOL_FP64, err
    assert st.gpu_launches > 0


def test_fp64_shuffled_spinors():
    p = synth.make_problem(6, 10, 5, seed=12)
    q = permute_spinors(p, np.random.default_rng(1).permutation(p.m))
    _, ref = ref_stream(q)
    got, _ = run_gpu(q)
    assert compare_streams(got, ref, TOL_FP64) <= TOL_FP64


def test_fp64_irrep_blocks():
    p = synth.make_problem(10, 14, 5, seed=13, n_irrep=4)
    _, ref = ref_stream(p)
    got, _ = run_gpu(p)
    assert compare_streams(got, ref, TOL_FP64) <= TOL_FP64


@pytest.mark.parametrize("thrgen,throut", [(1e-16, 1e-3), (1e-16, -1.0), (1e-5, 1e-16)])
def test_fp64_thresholds(thrgen, throut):
    p = synth.make_problem(6, 8, 4, seed=14)
    _, ref = ref_stream(p, thrgen=thrgen, throut=throut)
    got, _ = run_gpu(p, thrgen=thrgen, throut=throut)
    # TROUT's test |H| < THRGEN / (VMX(p) VMX(q)) (trout.F:30-43) is applied
    # to different intermediates: rotran's TRANS1 transforms bucket pq, which
    # holds only the integrals (rs|pq) sorted under pq (rs >= pq), and adds
    # the pair-interchanged part later (OUTPP2/PPSYM); the GPU's bucket holds
    # every (pq|rs), so its half-transformed value is the complete sum over
    # rs.  With the default THRGEN = 1e-16 (readin.F:93) both screens drop
    # only values below rounding and the streams agree to 1e-12; a coarse
    # THRGEN drops different values, hence the looser tolerance here.
    tol = TOL_FP64 if thrgen <= 1e-16 else 1e-4
    # with a large THROUT the reference drops canonical or pp-interchanged
    # halves below THROUT before summing them (outpp1.F:34, outpp2.F:40)
    tol = max(tol, throut)
    assert compare_streams(got, ref, tol, presence_tol=max(tol, 2 * throut)) <= tol


FP64, SPLIT = rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16


# (the split path screens in FP32, so a coarse THRGEN is checked on FP64)
@pytest.mark.parametrize("thrgen,throut,precision", [
    (1e-16, 1e-16, FP64), (1e-5, 1e-16, FP64), (1e-3, 1e-16, FP64), (1e-16, 1e-3, FP64), (1e-6, 1e-4, FP64),
    (1e-16, -1.0, FP64), (1e-16, 1e-16, SPLIT), (1e-16, 1e-3, SPLIT), (1e-16, -1.0, SPLIT)])
def test_half_buckets_are_rotrans_intermediate(thrgen, throut, precision):
    """half_buckets = 1: each integral under its LABEL1 pair only (SORT1), so
    TROUT's THRGEN screen sees rotran's own half-transformed values and the
    records add OUTPP1's and OUTPP2's halves, each tested against THROUT, as
    PPSYM does: the same stream as the oracle at any thresholds, and the same
    NHALFT."""
    p = synth.make_problem(6, 8, 4, seed=14)
    img, ref = ref_stream(p, thrgen=thrgen, throut=throut)
    got, st = run_gpu(p, precision=precision, thrgen=thrgen, throut=throut, half_buckets=True)
    tol = TOL_FP64 if precision == rotran.RT_PREC_FP64 else 1e-10
    # the split path's values differ from the oracle's by rounding, so an
    # element within that of THROUT may be present on one side only
    assert compare_streams(got, ref, tol, presence_tol=abs(throut) + tol) <= tol
    if precision == rotran.RT_PREC_FP64:
        assert st.nhalft == img.nhalft
        assert list(st.nfinal) == [int(x) for x in img.nfinal]


@pytest.mark.parametrize("precision", [FP64, SPLIT], ids=["fp64", "split"])
def test_half_buckets_irrep_blocks_and_shuffled_spinors(precision):
    """rotran's intermediate over the 4-irrep AO block structure and with the
    spinors in a shuffled order, at a coarse THRGEN (FP64) and the default
    (split)."""
    thrgen = 1e-5 if precision == FP64 else 1e-16
    tol = TOL_FP64 if precision == FP64 else 1e-10
    p = synth.make_problem(10, 14, 5, seed=13, n_irrep=4)
    img, ref = ref_stream(p, thrgen=thrgen)
    got, st = run_gpu(p, precision=precision, thrgen=thrgen, half_buckets=True)
    assert compare_streams(got, ref, tol) <= tol
    q = permute_spinors(synth.make_problem(6, 10, 5, seed=12), np.random.default_rng(1).permutation(10))
    img_q, ref_q = ref_stream(q, thrgen=thrgen)
    got_q, st_q = run_gpu(q, precision=precision, thrgen=thrgen, half_buckets=True)
    assert compare_streams(got_q, ref_q, tol) <= tol
    if precision == FP64:
        assert st.nhalft == img.nhalft and st_q.nhalft == img_q.nhalft


def test_per_record_calls_and_srt_files_match_bulk(tmp_path):
    p = synth.make_problem(6, 8, 4, seed=15)
    bulk, _ = run_gpu(p, bulk=True)
    per, _ = run_gpu(p, bulk=False)
    fortio.write_srt_files(p, str(tmp_path))
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        rt.read_srt_files(str(tmp_path))
        rt.transform()
        files = rt.result()
    for other in (per, files):
        assert np.array_equal(other[0], bulk[0]) and np.array_equal(other[1], bulk[1])
        assert np.max(np.abs(other[2] - bulk[2])) <= 1e-15


@pytest.mark.parametrize("precision", [rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16],
                         ids=["fp64", "split"])
def test_srtpq_files_match_the_oracle(tmp_path, precision):
    """The MPI version's pq-sorted files (three ranks, short records, repeated
    entries, Breit streams to skip) give the serial files' result."""
    p = synth.make_problem(7, 9, 4, seed=19)
    img, ref = ref_stream(p)
    fortio.write_srtpq_files(p, str(tmp_path), nranks=3, nbuf=24, split_every=4, breit_pairs=3)
    with rotran.Rotran.for_problem(p, precision=precision) as rt:
        rt.set_problem_coefficients(p)
        rt.read_srtpq_files(str(tmp_path), nranks=3)
        rt.transform()
        got = rt.result()
        st = rt.stats()
    fp64 = precision == rotran.RT_PREC_FP64
    tol = TOL_FP64 if fp64 else 1e-10
    assert compare_streams(got, ref, tol) <= tol
    if fp64:
        assert list(st.nfinal) == [int(x) for x in img.nfinal]


@pytest.mark.parametrize("precision", [rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16],
                         ids=["fp64", "split"])
def test_stream_reconstructs_the_tensor_as_a_reader_does(precision):
    """The GPU's MDCINT stream, expanded as goscip's RDTWO expands it
    (rdtwo.F:29-83), gives the whole dense (ij|kl): every quadruple reached,
    every implied value consistent."""
    p = permute_spinors(synth.make_problem(5, 7, 4, seed=20),
                        np.random.default_rng(3).permutation(8))
    (hdr, idx, val), _ = run_gpu(p, precision=precision)
    dense = dense_full(p)
    scale = max(1.0, float(np.abs(dense).max()))
    tol = (TOL_FP64 if precision == rotran.RT_PREC_FP64 else 1e-10) * scale
    check_rdtwo_reconstruction(hdr, idx, val, p.kra, p.krb, dense, tol=tol, throut=1e-16)


def test_no_integrals():
    """No records at all: every MDCINT record is written, with no elements,
    as the oracle writes it."""
    p = synth.make_problem(4, 5, 3, seed=21)
    empty = (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int64),
             np.zeros(0), np.zeros(0, np.int32), np.zeros(0, np.int32))
    img = pyoracle.run(p, records=empty)
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        rt.transform()
        hdr, idx, val = rt.result()
    assert np.array_equal(hdr, img.hdr) and idx.shape[0] == 0 == img.idx.shape[0]
    assert np.all(hdr[:, 2] == 0)


def test_files_above_mfil_are_not_read():
    """SORT1 reads files 1..MFIL only (sort1.F:60): (SS|SS) records added to
    an MFIL = 2 transform change nothing."""
    p2 = synth.make_problem(5, 6, 3, seed=22, mfil=2)
    p3 = synth.make_problem(5, 6, 3, seed=22, mfil=3)
    base, _ = run_gpu(p2)
    with rotran.Rotran.for_problem(p2) as rt:
        rt.set_problem_coefficients(p2)
        rt.add_problem_records(p2)
        for r in p3.files["SS"]:
            rt.add_record(3, r.it, r.rint, r.label2, r.label1)
        rt.transform()
        more = rt.result()
    assert all(np.array_equal(a, b) for a, b in zip(base[:2], more[:2]))
    assert np.max(np.abs(base[2] - more[2])) <= 1e-15


def test_mdcint_file(tmp_path):
    p = synth.make_problem(6, 8, 4, seed=16)
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        hdr, idx, val = rt.result()
        rt.write_mdcint(str(tmp_path / "MDCINT"), "03Dec2026", "12:00:00")
    datex, timex, nkr, pairs, h2, i2, v2 = fortio.read_mdcint(str(tmp_path / "MDCINT"))
    assert nkr == p.nkr and datex.startswith("03Dec2026") and timex == "12:00:00"
    assert np.array_equal(pairs, p.imoras_pairs())
    assert np.array_equal(h2, hdr) and np.array_equal(i2, idx) and np.array_equal(v2, val)


def test_repeat_transform_is_deterministic():
    p = synth.make_problem(6, 8, 4, seed=17)
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        rt.add_problem_records(p)
        rt.transform()
        a = rt.result()
        rt.transform()
        b = rt.result()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_bad_inputs_raise():
    p = synth.make_problem(3, 4, 2, seed=18)
    with rotran.Rotran.for_problem(p) as rt:
        rt.set_problem_coefficients(p)
        # label out of range
        rt.add_record(1, 12, [0.1], [(9 << 16) | 1], [(2 << 16) | 1])
        with pytest.raises(rotran.RotranError) as e:
            rt.transform()
        assert e.value.code == 2
        rt.clear_records()
        # mixed L/S pair in the r,s labels of an LL bucket
        rt.add_record(1, 12, [0.1], [(5 << 16) | 1], [(2 << 16) | 1])
        with pytest.raises(rotran.RotranError) as e:
            rt.transform()
        assert e.value.code == 2
        rt.clear_records()
        rt.add_problem_records(p)
        rt.transform()
    with rotran.Rotran.for_problem(p) as rt:
        bad = p.itrmo.copy()
        bad[0] = 3
        with pytest.raises(rotran.RotranError) as e:
            rt.set_coefficients(p.qa, bad, p.kra, p.krb, p.ikrmo)
        assert e.value.code == 6
