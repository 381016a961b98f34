"""tmoone's skeleton Fock build on the GPU (rt_fock_skeleton) against the
oracle's restatement of MFDFOCK/FOCK (needs a GB300).

The GPU adds every integral's terms with FP64 atomics, in another order
than FOCK's sequential loop, so the sets agree to rounding:
|F_gpu - F_oracle| <= 1e-12 max|F| per array.  Covered: all fourteen
integral types (every synthetic problem has them), one and two density sets,
MFIL = 1, 2, 3 (files above MFIL and the Gaunt file are not read), AO irrep
blocks, records given one by one (staged) or in bulk, host and device
arrays, and the label check."""

import numpy as np
import pytest
import torch

import pyoracle
from molfdir_gb300 import rotran, synth

pytestmark = pytest.mark.gpu

TOL = 1e-12


def random_density(n, nmat, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nmat, 4, n * (n + 1) // 2))


def check(got, want):
    """Per array: |got - want| <= 1e-12 of the array's largest element."""
    for s in range(want.shape[0]):
        for x in range(4):
            scale = np.abs(want[s, x]).max()
            assert scale > 0, (s, x)
            err = np.abs(got[s, x] - want[s, x]).max()
            assert err <= TOL * scale, (s, x, err, scale)


@pytest.mark.parametrize("nl,ns,nkr,seed,irrep,nmat", [(3, 4, 2, 0, 1, 1), (4, 6, 3, 1, 1, 2),
                                                       (6, 9, 3, 2, 4, 2), (12, 20, 4, 3, 1, 1),
                                                       (24, 40, 4, 4, 1, 2), (40, 60, 4, 5, 4, 1)])
def test_fock_skeleton_matches_the_oracle(nl, ns, nkr, seed, irrep, nmat):
    p = synth.make_problem(nl, ns, nkr, seed=seed, n_irrep=irrep)
    recs = p.flat_records()
    dens = random_density(p.n, nmat, seed)
    want = pyoracle.fock_skeleton(recs, p.n, dens, mfil=p.mfil)
    with rotran.Rotran.for_problem(p) as rt:
        rt.add_problem_records(p)
        got, ms = rt.fock_skeleton(dens)
    assert ms > 0
    check(got, want)


@pytest.mark.parametrize("mfil,ns", [(1, 0), (2, 9), (3, 9)])
def test_files_above_mfil_and_the_gaunt_file_are_not_read(mfil, ns):
    # MFIL = 1 contexts hold large-component functions only (NSC = NSC1)
    p = synth.make_problem(6, ns, 3, seed=7, breit=True)
    recs = p.flat_records()
    assert ns == 0 or 4 in set(recs[0].tolist())
    dens = random_density(p.n, 1, 7)
    want = pyoracle.fock_skeleton(recs, p.n, dens, mfil=mfil)
    cfg, keep = rotran.make_config(p.n, p.nsc1, p.nkr, mfil=mfil)
    with rotran.Rotran(cfg, keep) as rt:
        rt.add_problem_records(p)
        got, _ = rt.fock_skeleton(dens)
    check(got, want)


def test_staged_records_and_device_arrays():
    p = synth.make_problem(8, 12, 3, seed=9)
    recs = p.flat_records()
    dens = random_density(p.n, 2, 9)
    want = pyoracle.fock_skeleton(recs, p.n, dens, mfil=p.mfil)
    with rotran.Rotran.for_problem(p) as rt:
        rt.add_problem_records(p, bulk=False)   # one rt_add_ao_records call per record
        got, _ = rt.fock_skeleton(dens)
        check(got, want)
        dd = torch.from_numpy(dens).cuda()
        gd, _ = rt.fock_skeleton(dd)
        assert gd.is_cuda
        check(gd.cpu().numpy(), want)
        again, _ = rt.fock_skeleton(dens)   # repeatable: the Fock arrays start from zero
        check(again, want)


def test_label_outside_nsc_is_refused():
    p = synth.make_problem(3, 4, 2, seed=0)
    cls, its, nts, v, l2, l1 = p.flat_records()
    l1 = l1.copy()
    l1[5] = (p.n + 3) << 16 | 1
    with rotran.Rotran.for_problem(p) as rt:
        rt.add_records_bulk(cls, nts, its, v, l2, l1)
        with pytest.raises(rotran.RotranError) as e:
            rt.fock_skeleton(random_density(p.n, 1, 0))
        assert e.value.code == rotran.RT_ERR_USER and "label" in str(e.value)


# ---- tmoone's Gaunt contributions (MFDBREIT/GAUNT) ----

@pytest.mark.parametrize("nl,ns,nkr,seed,nmat", [(3, 4, 2, 0, 1), (6, 9, 3, 1, 2), (12, 20, 4, 2, 1),
                                                 (24, 40, 4, 3, 2)])
def test_gaunt_contributions_match_the_oracle(nl, ns, nkr, seed, nmat):
    """ONLYBRT (zeroed sets) and BREIT (added to MFDFOCK's sets)."""
    p = synth.make_problem(nl, ns, nkr, seed=seed, breit=True)
    recs = p.flat_records()
    dens = random_density(p.n, nmat, seed)
    coul = pyoracle.fock_skeleton(recs, p.n, dens, mfil=p.mfil)
    only = pyoracle.fock_gaunt(recs, p.n, dens)
    both = pyoracle.fock_gaunt(recs, p.n, dens, fock=coul)
    assert np.abs(only).max() > 0
    with rotran.Rotran.for_problem(p) as rt:   # a Coulomb context also holds file 4
        rt.add_problem_records(p)
        got_only, ms = rt.fock_gaunt(dens)
        f, _ = rt.fock_skeleton(dens)
        got_both, _ = rt.fock_gaunt(dens, f)
    assert ms > 0
    check(got_only, only)
    check(got_both, both)


def test_gaunt_refuses_the_types_gaunt_rejects():
    p = synth.make_problem(3, 4, 2, seed=0, breit=True)
    cls, its, nts, v, l2, l1 = p.flat_records()
    its = its.copy()
    its[np.nonzero(cls == 4)[0][0]] = 12
    with rotran.Rotran.for_problem(p) as rt:
        rt.add_records_bulk(cls, nts, its, v, l2, l1)
        with pytest.raises(rotran.RotranError) as e:
            rt.fock_gaunt(random_density(p.n, 1, 0))
        assert e.value.code == rotran.RT_ERR_PROGRAM and "INVALID TYPE IN BREIT" in str(e.value)
        rt.fock_skeleton(random_density(p.n, 1, 0))   # FOCK takes type 12
