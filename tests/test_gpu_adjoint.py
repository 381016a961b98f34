"""Adjoint (dE/dC) of the transformation through rt_adjoint, against an FP64
torch autograd reference and central finite differences (needs a GB300).

E(C) = sum_{ijkl} Gamma_ijkl (ij|kl) with (ij|kl) = sum Omega_ij G Omega_kl,
Omega_ij(p,q) = conj(C_pi) C_qj + s_ij conj(C_q jbar) C_p ibar.  The
reference evaluates it through the generator's low-rank factor
G(pq|rs) = sum_Q B_Q(p,q) B_Q(r,s), so it never forms the AO tensor."""

import numpy as np
import pytest

from molfdir_gb300 import rotran, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def b_factor(model, dev):
    """B_Q(p,q) as a (Q, n, n) symmetric tensor (zero on SL pairs)."""
    n, nq = model.n, model.bl.shape[1]
    b = torch.zeros((nq, n, n), dtype=torch.float64, device=dev)
    for pl, ql, bb in ((model.pl, model.ql, model.bl), (model.ps, model.qs, model.bs)):
        if len(pl) == 0:
            continue
        p = torch.as_tensor(pl - 1, device=dev)
        q = torch.as_tensor(ql - 1, device=dev)
        bt = torch.as_tensor(bb, device=dev).T
        b[:, p, q] = bt
        b[:, q, p] = bt
    return b


def make_gamma(m, seed, dev):
    """Random two-particle density with the integrals' symmetries: pair
    exchange and Hermiticity; entries N(0,1) exp(-0.05 (i+j+k+l))."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    shape = (m, m, m, m)
    x = torch.complex(torch.randn(shape, generator=g, dtype=torch.float64),
                      torch.randn(shape, generator=g, dtype=torch.float64)).to(dev)
    i = torch.arange(m, device=dev, dtype=torch.float64)
    w = torch.exp(-0.05 * (i[:, None, None, None] + i[None, :, None, None] +
                           i[None, None, :, None] + i[None, None, None, :]))
    x = x * w
    x = 0.5 * (x + x.permute(2, 3, 0, 1))
    x = 0.5 * (x + x.permute(1, 0, 3, 2).conj())
    return x.contiguous()


class EnergyRef:
    def __init__(self, prob, gamma, dev):
        self.b = b_factor(prob.model, dev).to(torch.complex128)
        itr = torch.as_tensor(prob.itrmo, device=dev)
        self.bar = itr.abs() - 1
        sg = torch.sign(itr).to(torch.float64)
        self.sig = (sg[:, None] * sg[None, :]).to(torch.complex128)
        m = gamma.shape[0]
        self.gmat = gamma.reshape(m * m, m * m)

    def __call__(self, c):
        t = c.conj().T @ (self.b @ c)                      # (Q, m, m): C^H B_Q C
        tt = t.transpose(1, 2)
        v = t + self.sig * tt[:, self.bar][:, :, self.bar]  # + s_ij T(jbar, ibar)
        vf = v.reshape(v.shape[0], -1)
        return ((vf @ self.gmat) * vf).sum().real


class TransformEnergy(torch.autograd.Function):
    """E(C) through rt_adjoint; backward returns the library's dE/dC."""

    @staticmethod
    def forward(ctx, c, rt, prob, gamma_ptr):
        rt.set_coefficients(c.detach().cpu().numpy(), prob.itrmo, prob.kra, prob.krb,
                            prob.ikrmo, prob.imoras_pairs())
        g, e = rt.adjoint(gamma_ptr)
        ctx.save_for_backward(torch.as_tensor(g, device=c.device))
        return torch.tensor(e, dtype=torch.float64, device=c.device)

    @staticmethod
    def backward(ctx, go):
        (g,) = ctx.saved_tensors
        return go * g, None, None, None


def fortran_ptr(gamma):
    """Device copy of gamma in Fortran order (i fastest); keep it alive."""
    gf = gamma.permute(3, 2, 1, 0).contiguous()
    return gf, gf.data_ptr()


FP64, SPLIT = rotran.RT_PREC_FP64, rotran.RT_PREC_SPLIT_BF16
# relative error bounds of E and of max|dE/dC| against the FP64 reference
TOL = {FP64: (1e-10, 1e-10), SPLIT: (2e-10, 2e-10)}  # split: 6 slices


def run_case(prob, records_on_device, seed, ndir, check_lib_fd=0, fd_tol=1e-7, precision=FP64,
             slices=6, tol=None, rich_tol=1e-8):
    dev = "cuda"
    m = prob.m
    gamma = make_gamma(m, seed, dev)
    gf, gptr = fortran_ptr(gamma)
    rt = rotran.Rotran.for_problem(prob, precision=precision,
                                   slices=slices if precision == SPLIT else 0)
    tol = tol or TOL[precision]
    if records_on_device:
        cls, its, nts, dv, dl2, dl1 = synth.device_records(prob, prob.mfil, device=dev)
        rt.add_records_bulk_device(cls, nts, its, dv, dl2, dl1)
        del dv, dl2, dl1
    else:
        rt.add_problem_records(prob)
    c0 = torch.as_tensor(prob.qa, device=dev).clone().requires_grad_(True)
    e_lib = TransformEnergy.apply(c0, rt, prob, gptr)
    e_lib.backward()
    g_lib = c0.grad.detach().clone()
    st = rt.stats()

    ref = EnergyRef(prob, gamma, dev)
    c1 = torch.as_tensor(prob.qa, device=dev).clone().requires_grad_(True)
    e_ref = ref(c1)
    e_ref.backward()
    g_ref = c1.grad.detach()
    rel_e = abs(e_lib.item() - e_ref.item()) / abs(e_ref.item())
    rel_g = (g_lib - g_ref).abs().max().item() / g_ref.abs().max().item()
    name = "split" if precision == SPLIT else "fp64"
    print(f"{name} n={prob.n} m={m}: E={e_ref.item():.12e} rel dE {rel_e:.2e}, "
          f"grad max rel {rel_g:.2e}, adjoint {st.ms_total:.1f} ms, "
          f"{st.flops_algorithmic / st.ms_total / 1e9:.3f} TFLOP/s "
          f"(stage A {st.ms_first:.1f} ms, contraction {st.ms_second:.1f} ms)")
    assert rel_e <= tol[0]
    assert rel_g <= tol[1]

    # central differences of E along random complex directions, h = 1e-5
    gen = torch.Generator(device="cpu").manual_seed(1000 + seed)
    h = 1e-5
    c = torch.as_tensor(prob.qa, device=dev)
    worst = worst_rich = 0.0
    with torch.no_grad():
        for d_i in range(ndir):
            d = torch.complex(torch.randn(c.shape, generator=gen, dtype=torch.float64),
                              torch.randn(c.shape, generator=gen, dtype=torch.float64)).to(dev)
            d = d / d.abs().max()
            fd = (ref(c + h * d) - ref(c - h * d)).item() / (2 * h)
            fd2 = (ref(c + 2 * h * d) - ref(c - 2 * h * d)).item() / (4 * h)
            an = (g_lib.conj() * d).sum().real.item()
            worst = max(worst, abs(fd - an) / abs(an))
            # E is quartic in C: (4 fd(h) - fd(2h)) / 3 cancels the h^2 term exactly
            worst_rich = max(worst_rich, abs((4 * fd - fd2) / 3 - an) / abs(an))
            if d_i < check_lib_fd:  # the same difference through the library's own E
                rt.set_coefficients((c + h * d).cpu().numpy(), prob.itrmo, prob.kra, prob.krb,
                                    prob.ikrmo, prob.imoras_pairs())
                _, ep = rt.adjoint(gptr)
                rt.set_coefficients((c - h * d).cpu().numpy(), prob.itrmo, prob.kra, prob.krb,
                                    prob.ikrmo, prob.imoras_pairs())
                _, em = rt.adjoint(gptr)
                fdl = (ep - em) / (2 * h)
                # the split path's E carries ~1e-12 relative rounding that is
                # not smooth in C; differences divide it by h
                assert abs(fdl - an) / abs(an) <= (1e-7 if precision == FP64 else 1e-5)
    print(f"  central differences (h = 1e-5): worst relative error {worst:.2e}, "
          f"Richardson {worst_rich:.2e}, over {ndir} directions")
    assert worst <= fd_tol
    assert worst_rich <= rich_tol  # rounding floor: eps |E| / h relative to the derivative
    rt.close()
    del gf


@pytest.mark.parametrize("precision", [FP64, SPLIT], ids=["fp64", "split"])
def test_adjoint_small(precision):
    prob = synth.make_problem(5, 7, 3, seed=11)
    run_case(prob, records_on_device=False, seed=1, ndir=20, check_lib_fd=3, fd_tol=1e-6,
             precision=precision)


def test_adjoint_small_default_slices():
    # 5 slices: errors about 2^7 larger than at 6
    prob = synth.make_problem(5, 7, 3, seed=11)
    run_case(prob, records_on_device=False, seed=1, ndir=10, check_lib_fd=2, fd_tol=1e-6,
             precision=SPLIT, slices=0, tol=(5e-8, 5e-8), rich_tol=1e-7)


@pytest.mark.parametrize("precision", [FP64, SPLIT], ids=["fp64", "split"])
def test_adjoint_shuffled_spinors(precision):
    from util import permute_spinors
    perm = np.random.default_rng(2).permutation(8)
    prob = permute_spinors(synth.make_problem(4, 6, 4, seed=5), perm)
    run_case(prob, records_on_device=False, seed=2, ndir=8, check_lib_fd=1, fd_tol=1e-6,
             precision=precision)


@pytest.mark.parametrize("precision", [FP64, SPLIT], ids=["fp64", "split"])
def test_adjoint_config4(precision):
    # 100 L + 156 S AOs (n = 256), 64 Kramers pairs
    prob = synth.make_spinor_problem(100, 156, 64, seed=0)
    run_case(prob, records_on_device=True, seed=0, ndir=20, precision=precision)


def test_adjoint_rejects_null_density():
    prob = synth.make_problem(3, 3, 2, seed=1)
    rt = rotran.Rotran.for_problem(prob, precision=FP64)
    rt.set_problem_coefficients(prob)
    rt.add_problem_records(prob)
    with pytest.raises(rotran.RotranError):
        rt.adjoint(0)
    rt.close()
