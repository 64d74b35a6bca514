"""Host logic of the FP64 engine and its adjoint on CPU, through the numpy model of the FP64
entry points (``tests/abi_model.py``): the builders' contraction plans, the residual's tape,
its forward sweep (the Jacobian action) and reverse sweep (Lambda), the density assembly.
The kernels themselves are covered by the ``-m gpu`` tests.

* The residual and the converged energy against the reference's (o5v19.npz).
* J.X against the reference's ``CCderiv._ccsd_jacobian`` at its converged amplitudes
  (o5v19_jacobian.npz), symmetrised doubles, 1e-12 relative.
* <l, J x> = <J^T l, x> and dE/dt . x from the two sweeps, to rounding.
* Lambda + gradient densities against the reference's D and Gamma (8-fold symmetric
  projection, 1e-9) and the energy identity E = <D,F> + <Gamma,ERI>.
"""
import numpy as np
import pytest
import torch

import abi_model
import pycc_gb300 as pg
from conftest import golden
from pycc_gb300.adjoint import CCSDAdjoint, symmetrize8


@pytest.fixture
def model(monkeypatch):
    m = abi_model.install(monkeypatch)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    return m


def rel(a, b):
    a = a.numpy() if isinstance(a, torch.Tensor) else a
    return np.abs(a - b).max() / np.abs(b).max()


def wavefunction(ham, t1=None, t2=None):
    _, F, ERI, L = ham
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    if t1 is not None:
        w.t1 = torch.from_numpy(np.ascontiguousarray(t1))
        w.t2 = torch.from_numpy(np.ascontiguousarray(t2))
    return w


def test_residual_and_solve(model, ham_o5v19, golden_o5v19):
    g = golden_o5v19
    w = wavefunction(ham_o5v19)
    r1, r2 = w.residuals(w.H.F, torch.from_numpy(g["probe_t1"].copy()),
                         torch.from_numpy(g["probe_t2"].copy()))
    assert rel(r1, g["r1"]) < 1e-13 and rel(r2, g["r2"]) < 1e-13
    e = w.solve_cc(1e-12, 1e-12)
    assert abs(e - float(g["ecc"])) < 1e-12
    assert w.niter == len(g["ecc_iters"]) - 1


def test_jacobian_vs_reference(model, ham_o5v19):
    g = golden("o5v19_jacobian.npz")
    adj = CCSDAdjoint(wavefunction(ham_o5v19, g["t1"], g["t2"]))
    s1, s2 = adj.jacobian(torch.from_numpy(g["X1"].copy()), torch.from_numpy(g["X2"].copy()))
    assert rel(s1, g["sigma1"]) < 1e-12
    assert rel(s2 + s2.permute(1, 0, 3, 2), g["sigma2_sym"]) < 1e-12
    assert torch.equal(s2, s2.permute(1, 0, 3, 2))          # half of the symmetric action
    with pytest.raises(ValueError):
        adj.jacobian(torch.zeros(5, 19), torch.zeros(5, 5, 19, 19))   # float32


def test_sweeps_are_transposes(model, ham_o5v19, golden_o5v19):
    adj = CCSDAdjoint(wavefunction(ham_o5v19, golden_o5v19["t1"], golden_o5v19["t2"]))
    rng = np.random.default_rng(9)
    x1, l1 = (torch.from_numpy(rng.standard_normal((5, 19))) for _ in range(2))
    x2, l2 = (torch.from_numpy(rng.standard_normal((5, 5, 19, 19))) for _ in range(2))
    dr1, dr2, dE = adj.jvp(x1, x2)
    lhs = float((l1 * dr1).sum() + (l2 * dr2).sum())
    G = adj.backward(l1=l1, l2=l2)
    rhs = float((G.get(adj.t1) * x1).sum() + (G.get(adj.t2) * x2).sum())
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)
    G = adj.backward(gE=1.0)
    ref = float((G.get(adj.t1) * x1).sum() + (G.get(adj.t2) * x2).sum())
    assert abs(float(dE) - ref) < 1e-12 * abs(ref)


def test_lambda_and_densities(model, ham_o5v19, golden_o5v19):
    g = golden_o5v19
    _, F, ERI, _ = ham_o5v19
    w = wavefunction(ham_o5v19)
    e = w.solve_cc(1e-12, 1e-12)
    adj = CCSDAdjoint(w)
    adj.solve_lambda(1e-12, 1e-12, 200)
    gF, Gam = adj.gradient()
    assert abs(float((gF.numpy() * F).sum() + (Gam.numpy() * ERI).sum()) - e) < 1e-10
    D, G = torch.from_numpy(g["D"]), torch.from_numpy(g["Gamma"])
    assert (0.5 * (gF + gF.T) - 0.5 * (D + D.T)).abs().max().item() < 1e-9
    assert (symmetrize8(Gam) - symmetrize8(G)).abs().max().item() < 1e-9


def test_reference_objects_chain(model, ham_o5v19, golden_o5v19):
    """cchbar -> cclambda -> ccdensity with the reference's constructors, methods and
    normalisation: pseudo-energy, l1 and l2 against the reference's cclambda, D and Gamma
    against its ccdensity.gradient_densities (symmetric projections), compute_energy
    against the converged energy."""
    g = golden_o5v19
    w = wavefunction(ham_o5v19)
    e = w.solve_cc(1e-12, 1e-12)
    hbar = pg.cchbar(w)
    with pytest.raises(AttributeError):
        hbar.Hxyzw
    lam = pg.cclambda(w, hbar)
    t1, t2 = g["t1"], g["t2"]
    assert rel(lam.l1, 2.0 * t1) < 1e-9                                # the reference's guess
    assert rel(lam.l2, 2.0 * (2.0 * t2 - t2.swapaxes(2, 3))) < 1e-9
    dens0 = pg.ccdensity(w, lam)                                      # any lambda: L = E at r = 0
    assert abs(dens0.compute_energy() - e) < 1e-10
    pseudo = lam.solve_lambda(1e-12, 1e-12, 200)
    assert abs(pseudo - float(g["lambda_pseudo"])) < 1e-10
    assert rel(lam.l1, g["l1"]) < 1e-9 and rel(lam.l2, g["l2"]) < 1e-9
    dens = pg.ccdensity(w, lam)
    D, G = dens.gradient_densities()
    Dr, Gr = torch.from_numpy(g["D"]), torch.from_numpy(g["Gamma"])
    assert (D - Dr).abs().max().item() < 1e-9                         # not symmetrised
    o, v = slice(0, 5), slice(5, 24)
    for blk, s in (("Doo", (o, o)), ("Dov", (o, v)), ("Dvo", (v, o)), ("Dvv", (v, v))):
        assert (getattr(dens, blk) - Dr[s]).abs().max().item() < 1e-9, blk
    assert (G - symmetrize8(Gr)).abs().max().item() < 1e-9
    assert abs(dens.compute_energy() - e) < 1e-10
    assert abs(dens.compute_energy() - float(g["E_from_densities"])) < 1e-10
    with pytest.raises(RuntimeError):
        pg.ccdensity(w, lam, onlyone=True).gradient_densities()


def test_density_symmetrisation_kernel_path(model):
    """The eight-fold projection on the combination kernel equals the torch definition."""
    from pycc_gb300.lagrangian import symmetrize_density2
    G = torch.from_numpy(np.random.default_rng(3).standard_normal((4, 5, 6, 7))[:, :4, :4, :4]
                         .copy()).contiguous()
    assert (symmetrize_density2(G) - symmetrize8(G)).abs().max().item() < 1e-15


def test_tensor_core_sweeps(model, ham_o5v19, golden_o5v19):
    """The 'tc' sweep engine (every GEMM-shaped contraction of the sweeps on the tensor-core
    engine, here with no size floor) plans the same products as the FP64 sweeps: with the
    pack and GEMM modelled exactly, J^T l, J x, Lambda and the densities agree to rounding."""
    g = golden_o5v19
    w = wavefunction(ham_o5v19, g["t1"], g["t2"])
    ref = CCSDAdjoint(w, sweep="fp64")
    tc = CCSDAdjoint(w, sweep="tc")
    tc.tc_min_flops = 0
    rng = np.random.default_rng(5)
    x1, l1 = (torch.from_numpy(rng.standard_normal((5, 19))) for _ in range(2))
    x2, l2 = (torch.from_numpy(rng.standard_normal((5, 5, 19, 19))) for _ in range(2))
    n0 = model.calls.count("pcg_tc_gemm")
    for a, b in zip(ref.jvp(x1, x2), tc.jvp(x1, x2)):
        assert (a - b).abs().max().item() <= 1e-12 * a.abs().max().item()
    Ga = [ref.backward(l1=l1, l2=l2).get(t).clone() for t in (ref.t1, ref.t2)]
    Gb = [tc.backward(l1=l1, l2=l2).get(t).clone() for t in (tc.t1, tc.t2)]
    for a, b in zip(Ga, Gb):
        assert (a - b).abs().max().item() <= 1e-12 * a.abs().max().item()
    assert model.calls.count("pcg_tc_gemm") - n0 > 20
    lam = pg.cclambda(w, pg.cchbar(w, sweep="tc"))
    lam.hbar.adjoint.tc_min_flops = 0
    assert abs(lam.solve_lambda(1e-12, 1e-12, 200) - float(g["lambda_pseudo"])) < 1e-10
    D, G = pg.ccdensity(w, lam).gradient_densities()
    assert (D - torch.from_numpy(g["D"])).abs().max().item() < 1e-9
    assert (G - symmetrize8(torch.from_numpy(g["Gamma"]))).abs().max().item() < 1e-9


def test_mixed_wavefunction_gets_a_dp_tape(model, ham_o5v19, golden_o5v19):
    """A MIXED wave function: the tape is recorded by a DP twin sharing its Hamiltonian and
    amplitudes, and the sweeps default to the tensor cores."""
    g = golden_o5v19
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"), precision="MIXED")
    w.t1 = torch.from_numpy(g["t1"].copy())
    w.t2 = torch.from_numpy(g["t2"].copy())
    hbar = pg.cchbar(w)
    assert hbar.adjoint.sweep == "tc" and hbar.adjoint.w is not w
    assert hbar.adjoint.w.H is w.H and torch.equal(hbar.adjoint.t2, w.t2)
    lam = pg.cclambda(w, hbar)
    assert abs(lam.solve_lambda(1e-12, 1e-12, 200) - float(g["lambda_pseudo"])) < 1e-10


@pytest.mark.parametrize("no,nv", [(1, 1), (2, 1), (1, 4), (3, 2)])
@pytest.mark.parametrize("sweep", ["fp64", "tc"])
def test_degenerate_sizes(model, no, nv, sweep):
    """Single occupied or virtual orbitals: J x against a five-point stencil of the residual
    (exact for the quartic map) and <l, J x> = <J^T l, x>, on both sweep engines."""
    fac = pg.SyntheticFactors(no, nv, 5)
    F, ERI, L = fac.hamiltonian()
    rng = np.random.default_rng(no * 7 + nv)
    t1 = torch.from_numpy(0.05 * rng.standard_normal((no, nv)))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = torch.from_numpy(t2 + t2.transpose(1, 0, 3, 2))
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, L=L, device="cpu"))
    w.t1, w.t2 = t1, t2
    adj = CCSDAdjoint(w, sweep=sweep)
    adj.tc_min_flops = 0
    x1, l1 = (torch.from_numpy(rng.standard_normal((no, nv))) for _ in range(2))
    x2, l2 = (torch.from_numpy(rng.standard_normal((no, no, nv, nv))) for _ in range(2))
    dr1, dr2, _ = adj.jvp(x1, x2)

    def r(e):
        return w.residuals(w.H.F, t1 + e * x1, t2 + e * x2)
    rp, rm, rp2, rm2 = r(1.0), r(-1.0), r(2.0), r(-2.0)
    for k, d in ((0, dr1), (1, dr2)):
        fd = (8 * (rp[k] - rm[k]) - (rp2[k] - rm2[k])) / 12
        assert (fd - d).abs().max().item() <= 1e-10 * max(1.0, fd.abs().max().item())
    G = adj.backward(l1=l1, l2=l2)
    lhs = float((l1 * dr1).sum() + (l2 * dr2).sum())
    rhs = float((G.get(adj.t1) * x1).sum() + (G.get(adj.t2) * x2).sum())
    assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(lhs))


def test_adjoint_adopts_the_last_forward_tape(model, ham_o5v19, golden_o5v19):
    """solve_cc(keep_tape=True): the adjoint adopts the converging iteration's taped
    residual instead of evaluating it again; Lambda and the densities still match the
    reference's.  Any later change of the amplitudes makes the adjoint record afresh."""
    g = golden_o5v19
    w = wavefunction(ham_o5v19)
    w.solve_cc(1e-12, 1e-12, keep_tape=True)
    n0 = len(model.calls)
    adj = CCSDAdjoint(w)
    assert adj.tape_reused
    assert "pcg_symmetrize_f64" not in model.calls[n0:]        # no residual evaluated
    lam = pg.cclambda(w, pg.cchbar(w))                        # the tape is used once
    assert not lam.hbar.adjoint.tape_reused
    adj.solve_lambda(1e-12, 1e-12, 200)
    gF, Gam = adj.gradient()
    assert (0.5 * (gF + gF.T) - 0.5 * (torch.from_numpy(g["D"]) + torch.from_numpy(g["D"]).T)
            ).abs().max().item() < 1e-9
    assert (symmetrize8(Gam) - symmetrize8(torch.from_numpy(g["Gamma"]))).abs().max().item() < 1e-9
    w.solve_cc(1e-12, 1e-12, keep_tape=True)
    w.t1[0, 0] += 1e-3
    assert not CCSDAdjoint(w).tape_reused


def test_hbar_blocks_vs_reference(model, ham_o5v19):
    """The eleven HBAR blocks of cchbar (pycc/cchbar.py:54-110) at the reference's converged
    amplitudes, against the reference's own blocks (o5v19_hbar.npz), 1e-12 relative."""
    g = golden("o5v19_hbar.npz")
    w = wavefunction(ham_o5v19, g["t1"], g["t2"])
    hbar = pg.cchbar(w)
    for name in ("Hov", "Hvv", "Hoo", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov",
                 "Hvvvo", "Hovoo"):
        got = getattr(hbar, name)
        assert tuple(got.shape) == g[name].shape, name
        assert rel(got, g[name]) < 1e-12, (name, rel(got, g[name]))
