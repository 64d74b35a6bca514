"""Adjoint of the converged CCSD energy (Lambda via the residual's tape, gradient densities).

Checked against the reference's own ccdensity.gradient_densities (D and Gamma, compared on the
8-fold symmetric projection that any real symmetric perturbation sees), against the energy
identity E_corr = <D,F> + <Gamma,ERI>, and against central finite differences along 16 random
symmetric Hamiltonian perturbations of norm 1: the fourth-order stencil
(8 (E(h) - E(-h)) - (E(2h) - E(-2h))) / 12h with h = 1e-3, every point converged to 1e-12
from the unperturbed amplitudes (truncation ~h^4, rounding ~1e-12 / h); tolerance 1e-6
relative to the derivative.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from pycc_gb300.adjoint import CCSDAdjoint, ccsd_energy, symmetrize8

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adj1(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    e = w.solve_cc(1e-12, 1e-12, 100)
    adj = CCSDAdjoint(w)
    adj.solve_lambda(1e-12, 1e-12, 200)
    gF, Gam = adj.gradient()
    return e, gF, Gam, adj


def test_energy_identity(adj1, ham_o5v19, cuda):
    e, gF, Gam, _ = adj1
    _, F, ERI, _ = ham_o5v19
    Ft, Et = torch.from_numpy(F).to(cuda), torch.from_numpy(ERI).to(cuda)
    lag = float((gF * Ft).sum() + (Gam * Et).sum())
    assert abs(lag - e) < 1e-10


def test_densities_vs_reference(adj1, golden_o5v19, cuda):
    _, gF, Gam, _ = adj1
    D = torch.from_numpy(golden_o5v19["D"]).to(cuda)
    G = torch.from_numpy(golden_o5v19["Gamma"]).to(cuda)
    sym2 = lambda X: 0.5 * (X + X.T)
    assert (sym2(gF) - sym2(D)).abs().max().item() < 1e-9
    d = (symmetrize8(Gam) - symmetrize8(G)).abs().max().item()
    assert d < 1e-9, d


def _rand_sym(rng, n):
    dF = rng.standard_normal((n, n))
    dF = 0.5 * (dF + dF.T)
    C = rng.standard_normal((n, n, n, n))
    C = 0.5 * (C + C.transpose(1, 0, 2, 3))
    C = 0.5 * (C + C.transpose(0, 1, 3, 2))
    C = 0.5 * (C + C.transpose(2, 3, 0, 1))
    dE = C.transpose(0, 2, 1, 3)
    nrm = np.sqrt(np.sum(dF * dF) + np.sum(dE * dE))
    return dF / nrm, np.ascontiguousarray(dE / nrm)


def _energy(F, ERI, no, cuda, t1, t2):
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, device=cuda))
    w.t1, w.t2 = t1, t2                     # warm start from the unperturbed amplitudes
    return w.solve_cc(1e-12, 1e-12, 200)


def test_finite_differences(adj1, ham_o5v19, cuda):
    _, gF, Gam, adj = adj1
    _, F, ERI, _ = ham_o5v19
    rng = np.random.default_rng(4)
    h = 1e-3
    gFn, Gn = gF.cpu().numpy(), Gam.cpu().numpy()
    worst = 0.0
    for _ in range(16):
        dF, dERI = _rand_sym(rng, F.shape[0])
        E = {s: _energy(F + s * h * dF, ERI + s * h * dERI, 5, cuda, adj.t1, adj.t2)
             for s in (1, -1, 2, -2)}
        fd = (8.0 * (E[1] - E[-1]) - (E[2] - E[-2])) / (12.0 * h)
        an = float(np.sum(gFn * dF) + np.sum(Gn * dERI))
        worst = max(worst, abs(fd - an) / abs(an))
        assert abs(fd - an) < 1e-6 * abs(an), (fd, an)
    print("finite differences: worst relative difference %.2e" % worst)


def test_autograd_function(adj1, ham_o5v19, cuda):
    e, gF, Gam, _ = adj1
    _, F, ERI, _ = ham_o5v19
    Ft = torch.from_numpy(F).to(cuda).requires_grad_(True)
    Et = torch.from_numpy(ERI).to(cuda).requires_grad_(True)
    E = ccsd_energy(Ft, Et, 5, 1e-12, 1e-12)
    assert abs(float(E.detach()) - e) < 1e-10
    E.backward()
    assert (Ft.grad - gF).abs().max().item() < 1e-9
    assert (Et.grad - Gam).abs().max().item() < 1e-9


def test_lambda_vjp_transpose(adj1, cuda):
    """<l, J x> = <J^T l, x>: the tape's reverse sweep is the transpose of the forward map."""
    _, _, _, adj = adj1
    w = adj.w
    g = torch.Generator(device=cuda).manual_seed(1)
    x1 = torch.randn(w.no, w.nv, dtype=torch.float64, device=cuda, generator=g) * 1e-5
    x2 = torch.randn(w.no, w.no, w.nv, w.nv, dtype=torch.float64, device=cuda, generator=g) * 1e-5
    l1 = torch.randn(w.no, w.nv, dtype=torch.float64, device=cuda, generator=g)
    l2 = torch.randn(w.no, w.no, w.nv, w.nv, dtype=torch.float64, device=cuda, generator=g)
    # J x by central differences of the residual (exact to O(eps^2) for the quartic map)
    t1, t2 = w.t1.clone(), w.t2.clone()
    rp = w.residuals(w.H.F, (t1 + x1).contiguous(), (t2 + x2).contiguous())
    rm = w.residuals(w.H.F, (t1 - x1).contiguous(), (t2 - x2).contiguous())
    lhs = float(((rp[0] - rm[0]) * l1).sum() + ((rp[1] - rm[1]) * l2).sum()) / 2.0
    G = adj.backward(l1=l1, l2=l2)
    rhs = float((G.get(adj.t1) * x1).sum() + (G.get(adj.t2) * x2).sum())
    assert abs(lhs - rhs) < 1e-7 * max(abs(lhs), 1e-12) + 1e-15
