"""The reference's adjoint objects on the GPU, over the FP64 residual's tape.

* J.X (forward sweep) against the reference's ``CCderiv._ccsd_jacobian``
  (pycc/ccderiv.py:149-180) at the reference's converged no=5, nv=19 amplitudes
  (tests/golden/o5v19_jacobian.npz): singles and symmetrised doubles within 1e-12 of the
  largest element; <l, J x> = <J^T l, x> between the forward and reverse sweeps.
* cchbar -> cclambda -> ccdensity with the reference's interface: pseudo-energy (1e-10),
  l1 / l2 (1e-9) against the reference's cclambda, D (as is) and Gamma (eight-fold
  projection) against its gradient_densities (1e-9), compute_energy against E_corr.
* The eleven HBAR blocks against the reference's cchbar (o5v19_hbar.npz), 1e-12 relative.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from conftest import golden
from pycc_gb300.adjoint import CCSDAdjoint, symmetrize8

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jac(cuda, ham_o5v19):
    g = golden("o5v19_jacobian.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    w.t1 = torch.from_numpy(g["t1"]).to(cuda)
    w.t2 = torch.from_numpy(g["t2"]).to(cuda)
    return g, CCSDAdjoint(w)


def test_jacobian_vs_reference(jac, cuda):
    g, adj = jac
    s1, s2 = adj.jacobian(torch.from_numpy(g["X1"]).to(cuda), torch.from_numpy(g["X2"]).to(cuda))
    torch.cuda.synchronize()
    s1 = s1.cpu().numpy()
    sym = (s2 + s2.permute(1, 0, 3, 2)).cpu().numpy()
    assert np.abs(s1 - g["sigma1"]).max() < 1e-12 * np.abs(g["sigma1"]).max()
    assert np.abs(sym - g["sigma2_sym"]).max() < 1e-12 * np.abs(g["sigma2_sym"]).max()


def test_forward_reverse_transpose(jac, cuda):
    _, adj = jac
    gen = torch.Generator(device=cuda).manual_seed(9)
    x1, l1 = (torch.randn(5, 19, dtype=torch.float64, device=cuda, generator=gen) for _ in range(2))
    x2, l2 = (torch.randn(5, 5, 19, 19, dtype=torch.float64, device=cuda, generator=gen)
              for _ in range(2))
    dr1, dr2, _ = adj.jvp(x1, x2)
    lhs = float((l1 * dr1).sum() + (l2 * dr2).sum())
    G = adj.backward(l1=l1, l2=l2)
    rhs = float((G.get(adj.t1) * x1).sum() + (G.get(adj.t2) * x2).sum())
    assert abs(lhs - rhs) < 1e-11 * abs(lhs)


def test_reference_objects_chain(cuda, ham_o5v19, golden_o5v19):
    g = golden_o5v19
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    e = w.solve_cc(1e-12, 1e-12, 100)
    lam = pg.cclambda(w, pg.cchbar(w))
    pseudo = lam.solve_lambda(1e-12, 1e-12, 200)
    assert abs(pseudo - float(g["lambda_pseudo"])) < 1e-10
    for got, want in ((lam.l1, g["l1"]), (lam.l2, g["l2"])):
        assert np.abs(got.cpu().numpy() - want).max() < 1e-9 * np.abs(want).max()
    dens = pg.ccdensity(w, lam)
    D, G = dens.gradient_densities()
    Dr = torch.from_numpy(g["D"]).to(cuda)
    Gr = torch.from_numpy(g["Gamma"]).to(cuda)
    assert (D - Dr).abs().max().item() < 1e-9                         # not symmetrised
    assert (G - symmetrize8(Gr)).abs().max().item() < 1e-9
    assert abs(dens.compute_energy() - e) < 1e-10


def test_hbar_blocks_vs_reference(cuda, ham_o5v19):
    """The reference's eleven HBAR blocks (pycc/cchbar.py:54-110), materialised on the GPU
    in FP64, against its own blocks at its converged amplitudes (o5v19_hbar.npz): 1e-12
    relative to each block's largest element."""
    g = golden("o5v19_hbar.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    w.t1 = torch.from_numpy(g["t1"]).to(cuda)
    w.t2 = torch.from_numpy(np.ascontiguousarray(g["t2"])).to(cuda)
    hbar = pg.cchbar(w)
    for name in ("Hov", "Hvv", "Hoo", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov",
                 "Hvvvo", "Hovoo"):
        got = getattr(hbar, name).cpu().numpy()
        assert got.shape == g[name].shape, name
        assert np.abs(got - g[name]).max() < 1e-12 * np.abs(g[name]).max(), name
