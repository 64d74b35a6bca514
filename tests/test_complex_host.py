"""Complex residuals on CPU through the numpy model of the entry points
(``tests/abi_model.py``): the reference's real-time propagation calls the same residual with a
complex Fock matrix and complex amplitudes (``residuals(F, t1, t2, real_time=True)``); the
engine forms it from five real residuals (a Lagrange interpolant evaluated at s = i, exact
for the residual's degree in s).  Pinned to the reference's own complex residual
(tests/golden/o5v19_complex.npz) in every precision stage.
"""
import numpy as np
import pytest
import torch

import abi_model
import pycc_gb300 as pg
from conftest import golden


@pytest.fixture
def model(monkeypatch):
    m = abi_model.install(monkeypatch)
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda *a: None)
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda *a: None)
    return m


def rel(a, b):
    return np.abs(a.numpy() - b).max() / np.abs(b).max()


@pytest.mark.parametrize("precision", ["DP", "MIXED", "SP"])
def test_complex_residual_vs_reference(model, ham_o5v19, precision):
    g = golden("o5v19_complex.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"), precision=precision,
                 real_time=True)
    Fc, t1, t2 = (torch.from_numpy(g[k]) for k in ("F", "t1", "t2"))
    stages = range(len(w.mixed_engine().stages)) if precision != "DP" else [None]
    for stage in stages:
        if stage is not None:
            w.mixed_engine().stage = stage
        r1, r2 = w.residuals(Fc, t1, t2, real_time=True)
        assert r1.dtype == torch.complex128 and r2.dtype == torch.complex128
        assert rel(r1, g["r1"]) < 1e-13 and rel(r2, g["r2"]) < 1e-13


def test_real_inputs_unchanged_by_the_flag(model, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    t1 = torch.from_numpy(golden_o5v19["probe_t1"].copy())
    t2 = torch.from_numpy(golden_o5v19["probe_t2"].copy())
    r1, r2 = w.residuals(w.H.F, t1, t2, real_time=True)
    assert r1.dtype == torch.float64
    assert rel(r1, golden_o5v19["r1"]) < 1e-13 and rel(r2, golden_o5v19["r2"]) < 1e-13
    # a complex call with zero imaginary parts equals the real one
    c1, c2 = w.residuals(w.H.F.to(torch.complex128), t1.to(torch.complex128), t2)
    assert (c1.real - r1).abs().max().item() < 1e-14 * r1.abs().max().item()
    assert c1.imag.abs().max().item() < 1e-14 * r1.abs().max().item()
    assert (c2.real - r2).abs().max().item() < 1e-14 * r2.abs().max().item()


def test_complex_energy_and_tau(model, ham_o5v19):
    """cc_energy and build_tau at complex amplitudes (the real-time propagation's energy)
    against the oracle's formulas evaluated in complex arithmetic; other dtypes are refused
    rather than misread by the FP64 kernels."""
    from oracle import ccsd as oc
    g = golden("o5v19_complex.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    Fc, t1, t2 = (torch.from_numpy(g[k]) for k in ("F", "t1", "t2"))
    o, v = w.o, w.v
    e = w.cc_energy(o, v, Fc, w.H.L, t1, t2)
    # E = 2 f_ia t_ia + (t2_ijab + t_ia t_jb) L_ijab (pycc/ccwfn.py:1122-1162), in complex
    # arithmetic (the oracle's cc_energy returns a real float)
    tau_c = g["t2"] + np.einsum("ia,jb->ijab", g["t1"], g["t1"])
    want = 2.0 * np.sum(g["F"][o, v] * g["t1"]) + np.sum(tau_c * L[o, o, v, v])
    assert e.dtype == torch.complex128 and abs(complex(e) - want) < 1e-13 * abs(want)
    tau = w.build_tau(t1, t2, 1.0, 0.5)
    want_tau = oc.build_tau(g["t1"], g["t2"], 1.0, 0.5)
    assert np.abs(tau.numpy() - want_tau).max() < 1e-14 * np.abs(want_tau).max()
    with pytest.raises(TypeError):
        w.build_tau(t1.real.float().contiguous(), t2.real.float().contiguous())
    with pytest.raises(TypeError):
        w.cc_energy(o, v, w.H.F, w.H.L, t1.real.float().contiguous(), t2.real.contiguous())


def test_single_precision_complex_refused(model, ham_o5v19):
    """complex64 (or float32 next to complex) inputs are refused, not misread as FP64."""
    g = golden("o5v19_complex.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    Fc, t1, t2 = (torch.from_numpy(g[k]) for k in ("F", "t1", "t2"))
    with pytest.raises(TypeError):
        w.residuals(Fc, t1.to(torch.complex64), t2)
    with pytest.raises(TypeError):
        w.residuals(Fc.real.float(), t1, t2)
