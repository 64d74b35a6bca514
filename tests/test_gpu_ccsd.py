"""FP64 GPU CCSD path against the oracle and the reference's golden fixtures.

Tolerances (the engine's FP64 contract): intermediates and residual tensors within 1e-12
relative to their largest element; converged correlation energy within 1e-10 Eh.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from oracle import ccsd as oc

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def wfn1(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)
    return pg.CCwfn(H, device="GPU", precision="DP")


def dev(x, cuda):
    return torch.from_numpy(np.ascontiguousarray(x)).to(cuda)


def test_mp2_guess(wfn1, golden_o5v19):
    e = float(wfn1.cc_energy(wfn1.o, wfn1.v, wfn1.H.F, wfn1.H.L, wfn1.t1, wfn1.t2))
    assert abs(e - float(golden_o5v19["ecc_mp2"])) < 1e-13


def test_builders_golden_o5v19(wfn1, golden_o5v19, cuda):
    w = wfn1
    o, v, F, ERI, L = w.o, w.v, w.H.F, w.H.ERI, w.H.L
    t1, t2 = dev(golden_o5v19["probe_t1"], cuda), dev(golden_o5v19["probe_t2"], cuda)
    assert rel(w.build_tau(t1, t2), golden_o5v19["tau"]) < RTOL
    assert rel(w.build_tau(t1, t2, 1.0, 0.5), golden_o5v19["taut"]) < RTOL
    assert rel(w.build_Fae(o, v, F, L, t1, t2), golden_o5v19["Fae"]) < RTOL
    assert rel(w.build_Fmi(o, v, F, L, t1, t2), golden_o5v19["Fmi"]) < RTOL
    assert rel(w.build_Fme(o, v, F, L, t1), golden_o5v19["Fme"]) < RTOL
    assert rel(w.build_Wmnij(o, v, ERI, t1, t2), golden_o5v19["Wmnij"]) < RTOL
    assert rel(w.build_Wmbej(o, v, ERI, L, t1, t2), golden_o5v19["Wmbej"]) < RTOL
    assert rel(w.build_Wmbje(o, v, ERI, t1, t2), golden_o5v19["Wmbje"]) < RTOL
    assert rel(w.build_Zmbij(o, v, ERI, t1, t2), golden_o5v19["Zmbij"]) < RTOL


def test_residuals_golden_o5v19(wfn1, golden_o5v19, cuda):
    t1, t2 = dev(golden_o5v19["probe_t1"], cuda), dev(golden_o5v19["probe_t2"], cuda)
    r1, r2 = wfn1.residuals(wfn1.H.F, t1, t2)
    assert rel(r1, golden_o5v19["r1"]) < RTOL
    assert rel(r2, golden_o5v19["r2"]) < RTOL
    e = float(wfn1.cc_energy(wfn1.o, wfn1.v, wfn1.H.F, wfn1.H.L, t1, t2))
    assert abs(e - float(golden_o5v19["ecc_probe"])) < 1e-13


def test_residual_vs_oracle_random_point(cuda, ham_o5v19):
    """A fresh seeded point (not in the fixtures): GPU FP64 vs the numpy oracle."""
    _, F, ERI, L = ham_o5v19
    rng = np.random.default_rng(99)
    t1 = 0.05 * rng.standard_normal((5, 19))
    t2 = 0.05 * rng.standard_normal((5, 5, 19, 19))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    o, v = slice(0, 5), slice(5, 24)
    r1o, r2o = oc.residuals(o, v, F, ERI, L, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, device=cuda))
    r1, r2 = w.residuals(w.H.F, dev(t1, cuda), dev(t2, cuda))
    assert rel(r1, r1o) < RTOL and rel(r2, r2o) < RTOL


def test_solve_cc_golden_o5v19(cuda, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    e = w.solve_cc(1e-12, 1e-12, 100)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-10
    assert len(w.energies) == len(golden_o5v19["ecc_iters"])
    assert np.abs(np.array(w.energies) - golden_o5v19["ecc_iters"]).max() < 1e-10
    assert rel(w.t2, golden_o5v19["t2"]) < 1e-8


def test_solve_cc_raises_on_maxiter(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    with pytest.raises(pg.ConvergenceError):
        w.solve_cc(1e-14, 1e-14, maxiter=3)


def test_gpu_built_blocks_match_host(cuda, ham_o5v19):
    fac, F, ERI, L = ham_o5v19
    Hg = pg.Hamiltonian.from_factors(fac, device=cuda)
    Hh = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)
    for pat, blk in Hh.ERI.blocks.items():
        assert rel(Hg.ERI.blocks[pat], blk.cpu().numpy()) < 1e-13, pat
    for pat, blk in Hh.L.blocks.items():
        assert rel(Hg.L.blocks[pat], blk.cpu().numpy()) < 1e-13, pat


@pytest.mark.parametrize("no,nv", [(2, 3), (3, 17), (7, 33)])
def test_ragged_sizes_vs_oracle(cuda, no, nv):
    """Sizes that are not multiples of any tile (tails in every dimension)."""
    fac = pg.SyntheticFactors(no, nv, seed=5)
    F, ERI, L = fac.hamiltonian()
    o, v = slice(0, no), slice(no, no + nv)
    rng = np.random.default_rng(no * 100 + nv)
    t1 = 0.05 * rng.standard_normal((no, nv))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    r1o, r2o = oc.residuals(o, v, F, ERI, L, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_factors(fac, device=cuda))
    r1, r2 = w.residuals(w.H.F, dev(t1, cuda), dev(t2, cuda))
    assert rel(r1, r1o) < 1e-11 and rel(r2, r2o) < 1e-11


def _probe(no, nv, t2_mp2, seed):
    rng = np.random.default_rng(1000 + seed)
    t1 = 0.02 * rng.standard_normal((no, nv))
    noise = 0.01 * rng.standard_normal((no, no, nv, nv))
    return t1, t2_mp2 + noise + noise.transpose(1, 0, 3, 2)


@pytest.fixture(scope="module")
def golden_o20v180_data():
    from conftest import golden
    return golden("o20v180.npz"), golden("o20v180_raw.npz")


@pytest.mark.parametrize("which", ["matched", "raw"])
def test_residual_o20v180_vs_reference(cuda, golden_o20v180_data, which):
    """no=20, nv=180: GPU FP64 residual against the reference's own output (both couplings)."""
    g = golden_o20v180_data[0] if which == "matched" else golden_o20v180_data[1]
    fac = pg.SyntheticFactors(20, 180, 1, coupling="matched" if which == "matched" else 1.0)
    H = pg.Hamiltonian.from_factors(fac, device=cuda)
    w = pg.CCwfn(H)
    t1, t2 = _probe(20, 180, w.t2.cpu().numpy(), 1)
    r1, r2 = w.residuals(H.F, dev(t1, cuda), dev(t2, cuda))
    r2 = r2.cpu().numpy()
    assert rel(r1, g["r1"]) < RTOL
    assert rel(r2[0, 1], g["r2_slice_ij01"]) < RTOL
    assert rel(r2[:, :, 0, 0], g["r2_slice_ab00"]) < RTOL
    assert rel(r2[3, 3, 10:20, 100:110], g["r2_slice_diag"]) < RTOL
    assert abs(np.linalg.norm(r2) - float(g["r2_norm"])) < RTOL * float(g["r2_norm"])


def test_solve_o20v180_vs_reference(cuda, golden_o20v180_data):
    """Converged FP64 GPU energy within 1e-10 Eh of the reference's at no=20, nv=180."""
    g = golden_o20v180_data[0]
    H = pg.Hamiltonian.from_factors(pg.SyntheticFactors(20, 180, 1, coupling="matched"), device=cuda)
    w = pg.CCwfn(H)
    e = w.solve_cc(1e-10, 1e-10, 100)
    assert abs(e - float(g["ecc"])) < 1e-10
    assert np.abs(np.array(w.energies) - g["ecc_iters"]).max() < 1e-9
    assert rel(w.t1, g["t1"]) < 1e-7
    wm = pg.CCwfn(H, precision="MIXED")
    em = wm.solve_cc(1e-8, 1e-7, 100)
    assert abs(em - float(g["ecc"])) < 1e-6
