"""Host logic of the mixed-precision engine on CPU, through the numpy model of the entry
points (``tests/abi_model.py``) with the tensor-core pack and GEMM in exact FP64.

Every contraction the engine plans -- operand combinations folded into packs (tau, 2 t2 -
t2~, W + W~), K orders, the symmetric / antisymmetric pair forms of the two ladders and of
Zmbij's and Wmnij's tau terms with their offset tables, K weights and assemblies, the o^3 v
tensors summed into Zmbij, the symmetrisation images -- is checked exactly: with no format rounding, each precision stage's residual must equal the
reference's FP64 residual (o5v19.npz) to rounding.  The formats' own accuracy is the subject
of the ``-m gpu`` tests.
"""
import numpy as np
import pytest
import torch

import abi_model
import pycc_gb300 as pg
from oracle import ccsd as oc


@pytest.fixture
def model(monkeypatch):
    m = abi_model.install(monkeypatch)
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda *a: None)
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda *a: None)
    return m


def rel(a, b):
    return np.abs(a.numpy() - b).max() / np.abs(b).max()


def hamiltonian(ham):
    _, F, ERI, L = ham
    return pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu")


@pytest.mark.parametrize("precision", ["MIXED", "SP"])
def test_every_stage_plans_the_exact_residual(model, ham_o5v19, golden_o5v19, precision):
    g = golden_o5v19
    w = pg.CCwfn(hamiltonian(ham_o5v19), precision=precision)
    eng = w.mixed_engine()
    t1 = torch.from_numpy(g["probe_t1"].copy())
    t2 = torch.from_numpy(g["probe_t2"].copy())
    for stage in range(len(eng.stages)):
        eng.stage = stage
        r1, r2 = w.residuals(w.H.F, t1, t2)
        assert rel(r1, g["r1"]) < 1e-13, eng.stages[stage]
        assert rel(r2, g["r2"]) < 1e-13, eng.stages[stage]
    assert "pcg_tc_gemm" in model.calls and "pcg_pack_operand" in model.calls


def test_ragged_sizes_vs_oracle(model):
    """Odd extents (no=3, nv=11) against the oracle's residual at a random point."""
    fac = pg.SyntheticFactors(3, 11, 7)
    F, ERI, L = fac.hamiltonian()
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 3, L=L, device="cpu"), precision="MIXED")
    rng = np.random.default_rng(1)
    t1 = 0.05 * rng.standard_normal((3, 11))
    t2 = 0.05 * rng.standard_normal((3, 3, 11, 11))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    o, v = slice(0, 3), slice(3, 14)
    want1, want2 = oc.residuals(o, v, F, ERI, L, t1, t2)
    r1, r2 = w.residuals(w.H.F, torch.from_numpy(t1), torch.from_numpy(t2))
    assert rel(r1, want1) < 1e-13 and rel(r2, want2) < 1e-13


def test_mixed_solve_control_flow(model, ham_o5v19, golden_o5v19):
    """The ladder's hand-overs and the final-stage refinement, in exact arithmetic: the
    solve walks every stage and ends at the reference's energy."""
    w = pg.CCwfn(hamiltonian(ham_o5v19), precision="MIXED")
    e = w.solve_cc(1e-12, 1e-12, 100)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-11
    hist = w.mixed_engine().history
    assert hist[0] == "fp8" and hist[-1] == "bf16x3s"
    assert not w.converged_at_floor


def test_swapped_integrals_are_repacked(model, ham_o5v19, golden_o5v19):
    """The reference's linear-in-H call (pycc/ccderiv.py:252-259): H.ERI / H.L swapped for
    other blocks around one residual.  The mixed engine must use the swapped blocks, and the
    original ones again afterwards."""
    g = golden_o5v19
    H = hamiltonian(ham_o5v19)
    w = pg.CCwfn(H, precision="MIXED")
    dp = pg.CCwfn(H)
    t1 = torch.from_numpy(g["probe_t1"].copy())
    t2 = torch.from_numpy(g["probe_t2"].copy())
    w.residuals(H.F, t1, t2)                                 # packs the original blocks
    rng = np.random.default_rng(2)
    n = 24
    dF = rng.standard_normal((n, n))
    dF = 0.5 * (dF + dF.T)
    C = rng.standard_normal((n, n, n, n))
    C = C + C.transpose(1, 0, 3, 2)
    C = C + C.transpose(2, 3, 0, 1)
    dERI = np.ascontiguousarray(C + C.transpose(2, 1, 0, 3))
    dH = pg.Hamiltonian.from_arrays(dF, dERI, 5, device="cpu")
    saved = H.ERI, H.L
    H.ERI, H.L = dH.ERI, dH.L
    try:
        m1, m2 = w.residuals(dH.F, t1, t2)
        d1, d2 = dp.residuals(dH.F, t1, t2)
    finally:
        H.ERI, H.L = saved
    assert rel(m1, d1.numpy()) < 1e-13 and rel(m2, d2.numpy()) < 1e-13
    r1, r2 = w.residuals(H.F, t1, t2)                        # the original blocks again
    assert rel(r1, g["r1"]) < 1e-13 and rel(r2, g["r2"]) < 1e-13


@pytest.mark.parametrize("no,nv", [(1, 1), (2, 1), (1, 3), (3, 2), (2, 7)])
@pytest.mark.parametrize("precision", ["DP", "MIXED", "SP"])
def test_degenerate_sizes(model, no, nv, precision):
    """Single occupied or virtual orbitals: every stage's residual against the oracle, twice
    in a row on one wave function (a buffer that aliased an input would show on the second
    call), and the Hamiltonian unchanged."""
    fac = pg.SyntheticFactors(no, nv, 3)
    F, ERI, L = fac.hamiltonian()
    rng = np.random.default_rng(no * 10 + nv)
    t1 = 0.05 * rng.standard_normal((no, nv))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    o, v = slice(0, no), slice(no, no + nv)
    want1, want2 = oc.residuals(o, v, F, ERI, L, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, L=L, device="cpu"), precision=precision)
    F0 = w.H.F.clone()
    stages = range(len(w.mixed_engine().stages)) if precision != "DP" else [None]
    for stage in stages:
        if stage is not None:
            w.mixed_engine().stage = stage
        for _ in range(2):
            r1, r2 = w.residuals(w.H.F, torch.from_numpy(t1), torch.from_numpy(t2))
            assert rel(r1, want1) < 1e-12 and rel(r2, want2) < 1e-12, stage
    assert torch.equal(w.H.F, F0)


@pytest.mark.parametrize("no,nv,nb", [(4, 6, 3), (1, 5, 2), (3, 1, 4)])
def test_pair_form_intermediate_through_the_model(model, no, nv, nb):
    """MixedResidual.pair_tau (Zmbij / Wmnij's tau_ijef X_r,ef in symmetric / antisymmetric
    pair form, with its tables, K weights and pcg_pair_pm_assemble) equals the plain
    contraction in the exact FP64 model, including no = 1 (no i < j pairs) and nv = 1 (no
    e < f pairs)."""
    from types import SimpleNamespace
    from pycc_gb300.mixed import MixedResidual
    from pycc_gb300.tc import FMT_BF16X3F
    rng = np.random.default_rng(no * 100 + nv * 10 + nb)
    X = torch.from_numpy(rng.standard_normal((no, nb, nv, nv)))
    t1 = torch.from_numpy(0.1 * rng.standard_normal((no, nv)))
    t2 = 0.1 * rng.standard_normal((no, no, nv, nv))
    t2 = torch.from_numpy(t2 + t2.transpose(1, 0, 3, 2)).contiguous()
    V = torch.zeros(nv, nv, nv, nv, dtype=torch.float64)
    w = SimpleNamespace(device1="cpu", stream=None, no=no, nv=nv, vvvv_fp8=True,
                        switch_threshold=1e-5,
                        H=SimpleNamespace(ERI=SimpleNamespace(blocks={"vvvv": V})))
    eng = MixedResidual(w)
    out = torch.ones((no, nb, no, no), dtype=torch.float64)
    eng.pair_tau(X, "mbef", "ovvv", t1, t2, out, FMT_BF16X3F)
    tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
    ref = 1.0 + torch.einsum("ijef,mbef->mbij", tau, X)
    assert torch.allclose(out, ref, rtol=0, atol=1e-13)
    assert "pcg_pair_pm_assemble" in model.calls


@pytest.mark.parametrize("no,nv", [(1, 4), (2, 1), (1, 1)])
def test_degenerate_pair_counts_vs_oracle(model, no, nv):
    """The pair forms with empty antisymmetric parts (no = 1: no i < j or m < n pairs;
    nv = 1: no a < b or e < f pairs) in the full mixed residual, every stage, against the
    oracle."""
    fac = pg.SyntheticFactors(no, nv, 3)
    F, ERI, L = fac.hamiltonian()
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, L=L, device="cpu"), precision="MIXED")
    rng = np.random.default_rng(no + 10 * nv)
    t1 = 0.05 * rng.standard_normal((no, nv))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    o, v = slice(0, no), slice(no, no + nv)
    want1, want2 = oc.residuals(o, v, F, ERI, L, t1, t2)
    eng = w.mixed_engine()
    for stage in range(len(eng.stages)):
        eng.stage = stage
        r1, r2 = w.residuals(w.H.F, torch.from_numpy(t1), torch.from_numpy(t2))
        assert rel(r1, want1) < 1e-13 and rel(r2, want2) < 1e-13, eng.stages[stage]
