"""Tensor-core (tcgen05) engine: exactness on integer data, error bounds per format, and the
mixed-precision CCSD residual / energy against the FP64 oracle.

Tolerances: BF16 relative Frobenius error < 2e-2, split-BF16x3 < 5e-5, FP8 (per-row scaled)
< 8e-2 on random normal operands; integer-valued operands are exact in every format whose
input type represents them.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from pycc_gb300.tc import FMT_BF16, FMT_BF16X3, FMT_FP8, Operand, TCEngine
from oracle import ccsd as oc

pytestmark = pytest.mark.gpu
TOL = {FMT_BF16: 2e-2, FMT_BF16X3: 5e-5, FMT_FP8: 8e-2}


def frob(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3, FMT_FP8])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (200, 70, 100), (37, 300, 513), (64, 180, 96),
                                   (100, 210, 64), (150, 150, 64), (300, 820, 200)])
def test_gemm_exact_integers(cuda, fmt, M, N, K):
    g = torch.Generator(device=cuda).manual_seed(M + N + K)
    A = torch.randint(-3, 4, (M, K), generator=g, device=cuda).double()
    B = torch.randint(-3, 4, (N, K), generator=g, device=cuda).double()
    if fmt == FMT_FP8:          # rows scaled by max|.|/448 stay exact for these magnitudes
        A[:, 0] = 3.0
        B[:, 0] = 3.0
    eng = TCEngine(cuda)
    out = torch.zeros(M, N, dtype=torch.float64, device=cuda)
    eng.contract("mk,nk->mn", Operand.of("mk", A), Operand.of("nk", B), out, fmt=fmt)
    torch.cuda.synchronize()
    eng.check_status()
    ref = A @ B.T
    assert torch.equal(out, ref)


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3, FMT_FP8])
def test_gemm_random_error(cuda, fmt):
    g = torch.Generator(device=cuda).manual_seed(5)
    A = torch.randn(333, 1000, generator=g, device=cuda, dtype=torch.float64)
    B = torch.randn(259, 1000, generator=g, device=cuda, dtype=torch.float64)
    eng = TCEngine(cuda)
    out = torch.ones(333, 259, dtype=torch.float64, device=cuda)
    eng.contract("mk,nk->mn", Operand.of("mk", A), Operand.of("nk", B), out, alpha=0.5,
                 beta=2.0, fmt=fmt)
    torch.cuda.synchronize()
    ref = 2.0 + 0.5 * (A @ B.T)
    assert frob(out, ref) < TOL[fmt]


def test_permuted_operands_and_output(cuda):
    """A ring-type term with composite operands: (t2 - t2') . W -> r[i,j,a,b]."""
    g = torch.Generator(device=cuda).manual_seed(9)
    o, v = 6, 21
    t2 = torch.randn(o, o, v, v, generator=g, device=cuda, dtype=torch.float64)
    W = torch.randn(o, v, v, o, generator=g, device=cuda, dtype=torch.float64)
    r = torch.randn(o, o, v, v, generator=g, device=cuda, dtype=torch.float64)
    ref = r + torch.einsum("imae,mbej->ijab", t2 - t2.transpose(2, 3), W)
    eng = TCEngine(cuda)
    eng.contract("imae,mbej->ijab", Operand("imae", (t2, "imae"), Y=(t2, "imea"), b=-1.0),
                 Operand.of("mbej", W), r, fmt=FMT_BF16X3)
    torch.cuda.synchronize()
    assert frob(r, ref) < TOL[FMT_BF16X3]


def test_split_k_small_output(cuda):
    g = torch.Generator(device=cuda).manual_seed(2)
    A = torch.randn(40, 60000, generator=g, device=cuda, dtype=torch.float64)
    B = torch.randn(30, 60000, generator=g, device=cuda, dtype=torch.float64)
    out = torch.full((40, 30), 3.0, dtype=torch.float64, device=cuda)
    eng = TCEngine(cuda)
    eng.contract("mk,nk->mn", Operand.of("mk", A), Operand.of("nk", B), out, beta=0.0,
                 fmt=FMT_BF16X3)
    torch.cuda.synchronize()
    assert frob(out, A @ B.T) < TOL[FMT_BF16X3]


@pytest.fixture(scope="module")
def h1(cuda, cfg1_ham):
    _, F, ERI, L = cfg1_ham
    return pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)


def test_mixed_residual_cfg1(cuda, h1, cfg1):
    t1 = torch.from_numpy(cfg1["probe_t1"]).to(cuda)
    t2 = torch.from_numpy(np.ascontiguousarray(cfg1["probe_t2"])).to(cuda)
    for mode, tol in (("bf16x3", 1e-4), ("fast", 5e-2)):
        w = pg.CCwfn(h1, precision="MIXED")
        w.mixed_engine().select_mode(0.0 if mode == "bf16x3" else 1.0)
        r1, r2 = w.residuals(h1.F, t1, t2)
        torch.cuda.synchronize()
        e1 = np.abs(r1.cpu().numpy() - cfg1["r1"]).max() / np.abs(cfg1["r1"]).max()
        e2 = np.abs(r2.cpu().numpy() - cfg1["r2"]).max() / np.abs(cfg1["r2"]).max()
        assert e1 < tol and e2 < tol, (mode, e1, e2)


def test_mixed_solve_cfg1(cuda, h1, cfg1):
    w = pg.CCwfn(h1, precision="MIXED")
    e = w.solve_cc(1e-9, 1e-7, 100)
    assert abs(e - float(cfg1["ecc"])) < 1e-6
    assert w.mixed_engine().is_final_mode()


def test_sp_solve_cfg1(cuda, h1, cfg1):
    """precision='SP' (split-BF16x3 throughout) within 1e-7 of DP, as the reference's SP test."""
    w = pg.CCwfn(h1, precision="SP")
    e = w.solve_cc(1e-9, 1e-7, 100)
    assert abs(e - float(cfg1["ecc"])) < 1e-7


@pytest.mark.parametrize("no,nv", [(3, 17), (7, 33)])
def test_mixed_ragged_vs_oracle(cuda, no, nv):
    fac = pg.SyntheticFactors(no, nv, seed=5)
    F, ERI, L = fac.hamiltonian()
    o, v = slice(0, no), slice(no, no + nv)
    rng = np.random.default_rng(no * 100 + nv)
    t1 = 0.05 * rng.standard_normal((no, nv))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    r1o, r2o = oc.residuals(o, v, F, ERI, L, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_factors(fac, device=cuda), precision="SP")
    r1, r2 = w.residuals(w.H.F, torch.from_numpy(t1).to(cuda), torch.from_numpy(t2).to(cuda))
    torch.cuda.synchronize()
    assert np.abs(r2.cpu().numpy() - r2o).max() / np.abs(r2o).max() < 1e-4
    assert np.abs(r1.cpu().numpy() - r1o).max() / np.abs(r1o).max() < 1e-4
