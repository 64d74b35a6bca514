"""The callers on either side of the residual, on the GPU.

* Complex residual (the reference's real-time propagation, pycc/rt/rtcc.py:139, which calls
  ``residuals(F, t1, t2, real_time=True)`` with complex F / t1 / t2): against the reference's
  own complex residual (tests/golden/o5v19_complex.npz), 1e-12 relative in FP64 and within
  the split-BF16x3 bound (5e-4 relative: five real residuals, Lagrange weights up to 2.5) in
  the mixed engine's final stage.
* Linear-in-H use (the derivative driver swaps H.ERI / H.L for derivative integrals around
  one residual call, pycc/ccderiv.py:252-259): the mixed engine re-packs the swapped blocks
  and matches the oracle's residual at the swapped integrals, then the original one after
  the swap back.
* psi4-free input (``Hamiltonian.from_npz``, full <pq|rs> or three-index factor) and the
  amplitude checkpoint (``save_amplitudes`` / ``load_amplitudes``): the same resident
  blocks as ``from_arrays``; a warm start converges at once to the reference's energy.
* The adjoint's tensor-core sweep engine (``sweep='tc'``, the default for MIXED / SP wave
  functions): J x against the reference's ``_ccsd_jacobian`` (o5v19_jacobian.npz) and J^T l
  against the FP64 sweep within 1e-4 relative (split-BF16x3 products); Lambda and the
  gradient densities against the reference's: within 1e-5 when the solve stops at the
  tensor cores' rounding floor, within 1e-9 (the FP64 bar) after the FP64 polish.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from conftest import golden
from oracle import ccsd as oc
from pycc_gb300.adjoint import CCSDAdjoint, symmetrize8

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def h1(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    return pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)


@pytest.mark.parametrize("precision,tol", [("DP", 1e-12), ("MIXED", 5e-4)])
def test_complex_residual_vs_reference(cuda, h1, precision, tol):
    g = golden("o5v19_complex.npz")
    w = pg.CCwfn(h1, precision=precision, real_time=True)
    if precision != "DP":
        w.mixed_engine().select_mode(0.0)          # the final (split-BF16x3) stage
    Fc, t1, t2 = (torch.from_numpy(g[k]).to(cuda) for k in ("F", "t1", "t2"))
    r1, r2 = w.residuals(Fc, t1, t2, real_time=True)
    torch.cuda.synchronize()
    assert r1.dtype == torch.complex128 and r2.dtype == torch.complex128
    e1, e2 = rel(r1, g["r1"]), rel(r2, g["r2"])
    print("complex residual %s: r1 %.2e r2 %.2e" % (precision, e1, e2))
    assert e1 < tol and e2 < tol


def test_swapped_integrals_mixed(cuda, h1, ham_o5v19, golden_o5v19):
    """The reference's linear-in-H call: derivative integrals (here a second synthetic
    Hamiltonian's blocks and a symmetric one-electron perturbation) swapped in for one
    residual call, then swapped back."""
    g = golden_o5v19
    no, nv = 5, 19
    o, v = slice(0, no), slice(no, no + nv)
    fac = pg.SyntheticFactors(no, nv, 9)
    _, dERI, dL = fac.hamiltonian()
    rng = np.random.default_rng(4)
    dF = rng.standard_normal((no + nv, no + nv))
    dF = 0.1 * (dF + dF.T)
    dH = pg.Hamiltonian.from_arrays(dF, dERI, no, L=dL, device=cuda)
    t1 = torch.from_numpy(g["probe_t1"]).to(cuda)
    t2 = torch.from_numpy(np.ascontiguousarray(g["probe_t2"])).to(cuda)
    w = pg.CCwfn(h1, precision="MIXED")
    w.mixed_engine().select_mode(0.0)
    r1a, r2a = w.residuals(w.H.F, t1, t2)                  # packs the original blocks
    saved = (w.H.ERI, w.H.L)
    w.H.ERI, w.H.L = dH.ERI, dH.L
    r1, r2 = w.residuals(dH.F, t1, t2)
    w.H.ERI, w.H.L = saved
    r1b, r2b = w.residuals(w.H.F, t1, t2)
    torch.cuda.synchronize()
    ro1, ro2 = oc.residuals(o, v, dF, dERI, dL, g["probe_t1"], g["probe_t2"])
    errs = [rel(r1, ro1), rel(r2, ro2), rel(r1b, g["r1"]), rel(r2b, g["r2"])]
    print("swapped integrals: %s" % ["%.2e" % x for x in errs])
    assert max(errs) < 1e-4
    # the same values as before the swap (split-K atomics may reorder the last bits)
    assert (r2b - r2a).abs().max().item() <= 1e-12 * r2a.abs().max().item()


def test_from_npz_and_warm_start(cuda, tmp_path, ham_o5v19, golden_o5v19):
    fac, F, ERI, L = ham_o5v19
    ref = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)
    np.savez(tmp_path / "full.npz", no=5, F=F, ERI=ERI)
    np.savez(tmp_path / "fac.npz", no=5, F=F, B=fac.B)
    for name in ("full.npz", "fac.npz"):
        H = pg.Hamiltonian.from_npz(tmp_path / name, device=cuda)
        assert torch.equal(H.F, ref.F)
        for X, Y in ((H.ERI, ref.ERI), (H.L, ref.L)):
            for pat, blk in Y.blocks.items():
                assert X.blocks[pat].is_cuda
                assert (X.blocks[pat] - blk).abs().max().item() < 1e-14, (name, pat)
    H = pg.Hamiltonian.from_npz(tmp_path / "fac.npz", device=cuda)
    w = pg.CCwfn(H)
    e = w.solve_cc(1e-12, 1e-12)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-10
    path = tmp_path / "amps.npz"
    w.save_amplitudes(path)
    w2 = pg.CCwfn(H)
    w2.load_amplitudes(path)
    assert torch.equal(w2.t2, w.t2) and torch.equal(w2.t1, w.t1)
    e2 = w2.solve_cc(1e-10, 1e-10)
    assert w2.niter <= 2 and abs(e2 - float(golden_o5v19["ecc"])) < 1e-10
    m = pg.CCwfn(H, precision="MIXED")
    m.load_amplitudes(path)
    em = m.solve_cc(1e-10, 1e-10, 40)
    assert m.mixed_engine().history[0] == "bf16x3s"
    assert abs(em - float(golden_o5v19["ecc"])) < 1e-6


def test_tensor_core_sweeps(cuda, h1, golden_o5v19):
    g = golden_o5v19
    jg = golden("o5v19_jacobian.npz")
    w = pg.CCwfn(h1)
    w.t1 = torch.from_numpy(jg["t1"]).to(cuda)
    w.t2 = torch.from_numpy(jg["t2"]).to(cuda)
    ref = CCSDAdjoint(w, sweep="fp64")
    tc = CCSDAdjoint(w, sweep="tc")
    tc.tc_min_flops = 0                                      # every GEMM-shaped product
    s1, s2 = tc.jacobian(torch.from_numpy(jg["X1"]).to(cuda), torch.from_numpy(jg["X2"]).to(cuda))
    sym = s2 + s2.permute(1, 0, 3, 2)
    ej = (rel(s1, jg["sigma1"]), rel(sym, jg["sigma2_sym"]))
    gen = torch.Generator(device=cuda).manual_seed(9)
    l1 = torch.randn(5, 19, dtype=torch.float64, device=cuda, generator=gen)
    l2 = torch.randn(5, 5, 19, 19, dtype=torch.float64, device=cuda, generator=gen)
    Ga = [ref.backward(l1=l1, l2=l2).get(t).clone() for t in (ref.t1, ref.t2)]
    Gb = [tc.backward(l1=l1, l2=l2).get(t).clone() for t in (tc.t1, tc.t2)]
    eb = [((a - b).abs().max() / a.abs().max()).item() for a, b in zip(Ga, Gb)]
    tc._check_tc()
    w2 = pg.CCwfn(h1)
    w2.t1 = torch.from_numpy(g["t1"]).to(cuda)
    w2.t2 = torch.from_numpy(np.ascontiguousarray(g["t2"])).to(cuda)
    res = {}
    sym2 = lambda X: 0.5 * (X + X.T)
    Dg = torch.from_numpy(g["D"]).to(cuda)
    Gg = symmetrize8(torch.from_numpy(g["Gamma"]).to(cuda))
    for polish in (False, True):
        adj = CCSDAdjoint(w2, sweep="tc")
        adj.tc_min_flops = 0
        adj.solve_lambda(1e-10, 1e-10, 200, polish=polish)
        gF, Gam = adj.gradient()
        res[polish] = ((sym2(gF) - sym2(Dg)).abs().max().item(),
                       (symmetrize8(Gam) - Gg).abs().max().item(),
                       adj.lambda_stages.count("tc"), adj.lambda_stages.count("fp64"))
    print("tc sweeps: J.x %.2e %.2e  J^T l %.2e %.2e  Lambda at the floor: D %.2e Gamma %.2e "
          "(%d tc iterations); polished: D %.2e Gamma %.2e (%d tc + %d fp64)"
          % (ej[0], ej[1], eb[0], eb[1], res[False][0], res[False][1], res[False][2],
             res[True][0], res[True][1], res[True][2], res[True][3]))
    assert max(ej) < 1e-4 and max(eb) < 1e-4
    assert res[False][0] < 1e-5 and res[False][1] < 1e-5
    assert res[True][0] < 1e-9 and res[True][1] < 1e-9


def test_tc_lambda_floor_refined_densities(cuda, h1, golden_o5v19):
    """Lambda stopped at the tensor cores' floor, then the FP64 density sweep with its
    one-step correction: the densities within 1e-10 of the reference's."""
    g = golden_o5v19
    w = pg.CCwfn(h1)
    w.t1 = torch.from_numpy(g["t1"]).to(cuda)
    w.t2 = torch.from_numpy(np.ascontiguousarray(g["t2"])).to(cuda)
    adj = CCSDAdjoint(w, sweep="tc")
    adj.tc_min_flops = 0
    adj.solve_lambda(1e-12, 1e-12, 200, polish=False)
    gF, Gam = adj.gradient()
    sym2 = lambda X: 0.5 * (X + X.T)
    ed = (sym2(gF) - sym2(torch.from_numpy(g["D"]).to(cuda))).abs().max().item()
    eg = (symmetrize8(Gam) - symmetrize8(torch.from_numpy(g["Gamma"]).to(cuda))).abs().max().item()
    print("tc Lambda at the floor (%s), refined: D %.2e Gamma %.2e"
          % (adj.lambda_at_floor, ed, eg))
    assert adj.lambda_refined == adj.lambda_at_floor
    assert ed < 1e-10 and eg < 1e-10
