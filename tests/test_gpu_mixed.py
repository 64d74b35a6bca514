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
from pycc_gb300.tc import (FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_FP8, Operand,
                           TCEngine)
from oracle import ccsd as oc

pytestmark = pytest.mark.gpu
TOL = {FMT_BF16: 2e-2, FMT_BF16X3: 5e-5, FMT_BF16X3F: 5e-5, FMT_BF16X3S: 5e-5, FMT_FP8: 8e-2}


def frob(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_FP8])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (200, 70, 100), (37, 300, 513), (64, 180, 96),
                                   (100, 210, 64), (150, 150, 64), (300, 820, 200),
                                   (3000, 2000, 64), (700, 1000, 128)])
def test_gemm_exact_integers(cuda, fmt, M, N, K):
    """N = 70, 150, 180, 210, 820 select the 96-, 160-, 192- and 224-column tiles (fused
    formats stop at 160); 3000 x 2000 walks several raster groups, the last one partial.
    N is cut into tiles of near-equal width below the tile's capacity (820 = 5 x 144 + 100
    and 1000 = 6 x 144 + 136 in 160-column tiles, 210 = 112 + 98)."""
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


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_FP8])
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


def _pack_inputs(cuda):
    """FP64 values across the cases the FP32 rounding of the pack meets: random magnitudes,
    exact FP32 ties (both parities), signed zeros, FP32's extremes and FP64 values beyond
    them (which round to zero or infinity)."""
    g = torch.Generator(device=cuda).manual_seed(11)
    v = torch.randn(37, 200, generator=g, device=cuda, dtype=torch.float64)
    v = v * torch.exp2(torch.randint(-60, 60, (37, 200), generator=g, device=cuda).double())
    ties = []
    for m in (1, 2, 3, 0x7fffff, 0x400000):              # FP32 mantissas, odd and even
        base = (1.0 + m * 2.0 ** -23)
        ties += [base + 2.0 ** -24, -(base + 2.0 ** -24), base + 2.0 ** -24 + 2.0 ** -40,
                 base + 2.0 ** -24 - 2.0 ** -40]
    edge = ties + [0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 1.1754943508222875e-38,
                   3.4028235677973366e38, 1e-300, -1e300]
    v[0, :len(edge)] = torch.tensor(edge, dtype=torch.float64, device=cuda)
    return v


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3])
def test_pack_rounding_bit_exact(cuda, fmt):
    """Packed pieces equal FP64 -> FP32 (round to nearest even) -> BF16 pieces, bit for bit:
    hi = bf16(f), lo = bf16(f - hi) with f the FP32 rounding of the value (zero below
    FP32's normal range, infinity above it)."""
    from pycc_gb300.tc import pack
    v = _pack_inputs(cuda)
    P = pack(Operand.of("rk", v), "r", "k", fmt)
    torch.cuda.synchronize()
    f = v.float()
    f = torch.where(f.abs() < 2.0 ** -126, f * 0.0, f)        # signed zero
    hi = f.bfloat16()
    K = v.shape[1]
    assert torch.equal(P.hi[:, :K].view(torch.int16), hi.view(torch.int16))
    assert torch.all(P.hi[:, K:].float() == 0)
    if fmt == FMT_BF16X3:
        lo = torch.where(torch.isinf(f), torch.full_like(f, float("nan")), f - hi.float())
        lo = lo.bfloat16()
        fin = torch.isfinite(f)
        assert torch.equal(P.lo[:, :K][fin].view(torch.int16), lo[fin].view(torch.int16))


@pytest.mark.parametrize("rows,ks", [("ij", "k"), ("k", "ij"), ("ki", "j")])
def test_pack_combination(cuda, rows, ks):
    """a*X + b*Y + c*P*Q with permuted sources and K padding, against FP64 within the FP32
    rounding of the operands; K along X's unit-stride index (the K-gathering pack), rows
    along it (the row-gathering pack), and rows whose unit-stride sub-index is the outer one
    (walked innermost, each walked row written to its own output row)."""
    from pycc_gb300.tc import pack
    g = torch.Generator(device=cuda).manual_seed(12)
    X = torch.randn(7, 9, 70, generator=g, device=cuda, dtype=torch.float64)
    Y = torch.randn(9, 7, 70, generator=g, device=cuda, dtype=torch.float64)
    Pm = torch.randn(7, 70, generator=g, device=cuda, dtype=torch.float64)
    Q = torch.randn(9, generator=g, device=cuda, dtype=torch.float64)
    op = Operand("ijk", (X, "ijk"), a=2.0, Y=(Y, "jik"), b=-0.5, P=(Pm, "ik"), Q=(Q, "j"), c=0.25)
    P = pack(op, rows, ks, FMT_BF16X3)
    torch.cuda.synchronize()
    parts = (2.0 * X, -0.5 * Y.transpose(0, 1), 0.25 * Pm[:, None, :] * Q[None, :, None])
    perm = ["ijk".index(c) for c in rows + ks]
    nr = int(np.prod([X.shape["ijk".index(c)] for c in rows]))
    ref = sum(parts).permute(*perm).reshape(nr, -1)
    scale = sum(q.abs() for q in parts).permute(*perm).reshape(nr, -1)
    K = ref.shape[1]
    got = P.hi[:, :K].double() + P.lo[:, :K].double()
    # split error 2^-17 of the value, FP32 combination 2^-24 of each operand (a few roundings)
    assert torch.all((got - ref).abs() <= 2.0 ** -16 * ref.abs() + 2.0 ** -21 * scale)
    assert torch.all(P.hi[:, K:].float() == 0) and torch.all(P.lo[:, K:].float() == 0)


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
def h1(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    return pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)


def test_mixed_residual_golden_o5v19(cuda, h1, golden_o5v19):
    t1 = torch.from_numpy(golden_o5v19["probe_t1"]).to(cuda)
    t2 = torch.from_numpy(np.ascontiguousarray(golden_o5v19["probe_t2"])).to(cuda)
    for mode, tol in (("bf16x3", 1e-4), ("fast", 5e-2)):
        w = pg.CCwfn(h1, precision="MIXED")
        w.mixed_engine().select_mode(0.0 if mode == "bf16x3" else 1.0)
        r1, r2 = w.residuals(h1.F, t1, t2)
        torch.cuda.synchronize()
        e1 = np.abs(r1.cpu().numpy() - golden_o5v19["r1"]).max() / np.abs(golden_o5v19["r1"]).max()
        e2 = np.abs(r2.cpu().numpy() - golden_o5v19["r2"]).max() / np.abs(golden_o5v19["r2"]).max()
        assert e1 < tol and e2 < tol, (mode, e1, e2)


def test_mixed_solve_golden_o5v19(cuda, h1, golden_o5v19):
    w = pg.CCwfn(h1, precision="MIXED")
    e = w.solve_cc(1e-9, 1e-7, 100)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-6
    assert w.mixed_engine().is_final_mode()


def test_sp_solve_golden_o5v19(cuda, h1, golden_o5v19):
    """precision='SP' (split-BF16x3 throughout) within 1e-7 of DP, as the reference's SP test."""
    w = pg.CCwfn(h1, precision="SP")
    e = w.solve_cc(1e-9, 1e-7, 100)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-7


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


def test_pack_tables_and_second_product(cuda):
    """a*X + b*Y + c*P*Q + d*R*S with explicit row and K offset tables and K multipliers
    (the pair form of the ladder: T+_ij,ef = tau_ijef + tau_ijfe over i <= j, e <= f),
    against FP64 within the FP32 rounding of the operands."""
    import numpy as np
    from pycc_gb300.tc import pack
    g = torch.Generator(device=cuda).manual_seed(13)
    no, nv = 5, 23
    t2 = torch.randn(no, no, nv, nv, generator=g, device=cuda, dtype=torch.float64)
    t1 = torch.randn(no, nv, generator=g, device=cuda, dtype=torch.float64)
    i, j = np.triu_indices(no)
    e, f = np.triu_indices(nv)
    s2, s1 = t2.stride(), t1.stride()
    rt = np.zeros((6, i.size), dtype=np.int64)
    rt[0] = rt[1] = i * s2[0] + j * s2[1]
    rt[2] = rt[4] = i * s1[0]
    rt[3] = rt[5] = j * s1[0]
    kt = np.zeros((6, e.size), dtype=np.int64)
    kt[0], kt[1] = e * s2[2] + f * s2[3], f * s2[2] + e * s2[3]
    kt[2], kt[3], kt[4], kt[5] = e, f, f, e
    kw = np.where(e == f, 0.5, 1.0).astype(np.float32)
    op = Operand("ijef", (t2, "ijef"), a=1.0, Y=(t2, "ijfe"), b=-1.0, P=(t1, "ie"), Q=(t1, "jf"),
                 c=1.0, R=(t1, "if"), S=(t1, "je"), d=-1.0)
    tt = lambda x: torch.from_numpy(x).to(cuda)
    P = pack(op, ["i", "j"], ["e", "f"], FMT_BF16X3, row_tab=tt(rt), k_tab=tt(kt), k_w=tt(kw))
    torch.cuda.synchronize()
    tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
    I, J, E, Fi = (torch.from_numpy(x).to(cuda) for x in (i, j, e, f))
    ref = (tau[I[:, None], J[:, None], E[None, :], Fi[None, :]]
           - tau[I[:, None], J[:, None], Fi[None, :], E[None, :]]) * tt(kw).double()[None, :]
    K = e.size
    got = P.hi[:, :K].double() + P.lo[:, :K].double()
    assert got.shape == ref.shape
    assert torch.all((got - ref).abs() <= 2.0 ** -16 * ref.abs() + 2.0 ** -19)
    assert torch.all(P.hi[:, K:].float() == 0)


def _ladder_setup(cuda, no, nv, integer=False, seed=3):
    g = torch.Generator(device=cuda).manual_seed(seed)
    if integer:
        V = torch.randint(-2, 3, (nv, nv, nv, nv), generator=g, device=cuda).double()
        t2 = torch.randint(-2, 3, (no, no, nv, nv), generator=g, device=cuda).double()
        t1 = torch.randint(-1, 2, (no, nv), generator=g, device=cuda).double()
    else:
        V = torch.randn(nv, nv, nv, nv, generator=g, device=cuda, dtype=torch.float64)
        t2 = 0.1 * torch.randn(no, no, nv, nv, generator=g, device=cuda, dtype=torch.float64)
        t1 = 0.1 * torch.randn(no, nv, generator=g, device=cuda, dtype=torch.float64)
    V = V + V.permute(1, 0, 3, 2)              # <ab|ef> = <ba|fe>
    t2 = t2 + t2.permute(1, 0, 3, 2)           # t2_ijab = t2_jiba
    tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
    ref = 0.5 * torch.einsum("ijef,abef->ijab", tau, V)
    ref = ref + ref.permute(1, 0, 3, 2)        # through the symmetrisation
    return V, t1, t2.contiguous(), ref


def _ladder_run(cuda, V, t1, t2, fmt):
    from types import SimpleNamespace
    from pycc_gb300.mixed import MixedResidual
    no, nv = t1.shape
    w = SimpleNamespace(device1=cuda, stream=None, no=no, nv=nv, vvvv_fp8=True,
                        switch_threshold=1e-5,
                        H=SimpleNamespace(ERI=SimpleNamespace(blocks={"vvvv": V})))
    eng = MixedResidual(w)
    h = torch.zeros(no, no, nv, nv, dtype=torch.float64, device=cuda)
    eng.ladder_pm(t1, t2, h, fmt)
    torch.cuda.synchronize()
    eng.tc.check_status()
    return h + h.permute(1, 0, 3, 2)


@pytest.mark.parametrize("no,nv", [(4, 24), (5, 37), (1, 9)])
def test_ladder_pair_form_exact_integers(cuda, no, nv):
    """The symmetric / antisymmetric pair form of the <ab|ef> ladder is exact on integer data
    in BF16 (every packed value and partial sum is an integer below 2^24)."""
    V, t1, t2, ref = _ladder_setup(cuda, no, nv, integer=True)
    got = _ladder_run(cuda, V, t1, t2, FMT_BF16)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3F, FMT_BF16X3S, FMT_FP8])
def test_ladder_pair_form_random(cuda, fmt):
    """The ladder's pair form in each format against FP64, within the format's bound."""
    V, t1, t2, ref = _ladder_setup(cuda, 6, 45)
    got = _ladder_run(cuda, V, t1, t2, fmt)
    assert frob(got, ref) < TOL[fmt]


def _pair_tau_run(cuda, X, t1, t2, fmt):
    """out[r, i, j] = sum_ef tau_ijef X[r.., e, f] through MixedResidual.pair_tau."""
    from types import SimpleNamespace
    from pycc_gb300.mixed import MixedResidual
    no, nv = t1.shape
    V = torch.zeros(nv, nv, nv, nv, dtype=torch.float64, device=cuda)  # only its strides
    w = SimpleNamespace(device1=cuda, stream=None, no=no, nv=nv, vvvv_fp8=True,
                        switch_threshold=1e-5,
                        H=SimpleNamespace(ERI=SimpleNamespace(blocks={"vvvv": V})))
    eng = MixedResidual(w)
    out = torch.ones(X.shape[:-2] + (no, no), dtype=torch.float64, device=cuda)
    eng.pair_tau(X, "mbef", "ovvv", t1, t2, out, fmt)
    torch.cuda.synchronize()
    eng.tc.check_status()
    return out


@pytest.mark.parametrize("no,nv,nb", [(4, 24, 3), (5, 37, 2), (1, 9, 4), (6, 1, 5)])
def test_pair_form_intermediate_exact_integers(cuda, no, nv, nb):
    """Zmbij-shaped tau_ijef X_mbef (X without any symmetry) in the pair form, added into an
    output of ones: exact on integer data in BF16, including no = 1 (no antisymmetric
    pairs) and nv = 1 (no e < f pairs)."""
    g = torch.Generator(device=cuda).manual_seed(no * nv + nb)
    X = torch.randint(-2, 3, (no, nb, nv, nv), generator=g, device=cuda).double()
    t2 = torch.randint(-2, 3, (no, no, nv, nv), generator=g, device=cuda).double()
    t1 = torch.randint(-1, 2, (no, nv), generator=g, device=cuda).double()
    t2 = (t2 + t2.permute(1, 0, 3, 2)).contiguous()
    tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
    ref = 1.0 + torch.einsum("ijef,mbef->mbij", tau, X)
    assert torch.equal(_pair_tau_run(cuda, X, t1, t2, FMT_BF16), ref)


@pytest.mark.parametrize("fmt", [FMT_BF16, FMT_BF16X3F, FMT_BF16X3S])
def test_pair_form_intermediate_random(cuda, fmt):
    g = torch.Generator(device=cuda).manual_seed(9)
    no, nv = 6, 45
    X = torch.randn(no, 7, nv, nv, generator=g, device=cuda, dtype=torch.float64)
    t2 = 0.1 * torch.randn(no, no, nv, nv, generator=g, device=cuda, dtype=torch.float64)
    t1 = 0.1 * torch.randn(no, nv, generator=g, device=cuda, dtype=torch.float64)
    t2 = (t2 + t2.permute(1, 0, 3, 2)).contiguous()
    tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
    ref = torch.einsum("ijef,mbef->mbij", tau, X)
    got = _pair_tau_run(cuda, X, t1, t2, fmt) - 1.0
    assert frob(got, ref) < TOL[fmt]
