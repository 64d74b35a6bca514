"""(T) correction on the GPU against the reference's energies and the CPU oracle.

Tolerances: FP64 path 1e-11 Eh (absolute) against t_tjl / t_vikings; the BF16 tensor-core
path within 1e-5 Eh of the reference at no=5, nv=19 and 1e-6 Eh of the FP64 path at no=10,
nv=80 (2e-3 relative on the small ragged cases); the grouped GEMM is exact on integer data.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from pycc_gb300 import _lib
from pycc_gb300.triples import t_energy_fp64
from pycc_gb300.triples_tc import GROUP_DTYPE, t_energy_tc
from pycc_gb300.tc import FMT_BF16, Operand, pack
from oracle import ccsd as oc
from oracle import triples as ot

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w1(cuda, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    w.t1.copy_(torch.from_numpy(golden_o5v19["t1"]))
    w.t2.copy_(torch.from_numpy(np.ascontiguousarray(golden_o5v19["t2"])))
    return w


def test_fp64_triples_golden_o5v19(w1, golden_o5v19):
    et = t_energy_fp64(w1)
    assert abs(et - float(golden_o5v19["et_tjl"])) < 1e-11
    assert abs(et - float(golden_o5v19["et_vikings"])) < 1e-11


def test_tc_triples_golden_o5v19(w1, golden_o5v19):
    et = t_energy_tc(w1, batch=7)
    ref = float(golden_o5v19["et_tjl"])
    # BF16 operands: at this size few terms average the rounding out (measured 6.0e-6 Eh,
    # 2e-4 relative; 6.5e-7 Eh at no=10, nv=80 and 8e-8 Eh at no=30, nv=240)
    print("(T) o5v19: tc %.12f reference %.12f diff %.2e" % (et, ref, et - ref))
    assert abs(et - ref) < 1e-5, (et, ref)


@pytest.mark.parametrize("no,nv", [(3, 17), (6, 23)])
def test_triples_vs_oracle(cuda, no, nv):
    fac = pg.SyntheticFactors(no, nv, seed=11, coupling="matched")
    F, ERI, L = fac.hamiltonian()
    t1, t2 = oc.mp2_guess(F, ERI, no)
    rng = np.random.default_rng(no + nv)
    t1 = 0.01 * rng.standard_normal((no, nv))
    ref = ot.t_tjl(no, nv, F, ERI, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, L=L, device=cuda))
    w.t1.copy_(torch.from_numpy(t1))
    et = t_energy_fp64(w)
    assert abs(et - ref) < 1e-11 * max(1.0, abs(ref) * 1e3)
    et_tc = t_energy_tc(w, batch=5)
    assert abs(et_tc - ref) < 2e-3 * abs(ref)


def test_ccsd_t_model(cuda, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda), model="CCSD(T)")
    e = w.solve_cc(1e-12, 1e-12, 100)
    assert abs(e - (float(golden_o5v19["ecc"]) + float(golden_o5v19["et_tjl"]))) < 1e-10


@pytest.mark.parametrize("layout", ["row", "col"])
def test_grouped_gemm_exact(cuda, layout):
    """Two groups with two K segments each, integer data: exact against torch, with the
    output row-major (ldm=N, ldn=1) or column-major (ldm=1, ldn=M, the (T) layout).  N=150
    takes the 160-wide tile (a 16-column remainder per epilogue warp)."""
    g = torch.Generator(device=cuda).manual_seed(3)
    M, N = 300, 150
    A0 = torch.randint(-3, 4, (2 * M, 64), generator=g, device=cuda).double()
    A1 = torch.randint(-3, 4, (M, 128), generator=g, device=cuda).double()
    B0 = torch.randint(-3, 4, (N + 20, 64), generator=g, device=cuda).double()
    B1 = torch.randint(-3, 4, (2 * N, 128), generator=g, device=cuda).double()
    pk = lambda X: pack(Operand.of("rk", X), ["r"], ["k"], FMT_BF16)
    pa, pb = [pk(A0), pk(A1)], [pk(B0), pk(B1)]
    gd = np.zeros(2, dtype=GROUP_DTYPE)
    # group 0: A0[0:M] B0[0:N] + A1 B1[N:2N];  group 1: A0[M:2M] B0[20:20+N]
    gd[0]["nseg"] = 2
    gd[0]["amap"][:2], gd[0]["arow"][:2] = [0, 1], [0, 0]
    gd[0]["bmap"][:2], gd[0]["brow"][:2], gd[0]["nkb"][:2] = [0, 1], [0, N], [1, 2]
    gd[0]["out"] = 0
    gd[1]["nseg"] = 1
    gd[1]["amap"][0], gd[1]["arow"][0], gd[1]["bmap"][0], gd[1]["brow"][0] = 0, M, 0, 20
    gd[1]["nkb"][0] = 1
    gd[1]["out"] = M * N
    gt = torch.from_numpy(gd.view(np.uint8)).to(cuda)
    shape = (2, M, N) if layout == "row" else (2, N, M)
    ldm, ldn = (N, 1) if layout == "row" else (1, M)
    out = torch.full(shape, float("nan"), dtype=torch.float32, device=cuda)
    st = torch.zeros(4, dtype=torch.int32, device=cuda)
    a_ptr = (C.c_void_p * 2)(*[x.hi.data_ptr() for x in pa])
    b_ptr = (C.c_void_p * 2)(*[x.hi.data_ptr() for x in pb])
    _lib.call("pcg_tc_grouped_gemm", 2, a_ptr, _lib.i64s([x.rows for x in pa]),
              _lib.i64s([x.Kp for x in pa]), 2, b_ptr, _lib.i64s([x.rows for x in pb]),
              _lib.i64s([x.Kp for x in pb]), gt.data_ptr(), 2, M, N, out.data_ptr(), ldm, ldn,
              st.data_ptr(), _lib.stream_handle())
    torch.cuda.synchronize()
    if layout == "col":
        out = out.transpose(1, 2)
    ref0 = A0[:M] @ B0[:N].T + A1 @ B1[N:].T
    ref1 = A0[M:] @ B0[20:20 + N].T
    assert torch.equal(out[0].double(), ref0)
    assert torch.equal(out[1].double(), ref1)
    assert int(st.abs().sum()) == 0


def test_tc_triples_mid_size_vs_fp64(cuda):
    """The tensor-core (T) (BF16 operands, FP32 accumulation, FP64 energy sum) against the
    FP64 (T) at no=10, nv=80 (MP2 doubles, small random singles): within 1e-6 Eh, the
    accuracy bar of the mixed-precision CCSD energy (measured: 6.5e-7 Eh, 1.8e-5 relative)."""
    fac = pg.SyntheticFactors(10, 80, seed=4, coupling="matched")
    w = pg.CCwfn(pg.Hamiltonian.from_factors(fac, device=cuda))
    g = torch.Generator(device=cuda).manual_seed(10)
    w.t1 = 0.01 * torch.randn(10, 80, dtype=torch.float64, device=cuda, generator=g)
    e64 = t_energy_fp64(w)
    etc = t_energy_tc(w, batch=32)
    print("(T) no=10 nv=80: fp64 %.12f tc %.12f diff %.2e" % (e64, etc, etc - e64))
    assert abs(etc - e64) < 1e-6


def test_t3_density_vs_reference(cuda, ham_o5v19):
    """(T) densities and Lambda sources on the GPU (FP64) against the reference's own
    t3_density (o5v19_t3density.npz): every block to 1e-12 relative, E(T) to 1e-12; and the
    CCSD(T) solve with make_t3_density=True returns the same E(T)."""
    from conftest import golden
    g = golden("o5v19_t3density.npz")
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)
    w = pg.CCwfn(H, model="CCSD(T)", make_t3_density=True)
    w.t1 = torch.from_numpy(g["t1"]).to(cuda)
    w.t2 = torch.from_numpy(np.ascontiguousarray(g["t2"])).to(cuda)
    et = w.t3_density()
    assert abs(et - float(g["et"])) < 1e-12
    for name in ("Doo", "Dvv", "Dov", "Goovv", "Gooov", "Gvvvo", "S1", "S2"):
        got = getattr(w, name).cpu().numpy()
        assert got.shape == g[name].shape, name
        assert np.abs(got - g[name]).max() <= 1e-12 * np.abs(g[name]).max(), name
    w2 = pg.CCwfn(H, model="CCSD(T)", make_t3_density=True)
    e = w2.solve_cc(1e-12, 1e-12, 100)
    assert abs(w2.et - float(g["et"])) < 1e-10 and hasattr(w2, "Gvvvo")
