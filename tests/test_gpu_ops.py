"""torch.ops.gbcc on the GPU against the reference's golden fixtures (o5v19.npz): every
builder, both residuals, the energy, the Jacobi update, the DIIS overlaps / combination and
the (T) energy, through the dispatcher.  FP64 bars: 1e-12 relative for tensors, 1e-12 Eh
for energies (1e-11 Eh for (T))."""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from pycc_gb300.ops import resident_blocks

pytestmark = pytest.mark.gpu
ops = torch.ops.gbcc


def rel(a, b):
    a = a.detach().cpu().numpy()
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def setup(cuda, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda)
    E, Lb = resident_blocks(H)
    g = golden_o5v19
    t1 = torch.from_numpy(g["probe_t1"]).to(cuda)
    t2 = torch.from_numpy(np.ascontiguousarray(g["probe_t2"])).to(cuda)
    return H, E, Lb, t1, t2, g


def test_builders_and_residuals(setup):
    H, E, Lb, t1, t2, g = setup
    F = H.F
    assert rel(ops.tau(t1, t2, 1.0, 1.0), g["tau"]) < 1e-12
    assert rel(ops.tau(t1, t2, 1.0, 0.5), g["taut"]) < 1e-12
    Fae, Fmi, Fme = ops.fae(F, Lb, t1, t2), ops.fmi(F, Lb, t1, t2), ops.fme(F, Lb, t1)
    W = (ops.wmnij(E, t1, t2), ops.wmbej(E, Lb, t1, t2), ops.wmbje(E, t1, t2),
         ops.zmbij(E, t1, t2))
    for got, key in zip((Fae, Fmi, Fme) + W, ("Fae", "Fmi", "Fme", "Wmnij", "Wmbej", "Wmbje",
                                              "Zmbij")):
        assert rel(got, g[key]) < 1e-12, key
    r1 = ops.r_t1(F, E, Lb, t1, t2, Fae, Fme, Fmi)
    r2 = ops.r_t2(F, E, t1, t2, Fae, Fme, Fmi, *W)
    assert rel(r1, g["r1"]) < 1e-12 and rel(r2, g["r2"]) < 1e-12
    q1, q2 = ops.residuals(F, E, Lb, t1, t2)
    assert rel(q1, g["r1"]) < 1e-12 and rel(q2, g["r2"]) < 1e-12
    e = ops.energy(F, H.L.blocks["oovv"], t1, t2)
    assert abs(float(e) - float(g["ecc_probe"])) < 1e-12
    c = ops.contract("ijab,ijab->", t2, t2)
    assert abs(float(c) - float((t2 * t2).sum())) < 1e-12 * float((t2 * t2).sum())


def test_update_diis_and_triples(setup, golden_o5v19):
    H, E, Lb, t1, t2, g = setup
    r1, r2 = ops.residuals(H.F, E, Lb, t1, t2)
    a1, a2 = t1.clone(), t2.clone()
    rms = ops.update_amps_(a1, a2, r1, r2, H.eps)
    eo, ev = H.eps[:5], H.eps[5:]
    D1 = eo[:, None] - ev[None, :]
    D2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev
    assert torch.allclose(a1, t1 + r1 / D1, rtol=1e-13, atol=1e-15)
    assert torch.allclose(a2, t2 + r2 / D2, rtol=1e-13, atol=1e-15)
    ref = torch.sqrt((r1 / D1).pow(2).sum() + (r2 / D2).pow(2).sum())
    assert abs(float(rms) - float(ref)) < 1e-12 * float(ref)
    x, ys = a2.reshape(-1), [t2.reshape(-1), r2.reshape(-1)]
    d = ops.diis_dots(x, ys)
    assert torch.allclose(d, torch.stack([torch.dot(x, y) for y in ys]), rtol=1e-12)
    lc = ops.lincomb([t2, r2], [0.25, -2.0])
    assert torch.allclose(lc, 0.25 * t2 - 2.0 * r2, rtol=1e-14, atol=1e-16)
    T1 = torch.from_numpy(golden_o5v19["t1"]).to(t1.device)
    T2 = torch.from_numpy(np.ascontiguousarray(golden_o5v19["t2"])).to(t1.device)
    et = ops.t_energy(H.F, E, T1, T2)
    assert abs(et - float(golden_o5v19["et_tjl"])) < 1e-11
