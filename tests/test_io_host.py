"""psi4-free input and the amplitude checkpoint, host logic on CPU through the numpy model of
the entry points (``tests/abi_model.py``).

* ``Hamiltonian.from_npz`` with the full <pq|rs> (the reference's layout) and with a
  three-index factor B: the same resident blocks as ``from_arrays``.
* ``save_amplitudes`` / ``load_amplitudes``: a warm start from converged amplitudes
  converges at once, to the reference's energy; mismatched sizes are refused.
"""
import numpy as np
import pytest
import torch

import abi_model
import pycc_gb300 as pg


@pytest.fixture
def model(monkeypatch):
    return abi_model.install(monkeypatch)


def test_hamiltonian_from_npz(model, tmp_path, ham_o5v19):
    fac, F, ERI, L = ham_o5v19
    ref = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu")
    np.savez(tmp_path / "full.npz", no=5, F=F, ERI=ERI)
    np.savez(tmp_path / "fac.npz", no=5, F=F, B=fac.B)
    for name in ("full.npz", "fac.npz"):
        H = pg.Hamiltonian.from_npz(tmp_path / name, device="cpu")
        assert torch.equal(H.F, ref.F)
        for X, Y in ((H.ERI, ref.ERI), (H.L, ref.L)):
            for pat, blk in Y.blocks.items():
                assert (X.blocks[pat] - blk).abs().max().item() < 1e-14, (name, pat)
    np.savez(tmp_path / "bad.npz", no=5, F=F)
    with pytest.raises(KeyError):
        pg.Hamiltonian.from_npz(tmp_path / "bad.npz", device="cpu")
    np.savez(tmp_path / "bad2.npz", no=5, F=F, B=fac.B[:, :3])
    with pytest.raises(ValueError):
        pg.Hamiltonian.from_npz(tmp_path / "bad2.npz", device="cpu")


def test_amplitude_checkpoint_warm_start(model, tmp_path, ham_o5v19, golden_o5v19):
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu")
    w = pg.CCwfn(H)
    e = w.solve_cc(1e-12, 1e-12)
    path = tmp_path / "amps.npz"
    w.save_amplitudes(path)
    w2 = pg.CCwfn(H)
    w2.load_amplitudes(path)
    assert torch.equal(w2.t2, w.t2) and torch.equal(w2.t1, w.t1)
    e2 = w2.solve_cc(1e-10, 1e-10)
    assert w2.niter <= 2 and abs(e2 - float(golden_o5v19["ecc"])) < 1e-11
    fac = pg.SyntheticFactors(4, 19, 0)
    F4, ERI4, L4 = fac.hamiltonian()
    w3 = pg.CCwfn(pg.Hamiltonian.from_arrays(F4, ERI4, 4, L=L4, device="cpu"))
    with pytest.raises(ValueError, match="no=5"):
        w3.load_amplitudes(path)


def test_mixed_warm_start_runs_the_final_stage(model, tmp_path, ham_o5v19, golden_o5v19,
                                               monkeypatch):
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda *a: None)
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda *a: None)
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu")
    w = pg.CCwfn(H)
    w.solve_cc(1e-12, 1e-12)
    path = tmp_path / "amps.npz"
    w.save_amplitudes(path)
    m = pg.CCwfn(H, precision="MIXED")
    m.load_amplitudes(path)
    e = m.solve_cc(1e-10, 1e-10)
    assert m.mixed_engine().history[0] == "bf16x3s"
    assert m.niter <= 2 and abs(e - float(golden_o5v19["ecc"])) < 1e-11


def test_reference_constructor_options(model, ham_o5v19):
    """The reference's constructor options: accepted at their defaults, validated like the
    reference validates them, refused when they switch on a feature outside the path."""
    _, F, ERI, L = ham_o5v19
    H = pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu")
    w = pg.CCwfn(H, model="ccsd", device="gpu", precision="dp", make_t3_density=False,
                 store_triples=False, field=False, field_strength=0.0, field_axis="Z",
                 real_time=False, local=None, local_cutoff=1e-5, it2_opt=True, filter=False,
                 localize_occ=False, local_mos="boys", orbital_basis="spatial", quiet=True)
    assert w.model == "CCSD" and w.local_mos == "BOYS" and w.make_t3_density is False
    assert pg.CCwfn(H, model="CCSD(T)", make_t3_density=True).make_t3_density is True
    for kw in ({"field": True},
               {"store_triples": True}, {"localize_occ": True}, {"local": "PNO"},
               {"model": "CC3"}, {"orbital_basis": "spinorbital"}, {"device": "CPU"}):
        with pytest.raises(NotImplementedError):
            pg.CCwfn(H, **kw)
    for kw in ({"it2_opt": 3}, {"local_mos": "EDMISTON"}, {"precision": "HP"},
               {"model": "CCSDT"}):
        with pytest.raises(pg.InvalidKeywordError):
            pg.CCwfn(H, **kw)
    with pytest.raises(TypeError):
        pg.CCwfn(H, frozen_core=True)
    with pytest.raises(pg.PyCCError):
        pg.CCwfn(H, no_such_option=1)


def test_reference_style_wavefunction(model, ham_o5v19, golden_o5v19):
    """CCwfn accepts a wave function shaped like the reference's (an active occupied count
    ``no`` and ``H`` with the full F, ERI and L arrays, as pycc's own CCwfn carries them): it
    uploads the blocks itself, and the residual equals the reference's."""
    from types import SimpleNamespace
    _, F, ERI, L = ham_o5v19
    g = golden_o5v19
    ref_like = SimpleNamespace(no=5, eref=-1.5, device1=torch.device("cpu"),
                               H=SimpleNamespace(F=F, ERI=ERI, L=L))
    w = pg.CCwfn(ref_like, precision="DP")
    assert w.no == 5 and w.nv == 19 and w.eref == -1.5
    r1, r2 = w.residuals(w.H.F, torch.from_numpy(g["probe_t1"].copy()),
                         torch.from_numpy(g["probe_t2"].copy()))
    assert np.abs(r1.numpy() - g["r1"]).max() / np.abs(g["r1"]).max() < 1e-12
    assert np.abs(r2.numpy() - g["r2"]).max() / np.abs(g["r2"]).max() < 1e-12
    with pytest.raises(TypeError):
        pg.CCwfn(SimpleNamespace(no=5, H=SimpleNamespace(F=F)), precision="DP")
