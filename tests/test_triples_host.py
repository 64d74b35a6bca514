"""Host logic of the (T) correction on CPU, through the numpy model of the entry points
(``tests/abi_model.py``), against the reference's own E(T) (``t_tjl``, o5v19.npz).

* FP64 path: the twelve t3 terms as three multi-term contractions per triple, written in the
  [z][x][y] partial layout, then the energy entry point -- to 1e-13.
* Tensor-core path: six operand packs, the group tables of the grouped GEMM (three
  orientations per triple, four K segments each), partial offsets inside a batch, FP32
  partials and per-batch reductions -- for batch sizes that divide the 35 triples of no=5
  and ones that leave a ragged last batch; within the FP32 storage of the partials (1e-9).
* ``model='CCSD(T)'`` through ``solve_cc`` in DP and MIXED.
"""
import numpy as np
import pytest
import torch

import abi_model
import pycc_gb300 as pg
from pycc_gb300.triples import t_energy_fp64
from pycc_gb300.triples_tc import t_energy_tc


@pytest.fixture
def model(monkeypatch):
    m = abi_model.install(monkeypatch)
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda *a: None)
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda *a: None)
    return m


def converged(ham, g, precision="DP", model_name="CCSD"):
    _, F, ERI, L = ham
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"), precision=precision,
                 model=model_name)
    w.t1 = torch.from_numpy(g["t1"].copy())
    w.t2 = torch.from_numpy(g["t2"].copy())
    return w


def test_fp64_path(model, ham_o5v19, golden_o5v19):
    w = converged(ham_o5v19, golden_o5v19)
    assert abs(t_energy_fp64(w) - float(golden_o5v19["et_tjl"])) < 1e-13
    assert "pcg_contract_multi_f64" in model.calls


@pytest.mark.parametrize("batch", [32, 35, 7, 4, 1])
def test_tensor_core_path_batches(model, ham_o5v19, golden_o5v19, batch):
    w = converged(ham_o5v19, golden_o5v19)
    et = t_energy_tc(w, batch=batch)
    assert abs(et - float(golden_o5v19["et_tjl"])) < 1e-9
    assert "pcg_tc_grouped_gemm" in model.calls


@pytest.mark.parametrize("precision,tol", [("DP", 1e-11), ("MIXED", 1e-9)])
def test_ccsd_t_model(model, ham_o5v19, golden_o5v19, precision, tol):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"), precision=precision,
                 model="CCSD(T)")
    e = w.solve_cc(1e-12, 1e-12, 100)
    g = golden_o5v19
    assert abs(e - (float(g["ecc"]) + float(g["et_tjl"]))) < tol
    assert abs(w.et - float(g["et_tjl"])) < tol


@pytest.mark.parametrize("no,nv", [(1, 1), (2, 1), (1, 5), (3, 2)])
def test_degenerate_sizes(model, no, nv):
    """Single occupied or virtual orbitals, both drivers, against the oracle's t_tjl."""
    from oracle import triples as ot
    fac = pg.SyntheticFactors(no, nv, 5)
    F, ERI, L = fac.hamiltonian()
    rng = np.random.default_rng(no * 7 + nv)
    t1 = 0.05 * rng.standard_normal((no, nv))
    t2 = 0.05 * rng.standard_normal((no, no, nv, nv))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    ref = ot.t_tjl(no, nv, F, ERI, t1, t2)
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, no, L=L, device="cpu"))
    w.t1, w.t2 = torch.from_numpy(t1), torch.from_numpy(t2)
    assert abs(t_energy_fp64(w) - ref) < 1e-13 * max(1.0, abs(ref))
    for batch in (1, 32):
        assert abs(t_energy_tc(w, batch=batch) - ref) < 1e-6 * max(abs(ref), 1e-8)


def test_reference_entry_point_names(model, ham_o5v19, golden_o5v19):
    from pycc_gb300.triples import t_tjl, t_vikings
    w = converged(ham_o5v19, golden_o5v19)
    assert abs(t_tjl(w) - float(golden_o5v19["et_tjl"])) < 1e-13
    assert abs(t_vikings(w) - float(golden_o5v19["et_vikings"])) < 1e-13


def test_t3_density_vs_reference(monkeypatch, ham_o5v19):
    """The (T) densities and Lambda sources (t3_density, pycc/cctriples.py:1063-1157) planned
    by the engine, through the numpy model of the entry points, against the reference's own
    (o5v19_t3density.npz): every block to 1e-12 relative, E(T) to 1e-13."""
    import abi_model
    from conftest import golden
    abi_model.install(monkeypatch)
    g = golden("o5v19_t3density.npz")
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"), model="CCSD(T)",
                 make_t3_density=True)
    w.t1 = torch.from_numpy(g["t1"].copy())
    w.t2 = torch.from_numpy(g["t2"].copy())
    et = w.t3_density()
    assert abs(et - float(g["et"])) < 1e-13
    for name in ("Doo", "Dvv", "Dov", "Goovv", "Gooov", "Gvvvo", "S1", "S2"):
        got = getattr(w, name).numpy()
        assert got.shape == g[name].shape, name
        assert np.abs(got - g[name]).max() <= 1e-12 * np.abs(g[name]).max(), name
