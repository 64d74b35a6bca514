"""Failure handling of the solver's host loop on CPU, through the numpy model of the entry
points: a NaN injected into t2 on the host raises NumericalError at the first iteration, and
an exhausted ``maxiter`` raises ConvergenceError (the reference returns None there,
pycc/ccwfn.py:268-319)."""
import pytest

import abi_model
import pycc_gb300 as pg


@pytest.fixture
def model(monkeypatch):
    return abi_model.install(monkeypatch)


def test_nan_in_t2_raises_numerical_error(model, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    w.t2[0, 1, 2, 3] = float("nan")
    with pytest.raises(pg.NumericalError, match="iteration 1"):
        w.solve_cc(1e-10, 1e-10, 10)


def test_maxiter_raises_convergence_error(model, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device="cpu"))
    with pytest.raises(pg.ConvergenceError) as e:
        w.solve_cc(1e-14, 1e-14, 2)
    assert e.value.maxiter == 2 and e.value.rms > 0
