"""The CPU legs of bench.py time the reference's own solve_cc iterations through
``oracle.reference.time_solve_iterations``: whole iterations only, the warm-up excluded,
the reference's code unchanged.  Runs when the reference is installed in ``baseline/_ref``
(or named by ``$PYCC_REF``)."""
import os

import numpy as np
import pytest

from oracle import reference as R
from pycc_gb300.synth import SyntheticFactors

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def pycc():
    for path in (os.environ.get("PYCC_REF"), os.path.join(ROOT, "baseline", "_ref")):
        try:
            return R.import_reference(path)
        except ImportError:
            continue
    pytest.skip("the reference is not installed (baseline/_ref) and PYCC_REF is unset")


def _wfn(pycc):
    fac = SyntheticFactors(5, 19, 0)
    F, ERI, L = fac.hamiltonian()
    return R.make_ref_ccwfn(pycc, F, ERI, L, 5, 19)


def test_iterations_timed_and_code_restored(pycc):
    w = _wfn(pycc)
    times, warm = R.time_solve_iterations(w, 2, 3)
    assert warm == 2 and len(times) == 3 and all(t > 0 for t in times)
    assert "residuals" not in vars(w)                 # the wrapper is gone
    # the reference's own solve_cc ran: t1/t2 moved from the MP2 guess
    assert np.abs(w.t1).max() > 0


def test_budget_stops_at_an_iteration_boundary(pycc):
    """With a fake clock advancing 10 s per call, a 25 s budget stops the loop after the
    third timed iteration; every counted iteration is whole."""
    w = _wfn(pycc)
    ticks = iter(range(0, 10000, 10))
    times, warm = R.time_solve_iterations(w, 1, 20, budget_s=25.0, clock=lambda: next(ticks))
    assert warm == 1 and times == [10, 10, 10]
