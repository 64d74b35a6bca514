"""Failure detection on the GPU, in the forms that fault, trap or hang nothing.

* Bounded device-side waits: with a 1 ms wait limit, the self-test kernel waits on an
  mbarrier that nothing completes; the wait expires, the kernel records status 4 in the
  engine's device status word and returns; the host's check raises EngineError; the context
  stays usable (a tensor-core GEMM afterwards is exact).
* Non-finite numbers injected on the host: a NaN in t2 makes solve_cc raise NumericalError
  in its first iteration, in FP64 and in the mixed engine.
* A solve that runs out of iterations raises ConvergenceError with the last dE and rms.
"""
import numpy as np
import pytest
import torch

import pycc_gb300 as pg
from pycc_gb300 import _lib
from pycc_gb300.tc import FMT_BF16X3S, Operand, TCEngine

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_and_the_context_survives(cuda):
    eng = TCEngine(cuda)
    prev = _lib.set_wait_limit_ns(1_000_000)                     # 1 ms
    try:
        _lib.call("pcg_wait_probe", eng.status.data_ptr(), _lib.stream_handle())
        torch.cuda.synchronize()
    finally:
        assert _lib.set_wait_limit_ns(prev) == 1_000_000
    assert eng.status.cpu().tolist() == [4, 0, 0, 0]
    with pytest.raises(_lib.EngineError, match="self-test"):
        eng.check_status()
    # the same context still runs the tensor-core kernels, with the default bound
    eng.status.zero_()
    g = torch.Generator(device=cuda).manual_seed(1)
    A = torch.randint(-3, 4, (300, 640), generator=g, device=cuda).double()
    B = torch.randint(-3, 4, (200, 640), generator=g, device=cuda).double()
    out = torch.zeros(300, 200, dtype=torch.float64, device=cuda)
    eng.contract("mk,nk->mn", Operand.of("mk", A), Operand.of("nk", B), out, fmt=FMT_BF16X3S)
    torch.cuda.synchronize()
    eng.check_status()
    assert torch.equal(out, A @ B.T)


def test_wait_limit_setter_defaults():
    prev = _lib.set_wait_limit_ns(0)          # <= 0: the 4 s default
    assert _lib.set_wait_limit_ns(prev) == 4_000_000_000


@pytest.mark.parametrize("precision", ["DP", "MIXED"])
def test_nan_injected_in_t2_raises(cuda, ham_o5v19, precision):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda), precision=precision)
    w.t2[1, 2, 3, 4] = float("nan")
    with pytest.raises(pg.NumericalError, match="iteration 1"):
        w.solve_cc(1e-10, 1e-10, 20)


def test_maxiter_raises_convergence_error(cuda, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    w = pg.CCwfn(pg.Hamiltonian.from_arrays(F, ERI, 5, L=L, device=cuda))
    with pytest.raises(pg.ConvergenceError) as e:
        w.solve_cc(1e-14, 1e-14, 3)
    assert "3" in str(e.value)
