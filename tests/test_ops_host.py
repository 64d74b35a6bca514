"""torch.ops.gbcc: the operators are registered with PyTorch's dispatcher for CUDA tensors
only; a call with CPU tensors raises instead of falling back to a CPU path."""
import pytest
import torch

import pycc_gb300  # noqa: F401  (registers the operators)

NAMES = ["contract", "tau", "fae", "fmi", "fme", "wmnij", "wmbej", "wmbje", "zmbij", "r_t1",
         "r_t2", "residuals", "energy", "update_amps_", "diis_dots", "lincomb", "t_energy"]


@pytest.mark.parametrize("name", NAMES)
def test_registered(name):
    op = getattr(torch.ops.gbcc, name)
    assert op.default._schema.name == "gbcc::" + name


def test_cpu_tensors_are_refused():
    t1 = torch.zeros(2, 3, dtype=torch.float64)
    t2 = torch.zeros(2, 2, 3, 3, dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        torch.ops.gbcc.tau(t1, t2, 1.0, 1.0)
    with pytest.raises(NotImplementedError):
        torch.ops.gbcc.contract("ij,jk->ik", t1.T.contiguous(), t1)
