"""pycc_gb300 -- a GB300-native RHF-CCSD amplitude engine.

Drop-in for the residual iteration of CrawfordGroup/pycc's ``CCwfn`` (``pycc/ccwfn.py``)
running on hand-written sm_103a CUDA kernels behind a C ABI (``include/pycc_gb300.h``).
"""
from .exceptions import PyCCError, InvalidKeywordError, ConvergenceError, NumericalError
from .hamiltonian import Hamiltonian, BlockTensor
from .synth import SyntheticFactors, WORKLOADS, synthetic_factors
from .ccwfn import CCwfn, ccwfn
from .contract import ContractionBackend, contract_f64
from .lagrangian import cchbar, cclambda, ccdensity
from ._lib import EngineError
from . import ops  # noqa: F401  (registers torch.ops.gbcc)

__all__ = [
    "CCwfn", "ccwfn", "Hamiltonian", "BlockTensor", "SyntheticFactors", "WORKLOADS",
    "synthetic_factors", "ContractionBackend", "contract_f64", "cchbar", "cclambda",
    "ccdensity", "PyCCError",
    "InvalidKeywordError", "ConvergenceError", "NumericalError", "EngineError",
]
