"""The reference's DIIS interface over the GPU DIIS (``pycc/utils.py:257-361``).

``helper_diis(t1, t2, max_diis, precision)`` with ``add_error_vector(t1, t2)`` and
``extrapolate(t1, t2) -> (t1, t2)``, the call pattern of the reference's solvers and of its
callers (e.g. ``CCderiv._perturbed_amplitudes``, ``pycc/ccderiv.py:262-276``).  The pair is
kept as one flat FP64 vector ``[t1 | t2]`` on the GPU (:class:`pycc_gb300.diis.DIIS`): error
vectors, overlaps and the extrapolation run on the library's kernels; the Pulay system is
the reference's (bordered, scaled by its largest entry).
"""
from __future__ import annotations

import torch

from .diis import DIIS


class helper_diis:
    """Rolling DIIS on an amplitude pair; ``precision`` 'DP' keeps FP64 error vectors,
    'SP' / 'MIXED' FP32 ones (the amplitudes stay FP64).  ``max_diis=0`` disables the
    extrapolation, as in the reference."""

    def __init__(self, t1, t2, max_diis, precision='DP'):
        self._check(t1, t2)
        self.shapes = (tuple(t1.shape), tuple(t2.shape))
        self.precision = str(precision).upper()
        edt = torch.float64 if self.precision == 'DP' else torch.float32
        self.max_diis = int(max_diis)
        self._diis = DIIS(self._flat(t1, t2), self.max_diis, error_dtype=edt)

    @staticmethod
    def _check(t1, t2):
        for t in (t1, t2):
            if not isinstance(t, torch.Tensor) or t.dtype != torch.float64:
                raise TypeError("helper_diis: FP64 torch tensors on the engine's device expected")

    def _flat(self, t1, t2):
        self._check(t1, t2)
        if (tuple(t1.shape), tuple(t2.shape)) != self.shapes:
            raise ValueError("helper_diis: amplitude shapes changed")
        return torch.cat([t1.reshape(-1), t2.reshape(-1)])

    def add_error_vector(self, t1, t2):
        """Store the pair and its error vector t - t_prev (``pycc/utils.py:284-295``)."""
        self._diis.add_error_vector(self._flat(t1, t2))

    def extrapolate(self, t1, t2):
        """The Pulay combination of the stored pairs (``pycc/utils.py:297-361``); returns
        new tensors (t1, t2), or the inputs unchanged when ``max_diis`` is 0."""
        if self.max_diis == 0:
            return t1, t2
        amps = self._diis.extrapolate(self._flat(t1, t2))
        n1 = t1.numel()
        return amps[:n1].view(self.shapes[0]), amps[n1:].view(self.shapes[1])
