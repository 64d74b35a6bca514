"""GPU DIIS extrapolation of the CCSD amplitudes (mirrors ``pycc/utils.py:257-361``).

Error vectors are the amplitude differences ``e_n = t_n - t_{n-1}`` of the flattened
``[t1 | t2]`` pair (``utils.py:284-295``).  The overlaps ``<e_m|e_n>`` are FP64 dot products
on the GPU, computed once per new vector against every stored one (the reference recomputes
the full matrix each call; the values are the same); the bordered (k+1)^2 Pulay system is
scaled by its largest |B| entry (``utils.py:341``) and solved in FP64; the new amplitudes
``sum_i c_i t_i`` are one fused linear-combination pass.

With ``error_dtype=torch.float32`` (the mixed-precision solver) the error vectors are kept
in FP32: each is the FP64 difference rounded once, and the overlaps come from FP32 products
accumulated in FP64.  The amplitudes stay FP64, and their extrapolation runs in
double-float arithmetic (about 48 bits, one FP64 instruction per element).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

WORK_LEN = 16 * 1024


class DIIS:
    def __init__(self, amps: torch.Tensor, max_diis: int, stream=None,
                 error_dtype=torch.float64):
        """``amps`` is the flat FP64 ``[t1 | t2]`` vector the solver iterates."""
        if error_dtype not in (torch.float64, torch.float32):
            raise ValueError("DIIS: error vectors are float64 or float32")
        self.max_diis = int(max_diis)
        self.stream = stream
        self.error_dtype = error_dtype
        self.old = amps.clone()
        self.vals = [amps.clone()]
        self.errors = []
        self.B = np.zeros((0, 0))
        self.work = torch.empty(WORK_LEN, dtype=torch.float64, device=amps.device)
        self.dots = torch.empty(16, dtype=torch.float64, device=amps.device)

    def add_error_vector(self, amps: torch.Tensor):
        self.vals.append(amps.clone())
        k = len(self.errors) + 1
        e = torch.empty(amps.shape, dtype=self.error_dtype, device=amps.device)
        # e = amps - old, written once, and its overlaps with every stored error vector
        # (itself included) in the same pass
        ptrs = (C.c_void_p * k)(*([x.data_ptr() for x in self.errors] + [0]))
        fn = "pcg_diis_error_f64" if self.error_dtype == torch.float64 else "pcg_diis_error_f32"
        _lib.call(fn, amps.data_ptr(), self.old.data_ptr(), e.data_ptr(), ptrs,
                  k, e.numel(), self.work.data_ptr(), self.work.numel(), self.dots.data_ptr(),
                  _lib.stream_handle(self.stream))
        self.errors.append(e)
        self.old = self.vals[-1]          # the stored copy of the current amplitudes
        d = self.dots[:k].cpu().numpy()
        B = np.zeros((k, k))
        B[:k - 1, :k - 1] = self.B
        B[k - 1, :] = d
        B[:, k - 1] = d
        self.B = B

    def extrapolate(self, amps: torch.Tensor) -> torch.Tensor:
        """New amplitudes sum_i c_i t_i, written into ``amps`` (which the history never aliases)."""
        if self.max_diis == 0:
            return amps
        if len(self.errors) > self.max_diis:
            del self.vals[0]
            del self.errors[0]
            self.B = self.B[1:, 1:]
        k = len(self.errors)
        Bb = -np.ones((k + 1, k + 1))
        Bb[-1, -1] = 0.0
        Bb[:k, :k] = self.B / np.abs(self.B).max()
        rhs = np.zeros(k + 1)
        rhs[-1] = -1.0
        c = np.linalg.solve(Bb, rhs)
        ptrs = (C.c_void_p * k)(*[x.data_ptr() for x in self.vals[1:]])
        coef = (C.c_double * k)(*[float(x) for x in c[:k]])
        fn = "pcg_lincomb_f64" if self.error_dtype == torch.float64 else "pcg_lincomb_f64_df"
        _lib.call(fn, ptrs, coef, k, amps.numel(), amps.data_ptr(), _lib.stream_handle(self.stream))
        self.old = amps.clone()
        return amps
