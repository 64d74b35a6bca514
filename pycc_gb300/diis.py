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

History length.  The reference trims one vector per ``extrapolate`` call, so its history
exceeds ``max_diis`` when extrapolation starts late (``start_diis`` past the window) and
stays that long; ``max_diis`` itself is not bounded.  The library's vector kernels take at
most ``MAX_VEC`` vectors per call, so longer histories run in chunks: one error-vector pass
per ``MAX_VEC - 1`` stored vectors (each pass writes the same difference), and a chain of
partial linear combinations through a scratch vector.  With ``max_diis == 0`` extrapolation
is off (``utils.py:318-319``) and no history is kept at all.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

WORK_LEN = 16 * 1024
MAX_VEC = 16            # vectors per call of pcg_diis_error_* / pcg_lincomb_*


class DIIS:
    def __init__(self, amps: torch.Tensor, max_diis: int, stream=None,
                 error_dtype=torch.float64):
        """``amps`` is the flat FP64 ``[t1 | t2]`` vector the solver iterates."""
        if error_dtype not in (torch.float64, torch.float32):
            raise ValueError("DIIS: error vectors are float64 or float32")
        self.max_diis = int(max_diis)
        if self.max_diis < 0:
            raise ValueError("DIIS: max_diis must be >= 0")
        self.stream = stream
        self.error_dtype = error_dtype
        self.old = amps.clone() if self.max_diis else None
        self.vals = [self.old.clone()] if self.max_diis else []
        self.errors = []
        self.B = np.zeros((0, 0))
        self.work = torch.empty(WORK_LEN, dtype=torch.float64, device=amps.device)
        self.dots = torch.empty(MAX_VEC, dtype=torch.float64, device=amps.device)

    def add_error_vector(self, amps: torch.Tensor):
        if self.max_diis == 0:
            return
        self.vals.append(amps.clone())
        e = torch.empty(amps.shape, dtype=self.error_dtype, device=amps.device)
        fn = "pcg_diis_error_f64" if self.error_dtype == torch.float64 else "pcg_diis_error_f32"
        # e = amps - old, written in the same pass as its overlaps with the stored error
        # vectors and with itself; a history of MAX_VEC or more takes one pass per chunk
        stored = self.errors
        step = MAX_VEC - 1
        d = np.empty(len(stored) + 1)
        for lo in range(0, max(len(stored), 1), step):
            chunk = stored[lo:lo + step]
            k = len(chunk) + 1
            ptrs = (C.c_void_p * k)(*([x.data_ptr() for x in chunk] + [0]))
            _lib.call(fn, amps.data_ptr(), self.old.data_ptr(), e.data_ptr(), ptrs,
                      k, e.numel(), self.work.data_ptr(), self.work.numel(), self.dots.data_ptr(),
                      _lib.stream_handle(self.stream))
            part = self.dots[:k].cpu().numpy()
            d[lo:lo + k - 1] = part[:k - 1]
            d[-1] = part[k - 1]
        self.errors.append(e)
        self.old = self.vals[-1]          # the stored copy of the current amplitudes
        k = len(self.errors)
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
        self._lincomb(self.vals[1:], [float(x) for x in c[:k]], amps)
        self.old = amps.clone()
        return amps

    def _lincomb(self, xs, cs, out):
        """out = sum_j cs[j] xs[j]; more than MAX_VEC terms chain partial sums, each carried
        into the next call with coefficient 1 (scratch vectors: the library's output never
        aliases an input)."""
        fn = "pcg_lincomb_f64" if self.error_dtype == torch.float64 else "pcg_lincomb_f64_df"
        scratch = []
        acc = None
        lo = 0
        while lo < len(xs):
            take = MAX_VEC if acc is None else MAX_VEC - 1
            terms, coefs = list(xs[lo:lo + take]), list(cs[lo:lo + take])
            lo += take
            if acc is not None:
                terms, coefs = [acc] + terms, [1.0] + coefs
            if lo >= len(xs):
                dst = out
            else:
                if len(scratch) < 2:
                    scratch.append(torch.empty_like(out))
                dst = scratch[0] if acc is not scratch[0] else scratch[1]
            k = len(terms)
            ptrs = (C.c_void_p * k)(*[x.data_ptr() for x in terms])
            coef = (C.c_double * k)(*coefs)
            _lib.call(fn, ptrs, coef, k, out.numel(), dst.data_ptr(),
                      _lib.stream_handle(self.stream))
            acc = dst
