"""Adjoint of the converged CCSD energy: Lambda equations and gradient densities.

The FP64 residual (``CCwfn.residuals``) and the energy are recorded on a tape as the
engine's own operations (strided contractions, copies, combinations, tau builds, the r2
symmetrisation).  Reverse accumulation through that tape, with the same CUDA kernels,
gives the vector-Jacobian products of the residual:

* J^T lambda (with respect to the amplitudes): one Lambda iteration.  The Lambda equations
  ``J^T lambda = -dE/dt`` replace the reference's hand-derived ``cclambda``
  (``pycc/cclambda.py:69-560``); they are solved by the same Jacobi + DIIS iteration as
  the amplitudes (``lambda += (dE/dt + J^T lambda) / D``).
* dE/dH at the converged (t, lambda): with respect to the Fock matrix and every
  integral block read by the residual.  Assembled into the full ``D`` (nmo x nmo) and
  ``Gamma`` (nmo^4, <pq|rs> order) they are the gradient densities of the reference's
  ``ccdensity.gradient_densities`` (``pycc/ccdensity.py:267-333``): E_corr = <D,F> + <Gamma,ERI>.
  The reference stores representative blocks and symmetrises them 4-fold; both agree on the
  8-fold permutationally symmetric projection, the part any symmetric perturbation sees.

* J x (the forward sweep over the same tape, each op's tangent rule): the CCSD Jacobian
  applied to an amplitude pair, the reference's ``CCderiv._ccsd_jacobian``
  (``pycc/ccderiv.py:149-180``), exact because every taped op is linear or bilinear.

The sweeps' contractions run on the FP64 DMMA kernel, or, with ``sweep='tc'``, the large
GEMM-shaped ones on the tcgen05 engine in split-BF16x3.  vvvv-sized cotangents are never
stored separately: the ladder's adjoint contractions write straight into the gradient
buffers of tau and of the <ab|ef> block.  ``pycc_gb300.lagrangian`` wraps the sweeps in the
reference's ``cchbar`` / ``cclambda`` / ``ccdensity`` objects.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import _lib
from .contract import contract_f64
from .diis import DIIS
from .exceptions import ConvergenceError
from .hamiltonian import ERI_BLOCKS, L_BLOCKS, _sl

WORK_LEN = 4096


class Tape:
    def __init__(self):
        self.ops = []

    def record(self, kind, *args):
        self.ops.append((kind, args))


def _base(t):
    return t._base if t._base is not None else t


def _key(t):
    return _base(t).untyped_storage().data_ptr()


class Grads:
    """Gradient buffers keyed by storage; views of a tensor map to views of its buffer."""

    def __init__(self):
        self.buf = {}

    def clear(self):
        self.buf = {}

    def get(self, t, create=True):
        b = _base(t)
        k = _key(t)
        g = self.buf.get(k)
        if g is None:
            if not create:
                return None
            g = torch.zeros(b.shape, dtype=torch.float64, device=b.device)
            self.buf[k] = g
        return g.as_strided(t.size(), t.stride(), t.storage_offset() - b.storage_offset())

    def has(self, t):
        return _key(t) in self.buf


def _as4(t):
    while t.dim() < 4:
        t = t.unsqueeze(0)
    return t


def accumulate(dst, src, a=1.0, perm=None, stream=None):
    """dst += a * src (src optionally read through ``perm``); in place, FP64 kernel."""
    d4 = _as4(dst)
    s = src.permute(*perm) if perm is not None else src
    s4 = _as4(s)
    _lib.call("pcg_combine4_f64", _lib.i64s(d4.shape), 1.0, d4.data_ptr(), _lib.i64s(d4.stride()),
              float(a), s4.data_ptr(), _lib.i64s(s4.stride()), d4.data_ptr(),
              _lib.i64s(d4.stride()), _lib.stream_handle(stream))


def _inverse(perm):
    inv = [0] * len(perm)
    for i, p in enumerate(perm):
        inv[p] = i
    return tuple(inv)


TC_MIN_FLOPS = 1 << 26     # M*N*K from which a sweep's contraction goes to the tensor cores


class CCSDAdjoint:
    """Tape of the FP64 residual + energy at the amplitudes of a converged ``CCwfn``.

    ``sweep`` selects the engine of the sweeps' contractions: ``'fp64'`` (the FP64 DMMA
    kernel; the default for ``precision='DP'``) or ``'tc'`` (GEMM-shaped contractions of at
    least ``TC_MIN_FLOPS`` multiply-adds on the tensor cores in split-BF16x3 with separate
    accumulators, the integral blocks as cached static packs; the default for 'MIXED' and
    'SP').  The tape is always recorded from the FP64 residual; for a MIXED / SP wave function
    a DP twin sharing its Hamiltonian and amplitudes records it.
    """

    def __init__(self, w, sweep=None):
        if sweep is None:
            sweep = 'fp64' if w.precision == 'DP' else 'tc'
        if sweep not in ('fp64', 'tc'):
            raise ValueError("sweep must be 'fp64' or 'tc', got %r" % (sweep,))
        if w.precision != 'DP':
            from .ccwfn import CCwfn
            twin = CCwfn(w.H, precision='DP')
            twin.t1, twin.t2 = w.t1, w.t2
            w = twin
        self.sweep = sweep
        self.tc_min_flops = TC_MIN_FLOPS
        self._tc = None
        self._tc_on = True        # a 'tc' sweep's contractions go to the tensor cores
        from .tc import FMT_BF16X3S
        self._tc_fmt = FMT_BF16X3S
        if sweep == 'tc':
            from .tc import TCEngine
            self._tc = TCEngine(w.device1, w.stream)
        self.w = w
        self.stream = w.stream
        H = w.H
        self.leaves_H = set()
        for t in [H.F] + list(H.ERI.blocks.values()) + list(H.L.blocks.values()):
            self.leaves_H.add(_key(t))
        self.t1, self.t2 = w.t1, w.t2
        last = getattr(w, "_last_tape", None)
        self.tape_reused = (last is not None and w._tape_version is not None
                            and w._tape_version == w._amps._version)
        if self.tape_reused:
            # the converging iteration of solve_cc(keep_tape=True) taped its residual
            tape, self.r1, self.r2 = last
        else:
            tape = Tape()
        w._tape = tape
        try:
            if not self.tape_reused:
                self.r1, self.r2 = w.residuals(H.F, self.t1, self.t2)
            self.E = w.cc_energy_contractions(w.o, w.v, H.F, H.L, self.t1, self.t2)
        finally:
            w._tape = None
        if self.tape_reused:
            w._last_tape = w._tape_version = None     # the tape now carries the energy ops
        self.tape = tape
        self.grads = Grads()
        self.wrt_H = False
        self._work = torch.empty(WORK_LEN, dtype=torch.float64, device=H.F.device)
        self._scal = torch.zeros(4, dtype=torch.float64, device=H.F.device)

    # -- the sweeps' contractions ----------------------------------------------------------
    def _mm(self, subs, A, B, out, alpha, beta, fp64=False):
        """out = beta*out + alpha*einsum(subs, A, B): on the FP64 kernel when ``fp64``, else on
        the tensor cores for a 'tc' sweep and a
        GEMM-shaped contraction (an output index, none in both operands and the output,
        K >= 64) of at least ``tc_min_flops`` multiply-adds whose output offsets stay below
        2^31 (the tensor-core epilogue's column offsets are 32-bit), else on the FP64 kernel."""
        if self._tc is not None and self._tc_on and not fp64:
            lhs, rhs = subs.replace(" ", "").split("->")
            la, lb = lhs.split(",")
            ext = dict(zip(la, A.shape))
            ext.update(zip(lb, B.shape))
            M = math.prod(ext[c] for c in la if c in rhs)
            N = math.prod(ext[c] for c in lb if c in rhs)
            K = math.prod(ext[c] for c in la if c in lb)
            span = sum((e - 1) * st for e, st in zip(out.shape, out.stride()))
            if (rhs and not (set(la) & set(lb) & set(rhs)) and K >= 64
                    and M * N * K >= self.tc_min_flops and span < 2 ** 31):
                from .tc import Operand
                opA = Operand(la, (A, la), key=self._static_key(A))
                opB = Operand(lb, (B, lb), key=self._static_key(B))
                self._tc.contract(subs, opA, opB, out, alpha=alpha, beta=beta, fmt=self._tc_fmt)
                return
        contract_f64(subs, A, B, out=out, alpha=alpha, beta=beta, stream=self.stream)

    def _static_key(self, t):
        """Integral blocks (and views of them) are packed once per sweep engine."""
        if _key(t) in self.leaves_H:
            return ("H", t.data_ptr(), tuple(t.shape), tuple(t.stride()))
        return None

    def _check_tc(self):
        if self._tc is not None:
            self._tc.check_status()

    # -- reverse accumulation -------------------------------------------------------------
    def _want(self, t):
        return self.wrt_H or _key(t) not in self.leaves_H

    def backward(self, gE=0.0, l1=None, l2=None, wrt_H=False, seed=None):
        """Accumulate cotangents (gE on E, l1 on r1, l2 on r2) back to the leaves.

        ``seed`` maps leaf tensors to initial gradient values (added before the sweep).
        """
        self.wrt_H = wrt_H
        G = self.grads
        G.clear()
        st = self.stream
        if seed:
            for t, val in seed.items():
                accumulate(G.get(t), val, stream=st)
        if gE != 0.0:
            gEt = G.get(self.E)
            gEt.fill_(float(gE))
        if l1 is not None:
            accumulate(G.get(self.r1), l1, stream=st)
        if l2 is not None:
            accumulate(G.get(self.r2), l2, stream=st)
        for kind, args in reversed(self.tape.ops):
            getattr(self, "_bw_" + kind)(*args)
        self._check_tc()
        return G

    def _bw_contract(self, subs, A, B, out, alpha, beta):
        G = self.grads
        if not G.has(out):
            return
        gZ = G.get(out)
        lhs, rhs = subs.replace(" ", "").split("->")
        la, lb = lhs.split(",")
        if self._want(A):
            self._mm("%s,%s->%s" % (rhs, lb, la), gZ, B, G.get(A), alpha, 1.0)
        if self._want(B):
            self._mm("%s,%s->%s" % (la, rhs, lb), A, gZ, G.get(B), alpha, 1.0)

    def _bw_copy(self, X, out):
        G = self.grads
        if G.has(out) and self._want(X):
            accumulate(G.get(X), G.get(out), stream=self.stream)

    def _bw_combine(self, a, X, b, Y, perm, out):
        G = self.grads
        if not G.has(out):
            return
        gO = G.get(out)
        if a != 0.0 and self._want(X):
            accumulate(G.get(X), gO, a, stream=self.stream)
        if Y is not None and b != 0.0 and self._want(Y):
            accumulate(G.get(Y), gO, b, perm=_inverse(perm), stream=self.stream)

    def _bw_tau(self, t1, t2, f1, f2, out):
        G = self.grads
        if not G.has(out):
            return
        gO = G.get(out)
        if f1 != 0.0:
            accumulate(G.get(t2), gO, f1, stream=self.stream)
        if f2 != 0.0:
            g1 = G.get(t1)
            self._mm("ijab,jb->ia", gO, t1, g1, f2, 1.0)
            self._mm("ijab,ia->jb", gO, t1, g1, f2, 1.0)

    def _bw_sym(self, h, out):
        G = self.grads
        if not G.has(out):
            return
        gO = G.get(out)
        gh = G.get(h)
        accumulate(gh, gO, stream=self.stream)
        accumulate(gh, gO, perm=(1, 0, 3, 2), stream=self.stream)

    # -- forward (tangent) sweep: the Jacobian action -------------------------------------
    def forward_tangent(self, x1, x2):
        """Tangents of every taped tensor along the amplitude direction (x1, x2), by one pass
        over the tape in recording order.  Each taped operation is linear or bilinear in its
        inputs, so the tangents are exact derivatives, not difference quotients.  Tensors
        with no tangent buffer (the integrals and everything built from them alone) are
        constant along (x1, x2)."""
        no, nv = self.w.no, self.w.nv
        for x, shape in ((x1, (no, nv)), (x2, (no, no, nv, nv))):
            if (not isinstance(x, torch.Tensor) or tuple(x.shape) != shape
                    or x.dtype != torch.float64 or x.device != self.t2.device):
                raise ValueError("jacobian: X1, X2 must be float64 tensors of shapes %s, %s on %s"
                                 % ((no, nv), (no, no, nv, nv), self.t2.device))
        T = Grads()
        accumulate(T.get(self.t1), x1, stream=self.stream)
        accumulate(T.get(self.t2), x2, stream=self.stream)
        for kind, args in self.tape.ops:
            getattr(self, "_fw_" + kind)(T, *args)
        self._check_tc()
        return T

    def _fw_contract(self, T, subs, A, B, out, alpha, beta):
        ta = T.get(A) if T.has(A) else None
        tb = T.get(B) if T.has(B) else None
        if ta is None and tb is None:
            return
        to = T.get(out)
        b = beta                      # 0 for a fresh output: the first term writes it
        if ta is not None:
            self._mm(subs, ta, B, to, alpha, b)
            b = 1.0
        if tb is not None:
            self._mm(subs, A, tb, to, alpha, b)

    def _fw_copy(self, T, X, out):
        if T.has(X):
            accumulate(T.get(out), T.get(X), stream=self.stream)

    def _fw_combine(self, T, a, X, b, Y, perm, out):
        use_x = a != 0.0 and T.has(X)
        use_y = Y is not None and b != 0.0 and T.has(Y)
        if not (use_x or use_y):
            return
        to = T.get(out)
        if use_x:
            accumulate(to, T.get(X), a, stream=self.stream)
        if use_y:
            accumulate(to, T.get(Y), b, perm=perm, stream=self.stream)

    def _fw_tau(self, T, t1, t2, f1, f2, out):
        use2 = f1 != 0.0 and T.has(t2)
        use1 = f2 != 0.0 and T.has(t1)
        if not (use1 or use2):
            return
        to = T.get(out)
        if use2:
            accumulate(to, T.get(t2), f1, stream=self.stream)
        if use1:
            d1 = T.get(t1)
            contract_f64("ia,jb->ijab", d1, t1, out=to, alpha=f2, beta=1.0, stream=self.stream)
            contract_f64("ia,jb->ijab", t1, d1, out=to, alpha=f2, beta=1.0, stream=self.stream)

    def _fw_sym(self, T, h, out):
        if T.has(h):
            to, th = T.get(out), T.get(h)
            accumulate(to, th, stream=self.stream)
            accumulate(to, th, perm=(1, 0, 3, 2), stream=self.stream)

    def jvp(self, x1, x2):
        """(dr1, dr2, dE): the derivatives of the residual (r2 symmetrised) and of the energy
        along (x1, x2) at the taped amplitudes."""
        T = self.forward_tangent(x1, x2)
        return T.get(self.r1).clone(), T.get(self.r2).clone(), T.get(self.E).clone()

    def jacobian(self, X1, X2):
        """The CCSD Jacobian applied to an amplitude pair, ``CCderiv._ccsd_jacobian(X1, X2,
        hbar)`` (pycc/ccderiv.py:149-180), without HBAR: the tangent of the residual itself.

        Returns (sigma1, sigma2) in the reference's convention: sigma2 is the doubles part
        before symmetrisation, so sigma2 + sigma2.swapaxes(0,1).swapaxes(2,3) is the doubles
        action, as the reference's callers form it (pycc/ccderiv.py:267-270).  Only that sum
        is defined by the residual; sigma2 is returned as half of it."""
        T = self.forward_tangent(X1, X2)
        s1 = T.get(self.r1).clone()
        d2 = T.get(self.r2)
        s2 = torch.empty_like(d2)
        _lib.call("pcg_combine4_f64", _lib.i64s(d2.shape), 0.5, d2.data_ptr(),
                  _lib.i64s(d2.stride()), 0.0, None, _lib.i64s([0, 0, 0, 0]), s2.data_ptr(),
                  _lib.i64s(s2.stride()), _lib.stream_handle(self.stream))
        return s1, s2

    # -- Lambda equations -----------------------------------------------------------------
    def dE_dt(self):
        G = self.backward(gE=1.0)
        return G.get(self.t1).clone(), G.get(self.t2).clone()

    def jt_lambda(self, l1, l2, g1, g2):
        """(dE/dt1 + J^T l)_1, (...)_2: the Lambda residual."""
        G = self.backward(l1=l1, l2=l2, seed={self.t1: g1, self.t2: g2})
        return G.get(self.t1), G.get(self.t2)

    def _sym_half(self, X):
        """(X_ijab + X_jiba) / 2 into a new buffer (FP64 kernel)."""
        out = torch.empty_like(X)
        _lib.call("pcg_combine4_f64", _lib.i64s(X.shape), 0.5, X.data_ptr(), _lib.i64s(X.stride()),
                  0.5, X.data_ptr(), _lib.i64s(X.permute(1, 0, 3, 2).stride()), out.data_ptr(),
                  _lib.i64s(out.stride()), _lib.stream_handle(self.stream))
        return out

    STALL_RATIO = 0.8     # a 'tc' Lambda iteration above this fraction of the best rms stalls
    STALL_ITERS = 2       # stalled iterations that end the tensor-core stage

    def solve_lambda(self, e_conv=1e-10, r_conv=1e-10, maxiter=100, max_diis=8, start_diis=1,
                     callback=None, polish=True):
        """Jacobi + DIIS on J^T lambda = -dE/dt; returns (l1, l2).

        With a 'tc' sweep the iterations start on the tensor cores.  Their split-BF16x3
        products leave a rounding floor in the update norm (about 1e-7 relative); once the
        norm stalls (``STALL_ITERS`` iterations above ``STALL_RATIO`` x its best) or the
        criteria are met there, ``polish`` switches the sweeps to the FP64 kernels, which
        converge the remaining digits.  Without ``polish`` the solve stops at the floor
        (``self.lambda_at_floor``); ``gradient`` then removes the floor's effect on the
        densities with one correction step (see there)."""
        t0 = time.time()
        self.lambda_times = []
        self.lambda_stages = []
        g1, g2 = self.dE_dt()
        l1, l2, niter, at_floor = self._jacobi(g1, g2, e_conv, r_conv, maxiter, max_diis,
                                               start_diis, callback, polish, "Lambda")
        self.l1, self.l2 = l1, l2
        self.lambda_niter = niter
        self.lambda_at_floor = at_floor
        self.timing_lambda = time.time() - t0
        return l1, l2

    def _jacobi(self, g1, g2, e_conv, r_conv, maxiter, max_diis, start_diis, callback, polish,
                what, rel_floor=None):
        """Solve (g + J^T x)_sym = 0 for x by Jacobi + DIIS on the sweep engine; returns
        (x1, x2, iterations, stopped at the tensor cores' floor).  ``rel_floor``: stop once
        the update norm is below this fraction of the first one."""
        w = self.w
        no, nv = w.no, w.nv
        tc_stage = self._tc is not None
        self._tc_on = True
        lam = torch.zeros(no * nv + no * no * nv * nv, dtype=torch.float64, device=g1.device)
        l1 = lam[:no * nv].view(no, nv)
        l2 = lam[no * nv:].view(no, no, nv, nv)
        diis = DIIS(lam, max_diis, self.stream)
        pseudo_last, rms = 0.0, float("inf")
        best, bad, first = float("inf"), 0, None
        for niter in range(1, maxiter + 1):
            ti = time.time()
            R1, R2 = self.jt_lambda(l1, l2, g1, g2)
            # t2 is constrained to t2_ijab = t2_jiba and r2 is symmetric, so the Lambda
            # equations live on the symmetric subspace: project the t2 part of the residual
            R2 = self._sym_half(R2)
            out = self._scal[1:2]
            _lib.call("pcg_update_amps_f64", l1.data_ptr(), l2.data_ptr(), R1.data_ptr(),
                      R2.data_ptr(), w.H.eps.data_ptr(), no, nv, self._work.data_ptr(),
                      self._work.numel(), out.data_ptr(), _lib.stream_handle(self.stream))
            # pseudo-energy: <lambda, dE/dt> (stationary at convergence)
            pe = contract_f64("ia,ia->", l1, g1, stream=self.stream)
            contract_f64("ijab,ijab->", l2, g2, out=pe, beta=1.0, stream=self.stream)
            vals = torch.stack([out.reshape(()), pe.reshape(())]).cpu().numpy()
            rms, pseudo = math.sqrt(max(float(vals[0]), 0.0)), float(vals[1])
            self._check_tc()
            first = rms if first is None else first
            self.lambda_times.append(time.time() - ti)
            self.lambda_stages.append("tc" if tc_stage else "fp64")
            if callback is not None:
                callback(niter, pseudo, pseudo - pseudo_last, rms)
            done = abs(pseudo - pseudo_last) < e_conv and rms < r_conv
            if rel_floor is not None and rms < rel_floor * first:
                done = True
            at_floor = False
            if tc_stage:
                bad = bad + 1 if rms > self.STALL_RATIO * best else 0
                best = min(best, rms)
                if polish and (done or bad >= self.STALL_ITERS):
                    # the rest on the FP64 kernels, from the tensor-core iterate
                    tc_stage = self._tc_on = False
                    self.lambda_switch = niter
                    if what == "Lambda":
                        g1, g2 = self.dE_dt()
                    diis = DIIS(lam, max_diis, self.stream)
                    pseudo_last = pseudo
                    continue
                if not done and bad >= 2 * self.STALL_ITERS:
                    at_floor = done = True          # the tensor cores' rounding floor
            if done:
                self._tc_on = True
                self.lambda_rms = rms
                return l1, l2, niter, at_floor
            pseudo_last = pseudo
            diis.add_error_vector(lam)
            if niter >= start_diis:
                diis.extrapolate(lam)
        self._tc_on = True
        raise ConvergenceError(what, maxiter, pseudo - pseudo_last, rms)

    # -- gradient densities ---------------------------------------------------------------
    def _densities(self, G):
        """(dL/dF, dL/d<pq|rs>) from a sweep's leaf gradients (L blocks folded into ERI)."""
        w = self.w
        H = w.H
        no, nv, n = w.no, w.nv, w.nmo
        gF = G.get(H.F).clone()
        Gam = torch.zeros((n, n, n, n), dtype=torch.float64, device=gF.device)
        for pat, blk in H.ERI.blocks.items():
            if G.has(blk):
                s = _sl(pat, no, nv)
                accumulate(Gam[s[0], s[1], s[2], s[3]], G.get(blk), stream=self.stream)
        for pat, blk in H.L.blocks.items():
            if G.has(blk):
                s = _sl(pat, no, nv)
                g = G.get(blk)
                accumulate(Gam[s[0], s[1], s[2], s[3]], g, 2.0, stream=self.stream)
                accumulate(Gam[s[0], s[1], s[3], s[2]], g, -1.0, perm=(0, 1, 3, 2),
                           stream=self.stream)
        return gF, Gam

    def gradient(self, e_conv=1e-10, r_conv=1e-10, maxiter=100, l1=None, l2=None, refine=True):
        """dL/dF (nmo x nmo) and dL/d<pq|rs> (nmo^4) of the Lagrangian L = E + <l, r> at the
        taped amplitudes: with the converged Lambda amplitudes (solved here when neither
        (l1, l2) nor an earlier solve gives them) these are dE/dF and dE/d<pq|rs>.

        The density sweep runs on the FP64 kernels for every sweep engine: the tensor cores'
        products (split-BF16x3 or x6, FP32 accumulation) leave 2-5e-6 of E in
        E = <D, F> + <Gamma, ERI> at no=20, nv=180, where the FP64 sweep keeps it to 1e-14.

        When Lambda stopped at the tensor cores' floor (``solve_lambda(polish=False)``) and
        ``refine`` is set, the same FP64 sweep also yields the Lambda residual
        R = dE/dt + J^T l at that Lambda (the sweep's gradient on t).  A correction d with
        J^T d = -R is solved on the tensor cores to 1e-5 of R -- the floor times that is far
        below FP64's own error -- and its densities <d, dr/dH> are added from one more
        tensor-core sweep: they are ~1e-7 of the total, so its rounding does not show."""
        if l1 is None or l2 is None:
            if not hasattr(self, "l1"):
                self.solve_lambda(e_conv, r_conv, maxiter)
            l1, l2 = self.l1, self.l2
            floor = getattr(self, "lambda_at_floor", False)
        else:
            floor = False
        t0 = time.time()
        tc_on = self._tc_on
        self._tc_on = False
        try:
            G = self.backward(gE=1.0, l1=l1, l2=l2, wrt_H=True)
        finally:
            self._tc_on = tc_on
        gF, Gam = self._densities(G)
        self.lambda_refined = False
        if floor and refine and self._tc is not None:
            R1 = G.get(self.t1).clone()
            R2 = self._sym_half(G.get(self.t2))
            self.grads.clear()
            d1, d2, _, _ = self._jacobi(R1, R2, 0.0, 0.0, 50, 8, 1, None, False,
                                        "Lambda correction", rel_floor=1e-5)
            G = self.backward(gE=0.0, l1=d1, l2=d2, wrt_H=True)
            dF, dGam = self._densities(G)
            gF += dF
            Gam += dGam
            self.l1 = l1 + d1
            self.l2 = l2 + d2
            self.lambda_refined = True
        torch.cuda.synchronize()
        self.timing_gradient = time.time() - t0
        self.grads.clear()
        return gF, Gam


def symmetrize8(G):
    """Projection of a <pq|rs> tensor onto the 8-fold permutational symmetry of real ERIs."""
    # <pq|rs> = (pr|qs); the chemist tensor is symmetric under p<->r, q<->s and (pr)<->(qs)
    C = G.permute(0, 2, 1, 3)
    C = 0.5 * (C + C.permute(1, 0, 2, 3))
    C = 0.5 * (C + C.permute(0, 1, 3, 2))
    C = 0.5 * (C + C.permute(2, 3, 0, 1))
    return C.permute(0, 2, 1, 3).contiguous()


class CCSDEnergy(torch.autograd.Function):
    """Converged FP64 CCSD correlation energy of (F, <pq|rs>) with its implicit adjoint.

    forward: ``CCwfn.solve_cc`` on the GPU, keeping the converging iteration's tape.
    backward: the Lambda equations through that tape on the tensor cores, then dE/dF and
    dE/d<pq|rs> (the gradient densities) from one FP64 sweep with the Lambda floor's
    correction: 2.2 forward iterations at no=20, nv=180, finite differences to 2e-8.
    """

    @staticmethod
    def forward(ctx, F, ERI, no, e_conv=1e-11, r_conv=1e-11):
        from .ccwfn import CCwfn
        from .hamiltonian import Hamiltonian
        H = Hamiltonian.from_full(F.detach(), ERI.detach(), int(no))
        w = CCwfn(H, precision='DP')
        e = w.solve_cc(e_conv, r_conv, 200, keep_tape=True)
        ctx.w = w
        ctx.conv = (e_conv, r_conv)
        return torch.tensor(e, dtype=torch.float64, device=F.device)

    @staticmethod
    def backward(ctx, gE):
        # Lambda on the tensor cores to their floor, the densities from one FP64 sweep with
        # the floor's correction (CCSDAdjoint.gradient), over the forward solve's own tape
        adj = CCSDAdjoint(ctx.w, sweep='tc')
        adj.solve_lambda(*ctx.conv, polish=False)
        gF, Gam = adj.gradient()
        return gE * gF, gE * Gam, None, None, None


def ccsd_energy(F, ERI, no, e_conv=1e-11, r_conv=1e-11):
    """Differentiable FP64 CCSD correlation energy (see :class:`CCSDEnergy`)."""
    return CCSDEnergy.apply(F, ERI, no, e_conv, r_conv)
