"""The reference's adjoint objects over the FP64 engine: ``cchbar``, ``cclambda`` and
``ccdensity`` (``pycc/cchbar.py:24-110``, ``pycc/cclambda.py:27-200, :547-570``,
``pycc/ccdensity.py:24-333``), with their constructors, methods and conventions.

The reference materialises eleven HBAR blocks (``Hvvvv`` is v^4), solves the Lambda equations
with hand-derived residuals and builds the densities block by block.  Here HBAR is the tape
of the FP64 residual at the current amplitudes (:class:`pycc_gb300.adjoint.CCSDAdjoint`): its
action is the tape's forward sweep (``cchbar.jacobian``), its transpose the reverse sweep,
which solves the Lambda equations; the densities are the derivatives of the Lagrangian
E + <lambda, r> with respect to F and <pq|rs>.

Conventions of the reference kept here:

* ``cclambda.l1``, ``cclambda.l2``: the reference's normalisation, l2 = 2 x the engine's
  lambda on r2 (the engine pairs lambda with the symmetrised r2); the starting guess
  l1 = 2 t1, l2 = 2 (2 t2 - t2.swapaxes(2,3)) (``pycc/cclambda.py:66-67``);
* ``solve_lambda(...)`` returns the pseudo-energy 1/2 <ij|ab> l2_ijab (``:547-570``);
* ``ccdensity.Doo / Dov / Dvo / Dvv`` and the D of ``gradient_densities()`` are the
  reference's one-particle density, not symmetrised: dL/dF_pq with F a general matrix, which
  is what the reference's blocks are (``pycc/ccdensity.py:335-470``);
* ``gradient_densities()`` returns (D, Gamma), nmo^2 and nmo^4 in <pq|rs> order, with
  E_corr = <D, F> + <Gamma, ERI>.  The reference stores representative two-particle blocks
  with per-block factors and symmetrises Gamma four-fold; the energy defines Gamma only up
  to the eight permutations under which real <pq|rs> are symmetric, so Gamma is returned
  symmetrised eight-fold.  It agrees with the reference's on that projection, which is all a
  real symmetric perturbation, and the generalised-Fock contraction, sees.
"""
from __future__ import annotations

import time

import torch

from . import _lib
from .adjoint import CCSDAdjoint


def _combine(a, X, b, perm, stream, out=None):
    """out = a X + b X.permute(perm) (b = 0: a X) on the FP64 combination kernel."""
    X4 = X.reshape((1,) * (4 - X.dim()) + tuple(X.shape)) if X.dim() < 4 else X
    if out is None:
        out = torch.empty(X4.shape, dtype=torch.float64, device=X.device)
    Y = X4.permute(*perm) if perm is not None else None
    _lib.call("pcg_combine4_f64", _lib.i64s(X4.shape), float(a), X4.data_ptr(),
              _lib.i64s(X4.stride()), float(b), X4.data_ptr() if Y is not None else None,
              _lib.i64s(Y.stride() if Y is not None else [0, 0, 0, 0]), out.data_ptr(),
              _lib.i64s(out.stride()), _lib.stream_handle(stream))
    return out.reshape(X.shape)


def symmetrize_density2(G, stream=None):
    """Projection of a <pq|rs>-ordered tensor onto the eight permutations that leave real
    two-electron integrals unchanged: averages over p<->r, q<->s and (pq)<->(rs) images."""
    for perm in ((2, 1, 0, 3), (0, 3, 2, 1), (1, 0, 3, 2)):
        G = _combine(0.5, G, 0.5, perm, stream)
    return G


class cchbar:
    """HBAR of the FP64 engine (``pycc/cchbar.py:54``), represented two ways.

    * The residual's tape: ``jacobian`` is HBAR's action on an amplitude pair
      (``CCderiv._ccsd_jacobian``) and the reverse sweep its transpose (Lambda); ``sweep``
      ('fp64' or 'tc') selects the engine of the sweeps (see :class:`CCSDAdjoint`).
    * The reference's eleven blocks ``Hov, Hvv, Hoo, Hoooo, Hvvvv, Hvovv, Hooov, Hovvo, Hovov,
      Hvvvo, Hovoo`` with its index layouts, built in FP64 on the GPU on first access
      (``pycc_gb300.hbar.HBAR``; ``Hvvvv`` is nv^4)."""

    def __init__(self, ccwfn, sweep=None):
        t0 = time.time()
        self.ccwfn = ccwfn
        self.contract = ccwfn.contract
        self.adjoint = CCSDAdjoint(ccwfn, sweep=sweep)
        self.timing = time.time() - t0

    def jacobian(self, X1, X2):
        return self.adjoint.jacobian(X1, X2)

    def __getattr__(self, name):
        from .hbar import HBAR, NAMES
        if name in NAMES:
            hb = self.__dict__.get("_hbar")
            if hb is None:
                hb = self.__dict__["_hbar"] = HBAR(self.ccwfn)
            return hb[name]
        raise AttributeError(name)


class cclambda:
    """Lambda amplitudes with the reference's interface (``pycc/cclambda.py:27-200``)."""

    def __init__(self, ccwfn, hbar=None):
        if not isinstance(hbar, cchbar):
            hbar = cchbar(ccwfn)
        self.ccwfn = ccwfn
        self.hbar = hbar
        self.contract = ccwfn.contract
        st = ccwfn.stream
        self.l1 = _combine(2.0, ccwfn.t1, 0.0, None, st)
        self.l2 = _combine(4.0, ccwfn.t2, -2.0, (0, 1, 3, 2), st)

    def solve_lambda(self, e_conv=1e-7, r_conv=1e-7, maxiter=100, max_diis=8, start_diis=1,
                     polish=True):
        """Solve the Lambda equations; returns the pseudo-energy (float).  ``polish``: see
        :meth:`CCSDAdjoint.solve_lambda` (tensor-core sweeps only)."""
        w = self.ccwfn
        l1, l2 = self.hbar.adjoint.solve_lambda(e_conv, r_conv, maxiter, max_diis, start_diis,
                                                polish=polish)
        self.l1 = l1.clone()
        self.l2 = _combine(2.0, l2, 0.0, None, w.stream)
        self.pseudo = self.pseudoenergy(w.o, w.v, w.H.ERI, self.l2)
        return self.pseudo

    def pseudoenergy(self, o, v, ERI, l2):
        """1/2 <ij|ab> l2_ijab (``pycc/cclambda.py:547-570``)."""
        return 0.5 * float(self.contract('ijab,ijab->', ERI[o, o, v, v], l2))


class ccdensity:
    """One- and two-particle densities at the current (t, lambda)
    (``pycc/ccdensity.py:58-111``): the derivatives of the Lagrangian E + <lambda, r> with
    respect to F and <pq|rs>, one reverse sweep over the residual's tape."""

    def __init__(self, ccwfn, cclambda, onlyone=False):
        t0 = time.time()
        self.ccwfn = ccwfn
        self.cclambda = cclambda
        self.contract = ccwfn.contract
        self.onlyone = onlyone
        adj = cclambda.hbar.adjoint
        l2 = _combine(0.5, cclambda.l2, 0.0, None, ccwfn.stream)     # the engine's lambda
        self._D, self._Gam = adj.gradient(l1=cclambda.l1, l2=l2)
        o, v = ccwfn.o, ccwfn.v
        self.Doo, self.Dov = self._D[o, o], self._D[o, v]
        self.Dvo, self.Dvv = self._D[v, o], self._D[v, v]
        self.timing = time.time() - t0

    def gradient_densities(self):
        """(D, Gamma) with E_corr = <D, F> + <Gamma, ERI> (``pycc/ccdensity.py:267-333``)."""
        if self.onlyone:
            raise RuntimeError("gradient_densities needs the two-particle density "
                               "(construct ccdensity with onlyone=False).")
        return self._D.clone(), symmetrize_density2(self._Gam, self.ccwfn.stream)

    def compute_energy(self):
        """The correlation energy from the densities (``pycc/ccdensity.py:113-211``): <D, F>,
        plus <Gamma, ERI> unless only the one-particle density was asked for.  Gamma is
        non-zero only on the integral blocks the residual reads, so the sum runs over those
        resident blocks."""
        w = self.ccwfn
        E = float(self.contract('pq,pq->', self._D, w.H.F))
        if self.onlyone:
            return E
        no, nv = w.no, w.nv
        sl = {"o": slice(0, no), "v": slice(no, no + nv)}
        for pat, blk in w.H.ERI.blocks.items():
            g = self._Gam[tuple(sl[c] for c in pat)]
            E += float(self.contract('pqrs,pqrs->', g, blk))
        return E
