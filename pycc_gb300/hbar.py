"""Materialised blocks of the similarity-transformed Hamiltonian (HBAR) of RHF-CCSD.

The reference builds eleven HBAR blocks in ``cchbar.__init__`` (``pycc/cchbar.py:54-110``,
spatial orbitals: ``build_Hov`` ... ``build_Hovoo``, ``:128-858``).  The engine's adjoint does
not need them -- J x and J^T l are the residual tape's sweeps -- but callers that read the
blocks themselves (EOM, response) do.  ``HBAR`` builds them on the GPU, in FP64 on the
engine's DMMA contraction kernel, from the wave function's amplitudes and resident integral
blocks, each block on first use (``Hvvvv`` alone is nv^4: 64.8 GB at nv = 300).

Blocks the residual does not read (<am|ef>, <am|ei>, <am|ie> and L_amef) are index
permutations of resident ones -- <am|ef> = <ma|fe>, <am|ei> = <ma|ie>, <am|ie> = <ma|ei>,
L_amef = L_mafe -- and enter the contractions as strided views, never copied.

Index layouts are the reference's: Hov[m,e], Hvv[a,e], Hoo[m,i], Hoooo[m,n,i,j],
Hvvvv[a,b,e,f], Hvovv[a,m,e,f], Hooov[m,n,i,e], Hovvo[m,b,e,j], Hovov[m,b,j,e],
Hvvvo[a,b,e,i], Hovoo[m,b,i,j].
"""
from __future__ import annotations

import torch

from . import _lib
from .contract import contract_f64

NAMES = ("Hov", "Hvv", "Hoo", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov", "Hvvvo",
         "Hovoo")


class HBAR:
    """The eleven HBAR blocks of a converged CCSD wave function, built on first access."""

    def __init__(self, w):
        self.w = w
        self.blocks = {}

    def __getitem__(self, name):
        if name not in NAMES:
            raise KeyError(name)
        if name not in self.blocks:
            self.blocks[name] = getattr(self, "_" + name)()
        return self.blocks[name]

    # -- helpers --------------------------------------------------------------------------
    def _c(self, subs, A, B, out=None, alpha=1.0, beta=1.0):
        return contract_f64(subs, A, B, out=out, alpha=alpha, beta=beta if out is not None else 0.0,
                            stream=self.w.stream)

    def _copy(self, X, a=1.0):
        out = torch.empty(X.shape, dtype=torch.float64, device=X.device)
        return self._axpy(out, a, X, 0.0, None, None, fresh=True)

    def _axpy(self, out, a, X, b, Y, perm, fresh=False):
        """out = a X + b Y.permute(perm) (4-index, FP64 kernel); in place when not fresh."""
        X4 = X if X.dim() == 4 else X.reshape((1,) * (4 - X.dim()) + tuple(X.shape))
        o4 = out if out.dim() == 4 else out.view((1,) * (4 - out.dim()) + tuple(out.shape))
        ys = [0, 0, 0, 0]
        yp = None
        if Y is not None:
            Yp = Y.permute(*perm)
            ys = list(Yp.stride())
            yp = Y.data_ptr()
        _lib.call("pcg_combine4_f64", _lib.i64s(X4.shape), float(a), X4.data_ptr(),
                  _lib.i64s(X4.stride()), float(b), yp, _lib.i64s(ys), o4.data_ptr(),
                  _lib.i64s(o4.stride()), _lib.stream_handle(self.w.stream))
        return out

    def _eri(self, pat):
        return self.w.H.ERI.blocks[pat]

    def _L(self, pat):
        return self.w.H.L.blocks[pat]

    def _amps(self):
        return self.w.t1.contiguous(), self.w.t2.contiguous()

    def _tau(self):
        t1, t2 = self._amps()
        return self.w.build_tau(t1, t2)

    # views of the blocks the residual does not keep
    def _vovv(self):        # <am|ef> = <ma|fe>
        return self._eri("ovvv").permute(1, 0, 3, 2)

    def _vovo(self):        # <am|ei> = <ma|ie>
        return self._eri("ovov").permute(1, 0, 3, 2)

    def _voov(self):        # <am|ie> = <ma|ei>
        return self._eri("ovvo").permute(1, 0, 3, 2)

    def _Lvovv(self):       # L_amef = L_mafe
        return self._L("ovvv").permute(1, 0, 3, 2)

    # -- one-body blocks (pycc/cchbar.py:128-301) ------------------------------------------
    def _Hov(self):
        """Hov_me = f_me + t_nf L_mnef."""
        t1, _ = self._amps()
        no = self.w.no
        H = self._copy(self.w.H.F[:no, no:])
        self._c('nf,mnef->me', t1, self._L("oovv"), out=H)
        return H

    def _Hvv(self):
        """Hvv_ae = f_ae - f_me t_ma + t_mf L_amef - tau_mnfa L_mnfe."""
        t1, _ = self._amps()
        no = self.w.no
        F = self.w.H.F
        H = self._copy(F[no:, no:])
        self._c('me,ma->ae', F[:no, no:], t1, out=H, alpha=-1.0)
        self._c('mf,amef->ae', t1, self._Lvovv(), out=H)
        self._c('mnfa,mnfe->ae', self._tau(), self._L("oovv"), out=H, alpha=-1.0)
        return H

    def _Hoo(self):
        """Hoo_mi = f_mi + t_ie f_me + t_ne L_mnie + tau_inef L_mnef."""
        t1, _ = self._amps()
        no = self.w.no
        F = self.w.H.F
        H = self._copy(F[:no, :no])
        self._c('ie,me->mi', t1, F[:no, no:], out=H)
        self._c('ne,mnie->mi', t1, self._L("ooov"), out=H)
        self._c('inef,mnef->mi', self._tau(), self._L("oovv"), out=H)
        return H

    # -- two-body blocks (pycc/cchbar.py:303-858) ------------------------------------------
    def _Hoooo(self):
        """<mn|ij> + (t_je <mn|ie> + t_ie <nm|je>) + tau_ijef <mn|ef>."""
        t1, _ = self._amps()
        X = self._c('je,mnie->mnij', t1, self._eri("ooov"))
        H = self._axpy(torch.empty_like(X), 1.0, X, 1.0, X, (1, 0, 3, 2), fresh=True)
        self._axpy(H, 1.0, H, 1.0, self._eri("oooo"), (0, 1, 2, 3))
        self._c('ijef,mnef->mnij', self._tau(), self._eri("oovv"), out=H)
        return H

    def _Hvvvv(self):
        """<ab|ef> - (t_mb <am|ef> + t_ma <bm|fe>) + tau_mnab <mn|ef>, accumulated into one
        nv^4 buffer (no nv^4 temporary)."""
        t1, _ = self._amps()
        H = self._copy(self._eri("vvvv"))
        self._c('mb,amef->abef', t1, self._vovv(), out=H, alpha=-1.0)
        self._c('ma,bmfe->abef', t1, self._vovv(), out=H, alpha=-1.0)
        self._c('mnab,mnef->abef', self._tau(), self._eri("oovv"), out=H)
        return H

    def _Hvovv(self):
        """<am|ef> - t_na <nm|ef>."""
        t1, _ = self._amps()
        H = self._copy(self._vovv())
        self._c('na,nmef->amef', t1, self._eri("oovv"), out=H, alpha=-1.0)
        return H

    def _Hooov(self):
        """<mn|ie> + t_if <nm|ef>."""
        t1, _ = self._amps()
        H = self._copy(self._eri("ooov"))
        self._c('if,nmef->mnie', t1, self._eri("oovv"), out=H)
        return H

    def _Hovvo(self):
        """<mb|ej> + t_jf <mb|ef> - t_nb <mn|ej> - tau_jnfb <mn|ef> + t2_njfb L_mnef."""
        t1, t2 = self._amps()
        H = self._copy(self._eri("ovvo"))
        self._c('jf,mbef->mbej', t1, self._eri("ovvv"), out=H)
        self._c('nb,mnej->mbej', t1, self._eri("oovo"), out=H, alpha=-1.0)
        self._c('jnfb,mnef->mbej', self._tau(), self._eri("oovv"), out=H, alpha=-1.0)
        self._c('njfb,mnef->mbej', t2, self._L("oovv"), out=H)
        return H

    def _Hovov(self):
        """<mb|je> + t_jf <bm|ef> - t_nb <mn|je> - tau_jnfb <nm|ef>."""
        t1, _ = self._amps()
        H = self._copy(self._eri("ovov"))
        self._c('jf,bmef->mbje', t1, self._vovv(), out=H)
        self._c('nb,mnje->mbje', t1, self._eri("ooov"), out=H, alpha=-1.0)
        self._c('jnfb,nmef->mbje', self._tau(), self._eri("oovv"), out=H, alpha=-1.0)
        return H

    def _Hvvvo(self):
        """<ab|ei> - Hov_me t2_miab + t_if Hvvvv_abef + tau_mnab <mn|ei>
        - t2_imfa <bm|fe> - t2_imfb <am|ef> + t2_mifb L_amef
        - t_mb (<am|ei> - t2_infa <mn|fe>)
        - t_ma (<bm|ie> - t2_infb <mn|ef> + t2_nifb L_mnef)."""
        t1, t2 = self._amps()
        ov = self._eri("oovv")
        H = self._copy(self._eri("vvvo"))
        self._c('me,miab->abei', self["Hov"], t2, out=H, alpha=-1.0)
        self._c('if,abef->abei', t1, self["Hvvvv"], out=H)
        self._c('mnab,mnei->abei', self._tau(), self._eri("oovo"), out=H)
        self._c('imfa,bmfe->abei', t2, self._vovv(), out=H, alpha=-1.0)
        self._c('imfb,amef->abei', t2, self._vovv(), out=H, alpha=-1.0)
        self._c('mifb,amef->abei', t2, self._Lvovv(), out=H)
        X = self._copy(self._vovo())
        self._c('infa,mnfe->amei', t2, ov, out=X, alpha=-1.0)
        self._c('mb,amei->abei', t1, X, out=H, alpha=-1.0)
        Y = self._copy(self._voov())
        self._c('infb,mnef->bmie', t2, ov, out=Y, alpha=-1.0)
        self._c('nifb,mnef->bmie', t2, self._L("oovv"), out=Y)
        self._c('ma,bmie->abei', t1, Y, out=H, alpha=-1.0)
        return H

    def _Hovoo(self):
        """<mb|ij> + Hov_me t2_ijeb - t_nb Hoooo_mnij + tau_ijef <mb|ef>
        - t2_ineb <nm|je> - t2_jneb <mn|ie> + t2_njeb L_mnie
        + t_je (<mb|ie> - t2_infb <mn|fe>)
        + t_ie (<bm|je> - t2_jnfb <mn|ef> + t2_njfb L_mnef)."""
        t1, t2 = self._amps()
        ov = self._eri("oovv")
        H = self._copy(self._eri("ovoo"))
        self._c('me,ijeb->mbij', self["Hov"], t2, out=H)
        self._c('nb,mnij->mbij', t1, self["Hoooo"], out=H, alpha=-1.0)
        self._c('ijef,mbef->mbij', self._tau(), self._eri("ovvv"), out=H)
        self._c('ineb,nmje->mbij', t2, self._eri("ooov"), out=H, alpha=-1.0)
        self._c('jneb,mnie->mbij', t2, self._eri("ooov"), out=H, alpha=-1.0)
        self._c('njeb,mnie->mbij', t2, self._L("ooov"), out=H)
        X = self._copy(self._eri("ovov"))
        self._c('infb,mnfe->mbie', t2, ov, out=X, alpha=-1.0)
        self._c('je,mbie->mbij', t1, X, out=H)
        Y = self._copy(self._voov())
        self._c('jnfb,mnef->bmje', t2, ov, out=Y, alpha=-1.0)
        self._c('njfb,mnef->bmje', t2, self._L("oovv"), out=Y)
        self._c('ie,bmje->mbij', t1, Y, out=H)
        return H
