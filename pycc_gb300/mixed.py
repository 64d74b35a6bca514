"""Mixed-precision RHF-CCSD residual on the tcgen05 tensor-core engine.

The same equations as ``CCwfn.residuals`` (``pycc/ccwfn.py:321-945``), with every
contraction of O(o^2 v^3) cost or more issued to the tensor cores (``pycc_gb300.tc``):

* fast mode: BF16 operands, FP32 accumulation in TMEM; the <ab|ef> ladder in FP8 E4M3
  with per-row scales when ``vvvv_fp8`` is set;
* final mode (update norm below ``switch_threshold``, or ``precision='SP'``): compensated
  split-BF16x3 products everywhere.

Amplitudes, intermediates, residuals, denominators, the energy, the update norm and DIIS stay
FP64 (the GEMM epilogue accumulates into FP64).  Matrix-vector shaped and O(o^2 v^2) terms
run on the FP64 kernels.  Two algebraically exact refactorings are shared with the FP64 path:
the t1 t1 <mb|ej> / <ma|je> terms of r2 are evaluated in two O(o^3 v^2) steps instead of one
O(o^3 v^3) step, and the Fme dressings of Fae / Fmi are folded into the dressed
one-body matrices before they multiply t2.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .contract import contract_f64
from .tc import (FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_BF16X6, FMT_FP8, Operand,
                 TCEngine, pack, static_pack_format)


class MixedResidual:
    """Precision ladder: FP8 ladder + BF16 -> BF16 -> split-BF16x3 fused -> split-BF16x3.

    A stage hands over to the next when the update norm drops below its threshold or
    stops decreasing (the stage's rounding floor): ``fp8_threshold`` (1e-3) for the FP8
    stage, ``switch_threshold`` (1e-5) for BF16.  The fused split-BF16x3 stage (all three
    products from one shared-memory stage) runs until its floor; the last stage issues the
    products as separate passes, whose FP32 chains carry less truncation bias, and
    fixes the converged energy.
    """

    STALL_RATIO = 0.8     # rms above this fraction of the stage's best counts as no progress
    STALL_ITERS = 2       # consecutive non-improving iterations that end a stage

    def __init__(self, w, mode="auto"):
        self.w = w
        self.tc = TCEngine(w.device1, w.stream)
        if mode == "bf16x6":
            self.stages = ["bf16x6"]
        elif mode == "bf16x3":
            self.stages = ["bf16x3"]
        else:
            self.stages = (["fp8", "bf16", "bf16x3f", "bf16x3s"] if w.vvvv_fp8
                           else ["bf16", "bf16x3f", "bf16x3s"])
        self.stage = 0
        self.thresholds = {"fp8": getattr(w, "fp8_threshold", 1e-3), "bf16": w.switch_threshold,
                           "bf16x3f": 0.0}
        self.best = float("inf")
        self.bad = 0
        self.history = []
        self.profile = None       # list of (subscripts, fmt, start, end) events when set
        self._pairs = None        # i <= j pair tables of the ladder
        self._hole_tab = None     # the pair columns of Wmnij for the hole ladder
        self._r_seed = None
        self._blocks = None       # the integral blocks the caches were built from

    def sync_integrals(self):
        """Drop the packed integrals and the 1/2 <ab|ij> seed when ``H.ERI`` / ``H.L`` no
        longer hold the blocks they were built from.  The reference's derivative driver swaps
        them for derivative integrals around one ``residuals`` call, using the residual's
        linearity in H (pycc/ccderiv.py:252-259); the next call after each swap re-packs.
        The blocks are referenced here, so their addresses cannot be reused unnoticed."""
        H = self.w.H
        try:
            blocks = list(H.ERI.blocks.values()) + list(H.L.blocks.values())
        except AttributeError:
            raise TypeError("H.ERI and H.L must be pycc_gb300 BlockTensors (resident o/v "
                            "blocks), e.g. Hamiltonian.from_arrays(...).ERI") from None
        if self._blocks is not None and len(blocks) == len(self._blocks) and all(
                a is b for a, b in zip(blocks, self._blocks)):
            return
        if self._blocks is not None:
            self.tc.cache.clear()
            self._r_seed = None
        self._blocks = blocks

    # -- precision schedule ---------------------------------------------------------------
    def select_mode(self, rms):
        """Pick the precision of the next residual from the last update norm."""
        if rms < float("inf"):
            name = self.stages[self.stage]
            if not self.is_final_mode() and rms < self.thresholds.get(name, 0.0):
                self._advance()
            else:
                if rms > self.STALL_RATIO * self.best:
                    self.bad += 1
                else:
                    self.bad = 0
                self.best = min(self.best, rms)
                if self.bad >= self.STALL_ITERS and not self.is_final_mode():
                    self._advance()
        if rms == 0.0:                      # explicit request for the final stage
            self.stage = len(self.stages) - 1
            self._prune()
        self.history.append(self.mode_name())

    def _advance(self):
        self.stage = min(self.stage + 1, len(self.stages) - 1)
        self.best = float("inf")
        self.bad = 0
        self._prune()

    def _prune(self):
        """Free the packed integrals of formats no remaining stage reads."""
        used = set()
        for name in self.stages[self.stage:]:
            used.add(static_pack_format(self.FMTS[name]))
            if name == "fp8":
                used.add(FMT_FP8)
        for key in [k for k in self.tc.cache if k[-1] not in used]:
            del self.tc.cache[key]

    def at_floor(self):
        """True once the final stage has stopped reducing the update norm."""
        return self.is_final_mode() and self.bad >= 2 * self.STALL_ITERS

    def force_final(self):
        self.stage = len(self.stages) - 1
        self._prune()

    def is_final_mode(self):
        return self.stage == len(self.stages) - 1

    def mode_name(self):
        return self.stages[self.stage]

    FMTS = {"bf16": FMT_BF16, "bf16x3f": FMT_BF16X3F, "bf16x3s": FMT_BF16X3S,
            "bf16x3": FMT_BF16X3, "bf16x6": FMT_BF16X6, "fp8": FMT_BF16}

    def fmt(self):
        return self.FMTS[self.mode_name()]

    def ladder_fmt(self):
        name = self.mode_name()
        return FMT_FP8 if name == "fp8" else self.FMTS[name]

    # -- helpers --------------------------------------------------------------------------
    def tcc(self, subs, A, B, out, alpha=1.0, beta=1.0, fmt=None):
        fmt = self.fmt() if fmt is None else fmt
        if self.profile is None:
            return self.tc.contract(subs, A, B, out, alpha=alpha, beta=beta, fmt=fmt)
        # per-term timing: CUDA events on the launching stream around pack + GEMM
        st = torch.cuda.current_stream() if self.w.stream is None else self.w.stream
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        res = self.tc.contract(subs, A, B, out, alpha=alpha, beta=beta, fmt=fmt)
        e1.record(st)
        self.profile.append((subs, fmt, e0, e1))
        return res

    def eri(self, pat, labels):
        return Operand.of(labels, self.w.H.ERI.blocks[pat], key=("ERI", pat))

    def ll(self, pat, labels):
        return Operand.of(labels, self.w.H.L.blocks[pat], key=("L", pat))

    # -- the <ab|ef> ladder over i <= j pairs (pycc/ccwfn.py:931) ---------------------------
    def _pair_tables(self):
        if self._pairs is None:
            no, nv = self.w.no, self.w.nv
            ii, jj = np.triu_indices(no)
            tab = np.zeros((4, ii.size), dtype=np.int64)
            tab[0] = ii * no * nv * nv + jj * nv * nv       # t2[i, j, :, :]
            tab[2] = ii * nv                                # t1[i, :]
            tab[3] = jj * nv                                # t1[j, :]
            cmap = (ii * no * nv * nv + jj * nv * nv).astype(np.int64)
            csc = np.where(ii == jj, 0.5, 1.0)
            dev = self.w.device1
            self._pairs = (torch.from_numpy(tab).to(dev), torch.from_numpy(cmap).to(dev),
                           torch.from_numpy(csc).to(dev))
        return self._pairs

    def ladder_pairs(self, t1, t2, r, fmt):
        """r_ijab += 1/2 tau_ijef <ab|ef> through the i <= j pairs only.

        tau_jife = tau_ijef and <ba|fe> = <ab|ef>, so the term is symmetric under
        (i<->j, a<->b) and the symmetrisation r2 = h + h' of r_T2 (ccwfn.py:790) doubles it.
        Writing the full term for i < j into h (and half of it for i = j) and nothing for
        i > j gives the same symmetrised residual with o(o+1)/2 instead of o^2 rows.
        """
        if not r.is_contiguous():
            raise ValueError("ladder_pairs: the half residual must be contiguous")
        tab, cmap, csc = self._pair_tables()
        tau = Operand('ijef', (t2, 'ijef'), P=(t1, 'ie'), Q=(t1, 'jf'), c=1.0)
        pb = pack(tau, ['i', 'j'], ['e', 'f'], fmt, self.w.stream, row_tab=tab)
        pa = self.tc._pack(self.eri('vvvv', 'abef'), ['a', 'b'], ['e', 'f'], fmt, 'A')
        torch.cuda.nvtx.range_push("ladder")     # selects this launch for profilers
        self.tc.run_gemm('ijef,abef->ijab', fmt, pa, pb, r, ['a', 'b'], [], 'ijab', 1.0, 1.0,
                         col_map=cmap, col_scale=csc)
        torch.cuda.nvtx.range_pop()

    def hole_ladder_pairs(self, t1, t2, Wmnij, r):
        """r_ijab += 1/2 tau_mnab W_mnij (pycc/ccwfn.py:930) through the i <= j pairs only.

        W_nmji = W_mnij and tau_nmba = tau_mnab, so the term is symmetric under
        (i<->j, a<->b), as the particle ladder is: the same output map and 1/2 diagonal weights
        (``ladder_pairs``) apply, with a row table selecting the pair columns of W_mnij.
        """
        no = self.w.no
        if self._hole_tab is None:
            ii, jj = np.triu_indices(no)
            tab = np.zeros((4, ii.size), dtype=np.int64)
            tab[0] = ii * no + jj                        # Wmnij[m, n, i, j]
            self._hole_tab = torch.from_numpy(tab).to(self.w.device1)
        _, cmap, csc = self._pair_tables()
        fmt = self.fmt()
        tau = Operand('mnab', (t2, 'mnab'), P=(t1, 'ma'), Q=(t1, 'nb'), c=1.0)
        pa = self.tc._pack(tau, ['a', 'b'], ['m', 'n'], fmt, 'A')
        pb = pack(Operand.of('mnij', Wmnij), ['i', 'j'], ['m', 'n'], fmt, self.w.stream,
                  row_tab=self._hole_tab)
        self.tc.run_gemm('mnab,mnij->ijab', fmt, pa, pb, r, ['a', 'b'], [], 'ijab', 1.0, 1.0,
                         col_map=cmap, col_scale=csc)

    # -- intermediates (pycc/ccwfn.py:458-715) -------------------------------------------
    def build_Fae(self, F, t1, t2):
        o, v = self.w.o, self.w.v
        Fae = F[v, v].clone()
        contract_f64('me,ma->ae', F[o, v], t1, out=Fae, alpha=-0.5, beta=1.0)
        self.tcc('mf,mafe->ae', Operand.of('mf', t1), self.ll('ovvv', 'mafe'), Fae)
        taut = Operand('mnaf', (t2, 'mnaf'), P=(t1, 'ma'), Q=(t1, 'nf'), c=0.5)
        self.tcc('mnaf,mnef->ae', taut, self.ll('oovv', 'mnef'), Fae, alpha=-1.0)
        return Fae

    def build_Fmi(self, F, t1, t2):
        o, v = self.w.o, self.w.v
        Fmi = F[o, o].clone()
        contract_f64('ie,me->mi', t1, F[o, v], out=Fmi, alpha=0.5, beta=1.0)
        self.tcc('ne,mnie->mi', Operand.of('ne', t1), self.ll('ooov', 'mnie'), Fmi)
        taut = Operand('inef', (t2, 'inef'), P=(t1, 'ie'), Q=(t1, 'nf'), c=0.5)
        self.tcc('inef,mnef->mi', taut, self.ll('oovv', 'mnef'), Fmi)
        return Fmi

    def build_Fme(self, F, t1):
        o, v = self.w.o, self.w.v
        Fme = F[o, v].clone()
        self.tcc('nf,mnef->me', Operand.of('nf', t1), self.ll('oovv', 'mnef'), Fme)
        return Fme

    def build_Wmnij(self, t1, t2):
        o = self.w.o
        W = self.w.H.ERI[o, o, o, o].clone()
        self.tcc('je,mnie->mnij', Operand.of('je', t1), self.eri('ooov', 'mnie'), W)
        self.tcc('ie,mnej->mnij', Operand.of('ie', t1), self.eri('oovo', 'mnej'), W)
        tau = Operand('ijef', (t2, 'ijef'), P=(t1, 'ie'), Q=(t1, 'jf'), c=1.0)
        self.tcc('ijef,mnef->mnij', tau, self.eri('oovv', 'mnef'), W)
        return W

    def build_Wmbej(self, t1, t2):
        o, v = self.w.o, self.w.v
        W = self.w.H.ERI[o, v, v, o].clone()
        self.tcc('jf,mbef->mbej', Operand.of('jf', t1), self.eri('ovvv', 'mbef'), W)
        self.tcc('nb,mnej->mbej', Operand.of('nb', t1), self.eri('oovo', 'mnej'), W, alpha=-1.0)
        X = Operand('jnfb', (t2, 'jnfb'), a=0.5, P=(t1, 'jf'), Q=(t1, 'nb'), c=1.0)
        self.tcc('jnfb,mnef->mbej', X, self.eri('oovv', 'mnef'), W, alpha=-1.0)
        self.tcc('njfb,mnef->mbej', Operand.of('njfb', t2), self.ll('oovv', 'mnef'), W, alpha=0.5)
        return W

    def build_Wmbje(self, t1, t2):
        o, v = self.w.o, self.w.v
        W = self.w._combine(-1.0, self.w.H.ERI[o, v, o, v], 0.0, None, None)
        self.tcc('jf,mbfe->mbje', Operand.of('jf', t1), self.eri('ovvv', 'mbfe'), W, alpha=-1.0)
        self.tcc('nb,mnje->mbje', Operand.of('nb', t1), self.eri('ooov', 'mnje'), W)
        X = Operand('jnfb', (t2, 'jnfb'), a=0.5, P=(t1, 'jf'), Q=(t1, 'nb'), c=1.0)
        self.tcc('jnfb,mnfe->mbje', X, self.eri('oovv', 'mnfe'), W)
        return W

    def build_Zmbij(self, t1, t2):
        """Z_mbij + <mb|ij> + t_ie <mb|ej> + t_je <mb|ie>: every o^3 v tensor the residual
        contracts with t_ma, summed so that one GEMM applies them (see r_T2_half)."""
        o, v = self.w.o, self.w.v
        Z = self.w._combine(1.0, self.w.H.ERI[o, v, o, o], 0.0, None, None, record=False)
        tau = Operand('ijef', (t2, 'ijef'), P=(t1, 'ie'), Q=(t1, 'jf'), c=1.0)
        self.tcc('mbef,ijef->mbij', self.eri('ovvv', 'mbef'), tau, Z)
        self.tcc('ie,mbej->mbij', Operand.of('ie', t1), self.eri('ovvo', 'mbej'), Z)
        self.tcc('je,mbie->mbij', Operand.of('je', t1), self.eri('ovov', 'mbie'), Z)
        return Z

    # -- residuals (pycc/ccwfn.py:718-945) ------------------------------------------------
    def r_T1(self, F, t1, t2, Fae, Fme, Fmi):
        o, v = self.w.o, self.w.v
        r = self.w._copy(F[v, o].transpose(0, 1))   # a fresh tensor, whatever F's layout
        contract_f64('ie,ae->ia', t1, Fae, out=r, beta=1.0)
        contract_f64('mi,ma->ia', Fmi, t1, out=r, alpha=-1.0, beta=1.0)
        t2s = Operand('imae', (t2, 'imae'), a=2.0, Y=(t2, 'imea'), b=-1.0)
        self.tcc('imae,me->ia', t2s, Operand.of('me', Fme), r)
        self.tcc('nf,nafi->ia', Operand.of('nf', t1), self.ll('ovvo', 'nafi'), r)
        t2s = Operand('mief', (t2, 'mief'), a=2.0, Y=(t2, 'mife'), b=-1.0)
        self.tcc('mief,maef->ia', t2s, self.eri('ovvv', 'maef'), r)
        self.tcc('mnae,nmei->ia', Operand.of('mnae', t2), self.ll('oovo', 'nmei'), r, alpha=-1.0)
        return r

    def r_T2_half(self, F, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
        o, v = self.w.o, self.w.v
        no, nv = self.w.no, self.w.nv
        ERI = self.w.H.ERI
        if self._r_seed is None:       # 1/2 <ab|ij> in the [i,j,a,b] layout, built once
            self._r_seed = self.w._combine(0.5, ERI[v, v, o, o].permute(2, 3, 0, 1), 0.0, None,
                                           None, record=False)
        r = self._r_seed.clone()
        # t2_ijae (F_be - 1/2 t_mb F_me) and - t2_imab (F_mj + 1/2 t_je F_me)
        Fbe = Fae.clone()
        contract_f64('mb,me->be', t1, Fme, out=Fbe, alpha=-0.5, beta=1.0)
        self.tcc('ijae,be->ijab', Operand.of('ijae', t2), Operand.of('be', Fbe), r)
        Fmj = Fmi.clone()
        contract_f64('je,me->mj', t1, Fme, out=Fmj, alpha=0.5, beta=1.0)
        self.tcc('imab,mj->ijab', Operand.of('imab', t2), Operand.of('mj', Fmj), r, alpha=-1.0)
        # ladders
        self.hole_ladder_pairs(t1, t2, Wmnij, r)
        self.ladder_pairs(t1, t2, r, self.ladder_fmt())
        # - t_ma (Z_mbij + <mb|ij>) - t_ie t_ma <mb|ej> - t_ie t_mb <ma|je>, the last written
        # as its (i<->j, a<->b) image - t_je t_ma <mb|ie>, which the symmetrisation
        # r2 = h + h' sums to the same residual; the o^3 v tensors are summed in Zmbij
        self.tcc('ma,mbij->ijab', Operand.of('ma', t1), Operand.of('mbij', Zmbij), r, alpha=-1.0)
        # rings
        # (t2 - t2~) W + t2 (W + W~) regrouped as (2 t2 - t2~) W + t2 W~: the first operand
        # is r_T1's, already packed this residual, and W~ is one source instead of two
        self.tcc('imae,mbej->ijab', Operand('imae', (t2, 'imae'), a=2.0, Y=(t2, 'imea'), b=-1.0),
                 Operand.of('mbej', Wmbej), r)
        self.tcc('imae,mbej->ijab', Operand.of('imae', t2), Operand('mbej', (Wmbje, 'mbje')), r)
        self.tcc('mjae,mbie->ijab', Operand.of('mjae', t2), Operand.of('mbie', Wmbje), r)
        self.tcc('ie,abej->ijab', Operand.of('ie', t1), self.eri('vvvo', 'abej'), r)
        return r

    def residuals(self, F, t1, t2):
        t1 = t1.contiguous()
        t2 = t2.contiguous()
        self.sync_integrals()
        # identical dynamic operands are packed once per call; the packs are released
        # when the call returns
        self.tc.dyn_cache = {}
        try:
            Fae = self.build_Fae(F, t1, t2)
            Fmi = self.build_Fmi(F, t1, t2)
            Fme = self.build_Fme(F, t1)
            Wmnij = self.build_Wmnij(t1, t2)
            Wmbej = self.build_Wmbej(t1, t2)
            Wmbje = self.build_Wmbje(t1, t2)
            Zmbij = self.build_Zmbij(t1, t2)
            r1 = self.r_T1(F, t1, t2, Fae, Fme, Fmi)
            half = self.r_T2_half(F, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij)
        finally:
            self.tc.dyn_cache = None
        r2 = torch.empty_like(half)
        _lib.call("pcg_symmetrize_f64", half.data_ptr(), self.w.no, self.w.nv, r2.data_ptr(),
                  _lib.stream_handle(self.w.stream))
        return r1, r2
