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
one-body matrices before they multiply t2.  Exact rearrangements of this path alone: the
particle and hole ladders and the tau terms of Wmnij and Zmbij in symmetric /
antisymmetric pair form (``ladder_pm``, ``pair_tau``), the ring terms regrouped, and r_T1's
(2 t2 - t2~) <ma|ef> as t2 L_maef.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .contract import contract_f64
from .tc import (FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_BF16X6, FMT_FP8, Operand,
                 TCEngine, static_pack_format)


class MixedResidual:
    """Precision ladder: FP8 ladder + BF16 -> BF16 -> split-BF16x3 fused -> split-BF16x3.

    A stage hands over to the next when the update norm drops below its threshold or
    stops decreasing (the stage's rounding floor): ``fp8_threshold`` (1e-3) for the FP8
    stage, ``switch_threshold`` (1e-5) for BF16.  The fused split-BF16x3 stage (all three
    products from one shared-memory stage, one FP32 accumulator) runs until its floor; the
    last stage keeps the two small products in an accumulator of their own over the tile's
    whole K, whose FP32 chain then carries less truncation bias, and fixes the converged
    energy.
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
        self._pm = None           # offset tables of the ladder's pair form
        self._kpm = {}            # K pair tables of the pair-form intermediates, per block
        self._hpm = None          # offset tables of the hole ladder's pair form
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
    def _pm_tables(self, t1, t2, V):
        """Offset tables of the symmetric / antisymmetric pair form of the ladder
        (``ladder_pm``): rows of V+- over the a <= b / a < b pairs, K over the e <= f /
        e < f pairs (with 1/2 on e = f for V+, whose <ab|ef> + <ab|fe> doubles it there),
        rows of T+- over the i <= j / i < j pairs.  Offsets follow the tensors' own strides
        (V: [a, b, e, f]; t2: [i, j, e, f]; t1: [i, e])."""
        key = (tuple(V.stride()), tuple(t2.stride()), tuple(t1.stride()))
        if self._pm is not None and self._pm[0] == key:
            return self._pm[1]
        no, nv = self.w.no, self.w.nv
        dev = self.w.device1
        sv, s2, s1 = V.stride(), t2.stride(), t1.stride()
        tabs = {}
        for sign, k in (("+", 0), ("-", 1)):
            a, b = np.triu_indices(nv, k)            # a <= b (+) or a < b (-) pairs
            i, j = np.triu_indices(no, k)
            vr = np.zeros((6, a.size), dtype=np.int64)
            vr[0] = vr[1] = a * sv[0] + b * sv[1]
            vk = np.zeros((6, a.size), dtype=np.int64)          # K pairs: e = a, f = b
            vk[0] = a * sv[2] + b * sv[3]
            vk[1] = b * sv[2] + a * sv[3]
            tr = np.zeros((6, i.size), dtype=np.int64)
            tr[0] = tr[1] = i * s2[0] + j * s2[1]
            tr[2] = tr[4] = i * s1[0]                            # t_ie, t_if
            tr[3] = tr[5] = j * s1[0]                            # t_jf, t_je
            tk = np.zeros((6, a.size), dtype=np.int64)
            tk[0] = a * s2[2] + b * s2[3]                        # tau_ijef
            tk[1] = b * s2[2] + a * s2[3]                        # tau_ijfe
            tk[2], tk[3] = a * s1[1], b * s1[1]                  # t_ie t_jf
            tk[4], tk[5] = b * s1[1], a * s1[1]                  # t_if t_je
            kw = np.where(a == b, 0.5, 1.0).astype(np.float32) if sign == "+" else None
            t = lambda x: torch.from_numpy(x).to(dev) if x is not None else None
            tabs[sign] = {"vrow": t(vr), "vk": t(vk), "kw": t(kw), "trow": t(tr), "tk": t(tk),
                          "rows": a.size, "cols": i.size}
        self._pm = (key, tabs)
        return tabs

    def _hole_pm_tables(self, t1, t2, W):
        """Offset tables of the hole ladder's pair form (``ladder_pm`` with Wmnij): rows of
        tau+- over the a <= b / a < b pairs and K over the m <= n / m < n pairs (sources
        tau_mnab = t2_mnab + t_ma t_nb and tau_mnba), rows of W+- over the i <= j / i < j pairs
        and K over the same (m, n) pairs (sources W_mnij and W_mnji, with 1/2 on m = n for
        W+).  Offsets follow the tensors' own strides (t2 and W: [m, n, ., .]; t1: [m, a])."""
        key = (tuple(W.stride()), tuple(t2.stride()), tuple(t1.stride()))
        if self._hpm is not None and self._hpm[0] == key:
            return self._hpm[1]
        no, nv = self.w.no, self.w.nv
        dev = self.w.device1
        sw, s2, s1 = W.stride(), t2.stride(), t1.stride()
        tabs = {}
        for sign, k in (("+", 0), ("-", 1)):
            a, b = np.triu_indices(nv, k)
            m, n = np.triu_indices(no, k)
            i, j = m, n                                          # the i <= j (i < j) pairs
            ur = np.zeros((6, a.size), dtype=np.int64)           # tau rows: (a, b)
            ur[0] = a * s2[2] + b * s2[3]                        # t2_mnab
            ur[1] = b * s2[2] + a * s2[3]                        # t2_mnba
            ur[2], ur[3] = a * s1[1], b * s1[1]                  # t_ma t_nb
            ur[4], ur[5] = b * s1[1], a * s1[1]                  # t_mb t_na
            uk = np.zeros((6, m.size), dtype=np.int64)           # tau K: (m, n)
            uk[0] = uk[1] = m * s2[0] + n * s2[1]
            uk[2], uk[3] = m * s1[0], n * s1[0]
            uk[4], uk[5] = m * s1[0], n * s1[0]
            wr = np.zeros((6, i.size), dtype=np.int64)           # W rows: (i, j)
            wr[0] = i * sw[2] + j * sw[3]                        # W_mnij
            wr[1] = j * sw[2] + i * sw[3]                        # W_mnji
            wk = np.zeros((6, m.size), dtype=np.int64)
            wk[0] = wk[1] = m * sw[0] + n * sw[1]
            kw = np.where(m == n, 0.5, 1.0).astype(np.float32) if sign == "+" else None
            t = lambda x: torch.from_numpy(x).to(dev) if x is not None else None
            tabs[sign] = {"urow": t(ur), "uk": t(uk), "wrow": t(wr), "wk": t(wk), "kw": t(kw),
                          "rows": a.size, "cols": i.size, "k": m.size}
        self._hpm = (key, tabs)
        return tabs

    def ladder_pm(self, t1, t2, r, fmt, Wmnij=None, hole_fmt=None):
        """r_ijab += 1/2 tau_ijef <ab|ef> (pycc/ccwfn.py:931) in symmetric / antisymmetric
        pair form: two GEMMs, G+- = T+- . V+-, over the e <= f (e < f) pairs of K, the
        a <= b (a < b) pairs of rows and the i <= j (i < j) pairs of columns, then
        ``pcg_ladder_pm_assemble`` adds S = 1/2 (G+ + sign(b - a) G-) = sum_ef tau_ijef <ab|ef>
        into the half residual for i < j (twice the term: h_jiba then carries none of it)
        and S / 2 for i = j, as the i <= j pair form of the ladder does.
        T+-_ij,ef = tau_ijef +- tau_ijfe (packed from t2 and t1 in one pass), V+-_ab,ef =
        <ab|ef> +- <ab|fe> (packed once per format and cached).  Half of the i <= j pair
        form's tensor-core work, and half of its packed integral bytes.

        With ``Wmnij`` the hole ladder r_ijab += 1/2 tau_mnab W_mnij (pycc/ccwfn.py:930) joins
        the same G+-: tau_nmab = tau_mnba and W_nmij = W_mnji, so over the m <= n (m < n)
        pairs sum_mn tau_mnab W_mnij = 1/2 (H+ + H-) with H+- = sum (tau_mnab +- tau_mnba)
        (W_mnij +- W_mnji) (1/2 on m = n for +), which has the symmetry of G+- under
        i<->j and a<->b.  Two small GEMMs (K = the occupied pairs, in ``hole_fmt``)
        accumulate into G+- before the one assembly."""
        if not r.is_contiguous():
            raise ValueError("ladder_pm: the half residual must be contiguous")
        no, nv = self.w.no, self.w.nv
        V = self.w.H.ERI.blocks['vvvv']
        tabs = self._pm_tables(t1, t2, V)
        dev = self.w.device1
        G = {}
        for sign, c in (("+", 1.0), ("-", -1.0)):
            tb = tabs[sign]
            if tb["rows"] == 0 or tb["cols"] == 0:
                G[sign] = None
                continue
            vop = Operand('abef', (V, 'abef'), a=1.0, Y=(V, 'abfe'), b=c,
                          key=("ERI", "vvvv", sign))
            pa = self.tc._pack(vop, ['a', 'b'], ['e', 'f'], fmt, 'A', row_tab=tb["vrow"],
                               k_tab=tb["vk"], k_w=tb["kw"])
            top = Operand('ijef', (t2, 'ijef'), a=1.0, Y=(t2, 'ijfe'), b=c, P=(t1, 'ie'),
                          Q=(t1, 'jf'), c=1.0, R=(t1, 'if'), S=(t1, 'je'), d=c)
            pb = self.tc._pack(top, ['i', 'j'], ['e', 'f'], fmt, 'B', row_tab=tb["trow"],
                               k_tab=tb["tk"])
            out = torch.empty((tb["cols"], tb["rows"]), dtype=torch.float64, device=dev)
            self.tc.run_gemm('ijef,abef->ijab' + sign, fmt, pa, pb, out, ['p'], ['q'], 'qp',
                             0.5, 0.0)
            G[sign] = out
            if Wmnij is not None:
                hb = self._hole_pm_tables(t1, t2, Wmnij)[sign]
                if hb["k"] == 0:
                    continue
                hf = fmt if hole_fmt is None else hole_fmt
                uop = Operand('mnab', (t2, 'mnab'), a=1.0, Y=(t2, 'mnba'), b=c, P=(t1, 'ma'),
                              Q=(t1, 'nb'), c=1.0, R=(t1, 'mb'), S=(t1, 'na'), d=c)
                pu = self.tc._pack(uop, ['a', 'b'], ['m', 'n'], hf, 'A', row_tab=hb["urow"],
                                   k_tab=hb["uk"])
                wop = Operand('mnij', (Wmnij, 'mnij'), a=1.0, Y=(Wmnij, 'mnji'), b=c)
                pw = self.tc._pack(wop, ['i', 'j'], ['m', 'n'], hf, 'B', row_tab=hb["wrow"],
                                   k_tab=hb["wk"], k_w=hb["kw"])
                self.tc.run_gemm('mnab,mnij->ijab' + sign, hf, pu, pw, out, ['p'], ['q'], 'qp',
                                 0.5, 1.0)
        _lib.call("pcg_ladder_pm_assemble", G["+"].data_ptr(),
                  G["-"].data_ptr() if G["-"] is not None else None, no, nv, r.data_ptr(),
                  _lib.stream_handle(self.w.stream))

    def _kpair_tables(self, X):
        """K tables of the e <= f (+) / e < f (-) pairs of the last two indices of a static
        block X[..., e, f], for the sources X[..., e, f] and X[..., f, e], with 1/2 on e = f
        for + (X_ee + X_ee counts it twice)."""
        key = (tuple(X.stride()), tuple(X.shape))
        if key in self._kpm:
            return self._kpm[key]
        nv = X.shape[-1]
        se, sf = X.stride()[-2], X.stride()[-1]
        dev = self.w.device1
        tabs = {}
        for sign, k in (("+", 0), ("-", 1)):
            e, f = np.triu_indices(nv, k)
            kt = np.zeros((6, e.size), dtype=np.int64)
            kt[0] = e * se + f * sf
            kt[1] = f * se + e * sf
            kw = np.where(e == f, 0.5, 1.0).astype(np.float32) if sign == "+" else None
            tabs[sign] = {"k": torch.from_numpy(kt).to(dev),
                          "kw": torch.from_numpy(kw).to(dev) if kw is not None else None,
                          "n": e.size}
        self._kpm[key] = tabs
        return tabs

    def pair_tau(self, X, labels, name, t1, t2, out, fmt):
        """out[r, i, j] += sum_ef tau_ijef X[r.., e, f] for a static block X whose last two
        indices are (e, f) and whose leading ones (``labels[:-2]``) are the rows r, in the
        ladder's symmetric / antisymmetric pair form: G+- = 1/2 sum over the e <= f (e < f)
        pairs of T+-_ij,ef (X_ef +- X_fe), over the i <= j (i < j) pairs, then
        ``pcg_pair_pm_assemble`` adds out_rij += G+ + G-, out_rji += G+ - G- (i < j) and
        out_rii += G+.  T+- are the ladder's own packed operands (packed once per residual
        call); X's pair combinations are packed once per format.  Half the tensor-core work
        of the plain contraction (Zmbij: tau_ijef <mb|ef>, pycc/ccwfn.py:715; Wmnij:
        tau_ijef <mn|ef>, pycc/ccwfn.py:603)."""
        if not out.is_contiguous():
            raise ValueError("pair_tau: the output must be contiguous")
        no = self.w.no
        nrow = X[..., 0, 0].numel()
        ttabs = self._pm_tables(t1, t2, self.w.H.ERI.blocks['vvvv'])
        ktabs = self._kpair_tables(X)
        dev = self.w.device1
        swapped = labels[:-2] + labels[-1] + labels[-2]
        G = {}
        for sign, c in (("+", 1.0), ("-", -1.0)):
            tb, kb = ttabs[sign], ktabs[sign]
            if tb["cols"] == 0:
                G[sign] = None
                continue
            if kb["n"] == 0:
                G[sign] = torch.zeros((tb["cols"], nrow), dtype=torch.float64, device=dev)
                continue
            xop = Operand(labels, (X, labels), a=1.0, Y=(X, swapped), b=c,
                          key=("ERI", name, sign, "pairs"))
            pa = self.tc._pack(xop, list(labels[:-2]), list(labels[-2:]), fmt, 'A',
                               k_tab=kb["k"], k_w=kb["kw"])
            top = Operand('ijef', (t2, 'ijef'), a=1.0, Y=(t2, 'ijfe'), b=c, P=(t1, 'ie'),
                          Q=(t1, 'jf'), c=1.0, R=(t1, 'if'), S=(t1, 'je'), d=c)
            pb = self.tc._pack(top, ['i', 'j'], ['e', 'f'], fmt, 'B', row_tab=tb["trow"],
                               k_tab=tb["tk"])
            g = torch.empty((tb["cols"], nrow), dtype=torch.float64, device=dev)
            self.tc.run_gemm('ijef,%s->%sij%s' % (labels, labels[:-2], sign), fmt, pa, pb, g,
                             ['p'], ['q'], 'qp', 0.5, 0.0)
            G[sign] = g
        _lib.call("pcg_pair_pm_assemble", G["+"].data_ptr(),
                  G["-"].data_ptr() if G["-"] is not None else None, no, nrow, out.data_ptr(),
                  _lib.stream_handle(self.w.stream))

    def timed(self, name, fn, *args):
        """Run one term; with ``self.profile`` set, CUDA events on the launching stream
        around it (pack + GEMM + assembly) join the per-term table, and an NVTX range named
        ``name`` ("ladder": both ladders' GEMMs and their assembly) selects its launches for
        profilers."""
        torch.cuda.nvtx.range_push(name)
        if self.profile is None:
            fn(*args)
        else:
            st = torch.cuda.current_stream() if self.w.stream is None else self.w.stream
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn(*args)
            e1.record(st)
            self.profile.append((name, self.fmt(), e0, e1))
        torch.cuda.nvtx.range_pop()

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
        W = self.w.H.ERI[o, o, o, o].clone(memory_format=torch.contiguous_format)
        self.tcc('je,mnie->mnij', Operand.of('je', t1), self.eri('ooov', 'mnie'), W)
        self.tcc('ie,mnej->mnij', Operand.of('ie', t1), self.eri('oovo', 'mnej'), W)
        # tau_ijef <mn|ef> in pair form
        self.pair_tau(self.w.H.ERI.blocks['oovv'], 'mnef', 'oovv', t1, t2, W, self.fmt())
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
        # tau_ijef <mb|ef> in pair form
        self.pair_tau(self.w.H.ERI.blocks['ovvv'], 'mbef', 'ovvv', t1, t2, Z, self.fmt())
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
        # (2 t2_mief - t2_mife) <ma|ef> summed over e, f is t2_mief (2 <ma|ef> - <ma|fe>)
        # = t2_mief L_maef (pycc/ccwfn.py:759): the resident L block takes the combination,
        # and t2 is gathered once instead of twice (once transposed)
        self.tcc('mief,maef->ia', Operand.of('mief', t2), self.ll('ovvv', 'maef'), r)
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
        self.timed("ladder", self.ladder_pm, t1, t2, r, self.ladder_fmt(), Wmnij, self.fmt())
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
