"""Host side of the tcgen05 tensor-core contraction engine (``pcg_pack_operand`` + ``pcg_tc_gemm``).

A contraction ``out = beta*out + alpha * einsum('A,B->C', opA, opB)`` is executed as

1. pack: each operand is gathered from its FP64 source(s) into a K-major row matrix
   ``[rows][Kp]`` in the GEMM's input format (BF16, BF16 hi+lo pair, or FP8 E4M3 with a
   per-row scale).  An operand may be a combination ``a*X + b*Y + c*P*Q + d*R*S`` of strided
   FP64 tensors (e.g. ``2 t2 - t2.swapaxes(2,3)``, ``t2 + t1 (x) t1``, or tau_ijef + tau_ijfe),
   so the combinations, index permutations and the conversion happen in one pass; rows and
   K may also be selected by explicit offset tables (index pairs such as i <= j);
2. GEMM: 128 x BN tiles on tcgen05 with TMEM accumulators; the epilogue writes FP64 with
   the output permutation expressed as per-row / per-column offsets.

Packed operands of static tensors (the integral blocks) are cached by the caller.
"""
from __future__ import annotations

import math

import torch

from . import _lib

FMT_BF16, FMT_BF16X3, FMT_FP8, FMT_BF16X6, FMT_BF16X3F, FMT_BF16X3S = 0, 1, 2, 3, 4, 5


def pack_format(fmt):
    """The operand pieces a GEMM format reads (the split-BF16x3 GEMMs, fused, fused with
    separate accumulators or by passes, share them)."""
    return FMT_BF16X3 if fmt in (FMT_BF16X3F, FMT_BF16X3S) else fmt


def static_pack_format(fmt):
    """The pieces cached for a static operand (an integral block).  A BF16 GEMM keeps the
    split-BF16x3 pair: its hi piece is the BF16 operand bit for bit (the same rounding of
    the same FP32 value), and the split-BF16x3 stages then reuse the cached pack instead of
    packing every integral block again."""
    f = pack_format(fmt)
    return FMT_BF16X3 if f == FMT_BF16 else f


MAX_SUB = 4


class Operand:
    """``a*X + b*Y + c*P*Q + d*R*S`` over the index labels ``labels``.

    Each component is ``(tensor, labels)``; labels of the operand a component lacks are
    broadcast (stride 0).
    """

    def __init__(self, labels, X, a=1.0, Y=None, b=0.0, P=None, Q=None, c=0.0, R=None, S=None,
                 d=0.0, key=None):
        self.labels = labels
        self.a, self.b, self.c, self.d = a, b, c, d
        self.X, self.Y, self.P, self.Q, self.R, self.S = X, Y, P, Q, R, S
        self.key = key            # cache key for static operands (None = dynamic)

    @staticmethod
    def of(labels, t, key=None):
        return Operand(labels, (t, labels), key=key)

    def sources(self):
        return [self.X, self.Y, self.P, self.Q, self.R, self.S]

    def extents(self):
        ext = {}
        for s in self.sources():
            if s is None:
                continue
            t, lab = s
            for c, n in zip(lab, t.shape):
                if ext.setdefault(c, n) != n:
                    raise ValueError("operand index %r has extents %d and %d" % (c, ext[c], n))
        return ext

    def strides(self, label):
        out = []
        for s in self.sources():
            if s is None:
                out.append(0)
                continue
            t, lab = s
            out.append(t.stride(lab.index(label)) if label in lab else 0)
        return out

    def device(self):
        return next(s for s in self.sources() if s is not None)[0].device


def _merge_multi(groups):
    """Merge consecutive (ext, [strides...]) groups contiguous in every stride set."""
    groups = [g for g in groups if g[0] != 1]
    out = []
    for e, s in groups:
        if out:
            pe, ps = out[-1]
            if all(p == e * q for p, q in zip(ps, s)):
                out[-1] = (pe * e, list(s))
                continue
        out.append((e, list(s)))
    return out


def _ptr(s):
    return s[0].data_ptr() if s is not None else None


class Packed:
    """A packed K-major operand: ``hi`` (and ``lo`` / ``scale``) of shape [rows, Kp]."""

    def __init__(self, fmt, rows, Kp, hi, lo=None, scale=None, mid=None):
        self.fmt, self.rows, self.Kp = fmt, rows, Kp
        self.hi, self.lo, self.scale, self.mid = hi, lo, scale, mid

    def nbytes(self):
        return sum(t.numel() * t.element_size() for t in (self.hi, self.mid, self.lo, self.scale)
                   if t is not None)


def kblock(fmt):
    return 128 if fmt == FMT_FP8 else 64


NSRC = 6   # sources of a packed operand: X, Y, P, Q, R, S


def pack(op: Operand, row_labels, k_labels, fmt, stream=None, row_tab=None, k_tab=None,
         k_w=None) -> Packed:
    """Pack ``op`` with rows over ``row_labels`` (or the explicit per-source row offsets
    ``row_tab``, an int64 [6, R] device tensor) and K over ``k_labels`` (or the per-source K
    offsets ``k_tab``, int64 [6, K], with optional float32 K multipliers ``k_w``).  With a
    table the labels' strides still tell the kernel which side is unit-stride."""
    fmt = pack_format(fmt)
    ext = op.extents()
    rows = [(ext[c], op.strides(c)) for c in row_labels]
    ks = [(ext[c], op.strides(c)) for c in k_labels]
    R = math.prod(ext[c] for c in row_labels) if row_tab is None else int(row_tab.shape[1])
    K = math.prod(ext[c] for c in k_labels) if k_tab is None else int(k_tab.shape[1])
    rows, ks = _merge_multi(rows), _merge_multi(ks)
    if len(rows) > MAX_SUB or len(ks) > MAX_SUB:
        raise ValueError("pack: more than %d sub-indices" % MAX_SUB)
    for tab in (row_tab, k_tab):
        if tab is not None and (tab.dtype != torch.int64 or tab.shape[0] != NSRC
                                or not tab.is_contiguous()):
            raise ValueError("pack: offset tables are contiguous int64 [%d, n] tensors" % NSRC)
    if k_w is not None and (k_tab is None or k_w.dtype != torch.float32
                            or k_w.numel() != K or not k_w.is_contiguous()):
        raise ValueError("pack: K multipliers need a K table and K float32 entries")
    kb = kblock(fmt)
    Kp = ((K + kb - 1) // kb) * kb
    dev = op.device()
    mid = None
    if fmt == FMT_FP8:
        hi = torch.empty((R, Kp), dtype=torch.uint8, device=dev)
        lo = None
        scale = torch.empty(R, dtype=torch.float32, device=dev)
    else:
        hi = torch.empty((R, Kp), dtype=torch.bfloat16, device=dev)
        lo = torch.empty_like(hi) if fmt in (FMT_BF16X3, FMT_BF16X6) else None
        mid = torch.empty_like(hi) if fmt == FMT_BF16X6 else None
        scale = None

    def flat(groups):
        e = [g[0] for g in groups]
        st = [0] * (NSRC * MAX_SUB)
        for q, (_, s) in enumerate(groups):
            for src in range(NSRC):
                st[src * MAX_SUB + q] = s[src]
        return len(groups), _lib.i64s(e), _lib.i64s(st)

    def ptr(t):
        return t.data_ptr() if t is not None else None

    rn, re_, rs = flat(rows)
    kn, ke, kst = flat(ks)
    _lib.call("pcg_pack_operand", int(fmt), rn, re_, rs, kn, ke, kst, Kp,
              float(op.a), _ptr(op.X), float(op.b), _ptr(op.Y), float(op.c), _ptr(op.P),
              _ptr(op.Q), float(op.d), _ptr(op.R), _ptr(op.S), hi.data_ptr(), ptr(mid), ptr(lo),
              ptr(scale), ptr(row_tab), R if row_tab is not None else 0, ptr(k_tab), ptr(k_w),
              K if k_tab is not None else 0, _lib.stream_handle(stream))
    return Packed(fmt, R, Kp, hi, lo, scale, mid)


def gemm(fmt, A: Packed, B: Packed, out, row_labels, col_labels, out_labels, alpha=1.0,
         beta=1.0, status=None, stream=None, col_map=None, col_scale=None):
    """out = beta*out + alpha * A . B^T with rows/cols mapped to ``out`` through labels
    (or, for the columns, the explicit offsets ``col_map`` and multipliers ``col_scale``)."""
    if A.Kp != B.Kp:
        raise ValueError("gemm: K mismatch %d vs %d" % (A.Kp, B.Kp))
    ost = dict(zip(out_labels, out.stride()))
    oext = dict(zip(out_labels, out.shape))
    mg = _merge_multi([(oext[c], [ost[c]]) for c in row_labels])
    ng = _merge_multi([(oext[c], [ost[c]]) for c in col_labels]) if col_map is None else []
    if len(mg) > MAX_SUB or len(ng) > MAX_SUB:
        raise ValueError("gemm: more than %d output sub-indices" % MAX_SUB)
    i64 = _lib.i64s
    def p(t):
        return t.data_ptr() if t is not None else None
    _lib.call("pcg_tc_gemm", int(fmt), p(A.hi), p(A.mid), p(A.lo), A.rows, A.Kp,
              p(B.hi), p(B.mid), p(B.lo), B.rows, B.Kp, A.Kp,
              A.scale.data_ptr() if A.scale is not None else None,
              B.scale.data_ptr() if B.scale is not None else None,
              len(mg), i64([g[0] for g in mg]), i64([g[1][0] for g in mg]),
              len(ng), i64([g[0] for g in ng]), i64([g[1][0] for g in ng]),
              col_map.data_ptr() if col_map is not None else None,
              col_scale.data_ptr() if col_scale is not None else None,
              float(alpha), float(beta), out.data_ptr(), status.data_ptr(),
              _lib.stream_handle(stream))


class TCEngine:
    """Plans and runs einsum-style contractions on the tensor-core engine."""

    def __init__(self, device, stream=None):
        self.device = device
        self.stream = stream
        self.status = torch.zeros(4, dtype=torch.int32, device=device)
        self.cache = {}
        self.timing = None        # list of GEMM launch records (CUDA events) when set
        self.dyn_cache = None     # per-residual cache of packed dynamic operands

    def contract(self, subscripts, A: Operand, B: Operand, out, alpha=1.0, beta=1.0, fmt=FMT_BF16):
        lhs, rhs = subscripts.replace(" ", "").split("->")
        la, lb = lhs.split(",")
        if la != A.labels or lb != B.labels:
            raise ValueError("contract: operand labels %s,%s do not match %s" % (A.labels, B.labels, lhs))
        ost = dict(zip(rhs, out.stride()))
        ea, eb = A.extents(), B.extents()
        ma = [c for c in rhs if c in la and c not in lb]
        nb = [c for c in rhs if c in lb and c not in la]
        kk = [c for c in la if c in lb and c not in rhs]
        if len(ma) + len(nb) != len(rhs):
            raise ValueError("contract: batch indices are not supported (%s)" % subscripts)
        # rows / cols in output-stride order (innermost last); K by the dynamic operand
        ma.sort(key=lambda c: -ost[c])
        nb.sort(key=lambda c: -ost[c])
        dyn = A if A.key is None else B
        dst = {c: max(abs(s) for s in dyn.strides(c)) for c in kk}
        kk.sort(key=lambda c: -dst[c])
        mA = math.prod(ea[c] for c in ma) if ma else 1
        nB = math.prod(eb[c] for c in nb) if nb else 1
        # The 128-row tile side: the side holding the output's unit-stride index (so a warp's
        # 32 consecutive rows store to consecutive addresses), unless it is too short.
        inner = min(rhs, key=lambda c: abs(ost[c]))
        if inner in nb and nB >= 128:
            swap = True
        elif inner in ma and mA >= 128:
            swap = False
        else:
            swap = nB > mA
        if swap:
            A, B, ma, nb = B, A, nb, ma
        pa = self._pack(A, ma, kk, fmt, "A")
        pb = self._pack(B, nb, kk, fmt, "B")
        self.run_gemm(subscripts, fmt, pa, pb, out, ma, nb, rhs, alpha, beta)
        return out

    def run_gemm(self, subscripts, fmt, pa, pb, out, rows, cols, rhs, alpha, beta,
                 col_map=None, col_scale=None):
        """One tensor-core GEMM launch, timed with CUDA events when ``self.timing`` is set."""
        ev = None
        if self.timing is not None:
            st = torch.cuda.current_stream() if self.stream is None else self.stream
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record(st)
        gemm(fmt, pa, pb, out, rows, cols, rhs, alpha=alpha, beta=beta, status=self.status,
             stream=self.stream, col_map=col_map, col_scale=col_scale)
        if ev is not None:
            ev[1].record(st)
            self.timing.append({"subs": subscripts, "fmt": fmt, "M": pa.rows, "N": pb.rows,
                                "Kp": pa.Kp, "start": ev[0], "end": ev[1]})

    def _pack(self, op, rows, ks, fmt, side, row_tab=None, k_tab=None, k_w=None):
        tabs = tuple(t.data_ptr() if t is not None else None for t in (row_tab, k_tab, k_w))
        if op.key is None:
            if self.dyn_cache is None:
                return pack(op, rows, ks, fmt, self.stream, row_tab, k_tab, k_w)
            # the key is the gather itself: each source's address, and the extent and
            # per-source strides of every row and K index, so one matrix reached through
            # differently named labels is packed once
            ext = op.extents()
            src = tuple(s[0].data_ptr() if s is not None else None for s in op.sources())
            geo = tuple((ext[c], tuple(op.strides(c))) for c in rows)
            kgeo = tuple((ext[c], tuple(op.strides(c))) for c in ks)
            dkey = (src, op.a, op.b, op.c, op.d, geo, kgeo, tabs, pack_format(fmt))
            hit = self.dyn_cache.get(dkey)
            if hit is None:
                # the entry holds its source tensors and tables, so no later tensor can reuse
                # their addresses while the cache lives
                hit = (pack(op, rows, ks, fmt, self.stream, row_tab, k_tab, k_w),
                       [s[0] for s in op.sources() if s is not None] + [row_tab, k_tab, k_w])
                self.dyn_cache[dkey] = hit
            return hit[0]
        # the operand's own label string fixes which tensor axis each label names; the key
        # (op.key) names the static tensor and any tables that select from it
        sf = static_pack_format(fmt)
        key = (op.key, op.labels, tuple(rows), tuple(ks), sf)
        p = self.cache.get(key)
        if p is None:
            p = pack(op, rows, ks, sf, self.stream, row_tab, k_tab, k_w)
            self.cache[key] = p
        return p

    STATUS_TEXT = {1: "a stage's TMA data never arrived", 2: "a stage or accumulator was "
                   "never released", 3: "an accumulator was never completed",
                   4: "the self-test's wait expired"}

    def check_status(self, values=None):
        """Raise EngineError when a kernel recorded an expired device-side wait.  ``values``:
        the status words already read to the host (read here otherwise)."""
        s = [int(x) for x in (self.status.cpu().tolist() if values is None else values)]
        if any(s):
            what = "; ".join(sorted({self.STATUS_TEXT.get(abs(x), "code %d" % x)
                                     for x in s if x}))
            raise _lib.EngineError("tensor-core kernel reported an expired wait (%s; status %s)"
                                   % (what, s))
