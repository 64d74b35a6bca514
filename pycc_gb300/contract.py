"""GPU drop-in for the reference's contraction backend.

``ContractionBackend.__call__(subscripts, *operands)`` keeps the einsum-string interface of
``pycc/device.py:64-87`` (the ``self.contract`` every CCSD builder calls), but executes each
pairwise contraction as ONE launch of the FP64 strided DMMA kernel in the CUDA library:
operand and output permutations become element strides, nothing is transposed or copied
and nothing crosses PCIe/C2C (the reference copies CPU-resident integrals per call,
``pycc/device.py:71-74``).

Two keyword-only extensions make the builders allocation-free: ``out=`` accumulates into an
existing tensor and ``alpha``/``beta`` give ``out = beta*out + alpha*contract(...)``.
"""
from __future__ import annotations

import torch

from . import _lib

MAX_SUB = 4


def _merge(groups):
    """Merge consecutive sub-indices that are contiguous in both tensors (outer -> inner)."""
    groups = [g for g in groups if g[0] != 1]
    out = []
    for e, s0, s1 in groups:
        if out:
            pe, p0, p1 = out[-1]
            if p0 == e * s0 and p1 == e * s1:
                out[-1] = (pe * e, s0, s1)
                continue
        out.append((e, s0, s1))
    return out


def _parse(subscripts):
    s = subscripts.replace(" ", "")
    if "->" not in s:
        raise ValueError("contract: explicit output ('->') required, got %r" % subscripts)
    lhs, rhs = s.split("->")
    ins = lhs.split(",")
    return ins, rhs


class ContractPlan:
    """Sub-index groups of one pairwise contraction for given operand strides."""

    def __init__(self, subscripts, a, b, out_shape=None):
        ins, rhs = _parse(subscripts)
        if len(ins) != 2:
            raise ValueError("contract: exactly two operands supported, got %d" % len(ins))
        sa, sb = ins
        for sub, t in ((sa, a), (sb, b)):
            if len(sub) != t.dim():
                raise ValueError("contract: %r does not match operand of rank %d" % (sub, t.dim()))
            if len(set(sub)) != len(sub):
                raise ValueError("contract: repeated index within an operand (%r)" % sub)
        if len(set(rhs)) != len(rhs):
            raise ValueError("contract: repeated output index (%r)" % rhs)
        ext = {}
        for sub, t in ((sa, a), (sb, b)):
            for c, n in zip(sub, t.shape):
                if ext.setdefault(c, n) != n:
                    raise ValueError("contract: index %r has extents %d and %d" % (c, ext[c], n))
        for c in rhs:
            if c not in ext:
                raise ValueError("contract: output index %r absent from the operands" % c)
        for c in set(sa) | set(sb):
            if c not in rhs and not (c in sa and c in sb):
                raise ValueError("contract: index %r summed over a single operand" % c)
        self.sa, self.sb, self.rhs = sa, sb, rhs
        self.shape = tuple(ext[c] for c in rhs)
        self.ext = ext

    def groups(self, a, b, out):
        sa, sb, rhs, ext = self.sa, self.sb, self.rhs, self.ext
        ast = dict(zip(sa, a.stride()))
        bst = dict(zip(sb, b.stride()))
        cst = dict(zip(rhs, out.stride()))
        M, N, batch = [], [], []
        for c in rhs:
            ia, ib = c in ast, c in bst
            if ia and ib:
                batch.append(c)
            elif ia:
                M.append((ext[c], ast[c], cst[c]))
            else:
                N.append((ext[c], bst[c], cst[c]))
        K = [(ext[c], ast[c], bst[c]) for c in sa if c in bst and c not in cst]
        K.sort(key=lambda g: (-g[1], -g[2]))
        M, N, K = _merge(M), _merge(N), _merge(K)
        if max(len(M), len(N), len(K)) > MAX_SUB:
            raise ValueError("contract: more than %d sub-indices after merging" % MAX_SUB)
        return M, N, K, batch, ast, bst, cst


def _check(t, name):
    if not isinstance(t, torch.Tensor):
        raise TypeError("contract: %s must be a torch.Tensor" % name)
    if not t.is_cuda:
        raise ValueError("contract: %s must be resident on the GPU (no host copies)" % name)
    if t.dtype != torch.float64:
        raise TypeError("contract: %s must be float64, got %s" % (name, t.dtype))


def contract_f64(subscripts, a, b, out=None, alpha=1.0, beta=0.0, stream=None):
    """``out = beta*out + alpha * einsum(subscripts, a, b)`` on the FP64 DMMA kernel."""
    _check(a, "operand 0")
    _check(b, "operand 1")
    plan = ContractPlan(subscripts, a, b)
    if out is None:
        out = torch.empty(plan.shape, dtype=torch.float64, device=a.device)
        beta = 0.0
    else:
        _check(out, "out")
        if tuple(out.shape) != plan.shape:
            raise ValueError("contract: out has shape %s, expected %s" % (tuple(out.shape), plan.shape))
    M, N, K, batch, ast, bst, cst = plan.groups(a, b, out)
    st = _lib.stream_handle(stream)
    if not batch:
        _launch(M, N, K, alpha, a.data_ptr(), b.data_ptr(), beta, out.data_ptr(), st)
        return out
    # batch indices (present in both operands and the output): one launch per value
    import itertools
    rngs = [range(plan.ext[c]) for c in batch]
    for vals in itertools.product(*rngs):
        oa = sum(v * ast[c] for v, c in zip(vals, batch)) * 8
        ob = sum(v * bst[c] for v, c in zip(vals, batch)) * 8
        oc = sum(v * cst[c] for v, c in zip(vals, batch)) * 8
        _launch(M, N, K, alpha, a.data_ptr() + oa, b.data_ptr() + ob, beta,
                out.data_ptr() + oc, st)
    return out


def _launch(M, N, K, alpha, pa, pb, beta, pc, st):
    i64 = _lib.i64s
    _lib.call("pcg_contract_f64",
              len(M), i64([g[0] for g in M]), i64([g[1] for g in M]), i64([g[2] for g in M]),
              len(N), i64([g[0] for g in N]), i64([g[1] for g in N]), i64([g[2] for g in N]),
              len(K), i64([g[0] for g in K]), i64([g[1] for g in K]), i64([g[2] for g in K]),
              float(alpha), pa, pb, float(beta), pc, st)


class ContractionBackend:
    """``self.contract`` of the GPU CCSD engine (mirrors ``pycc/device.py:38-87``)."""

    def __init__(self, device1=None, stream=None):
        self.device = "GPU"
        self.device1 = device1 if device1 is not None else torch.device("cuda:0")
        self.stream = stream

    def __call__(self, subscripts, *operands, out=None, alpha=1.0, beta=0.0):
        if len(operands) != 2:
            raise ValueError("contract: the GPU engine contracts operand pairs (got %d)" % len(operands))
        return contract_f64(subscripts, operands[0], operands[1], out=out, alpha=alpha,
                            beta=beta, stream=self.stream)
