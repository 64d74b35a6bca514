"""(T) correction on the GPU (the reference's ``t_tjl``, ``pycc/cctriples.py:177-240``).

For every triple i >= j >= k the connected triples W[a,b,c] (``t3c_ijk``, :27-72) are
built as three partial tensors, one per output orientation of the twelve t3 terms:

* orientation 1, P1[a,b,c]: t2_kj <ba|ei>, t2_ki <ab|ej>, -t2_imab <mc|jk>, -t2_jmba <mc|ik>
* orientation 2, P2[a,c,b]: t2_jk <ca|ei>, t2_ji <ac|ek>, -t2_imac <mb|kj>, -t2_kmca <mb|ij>
* orientation 3, P3[b,c,a]: t2_ij <bc|ek>, t2_ik <cb|ej>, -t2_kmcb <ma|ji>, -t2_jmbc <ma|ki>

so each partial is written once by one multi-term contraction.  A partial is stored with its
last (column) index slowest, P[z][x][y] for the logical P[x,y,z], the layout in which the
tensor-core GEMM writes it with coalesced stores.  The energy kernel
(``csrc/triples.cu``) adds the partials, the disconnected triples (``t3d_ijk``) and the
Lee-Rendell weights, and accumulates E(T) in FP64.

``precision='DP'`` uses the FP64 DMMA multi-term contraction; the mixed path
(``t_energy_tc``) builds the partials for batches of triples with the grouped tcgen05 GEMM.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

MAX_SUB = 4


def orientation_terms(i, j, k, t2, V, O):
    """The four terms of each orientation: (alpha, A, A labels, B, B labels).

    V = <pq|ex> (the vvvo block), O = <mp|xy> (the ovoo block).
    """
    return [
        ("abc", [(1.0, V[:, :, :, i], "bae", t2[k, j], "ce"),
                 (1.0, V[:, :, :, j], "abe", t2[k, i], "ce"),
                 (-1.0, t2[i], "mab", O[:, :, j, k], "mc"),
                 (-1.0, t2[j], "mba", O[:, :, i, k], "mc")]),
        ("acb", [(1.0, V[:, :, :, i], "cae", t2[j, k], "be"),
                 (1.0, V[:, :, :, k], "ace", t2[j, i], "be"),
                 (-1.0, t2[i], "mac", O[:, :, k, j], "mb"),
                 (-1.0, t2[k], "mca", O[:, :, i, j], "mb")]),
        ("bca", [(1.0, V[:, :, :, k], "bce", t2[i, j], "ae"),
                 (1.0, V[:, :, :, j], "cbe", t2[i, k], "ae"),
                 (-1.0, t2[k], "mcb", O[:, :, j, i], "ma"),
                 (-1.0, t2[j], "mbc", O[:, :, k, i], "ma")]),
    ]


def contract_multi(out, out_labels, terms, beta=0.0, stream=None):
    """out = beta*out + sum_t alpha_t einsum(A_t, B_t) on the FP64 multi-term kernel."""
    nt = len(terms)
    if not 1 <= nt <= 4:
        raise ValueError("contract_multi: 1..4 terms")
    ost = dict(zip(out_labels, out.stride()))
    oext = dict(zip(out_labels, out.shape))
    alab0, blab0 = terms[0][2], terms[0][4]
    Ml = [c for c in out_labels if c in alab0]
    Nl = [c for c in out_labels if c in blab0]
    m_sa, n_sb, k_n, k_ext, k_sa, k_sb, alphas, As, Bs = [], [], [], [], [], [], [], [], []
    for alpha, A, alab, B, blab in terms:
        if [c for c in out_labels if c in alab] != Ml or [c for c in out_labels if c in blab] != Nl:
            raise ValueError("contract_multi: terms disagree on the output index split")
        ast = dict(zip(alab, A.stride()))
        bst = dict(zip(blab, B.stride()))
        aex = dict(zip(alab, A.shape))
        m_sa += [ast[c] for c in Ml] + [0] * (MAX_SUB - len(Ml))
        n_sb += [bst[c] for c in Nl] + [0] * (MAX_SUB - len(Nl))
        kl = [c for c in alab if c in blab and c not in out_labels]
        kl.sort(key=lambda c: -ast[c])
        k_n.append(len(kl))
        k_ext += [aex[c] for c in kl] + [1] * (MAX_SUB - len(kl))
        k_sa += [ast[c] for c in kl] + [0] * (MAX_SUB - len(kl))
        k_sb += [bst[c] for c in kl] + [0] * (MAX_SUB - len(kl))
        alphas.append(float(alpha))
        As.append(A.data_ptr())
        Bs.append(B.data_ptr())
    i64 = _lib.i64s
    _lib.call("pcg_contract_multi_f64", nt, len(Ml), i64([oext[c] for c in Ml]),
              i64([ost[c] for c in Ml]), i64(m_sa), len(Nl), i64([oext[c] for c in Nl]),
              i64([ost[c] for c in Nl]), i64(n_sb), (C.c_int * nt)(*k_n), i64(k_ext), i64(k_sa),
              i64(k_sb), (C.c_double * nt)(*alphas), (C.c_void_p * nt)(*As),
              (C.c_void_p * nt)(*Bs), float(beta), out.data_ptr(), _lib.stream_handle(stream))
    return out


def triples_list(no):
    return [(i, j, k) for i in range(no) for j in range(i + 1) for k in range(j + 1)]


def _energy(fp32, P1, P2, P3, pstride, ijk_dev, ntrip, w, t1, t2, part, stream):
    H = w.H
    o, v = w.o, w.v
    fov = H.F[o, v].contiguous()
    fov_ptr = fov.data_ptr() if bool(fov.abs().max() > 0) else None
    _lib.call("pcg_triples_energy", int(fp32), P1.data_ptr(), P2.data_ptr(), P3.data_ptr(),
              int(pstride), ijk_dev.data_ptr(), int(ntrip), H.eps.data_ptr(),
              H.ERI[o, o, v, v].data_ptr(), t1.data_ptr(), t2.data_ptr(), fov_ptr, w.no, w.nv,
              part.data_ptr(), _lib.stream_handle(stream))


def t_energy_fp64(w, t1=None, t2=None):
    """E(T) with FP64 partials (DMMA) and FP64 energy arithmetic."""
    t1 = (w.t1 if t1 is None else t1).contiguous()
    t2 = (w.t2 if t2 is None else t2).contiguous()
    no, nv = w.no, w.nv
    o, v = w.o, w.v
    V = w.H.ERI[v, v, v, o]
    O = w.H.ERI[o, v, o, o]
    dev = t2.device
    P = torch.empty((3, nv, nv, nv), dtype=torch.float64, device=dev)
    trips = triples_list(no)
    part = torch.empty((len(trips), nv), dtype=torch.float64, device=dev)
    ijk = torch.tensor(trips, dtype=torch.int32, device=dev)
    for t, (i, j, k) in enumerate(trips):
        for q, (lab, terms) in enumerate(orientation_terms(i, j, k, t2, V, O)):
            contract_multi(P[q].permute(1, 2, 0), lab, terms, stream=w.stream)
        _energy(False, P[0], P[1], P[2], 0, ijk[t:t + 1], 1, w, t1, t2, part[t:t + 1], w.stream)
    out = torch.zeros((), dtype=torch.float64, device=dev)
    _lib.call("pcg_reduce_sum_f64", part.data_ptr(), part.numel(), out.data_ptr(),
              _lib.stream_handle(w.stream))
    return float(out)


def t_energy(w, t1=None, t2=None):
    """E(T) for the converged amplitudes of ``w`` in ``w``'s precision."""
    if w.precision == 'DP':
        return t_energy_fp64(w, t1, t2)
    from .triples_tc import t_energy_tc
    return t_energy_tc(w, t1, t2)


def t_tjl(ccwfn):
    """The reference's entry point ``t_tjl(ccwfn) -> float`` (``pycc/cctriples.py:177-240``):
    E(T) at ``ccwfn``'s amplitudes, in its precision (``t_energy``)."""
    return t_energy(ccwfn)


def t_vikings(ccwfn):
    """``t_vikings(ccwfn) -> float`` (``pycc/cctriples.py:243-308``): the reference's
    full-(i,j,k) formulation of the same E(T); the engine evaluates it over i >= j >= k with
    the Lee-Rendell weights, which gives the same value (``t_energy``)."""
    return t_energy(ccwfn)
