"""CPU oracle for the (T) correction -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's closed-shell (T) drivers (CrawfordGroup/pycc,
``pycc/cctriples.py``): the connected and disconnected triples for fixed (i, j, k)
(``t3c_ijk`` :27-72, ``t3d_ijk`` :108-147) and the Lee-Rendell energy over i >= j >= k and
a >= b >= c (``t_tjl`` :177-240), with the per-element Python loops of the reference
replaced by whole-array numpy expressions over (a, b, c).  ``t_vikings`` (:243-308) is the
full-(i, j, k) formulation, used to cross-check.  Pinned against the reference's own
energies in ``tests/golden/o5v19.npz``.
"""
from __future__ import annotations

import numpy as np


def t3c_ijk(o, v, i, j, k, t2, Vvvvo, Vovoo, F, with_denom=True):
    """Connected triples W3[a,b,c] for fixed i,j,k (cctriples.py:56-72)."""
    e = np.einsum
    t3 = e('bae,ce->abc', Vvvvo[:, :, :, i], t2[k, j])
    t3 += e('cae,be->abc', Vvvvo[:, :, :, i], t2[j, k])
    t3 += e('ace,be->abc', Vvvvo[:, :, :, k], t2[j, i])
    t3 += e('bce,ae->abc', Vvvvo[:, :, :, k], t2[i, j])
    t3 += e('cbe,ae->abc', Vvvvo[:, :, :, j], t2[i, k])
    t3 += e('abe,ce->abc', Vvvvo[:, :, :, j], t2[k, i])
    t3 -= e('mc,mab->abc', Vovoo[:, :, j, k], t2[i])
    t3 -= e('mb,mac->abc', Vovoo[:, :, k, j], t2[i])
    t3 -= e('mb,mca->abc', Vovoo[:, :, i, j], t2[k])
    t3 -= e('ma,mcb->abc', Vovoo[:, :, j, i], t2[k])
    t3 -= e('ma,mbc->abc', Vovoo[:, :, k, i], t2[j])
    t3 -= e('mc,mba->abc', Vovoo[:, :, i, k], t2[j])
    if with_denom:
        t3 = t3 / denom_ijk(o, v, i, j, k, F)
    return t3


def t3d_ijk(o, v, i, j, k, t1, t2, Voovv, F):
    """Disconnected triples for fixed i,j,k without denominator (cctriples.py:133-140)."""
    Fov = F[o, v]
    e = np.einsum
    t3 = e('ab,c->abc', Voovv[i, j], t1[k])
    t3 += e('ac,b->abc', Voovv[i, k], t1[j])
    t3 += e('bc,a->abc', Voovv[j, k], t1[i])
    t3 += e('ab,c->abc', t2[i, j], Fov[k])
    t3 += e('ac,b->abc', t2[i, k], Fov[j])
    t3 += e('bc,a->abc', t2[j, k], Fov[i])
    return t3


def denom_ijk(o, v, i, j, k, F):
    fo = np.diag(F)[o]
    fv = np.diag(F)[v]
    return fo[i] + fo[j] + fo[k] - fv.reshape(-1, 1, 1) - fv.reshape(-1, 1) - fv


def ijk_energy(o, v, i, j, k, W, t1, t2, Voovv, F):
    """The Lee-Rendell contribution of one triple i >= j >= k (cctriples.py:207-238) from its
    connected triples W[a,b,c] without denominator: V = (W + t3d) / (1 + d_ab + d_ac + d_bc),
    the X / Y / Z symmetry intermediates, and the a >= b >= c sum with weight
    2 - d_ij - d_ik - d_jk."""
    nv = W.shape[0]
    a = np.arange(nv)
    w = 1.0 + (a[:, None, None] == a[None, :, None]) + (a[:, None, None] == a[None, None, :]) \
        + (a[None, :, None] == a[None, None, :])
    tri = (a[:, None, None] >= a[None, :, None]) & (a[None, :, None] >= a[None, None, :])
    V = (t3d_ijk(o, v, i, j, k, t1, t2, Voovv, F) + W) / w
    tr = lambda X, p: X.transpose(p)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    X = sum(tr(W, p) * tr(V, p) for p in perms)
    Y = V + tr(V, (1, 2, 0)) + tr(V, (2, 0, 1))
    Z = tr(V, (0, 2, 1)) + tr(V, (1, 0, 2)) + tr(V, (2, 1, 0))
    Wc = W + tr(W, (1, 2, 0)) + tr(W, (2, 0, 1))
    Wa = tr(W, (0, 2, 1)) + tr(W, (1, 0, 2)) + tr(W, (2, 1, 0))
    S = (Y - 2 * Z) * Wc + (Z - 2 * Y) * Wa + 3 * X
    fac = 2.0 - ((i == j) + (i == k) + (j == k))
    return fac * np.sum((S / denom_ijk(o, v, i, j, k, F))[tri])


def t_tjl(no, nv, F, ERI, t1, t2):
    """Lee-Rendell E(T) (cctriples.py:177-240), vectorised over a, b, c."""
    n = no + nv
    o, v = slice(0, no), slice(no, n)
    Vvvvo, Vovoo, Voovv = ERI[v, v, v, o], ERI[o, v, o, o], ERI[o, o, v, v]
    ET = 0.0
    for i in range(no):
        for j in range(i + 1):
            for k in range(j + 1):
                W = t3c_ijk(o, v, i, j, k, t2, Vvvvo, Vovoo, F, with_denom=False)
                ET += ijk_energy(o, v, i, j, k, W, t1, t2, Voovv, F)
    return ET


def t_vikings(no, nv, F, ERI, L, t1, t2):
    """Vikings E(T) (cctriples.py:243-308): full i,j,k loops, X1/X2 intermediates."""
    n = no + nv
    o, v = slice(0, no), slice(no, n)
    Vvvvo, Vovoo = ERI[v, v, v, o], ERI[o, v, o, o]
    Loovv, Vvovv, Vooov, Fov = L[o, o, v, v], ERI[v, o, v, v], ERI[o, o, o, v], F[o, v]
    X1 = np.zeros_like(t1)
    X2 = np.zeros_like(t2)
    e = np.einsum
    for i in range(no):
        for j in range(no):
            for k in range(no):
                t3 = t3c_ijk(o, v, i, j, k, t2, Vvvvo, Vovoo, F)
                X1[i] += e('abc,bc->a', t3 - t3.swapaxes(0, 2), Loovv[j, k])
                s = 2.0 * t3 - t3.swapaxes(1, 2) - t3.swapaxes(0, 2)
                X2[i, j] += e('abc,dbc->ad', s, Vvovv[:, k])
                X2[i] -= e('abc,lc->lab', s, Vooov[j, k])
                X2[i, j] += e('abc,c->ab', t3 - t3.swapaxes(0, 2), Fov[k])
    return 2.0 * e('ia,ia->', t1, X1) + e('ijab,ijab->', 4.0 * t2 - 2.0 * t2.swapaxes(2, 3), X2)
