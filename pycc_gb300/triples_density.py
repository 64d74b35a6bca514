"""(T) densities and Lambda sources on the GPU (the reference's ``t3_density``,
``pycc/cctriples.py:1063-1157``; cached on the wave function by ``CCwfn.t3_density``,
``pycc/ccwfn.py:1819-1829``): the (T) contributions to the one- and two-particle densities
and to the Lambda residuals of CCSD(T) gradients, and the (T) energy.

For every ordered triple (i, j, k) -- all no^3 of them, as the reference loops -- the connected
partials of the (T) energy path (``triples.orientation_terms``, FP64 multi-term DMMA
contraction) and ``pcg_t3_ijk_f64`` give M3 = t3c_ijk / D and N3 = t3d_ijk / D;
``pcg_t3_density_terms_f64`` forms their permutation combinations, and the FP64 contraction
kernel accumulates every density block.  FP64 throughout; the result has the reference's
keys and layouts:

* ``Doo`` [o,o], ``Dvv`` [v,v] (diagonal), ``Dov`` [o,v];
* ``Goovv`` [o,o,v,v], ``Gooov`` [o,o,o,v], ``Gvvvo`` [v,v,v,o];
* ``S1`` [o,v], ``S2`` [o,o,v,v] (symmetrised, S2 + S2.swap(0,1).swap(2,3));
* the (T) energy ``t1 . S1 + (4 t2 - 2 t2.swap(2,3)) . X2``.
"""
from __future__ import annotations

import torch

from . import _lib
from .contract import contract_f64
from .triples import contract_multi, orientation_terms


def t3_density(w, t1=None, t2=None):
    """(ET, {Doo, Dvv, Dov, Goovv, Gooov, Gvvvo, S1, S2}) at the amplitudes of ``w`` (FP64)."""
    t1 = (w.t1 if t1 is None else t1).contiguous()
    t2 = (w.t2 if t2 is None else t2).contiguous()
    H = w.H
    no, nv = w.no, w.nv
    o, v = w.o, w.v
    dev = t2.device
    st = w.stream
    sh = _lib.stream_handle(st)
    f64 = dict(dtype=torch.float64, device=dev)
    V = H.ERI[v, v, v, o]                   # <ab|ei>
    O = H.ERI[o, v, o, o]                   # <ma|ij>
    Woovv = H.ERI[o, o, v, v].contiguous()  # <ij|ab>
    ooov = H.ERI[o, o, o, v]                # <jk|lc>
    ovvv = H.ERI[o, v, v, v]                # <kd|cb>
    vovv = ovvv.permute(1, 0, 3, 2)         # <dk|bc> = <kd|cb>
    Loovv = H.L[o, o, v, v]
    fov = H.F[o, v].contiguous()
    fov_ptr = fov.data_ptr() if bool(fov.abs().max() > 0) else None
    eps = H.eps.contiguous()

    dvv = torch.zeros(nv, **f64)
    doo = torch.zeros(no, **f64)
    Dov = torch.zeros(no, nv, **f64)
    Goovv = torch.zeros(no, no, nv, nv, **f64)
    Gooov = torch.zeros(no, no, no, nv, **f64)
    Gvvvo = torch.zeros(nv, nv, nv, no, **f64)
    S1 = torch.zeros(no, nv, **f64)
    S2 = torch.zeros(no, no, nv, nv, **f64)
    X2 = torch.zeros(no, no, nv, nv, **f64)
    T4 = w._combine(4.0, t2, -2.0, t2, (0, 1, 3, 2), record=False)   # 4 t2 - 2 t2.swap(2,3)

    P = torch.empty(3, nv, nv, nv, **f64)
    M3, N3, A, S, Z, Ma, Mb, Mc = (torch.empty(nv, nv, nv, **f64) for _ in range(8))

    def c(subs, X, Y, out, alpha=1.0):
        contract_f64(subs, X, Y, out=out, alpha=alpha, beta=1.0, stream=st)

    for i in range(no):
        for j in range(no):
            for k in range(no):
                for q, (lab, terms) in enumerate(orientation_terms(i, j, k, t2, V, O)):
                    contract_multi(P[q].permute(1, 2, 0), lab, terms, stream=st)
                _lib.call("pcg_t3_ijk_f64", P.data_ptr(), eps.data_ptr(), i, j, k, no, nv,
                          Woovv.data_ptr(), t1.data_ptr(), t2.data_ptr(), fov_ptr,
                          M3.data_ptr(), N3.data_ptr(), sh)
                _lib.call("pcg_t3_density_terms_f64", M3.data_ptr(), N3.data_ptr(), nv,
                          A.data_ptr(), S.data_ptr(), Z.data_ptr(), Ma.data_ptr(),
                          Mb.data_ptr(), Mc.data_ptr(), sh)
                # doubles part of the (T) energy (the reference's X2)
                c('abc,c->ab', Ma, fov[k], X2[i, j])
                c('abc,dbc->ad', Mb, vovv[:, k], X2[i, j])
                c('abc,lc->lab', Mb, ooov[j, k], X2[i], alpha=-1.0)
                # one-particle (T) density: diagonal oo / vv, and ov
                c('acd,acd->a', M3, S, dvv, alpha=0.5)
                c('abc,abc->', M3, S, doo[i], alpha=-0.5)
                c('abc,bc->a', Ma, T4[j, k], Dov[i])
                # two-particle (T) density
                c('c,abc->ab', t1[k], Z, Goovv[i, j], alpha=4.0)
                c('abc,lbc->la', A, t2[:, k], Gooov[j, i], alpha=-1.0)
                c('abc,cd->abd', A, t2[k, i], Gvvvo[:, :, :, j])
                # (T) sources of the Lambda residuals
                c('abc,bc->a', Mc, Loovv[j, k], S1[i])
                c('abc,lc->lab', A, ooov[j, k], S2[i], alpha=-1.0)
                c('abc,dcb->ad', A, ovvv[k], S2[i, j])
    S2 = w._combine(1.0, S2, 1.0, S2, (1, 0, 3, 2), record=False)
    et = contract_f64('ia,ia->', t1, S1, stream=st)
    contract_f64('ijab,ijab->', T4, X2, out=et, beta=1.0, stream=st)
    return float(et), {'Doo': torch.diag(doo), 'Dvv': torch.diag(dvv), 'Dov': Dov,
                       'Goovv': Goovv, 'Gooov': Gooov, 'Gvvvo': Gvvvo, 'S1': S1, 'S2': S2}
