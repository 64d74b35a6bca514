"""(T) on the tensor cores: grouped BF16 tcgen05 GEMMs build the connected triples of a
batch of (i, j, k) triples, the energy kernel reduces them in FP64.

The twelve t3 terms of ``t3c_ijk`` (``pycc/cctriples.py:56-67``) are products of six
operand matrices, packed once from the converged amplitudes and the integrals (BF16,
K-major):

* A side (rows x*v^2 + p*v + q):  VT[x] = <qp|ex>,  VN[x] = <pq|ex>  (K = e),
                                   TM[x] = t2_xmpq,  TMT[x] = t2_xmqp (K = m)
* B side (rows (x*o + y)*v + p):  T2P = t2_xype (K = e),  OB = -<mp|xy> (K = m)

Each (triple, orientation) is one GEMM group with four K segments (see
``pycc_gb300.triples.orientation_terms``), so every partial tensor is written once, in FP32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .tc import FMT_BF16, Operand, pack
from .triples import triples_list

GROUP_DTYPE = np.dtype({
    "names": ["nseg", "amap", "arow", "bmap", "brow", "nkb", "out"],
    "formats": [np.int32, (np.int32, 4), (np.int32, 4), (np.int32, 4), (np.int32, 4),
                (np.int32, 4), np.int64],
    "offsets": [0, 4, 20, 36, 52, 68, 88],
    "itemsize": 96,
})

VT, VN, TM, TMT = 0, 1, 2, 3
T2P, OB = 0, 1


class TriplesTC:
    """Packed (T) operands for one set of amplitudes, and the batched driver."""

    def __init__(self, w, t1, t2, batch=32):
        self.w = w
        no, nv = w.no, w.nv
        o, v = w.o, w.v
        self.no, self.nv = no, nv
        self.batch = batch
        self.t1 = t1.contiguous()
        self.t2 = t2.contiguous()
        V = w.H.ERI[v, v, v, o]          # <pq|ex>
        O = w.H.ERI[o, v, o, o]          # <mp|xy>
        st = w.stream
        f = FMT_BF16
        self.A = [
            pack(Operand("xpqe", (V, "qpex")), ["x", "p", "q"], ["e"], f, st),
            pack(Operand("xpqe", (V, "pqex")), ["x", "p", "q"], ["e"], f, st),
            pack(Operand("xpqm", (self.t2, "xmpq")), ["x", "p", "q"], ["m"], f, st),
            pack(Operand("xpqm", (self.t2, "xmqp")), ["x", "p", "q"], ["m"], f, st),
        ]
        self.B = [
            pack(Operand("xype", (self.t2, "xype")), ["x", "y", "p"], ["e"], f, st),
            pack(Operand("xypm", (O, "mpxy"), a=-1.0), ["x", "y", "p"], ["m"], f, st),
        ]
        self.nkb_v = self.A[VT].Kp // 64
        self.nkb_o = self.A[TM].Kp // 64
        self.status = torch.zeros(4, dtype=torch.int32, device=t2.device)
        if _lib.load().pcg_tc_group_desc_size() != GROUP_DTYPE.itemsize:
            raise _lib.EngineError("GroupDesc layout mismatch")

    def groups(self, trips):
        """GroupDesc records of the three orientations of every triple (numpy, vectorised)."""
        no, nv = self.no, self.nv
        v2, v3 = nv * nv, nv ** 3
        kv, ko = self.nkb_v, self.nkb_o
        tr = np.asarray(trips, dtype=np.int64).reshape(-1, 3)
        i, j, k = tr[:, 0], tr[:, 1], tr[:, 2]
        nt = len(tr)
        g = np.zeros(3 * nt, dtype=GROUP_DTYPE)

        def row_b(x, y):
            return (x * no + y) * nv

        # per orientation: four (A map, A triple index, B map, B row, K blocks) segments
        segs = [
            [(VT, i, T2P, row_b(k, j), kv), (VN, j, T2P, row_b(k, i), kv),
             (TM, i, OB, row_b(j, k), ko), (TMT, j, OB, row_b(i, k), ko)],
            [(VT, i, T2P, row_b(j, k), kv), (VN, k, T2P, row_b(j, i), kv),
             (TM, i, OB, row_b(k, j), ko), (TMT, k, OB, row_b(i, j), ko)],
            [(VN, k, T2P, row_b(i, j), kv), (VT, j, T2P, row_b(i, k), kv),
             (TMT, k, OB, row_b(j, i), ko), (TM, j, OB, row_b(k, i), ko)],
        ]
        t = np.arange(nt)
        for q in range(3):
            r = g[q::3]
            r["nseg"] = 4
            for s, (am, ax, bm, brow, nk) in enumerate(segs[q]):
                r["amap"][:, s] = am
                r["arow"][:, s] = ax * v2
                r["bmap"][:, s] = bm
                r["brow"][:, s] = brow
                r["nkb"][:, s] = nk
            r["out"] = (3 * (t % self.batch) + q) * v3
        return g

    def energy(self):
        w, no, nv = self.w, self.no, self.nv
        dev = self.t2.device
        trips = triples_list(no)
        nb = self.batch
        P = torch.empty((nb, 3, nv, nv, nv), dtype=torch.float32, device=dev)
        plen = int(_lib.load().pcg_triples_part_len(1, nv))
        part = torch.empty((nb, plen), dtype=torch.float64, device=dev)   # one batch
        out = torch.zeros((), dtype=torch.float64, device=dev)
        ijk_all = torch.tensor(trips, dtype=torch.int32, device=dev)
        st = _lib.stream_handle(w.stream)
        A, B = self.A, self.B
        a_ptr = (C.c_void_p * 4)(*[x.hi.data_ptr() for x in A])
        a_rows = _lib.i64s([x.rows for x in A])
        a_ld = _lib.i64s([x.Kp for x in A])
        b_ptr = (C.c_void_p * 2)(*[x.hi.data_ptr() for x in B])
        b_rows = _lib.i64s([x.rows for x in B])
        b_ld = _lib.i64s([x.Kp for x in B])
        H = w.H
        o, v = w.o, w.v
        fov = H.F[o, v].contiguous()
        fov_ptr = fov.data_ptr() if bool(fov.abs().max() > 0) else None
        eoovv = H.ERI[o, o, v, v].float()          # the FP32 energy kernel's copies
        t2f = self.t2.float()
        # every batch's group records, uploaded once; a batch's partials start at P[0]
        gall = torch.from_numpy(self.groups(trips).view(np.uint8)).to(dev)
        gsz = GROUP_DTYPE.itemsize
        for b0 in range(0, len(trips), nb):
            chunk = trips[b0:b0 + nb]
            _lib.call("pcg_tc_grouped_gemm", 4, a_ptr, a_rows, a_ld, 2, b_ptr, b_rows, b_ld,
                      gall.data_ptr() + 3 * b0 * gsz, 3 * len(chunk), nv * nv, nv,
                      P.data_ptr(), 1, nv * nv, self.status.data_ptr(), st)
            _lib.call("pcg_triples_energy", 1, P.data_ptr(), P[:, 1].data_ptr(),
                      P[:, 2].data_ptr(), 3 * nv ** 3, ijk_all[b0:].data_ptr(), len(chunk),
                      H.eps.data_ptr(), eoovv.data_ptr(), self.t1.data_ptr(), t2f.data_ptr(),
                      fov_ptr, no, nv, part.data_ptr(), st)
            _lib.call("pcg_reduce_sum_f64", part.data_ptr(), len(chunk) * plen, out.data_ptr(),
                      st)
        s = self.status.cpu()
        if int(s.abs().sum()):
            raise _lib.EngineError("grouped GEMM reported a wait timeout (status %s)" % s.tolist())
        return float(out)


def t_energy_tc(w, t1=None, t2=None, batch=32):
    t1 = w.t1 if t1 is None else t1
    t2 = w.t2 if t2 is None else t2
    return TriplesTC(w, t1, t2, batch=batch).energy()
