"""Host logic of the tensor-core (T): the GroupDesc table of every (triple, orientation).

Each record's four K segments must be the four t3 terms of that orientation
(pycc/cctriples.py:56-67, grouped as in pycc_gb300.triples.orientation_terms): A operand,
its triple index, B operand row and K blocks; partials of a batch are laid out
consecutively.  Checked record by record against the per-triple formulas, no GPU.
"""
import numpy as np

from pycc_gb300.triples import triples_list
from pycc_gb300.triples_tc import OB, T2P, TM, TMT, VN, VT, GROUP_DTYPE, TriplesTC


def test_group_table():
    no, nv, batch = 7, 13, 32
    t = TriplesTC.__new__(TriplesTC)
    t.no, t.nv, t.nkb_v, t.nkb_o, t.batch = no, nv, 4, 1, batch
    trips = triples_list(no)
    g = t.groups(trips)
    assert g.dtype == GROUP_DTYPE and len(g) == 3 * len(trips)
    v2, v3 = nv * nv, nv ** 3

    def rb(x, y):
        return (x * no + y) * nv

    for n, (i, j, k) in enumerate(trips):
        want = [
            [(VT, i, T2P, rb(k, j), 4), (VN, j, T2P, rb(k, i), 4),
             (TM, i, OB, rb(j, k), 1), (TMT, j, OB, rb(i, k), 1)],
            [(VT, i, T2P, rb(j, k), 4), (VN, k, T2P, rb(j, i), 4),
             (TM, i, OB, rb(k, j), 1), (TMT, k, OB, rb(i, j), 1)],
            [(VN, k, T2P, rb(i, j), 4), (VT, j, T2P, rb(i, k), 4),
             (TMT, k, OB, rb(j, i), 1), (TM, j, OB, rb(k, i), 1)],
        ]
        for q in range(3):
            r = g[3 * n + q]
            assert r["nseg"] == 4
            assert r["out"] == (3 * (n % batch) + q) * v3
            got = [(r["amap"][s], r["arow"][s], r["bmap"][s], r["brow"][s], r["nkb"][s])
                   for s in range(4)]
            assert got == [(am, ax * v2, bm, brow, nk) for am, ax, bm, brow, nk in want[q]]
