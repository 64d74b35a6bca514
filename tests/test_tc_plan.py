"""Host logic of the tensor-core engine, on CPU with the pack and GEMM launches recorded
instead of run: the GEMM orientation (the output's unit-stride index on the 128-row side),
the K order, the caches of packed operands and the precision ladder's release of packed
integrals no later stage reads.
"""
import pytest
import torch

import pycc_gb300.tc as tc
from pycc_gb300.tc import (FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_BF16X6, FMT_FP8,
                           Operand, Packed, TCEngine, static_pack_format)


@pytest.fixture
def recorder(monkeypatch):
    calls = {"pack": [], "gemm": []}

    def fake_pack(op, rows, ks, fmt, stream=None, row_tab=None, k_tab=None, k_w=None):
        ext = op.extents()
        R = 1
        for c in rows:
            R *= ext[c]
        calls["pack"].append((op.labels, tuple(rows), tuple(ks), fmt, op.key))
        return Packed(fmt, R, 64, None)

    def fake_gemm(fmt, A, B, out, rows, cols, rhs, **kw):
        calls["gemm"].append((fmt, A.rows, B.rows, tuple(rows), tuple(cols), rhs))

    monkeypatch.setattr(tc, "pack", fake_pack)
    monkeypatch.setattr(tc, "gemm", fake_gemm)
    return calls


def t(*shape):
    return torch.zeros(shape, dtype=torch.float64)


def test_orientation_follows_output_unit_stride(recorder):
    """The operand holding the output's unit-stride index supplies the 128-row side (a
    warp's 32 rows are then 32 consecutive output addresses), unless that side is shorter
    than one 128-row tile."""
    eng = TCEngine("cpu")
    # mbej, j unit-stride and j held by t1: 200 occupied orbitals fill the rows
    o, v = 200, 3
    eng.contract("jf,mbef->mbej", Operand.of("jf", t(o, v)), Operand.of("mbef", t(o, v, v, v)),
                 t(o, v, v, o))
    fmt, M, N, rows, cols, rhs = recorder["gemm"][-1]
    assert rows == ("j",) and M == o and cols == ("m", "b", "e")
    # the same term with 4 occupied orbitals: j is too short, (m, b, e) takes the rows
    o, v = 4, 300
    eng.contract("jf,mbef->mbej", Operand.of("jf", t(o, v)), Operand.of("mbef", t(o, v, v, v)),
                 t(o, v, v, o))
    fmt, M, N, rows, cols, rhs = recorder["gemm"][-1]
    assert rows == ("m", "b", "e") and M == o * v * v and cols == ("j",)
    # ijab, b unit-stride and held by F_be (300 rows)
    eng.contract("ijae,be->ijab", Operand.of("ijae", t(o, o, v, v)), Operand.of("be", t(v, v)),
                 t(o, o, v, v))
    fmt, M, N, rows, cols, rhs = recorder["gemm"][-1]
    assert rows == ("b",) and M == v and cols == ("i", "j", "a")


def test_k_order_follows_dynamic_operand_strides(recorder):
    """K is ordered by the dynamic operand's strides, slowest first, so its gather runs
    along its own memory order."""
    o, v = 3, 5
    eng = TCEngine("cpu")
    t2 = t(o, o, v, v)
    L = Operand.of("mnef", t(o, o, v, v), key=("L", "oovv"))
    eng.contract("inef,mnef->mi", Operand.of("inef", t2), L, t(o, o))
    ks = [c[2] for c in recorder["pack"]]
    assert all(k == ("n", "e", "f") for k in ks)


def test_static_and_dynamic_caches(recorder):
    """Static operands are packed once per (block, labels, layout, pieces) and BF16 GEMMs
    reuse the split-BF16x3 pack; dynamic operands are packed once per residual."""
    o, v = 3, 5
    eng = TCEngine("cpu")
    V = Operand.of("mbef", t(o, v, v, v), key=("ERI", "ovvv"))
    t1 = t(o, v)
    for fmt in (FMT_BF16, FMT_BF16X3F, FMT_BF16X3, FMT_BF16):
        eng.contract("jf,mbef->mbej", Operand.of("jf", t1), V, t(o, v, v, o), fmt=fmt)
    static = [c for c in recorder["pack"] if c[4] is not None]
    assert len(static) == 1 and static[0][3] == FMT_BF16X3
    assert len(eng.cache) == 1
    eng.dyn_cache = {}
    n0 = len(recorder["pack"])
    for _ in range(3):
        eng.contract("jf,mbef->mbej", Operand.of("jf", t1), V, t(o, v, v, o), fmt=FMT_BF16X3)
    assert len(recorder["pack"]) == n0 + 1                # t1 packed once per residual
    # the entry keeps its source alive, so its address cannot be reused for another tensor
    (entry,) = eng.dyn_cache.values()
    assert any(s is t1 for s in entry[1])


def test_dynamic_cache_keys_the_gather_not_the_labels(recorder):
    """Spellings of one gather (the same tensor, extents and strides per row and K index,
    under other label names or with the K order following the source's strides) share a pack
    within a residual; a different combination coefficient or transposed rows do not."""
    o, v = 3, 5
    eng = TCEngine("cpu")
    eng.dyn_cache = {}
    x = t(o, o, v, v)
    V = Operand.of("mbef", t(o, v, v, v), key=("ERI", "ovvv"))
    n0 = len(recorder["pack"])
    eng.contract("ijef,mbef->mbij", Operand.of("ijef", x), V, t(o, v, o, o), fmt=FMT_BF16X3)
    eng.contract("klef,mbef->mbkl", Operand.of("klef", x), V, t(o, v, o, o), fmt=FMT_BF16X3)
    dyn = [c for c in recorder["pack"][n0:] if c[4] is None]
    assert len(dyn) == 1
    # x read as x[i, j, f, e]: K runs (f, e) by the source's strides, the same bytes
    eng.contract("ijef,mbef->mbij", Operand("ijef", (x, "ijfe")), V, t(o, v, o, o),
                 fmt=FMT_BF16X3)
    dyn = [c for c in recorder["pack"][n0:] if c[4] is None]
    assert len(dyn) == 1
    eng.contract("ijef,mbef->mbij", Operand("ijef", (x, "ijef"), a=2.0), V, t(o, v, o, o),
                 fmt=FMT_BF16X3)
    eng.contract("ijef,mbef->mbij", Operand("ijef", (x, "jief")), V, t(o, v, o, o),
                 fmt=FMT_BF16X3)
    dyn = [c for c in recorder["pack"][n0:] if c[4] is None]
    assert len(dyn) == 3


def test_static_pack_formats():
    assert static_pack_format(FMT_BF16) == FMT_BF16X3
    assert static_pack_format(FMT_BF16X3F) == FMT_BF16X3
    assert static_pack_format(FMT_BF16X3S) == FMT_BF16X3
    assert static_pack_format(FMT_BF16X3) == FMT_BF16X3
    assert static_pack_format(FMT_FP8) == FMT_FP8
    assert static_pack_format(FMT_BF16X6) == FMT_BF16X6


def test_ladder_prunes_formats_no_later_stage_reads():
    """Advancing the precision ladder frees the packed integrals of formats that no later
    stage reads (the FP8 ladder operand after the FP8 stage)."""
    from pycc_gb300.mixed import MixedResidual

    class W:
        device1, stream, vvvv_fp8, switch_threshold = "cpu", None, True, 1e-5

    m = MixedResidual(W())
    assert m.stages == ["fp8", "bf16", "bf16x3f", "bf16x3s"]
    m.tc.cache = {("ERI", "vvvv", FMT_FP8): 1, ("ERI", "ovvv", FMT_BF16X3): 2}
    m._advance()                                         # fp8 -> bf16
    assert list(m.tc.cache) == [("ERI", "ovvv", FMT_BF16X3)]
    m._advance()
    m._advance()                                         # split stages keep the pack
    assert list(m.tc.cache) == [("ERI", "ovvv", FMT_BF16X3)]


def test_swapped_integrals_drop_the_packs():
    """A caller that swaps H.ERI / H.L for other blocks (the reference's linear-in-H use of
    the residual, pycc/ccderiv.py:252-259) gets its integrals re-packed, not the cached
    packs of the previous blocks."""
    from pycc_gb300.hamiltonian import BlockTensor
    from pycc_gb300.mixed import MixedResidual

    def blocks(name):
        return BlockTensor(name, 2, 3, {"oovv": t(2, 2, 3, 3), "ovvv": t(2, 3, 3, 3)})

    class Ham:
        def __init__(self):
            self.ERI, self.L = blocks("ERI"), blocks("L")

    class W:
        device1, stream, vvvv_fp8, switch_threshold = "cpu", None, True, 1e-5

        def __init__(self):
            self.h = self.H = Ham()

    w = W()
    m = MixedResidual(w)
    m.sync_integrals()
    m.tc.cache = {("ERI", "ovvv", FMT_BF16X3): 1}
    m._r_seed = "seed"
    m.sync_integrals()                                  # same blocks: caches kept
    assert m.tc.cache and m._r_seed == "seed"
    saved = w.h.ERI
    w.h.ERI = blocks("ERI")                             # derivative integrals swapped in
    m.sync_integrals()
    assert not m.tc.cache and m._r_seed is None
    m.tc.cache = {("ERI", "ovvv", FMT_BF16X3): 2}
    w.h.ERI = saved                                     # and swapped back
    m.sync_integrals()
    assert not m.tc.cache
    w.h.ERI = t(5, 5, 5, 5)                             # a plain array is refused
    with pytest.raises(TypeError):
        m.sync_integrals()


def test_random_contractions_through_the_entry_point_model(monkeypatch):
    """Seeded random contractions on the tensor-core engine -- operand combinations
    a X + b Y' (Y in another label order) and c P (x) Q, static and dynamic operands, every
    GEMM format, sliced views, extents 1..6 -- packed and multiplied by the exact FP64 model
    of pcg_pack_operand / pcg_tc_gemm, against numpy.einsum of the same combinations."""
    import random
    import string
    import numpy as np
    import abi_model
    abi_model.install(monkeypatch)
    random.seed(2)
    rng = np.random.default_rng(2)
    eng = TCEngine("cpu")
    fmts = [FMT_BF16, FMT_BF16X3, FMT_BF16X3F, FMT_BF16X3S, FMT_BF16X6, FMT_FP8]
    ran = 0
    while ran < 200:
        letters = random.sample(string.ascii_lowercase, 8)
        nm, nn, nk = random.randint(0, 3), random.randint(0, 3), random.randint(1, 3)
        if nm + nk > 4 or nn + nk > 4 or nm + nn == 0:
            continue
        M, N, K = letters[:nm], letters[nm:nm + nn], letters[nm + nn:nm + nn + nk]
        ext = {c: random.randint(1, 6) for c in M + N + K}
        la, lb, rhs = M + K, N + K, M + N
        for lab in (la, lb, rhs):
            random.shuffle(lab)

        def view(labels):
            base = torch.from_numpy(rng.standard_normal([ext[c] + random.randint(0, 2)
                                                         for c in labels]))
            return base[tuple(slice(0, ext[c]) for c in labels)]

        def operand(labels, key):
            s = "".join(labels)
            X = view(labels)
            op, val = Operand(s, (X, s), key=key), X.numpy().copy()
            if len(labels) >= 2 and random.random() < 0.5:
                perm = labels[:]
                random.shuffle(perm)
                Y = view(perm)
                op.Y, op.b = (Y, "".join(perm)), -0.5
                val = val - 0.5 * np.einsum("%s->%s" % ("".join(perm), s), Y.numpy())
            if len(labels) >= 2 and random.random() < 0.5:
                cut = random.randint(1, len(labels) - 1)
                P, Q = view(labels[:cut]), view(labels[cut:])
                op.P, op.Q, op.c = (P, "".join(labels[:cut])), (Q, "".join(labels[cut:])), 0.75
                val = val + 0.75 * np.einsum("%s,%s->%s" % ("".join(labels[:cut]),
                                                              "".join(labels[cut:]), s),
                                             P.numpy(), Q.numpy())
            return op, val
        A, va = operand(la, None)
        B, vb = operand(lb, ("static", ran) if random.random() < 0.5 else None)
        out = torch.from_numpy(rng.standard_normal([ext[c] for c in rhs]))
        subs = "%s,%s->%s" % ("".join(la), "".join(lb), "".join(rhs))
        want = 0.25 * out.numpy() + 2.0 * np.einsum(subs, va, vb)
        eng.contract(subs, A, B, out, alpha=2.0, beta=0.25, fmt=random.choice(fmts))
        assert np.allclose(out.numpy(), want, rtol=1e-11, atol=1e-11), subs
        ran += 1
