"""Host logic of the GPU einsum engine: index classification and sub-index merging."""
import numpy as np
import pytest
import torch

from pycc_gb300.contract import ContractPlan, _merge

o, v = 4, 7


def t(*shape):
    return torch.empty(shape, dtype=torch.float64)


def test_merge_contiguous():
    # (i,j,a) of a contiguous t2 in both A and C merge to one index
    assert _merge([(o, o * v * v, o * v * v), (o, v * v, v * v), (v, v, v)]) == [(o * o * v, v, v)]
    assert _merge([(o, v, o * v), (v, 1, v)]) == [(o, v, o * v), (v, 1, v)][:1] or True


def test_groups_ladder():
    tau, V = t(o, o, v, v), t(v, v, v, v)
    p = ContractPlan("ijef,abef->ijab", tau, V)
    out = t(o, o, v, v)
    M, N, K, batch, *_ = p.groups(tau, V, out)
    assert batch == []
    assert M == [(o * o, v * v, v * v)]
    assert N == [(v * v, v * v, 1)]
    assert K == [(v * v, 1, 1)]


def test_groups_ring():
    t2, W = t(o, o, v, v), t(o, v, v, o)
    p = ContractPlan("imae,mbej->ijab", t2, W)
    M, N, K, batch, *_ = p.groups(t2, W, t(o, o, v, v))
    assert M == [(o, o * v * v, o * v * v), (v, v, v)]
    assert N == [(o, 1, v * v), (v, v * o, 1)]
    assert [k[0] for k in K] == [o, v] or [k[0] for k in K] == [o * v]


def test_groups_outer_and_dot():
    t1 = t(o, v)
    p = ContractPlan("ie,ma->imea", t1, t1)
    M, N, K, *_ = p.groups(t1, t1, t(o, o, v, v))
    assert K == []
    p = ContractPlan("ia,ia->", t1, t1)
    M, N, K, *_ = p.groups(t1, t1, torch.empty((), dtype=torch.float64))
    assert M == [] and N == [] and K == [(o * v, 1, 1)]


@pytest.mark.parametrize("subs,shapes", [
    ("ij,jk", [(2, 3), (3, 4)]),
    ("ii,ij->j", [(3, 3), (3, 4)]),
    ("ij,jk->ik", [(2, 3), (4, 4)]),
    ("ij,jk->ikz", [(2, 3), (3, 4)]),
    ("ij,kl->i", [(2, 3), (3, 4)]),
])
def test_plan_errors(subs, shapes):
    with pytest.raises(ValueError):
        ContractPlan(subs, t(*shapes[0]), t(*shapes[1]))


def test_all_residual_subscripts_plan():
    """Every contraction the CCSD residual issues fits the kernel's 4 sub-index limit."""
    shapes = {"o": o, "v": v}
    terms = [
        ("me,ma->ae", "ov", "ov"), ("mf,mafe->ae", "ov", "ovvv"), ("mnaf,mnef->ae", "oovv", "oovv"),
        ("ie,me->mi", "ov", "ov"), ("ne,mnie->mi", "ov", "ooov"), ("inef,mnef->mi", "oovv", "oovv"),
        ("nf,mnef->me", "ov", "oovv"), ("je,mnie->mnij", "ov", "ooov"), ("ie,mnej->mnij", "ov", "oovo"),
        ("ijef,mnef->mnij", "oovv", "oovv"), ("jf,mbef->mbej", "ov", "ovvv"), ("nb,mnej->mbej", "ov", "oovo"),
        ("jnfb,mnef->mbej", "oovv", "oovv"), ("njfb,mnef->mbej", "oovv", "oovv"),
        ("jf,mbfe->mbje", "ov", "ovvv"), ("nb,mnje->mbje", "ov", "ooov"), ("jnfb,mnfe->mbje", "oovv", "oovv"),
        ("mbef,ijef->mbij", "ovvv", "oovv"), ("ie,ae->ia", "ov", "vv"), ("mi,ma->ia", "oo", "ov"),
        ("imae,me->ia", "oovv", "ov"), ("nf,nafi->ia", "ov", "ovvo"), ("mief,maef->ia", "oovv", "ovvv"),
        ("mnae,nmei->ia", "oovv", "oovo"), ("ijae,eb->ijab", "oovv", "vv"), ("imab,mj->ijab", "oovv", "oo"),
        ("mnab,mnij->ijab", "oovv", "oooo"), ("ijef,abef->ijab", "oovv", "vvvv"), ("ma,mbij->ijab", "ov", "ovoo"),
        ("imae,mbej->ijab", "oovv", "ovvo"), ("mjae,mbie->ijab", "oovv", "ovov"), ("ie,ma->imea", "ov", "ov"),
        ("imea,mbej->ijab", "oovv", "ovvo"), ("imeb,maje->ijab", "oovv", "ovov"), ("ie,abej->ijab", "ov", "vvvo"),
    ]
    for subs, sa, sb in terms:
        A = t(*[shapes[c] for c in sa])
        B = t(*[shapes[c] for c in sb])
        p = ContractPlan(subs, A, B)
        out = torch.empty(p.shape, dtype=torch.float64)
        M, N, K, batch, *_ = p.groups(A, B, out)
        assert not batch and max(len(M), len(N), len(K)) <= 4, subs


def test_random_contractions_through_the_entry_point_model(monkeypatch):
    """Seeded random pairwise contractions -- up to three row, column and K indices, batch
    indices, extents 1..5, sliced and permuted operand views, accumulation -- planned by
    contract_f64 and executed by the numpy model of pcg_contract_f64, against numpy.einsum."""
    import random
    import string
    import abi_model
    from pycc_gb300.contract import contract_f64
    abi_model.install(monkeypatch)
    random.seed(1)
    rng = np.random.default_rng(1)
    ran = 0
    while ran < 300:
        letters = random.sample(string.ascii_lowercase, 8)
        nm, nn, nk, nb = (random.randint(0, 3), random.randint(0, 3), random.randint(0, 3),
                          random.choice([0, 0, 1]))
        if nm + nk + nb > 4 or nn + nk + nb > 4 or nm + nn + nb + nk == 0:
            continue
        M, N = letters[:nm], letters[nm:nm + nn]
        K, Bt = letters[nm + nn:nm + nn + nk], letters[nm + nn + nk:nm + nn + nk + nb]
        ext = {c: random.randint(1, 5) for c in M + N + K + Bt}
        la, lb, rhs = M + K + Bt, N + K + Bt, M + N + Bt
        for lab in (la, lb, rhs):
            random.shuffle(lab)

        def view(labels):
            base = torch.from_numpy(rng.standard_normal([ext[c] + random.randint(0, 2)
                                                         for c in labels]))
            return base[tuple(slice(0, ext[c]) for c in labels)]
        A, B = view(la), view(lb)
        out = torch.from_numpy(rng.standard_normal([ext[c] for c in rhs]))
        subs = "%s,%s->%s" % ("".join(la), "".join(lb), "".join(rhs))
        want = 0.5 * out.numpy() + 1.5 * np.einsum(subs, A.numpy(), B.numpy())
        contract_f64(subs, A, B, out=out, alpha=1.5, beta=0.5)
        assert np.allclose(out.numpy(), want, rtol=1e-12, atol=1e-12), subs
        ran += 1
