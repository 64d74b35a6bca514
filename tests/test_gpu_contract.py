"""FP64 strided contraction kernel against torch's FP64 einsum on the same GPU tensors."""
import pytest
import torch

from pycc_gb300.contract import contract_f64

pytestmark = pytest.mark.gpu

SHAPES = {"o": 5, "v": 37}
TERMS = [
    ("mnaf,mnef->ae", "oovv", "oovv"), ("ijef,mnef->mnij", "oovv", "oovv"),
    ("jf,mbef->mbej", "ov", "ovvv"), ("jnfb,mnef->mbej", "oovv", "oovv"),
    ("mbef,ijef->mbij", "ovvv", "oovv"), ("mief,maef->ia", "oovv", "ovvv"),
    ("ijae,eb->ijab", "oovv", "vv"), ("mnab,mnij->ijab", "oovv", "oooo"),
    ("ijef,abef->ijab", "oovv", "vvvv"), ("imae,mbej->ijab", "oovv", "ovvo"),
    ("mjae,mbie->ijab", "oovv", "ovov"), ("ie,ma->imea", "ov", "ov"),
    ("ie,abej->ijab", "ov", "vvvo"), ("ia,ia->", "ov", "ov"),
    # matrix-vector shapes (thread- and warp-per-output paths)
    ("mf,mafe->ae", "ov", "ovvv"), ("nf,nafi->ia", "ov", "ovvo"), ("nf,mnef->me", "ov", "oovv"),
    ("imae,me->ia", "oovv", "ov"), ("mafe,mf->ae", "ovvv", "ov"),
]


def rand(pat, dev, gen):
    return torch.randn([SHAPES[c] for c in pat], dtype=torch.float64, device=dev, generator=gen)


@pytest.mark.parametrize("subs,sa,sb", TERMS)
def test_contract_vs_torch(cuda, subs, sa, sb):
    gen = torch.Generator(device=cuda).manual_seed(7)
    A, B = rand(sa, cuda, gen), rand(sb, cuda, gen)
    ref = torch.einsum(subs, A, B)
    got = contract_f64(subs, A, B)
    torch.cuda.synchronize()
    assert torch.allclose(got, ref, rtol=1e-12, atol=1e-12 * ref.abs().max().item())


def test_accumulate_and_strided_views(cuda):
    gen = torch.Generator(device=cuda).manual_seed(3)
    n = 37
    X = torch.randn(n, n, n, n, dtype=torch.float64, device=cuda, generator=gen)
    A = X[:5, 5:16, 3:9, :11]                # non-contiguous views of one tensor
    B = X[5:16, 10:16, 3:9, 20:31]
    out = torch.randn(5, 11, 11, 6, dtype=torch.float64, device=cuda, generator=gen)
    ref = 0.25 * out - 1.5 * torch.einsum("iaeb,jfea->ibjf", A, B)
    got = contract_f64("iaeb,jfea->ibjf", A, B, out=out, alpha=-1.5, beta=0.25)
    torch.cuda.synchronize()
    assert got.data_ptr() == out.data_ptr()
    assert torch.allclose(out, ref, rtol=1e-12, atol=1e-12)


def test_split_k_large_k(cuda):
    gen = torch.Generator(device=cuda).manual_seed(11)
    A = torch.randn(3, 20000, dtype=torch.float64, device=cuda, generator=gen)
    B = torch.randn(2, 20000, dtype=torch.float64, device=cuda, generator=gen)
    out = torch.ones(3, 2, dtype=torch.float64, device=cuda)
    ref = 2.0 * out + torch.einsum("mk,nk->mn", A, B)
    contract_f64("mk,nk->mn", A, B, out=out, beta=2.0)
    torch.cuda.synchronize()
    assert torch.allclose(out, ref, rtol=1e-12, atol=1e-10)


def test_rejects_host_and_fp32(cuda):
    A = torch.randn(3, 4, dtype=torch.float64)
    with pytest.raises(ValueError):
        contract_f64("ij,jk->ik", A, A.T.contiguous())
    B = torch.randn(3, 4, device=cuda)
    with pytest.raises(TypeError):
        contract_f64("ij,kj->ik", B, B)
