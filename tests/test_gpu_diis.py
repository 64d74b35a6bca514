"""GPU DIIS against the oracle's restatement of helper_diis (pycc/utils.py:257-361).

* FP64 error vectors: the extrapolated amplitudes of a converging sequence equal the
  oracle's to 1e-10 (same error vectors, same bordered Pulay system; the overlaps differ
  in summation order only, in the last digits, which the system's conditioning magnifies).
* FP32 error vectors (the mixed-precision solver): each error vector is the FP64
  difference rounded once to FP32, bit for bit; the overlaps are within the FP32 rounding
  of the products (1e-6 of sum |e_i y_i|); the extrapolation stays within 1e-4 of the FP64
  one on the same sequence (the Pulay system of a converging sequence is ill-conditioned,
  so the coefficients move by more than the overlaps' 1e-7, but only along the small
  differences between the stored amplitudes).
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pycc_gb300 import _lib
from pycc_gb300.diis import DIIS
from oracle import ccsd as oc

pytestmark = pytest.mark.gpu


def _sequence(n1, n2, steps, seed):
    """Amplitude iterates converging geometrically with noise, as host arrays."""
    rng = np.random.default_rng(seed)
    t1s, t2s = [rng.standard_normal(n1) * 0.05], [rng.standard_normal(n2) * 0.01]
    lim1, lim2 = rng.standard_normal(n1) * 0.05, rng.standard_normal(n2) * 0.01
    for s in range(steps):
        f = 0.5 ** (s + 1)
        t1s.append(lim1 + f * (t1s[0] - lim1) + 1e-4 * f * rng.standard_normal(n1))
        t2s.append(lim2 + f * (t2s[0] - lim2) + 1e-4 * f * rng.standard_normal(n2))
    return t1s, t2s


def _run_gpu(t1s, t2s, cuda, error_dtype, max_diis=4):
    amps = torch.from_numpy(np.concatenate([t1s[0], t2s[0]])).to(cuda)
    d = DIIS(amps, max_diis, error_dtype=error_dtype)
    out = []
    for a, b in zip(t1s[1:], t2s[1:]):
        amps = torch.from_numpy(np.concatenate([a, b])).to(cuda)
        d.add_error_vector(amps)
        amps = d.extrapolate(amps)
        out.append(amps.cpu().numpy().copy())
    return out


@pytest.mark.parametrize("n1,n2", [(12, 403), (40, 4001)])
def test_diis_fp64_matches_oracle(cuda, n1, n2):
    t1s, t2s = _sequence(n1, n2, 7, n1 + n2)
    got = _run_gpu(t1s, t2s, cuda, torch.float64)
    ref = oc.DIIS(t1s[0], t2s[0], 4)
    for k, (a, b) in enumerate(zip(t1s[1:], t2s[1:])):
        ref.add_error_vector(a, b)
        r1, r2 = ref.extrapolate(a, b)
        want = np.concatenate([r1, r2])
        assert np.abs(got[k] - want).max() < 1e-10 * max(1.0, np.abs(want).max())


@pytest.mark.parametrize("n", [4096, 4099, 1 << 20])
def test_diis_error_f32_pass(cuda, n):
    g = torch.Generator(device=cuda).manual_seed(n)
    x = torch.randn(n, generator=g, dtype=torch.float64, device=cuda)
    old = x + 1e-3 * torch.randn(n, generator=g, dtype=torch.float64, device=cuda)
    ys = [torch.randn(n, generator=g, dtype=torch.float64, device=cuda).float() for _ in range(5)]
    k = len(ys) + 1
    e = torch.empty(n, dtype=torch.float32, device=cuda)
    work = torch.empty(1024 * k, dtype=torch.float64, device=cuda)
    out = torch.empty(k, dtype=torch.float64, device=cuda)
    ptrs = (C.c_void_p * k)(*([y.data_ptr() for y in ys] + [0]))
    _lib.call("pcg_diis_error_f32", x.data_ptr(), old.data_ptr(), e.data_ptr(), ptrs, k, n,
              work.data_ptr(), work.numel(), out.data_ptr(), None)
    torch.cuda.synchronize()
    want_e = (x - old).float()
    assert torch.equal(e.view(torch.int32), want_e.view(torch.int32))
    e64 = want_e.double()
    for j, y in enumerate(ys + [want_e]):
        ref = float((e64 * y.double()).sum())
        scale = float((e64 * y.double()).abs().sum())
        assert abs(out[j].item() - ref) <= 1e-6 * scale, (j, out[j].item(), ref)


def test_diis_error_f32_rejects_misaligned(cuda):
    x = torch.zeros(64, dtype=torch.float64, device=cuda)
    e = torch.empty(65, dtype=torch.float32, device=cuda)
    work = torch.empty(1024, dtype=torch.float64, device=cuda)
    out = torch.empty(1, dtype=torch.float64, device=cuda)
    ptrs = (C.c_void_p * 1)(0)
    with pytest.raises(_lib.EngineError, match="aligned"):
        _lib.call("pcg_diis_error_f32", x.data_ptr(), x.data_ptr(), e.data_ptr() + 4, ptrs, 1,
                  64, work.data_ptr(), work.numel(), out.data_ptr(), None)


def test_diis_fp32_errors_extrapolation(cuda):
    t1s, t2s = _sequence(40, 20001, 7, 3)          # 20041 elements: a ragged tail
    a = _run_gpu(t1s, t2s, cuda, torch.float64)
    b = _run_gpu(t1s, t2s, cuda, torch.float32)
    for u, v in zip(a, b):
        assert np.abs(u - v).max() < 1e-4 * np.abs(u).max()


@pytest.mark.parametrize("k,n", [(1, 1000), (3, 4099), (8, 1 << 20)])
def test_lincomb_double_float(cuda, k, n):
    """sum_j c_j x_j in double-float arithmetic against the FP64 sum: within 1e-13 of
    sum_j |c_j x_j|, over magnitudes from 1e-12 to 1e6, signed zeros and DIIS-like
    coefficients of both signs."""
    g = torch.Generator(device=cuda).manual_seed(k * 7 + n)
    xs = []
    for j in range(k):
        x = torch.randn(n, generator=g, dtype=torch.float64, device=cuda)
        x *= torch.exp2(torch.randint(-40, 20, (n,), generator=g, device=cuda).double())
        x[:4] = torch.tensor([0.0, -0.0, 1.0, -3.0], dtype=torch.float64)
        xs.append(x)
    c = np.array([(-1.0) ** j * (1.5 + j) for j in range(k)]) / k
    out = torch.empty(n, dtype=torch.float64, device=cuda)
    ptrs = (C.c_void_p * k)(*[x.data_ptr() for x in xs])
    coef = (C.c_double * k)(*[float(v) for v in c])
    _lib.call("pcg_lincomb_f64_df", ptrs, coef, k, n, out.data_ptr(), None)
    torch.cuda.synchronize()
    ref = sum(float(c[j]) * xs[j] for j in range(k))
    scale = sum(abs(float(c[j])) * xs[j].abs() for j in range(k))
    assert torch.all((out - ref).abs() <= 1e-13 * scale)
