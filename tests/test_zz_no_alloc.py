"""The allocation-free overlap entry point, pcg_dots_f64_noalloc.

It exists for host programs that cannot give the library device scratch (they own all
device memory, or must avoid cudaMalloc's implicit synchronisation): its partial sums live
in a fixed array inside the library.  Checked here through the C ABI against the regular
pcg_dots_f64 (caller-provided work buffer) and, independently of both, against torch's FP64
dot products, on two calls in a row, with different inputs and vector counts, so the second
call runs on the array the first one left behind.  This file is collected last.
"""
import ctypes as C

import pytest
import torch

from pycc_gb300 import _lib

pytestmark = pytest.mark.gpu
RTOL = 1e-12      # the FP64 tolerance of the engine's other tests


def _dots_regular(lib, x, ys, work, out, st):
    ptrs = (C.c_void_p * len(ys))(*[y.data_ptr() for y in ys])
    rc = lib.pcg_dots_f64(x.data_ptr(), ptrs, len(ys), x.numel(), work.data_ptr(), work.numel(),
                          out.data_ptr(), st)
    assert rc == 0, lib.pcg_last_error()


def _dots_noalloc(lib, x, ys, out, st):
    ptrs = (C.c_void_p * len(ys))(*[y.data_ptr() for y in ys])
    rc = lib.pcg_dots_f64_noalloc(x.data_ptr(), ptrs, len(ys), x.numel(), out.data_ptr(), st)
    assert rc == 0, lib.pcg_last_error()


def test_noalloc_matches_regular_two_calls(cuda):
    lib = _lib.load()
    st = _lib.stream_handle()
    g = torch.Generator(device=cuda).manual_seed(2024)
    work = torch.empty(16 * 1024, dtype=torch.float64, device=cuda)
    for k, n in ((3, 1_000_003), (8, 2_500_000)):
        x = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
        ys = [torch.randn(n, dtype=torch.float64, device=cuda, generator=g) for _ in range(k)]
        ref = torch.empty(k, dtype=torch.float64, device=cuda)
        got = torch.full((k,), float("nan"), dtype=torch.float64, device=cuda)
        _dots_regular(lib, x, ys, work, ref, st)
        _dots_noalloc(lib, x, ys, got, st)
        torch.cuda.synchronize()
        assert torch.allclose(got, ref, rtol=RTOL, atol=RTOL * ref.abs().max().item()), (k, got, ref)
        # an independent FP64 reference: torch's dot products of the same vectors
        tdot = torch.stack([torch.dot(x, y) for y in ys])
        scale = max(float(torch.linalg.norm(x)) * max(float(torch.linalg.norm(y)) for y in ys), 1.0)
        assert (got - tdot).abs().max().item() < RTOL * scale, (k, got, tdot)


def test_noalloc_rejects_too_many_vectors(cuda):
    lib = _lib.load()
    x = torch.zeros(16, dtype=torch.float64, device=cuda)
    ys = [x] * 9
    ptrs = (C.c_void_p * 9)(*[y.data_ptr() for y in ys])
    out = torch.zeros(9, dtype=torch.float64, device=cuda)
    rc = lib.pcg_dots_f64_noalloc(x.data_ptr(), ptrs, 9, 16, out.data_ptr(), _lib.stream_handle())
    assert rc != 0
    assert b"k=9" in lib.pcg_last_error()
