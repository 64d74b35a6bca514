"""The C-ABI's error behaviour, on CPU: every entry point that takes device pointers rejects
null pointers (and the other arguments it cannot use) before it touches CUDA, returns a
non-zero code and leaves a message that names it in ``pcg_last_error()``.
"""
import ctypes as C

import pytest
import torch

from pycc_gb300 import _lib

# The calls below hand the library null or made-up device addresses on purpose.  They run on
# hosts without a GPU only: there, an entry point that lacked a check could not reach a
# device at all, while on a GPU host it would launch a kernel on those addresses.
pytestmark = pytest.mark.skipif(torch.cuda.is_available(),
                                reason="host-side argument checks, run without a GPU")

# entry points without device pointers, or whose job is a CUDA call
PLUMBING = {"pcg_last_error", "pcg_abi_version", "pcg_launch_count", "pcg_device_cc",
            "pcg_stream_sync", "pcg_tc_group_desc_size", "pcg_triples_part_len",
            "pcg_set_wait_limit_ns"}
# argument values of the "plausible sizes, null pointers" call, by ctypes type
DEFAULTS = {C.c_int: 1, C.c_longlong: 4, C.c_double: 1.0}


@pytest.fixture(scope="module")
def lib():
    from pycc_gb300 import build
    build.build()
    return _lib.load()


def null_call_args(argtypes):
    return [DEFAULTS.get(t) for t in argtypes]      # pointers and arrays -> None


@pytest.mark.parametrize("name", sorted(set(_lib.SIGNATURES) - PLUMBING))
def test_null_pointers_rejected(lib, name):
    restype, argtypes = _lib.SIGNATURES[name]
    rc = getattr(lib, name)(*null_call_args(argtypes))
    assert rc != 0
    msg = lib.pcg_last_error().decode()
    assert msg.startswith(name.replace("_noalloc", "")) or msg.startswith(name), msg


def test_size_limits(lib):
    """Sizes the kernels cannot index: o^2 v^2 >= 2^31 for the amplitude kernels, more
    than 16 vectors for the DIIS kernels, an unknown GEMM format, k above the fixed scratch
    of the allocation-free overlaps."""
    p = C.c_void_p(16)                                # never dereferenced on these paths
    big = 216                                         # 216^4 > 2^31
    assert lib.pcg_symmetrize_f64(p, big, big, C.c_void_p(32), None) != 0
    assert b"2^31" in lib.pcg_last_error()
    assert lib.pcg_tau_f64(p, p, big, big, 1.0, 1.0, C.c_void_p(32), None) != 0
    ptrs = (C.c_void_p * 17)(*([16] * 17))
    coef = (C.c_double * 17)(*([0.1] * 17))
    assert lib.pcg_lincomb_f64(ptrs, coef, 17, 8, C.c_void_p(64), None) != 0
    assert b"k=17" in lib.pcg_last_error()
    assert lib.pcg_lincomb_f64_df(ptrs, coef, 17, 8, C.c_void_p(64), None) != 0
    assert lib.pcg_dots_f64_noalloc(p, ptrs, 9, 8, C.c_void_p(64), None) != 0
    assert b"k=9" in lib.pcg_last_error()
    z = (C.c_longlong * 4)(1, 1, 1, 1)
    assert lib.pcg_tc_gemm(9, p, p, p, 4, 64, p, p, p, 4, 64, 64, None, None, 1, z, z, 1, z, z,
                           None, None, 1.0, 0.0, C.c_void_p(64), C.c_void_p(64), None) != 0
    assert b"unknown format 9" in lib.pcg_last_error()


def test_misaligned_vectors_rejected(lib):
    """The 16-byte vector paths refuse unaligned pointers instead of faulting."""
    ptrs = (C.c_void_p * 2)(16, 24)                   # the second is 8-byte aligned only
    coef = (C.c_double * 2)(0.5, 0.5)
    assert lib.pcg_lincomb_f64_df(ptrs, coef, 2, 8, C.c_void_p(64), None) != 0
    assert b"aligned" in lib.pcg_last_error()
    work = C.c_void_p(128)
    assert lib.pcg_diis_error_f32(C.c_void_p(16), C.c_void_p(32), C.c_void_p(52), None, 1, 8,
                                  work, 4096, C.c_void_p(256), None) != 0
    assert b"aligned" in lib.pcg_last_error()
