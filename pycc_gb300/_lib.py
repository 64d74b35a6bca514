"""ctypes binding of ``libpycc_gb300.so`` (the C-ABI declared in ``include/pycc_gb300.h``).

The engine has no CPU fallback: if the shared library is missing or fails to load, every
GPU entry point raises.  Tensors cross the boundary as raw device pointers (``data_ptr()``),
element strides and sizes; streams as ``cudaStream_t`` handles.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpycc_gb300.so")

_i64 = C.c_longlong
_p = C.c_void_p
_pi64 = C.POINTER(C.c_longlong)
_d = C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "pcg_last_error": (C.c_char_p, []),
    "pcg_abi_version": (C.c_int, []),
    "pcg_launch_count": (C.c_longlong, []),
    "pcg_device_cc": (C.c_int, []),
    "pcg_stream_sync": (C.c_int, [_p]),
    "pcg_set_wait_limit_ns": (C.c_longlong, [_i64]),
    "pcg_wait_probe": (C.c_int, [_p, _p]),
    "pcg_contract_f64": (C.c_int, [C.c_int, _pi64, _pi64, _pi64, C.c_int, _pi64, _pi64, _pi64,
                                   C.c_int, _pi64, _pi64, _pi64, _d, _p, _p, _d, _p, _p]),
    "pcg_tau_f64": (C.c_int, [_p, _p, _i64, _i64, _d, _d, _p, _p]),
    "pcg_combine4_f64": (C.c_int, [_pi64, _d, _p, _pi64, _d, _p, _pi64, _p, _pi64, _p]),
    "pcg_symmetrize_f64": (C.c_int, [_p, _i64, _i64, _p, _p]),
    "pcg_update_amps_f64": (C.c_int, [_p, _p, _p, _p, _p, _i64, _i64, _p, _i64, _p, _p]),
    "pcg_inv_denominators_f64": (C.c_int, [_p, _i64, _i64, _p, _p, _p]),
    "pcg_update_inv_f64": (C.c_int, [_p, _p, _p, _i64, _p, _i64, _p, _p]),
    "pcg_energy_f64": (C.c_int, [_p, _pi64, _p, _pi64, _p, _p, _i64, _i64, _p, _i64, _p, _p]),
    "pcg_dots_f64": (C.c_int, [_p, C.POINTER(_p), C.c_int, _i64, _p, _i64, _p, _p]),
    "pcg_dots_f64_noalloc": (C.c_int, [_p, C.POINTER(_p), C.c_int, _i64, _p, _p]),
    "pcg_lincomb_f64": (C.c_int, [C.POINTER(_p), C.POINTER(_d), C.c_int, _i64, _p, _p]),
    "pcg_lincomb_f64_df": (C.c_int, [C.POINTER(_p), C.POINTER(_d), C.c_int, _i64, _p, _p]),
    "pcg_diis_error_f64": (C.c_int, [_p, _p, _p, C.POINTER(_p), C.c_int, _i64, _p, _i64, _p, _p]),
    "pcg_diis_error_f32": (C.c_int, [_p, _p, _p, C.POINTER(_p), C.c_int, _i64, _p, _i64, _p, _p]),
    "pcg_contract_multi_f64": (C.c_int, [C.c_int, C.c_int, _pi64, _pi64, _pi64, C.c_int, _pi64,
                                         _pi64, _pi64, C.POINTER(C.c_int), _pi64, _pi64, _pi64,
                                         C.POINTER(_d), C.POINTER(_p), C.POINTER(_p), _d, _p,
                                         _p]),
    "pcg_triples_energy": (C.c_int, [C.c_int, _p, _p, _p, _i64, _p, C.c_int, _p, _p, _p, _p, _p,
                                     _i64, _i64, _p, _p]),
    "pcg_triples_part_len": (C.c_longlong, [C.c_int, _i64]),
    "pcg_reduce_sum_f64": (C.c_int, [_p, _i64, _p, _p]),
    "pcg_tc_grouped_gemm": (C.c_int, [C.c_int, C.POINTER(_p), _pi64, _pi64, C.c_int, C.POINTER(_p),
                                      _pi64, _pi64, _p, C.c_int, _i64, _i64, _p, _i64, _i64, _p,
                                      _p]),
    "pcg_tc_group_desc_size": (C.c_int, []),
    "pcg_pack_operand": (C.c_int, [C.c_int, C.c_int, _pi64, _pi64, C.c_int, _pi64, _pi64, _i64,
                                   _d, _p, _d, _p, _d, _p, _p, _d, _p, _p, _p, _p, _p, _p, _p,
                                   _i64, _p, _p, _i64, _p]),
    "pcg_ladder_pm_assemble": (C.c_int, [_p, _p, _i64, _i64, _p, _p]),
    "pcg_pair_pm_assemble": (C.c_int, [_p, _p, _i64, _i64, _p, _p]),
    "pcg_t3_ijk_f64": (C.c_int, [_p, _p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _p, _p,
                                 _p, _p, _p, _p, _p]),
    "pcg_t3_density_terms_f64": (C.c_int, [_p, _p, C.c_int, _p, _p, _p, _p, _p, _p, _p]),
    "pcg_tc_gemm": (C.c_int, [C.c_int, _p, _p, _p, _i64, _i64, _p, _p, _p, _i64, _i64, _i64,
                              _p, _p, C.c_int, _pi64, _pi64, C.c_int, _pi64, _pi64, _p, _p, _d,
                              _d, _p, _p, _p]),
}

_lib = None


class EngineError(RuntimeError):
    """A C-ABI entry point of the CUDA engine reported a failure."""


def load(path: str = LIB_PATH):
    """Load the shared library (once) and attach the argument types."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise EngineError(
            "pycc_gb300 CUDA library not found at %s; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES)


def i64s(vals):
    vals = [int(x) for x in vals]
    return (C.c_longlong * max(1, len(vals)))(*vals)


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.pcg_last_error().decode(errors="replace")
        raise EngineError("%s failed (%d): %s" % (name, rc, msg))
    return rc


def set_wait_limit_ns(ns: int) -> int:
    """Bound (ns) on any single device-side wait of the tensor-core kernels launched from now
    on (<= 0 restores the 4 s default); returns the previous bound."""
    return int(load().pcg_set_wait_limit_ns(int(ns)))


def launch_count() -> int:
    """Kernels the CUDA library has launched since it was loaded."""
    return int(load().pcg_launch_count())


def stream_handle(stream=None):
    """cudaStream_t of a torch stream (default: the current stream)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
