"""The C-ABI library builds, loads without a GPU and exports every declared entry point."""
import ctypes
import os
import re

import pytest

from pycc_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "pycc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcg_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from pycc_gb300 import build
    build.build()
    return _lib.load()


def test_header_matches_binding():
    assert declared() == sorted(_lib.exported_symbols())


def test_library_exports_all(lib):
    for name in declared():
        assert hasattr(lib, name), name
    raw = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared():
        getattr(raw, name)


def test_abi_version(lib):
    assert lib.pcg_abi_version() == 2


@pytest.mark.skipif(__import__("torch").cuda.is_available(),
                    reason="hands the library null pointers; host-side checks, run without a GPU")
def test_argument_errors_without_gpu(lib):
    # host-side validation happens before any CUDA call
    n = (ctypes.c_longlong * 1)(5)
    rc = lib.pcg_contract_f64(5, n, n, n, 0, n, n, n, 0, n, n, n, 1.0, None, None, 0.0, None, None)
    assert rc != 0
    assert b"sub-indices" in lib.pcg_last_error()
    rc = lib.pcg_dots_f64(None, None, 0, 10, None, 0, None, None)
    assert rc != 0
    assert b"k=0" in lib.pcg_last_error()


def test_entry_point_model_matches_the_abi():
    """The CPU tests' numpy model of the entry points (tests/abi_model.py) takes the same
    arguments as each entry point's ctypes signature, so host-logic tests call it exactly
    as they would call the library."""
    import inspect
    import abi_model
    modelled = 0
    for name, (_res, argtypes) in _lib.SIGNATURES.items():
        fn = getattr(abi_model.ABIModel, name[4:], None)
        if fn is None:
            continue
        params = list(inspect.signature(fn).parameters)[1:]        # drop self
        assert len(params) == len(argtypes), (name, len(params), len(argtypes))
        modelled += 1
    assert modelled >= 15
