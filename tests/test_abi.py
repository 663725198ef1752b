"""The C-ABI library loads (no GPU needed) and exports every entry point
include/fsph.h declares; the ctypes mirror matches the header layout."""
import ctypes as C
import os
import re

import pytest

from flecsph_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fsph.h")).read()
    return sorted(set(re.findall(r"\b(fsph_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return C.CDLL(build.LIB)


def test_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version(lib):
    lib.fsph_abi_version.restype = C.c_int32
    assert lib.fsph_abi_version() == 1


def test_params_defaults_match_header(lib):
    p = abi.Params()
    lib.fsph_params_default(C.byref(p))
    q = abi.Params.defaults()
    for name, _ in abi.Params._fields_:
        if name == "reserved":
            continue
        assert getattr(p, name) == getattr(q, name), name


def test_struct_sizes():
    # fsph_soa_view: n + 29 double pointers + id + key
    assert C.sizeof(abi.SoAView) == 8 * 32
    assert C.sizeof(abi.Conserved) == 8 * 8


def test_create_without_device_fails_cleanly(lib):
    """On a host without a GPU fsph_create must return NULL with a status,
    never crash; on a GPU host it succeeds."""
    lib.fsph_create.restype = C.c_void_p
    lib.fsph_create.argtypes = [C.POINTER(abi.Params), C.c_int32, C.c_int64,
                                C.POINTER(C.c_int)]
    st = C.c_int(-1)
    p = abi.Params.defaults()
    ctx = lib.fsph_create(C.byref(p), 0, 1024, C.byref(st))
    if ctx:
        lib.fsph_destroy.argtypes = [C.c_void_p]
        lib.fsph_destroy(ctx)
        assert st.value == 0
    else:
        assert st.value in (abi.STATUS_NAMES and 13, 2)


def test_bad_params_rejected(lib):
    lib.fsph_create.restype = C.c_void_p
    lib.fsph_create.argtypes = [C.POINTER(abi.Params), C.c_int32, C.c_int64,
                                C.POINTER(C.c_int)]
    st = C.c_int(-1)
    p = abi.Params.defaults(dimension=5)
    assert not lib.fsph_create(C.byref(p), 0, 1024, C.byref(st))
    assert st.value == 1
