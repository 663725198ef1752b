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
    assert lib.fsph_abi_version() == 4


def test_params_defaults_match_header(lib):
    p = abi.Params()
    lib.fsph_params_default(C.byref(p))
    q = abi.Params.defaults()
    for name, _ in abi.Params._fields_:
        if name in ("reserved", "reserved_pad"):
            continue
        assert getattr(p, name) == getattr(q, name), name


def test_struct_sizes():
    # fsph_soa_view: n + 32 double pointers + id + key
    assert C.sizeof(abi.SoAView) == 8 * 35
    assert C.sizeof(abi.Conserved) == 8 * 8


def test_struct_layout_matches_c(tmp_path):
    """sizeof and the offsets of the last fields, as the C compiler lays
    the header out, equal the ctypes mirror's."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "fsph.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(fsph_params), '
        'offsetof(fsph_params, sph_viscosity_delta), sizeof(fsph_soa_view), '
        'offsetof(fsph_soa_view, ddivvdt), offsetof(fsph_soa_view, key)); return 0; }\n')
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [C.sizeof(abi.Params), abi.Params.sph_viscosity_delta.offset,
            C.sizeof(abi.SoAView), abi.SoAView.ddivvdt.offset, abi.SoAView.key.offset]
    assert got == want


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
