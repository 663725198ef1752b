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
    assert lib.fsph_abi_version() == 6


def test_params_defaults_match_header(lib):
    p = abi.Params()
    lib.fsph_params_default(C.byref(p))
    q = abi.Params.defaults()
    for name, _ in abi.Params._fields_:
        if name in ("reserved", "reserved_pad2"):
            continue
        a, b = getattr(p, name), getattr(q, name)
        if name == "external_force":
            a, b = list(a), list(b)
        assert a == b, name


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
        'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(fsph_params), '
        'offsetof(fsph_params, sph_viscosity_delta), '
        'offsetof(fsph_params, external_force), '
        'offsetof(fsph_params, relaxation_repulsion_gamma), sizeof(fsph_soa_view), '
        'offsetof(fsph_soa_view, ddivvdt), offsetof(fsph_soa_view, key)); return 0; }\n')
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [C.sizeof(abi.Params), abi.Params.sph_viscosity_delta.offset,
            abi.Params.external_force.offset, abi.Params.relaxation_repulsion_gamma.offset,
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


@pytest.mark.parametrize("spec,codes", [
    ("none", []), ("Zero", []),
    ("spherical wall,walls:xyz,gravity",
     [abi.EFORCE_SPHERICAL_WALL, abi.EFORCE_WALLS_X, abi.EFORCE_WALLS_Y,
      abi.EFORCE_WALLS_Z, abi.EFORCE_GRAVITY]),
    ("Airfoil,ORBIT,poison,Spherical Density Support",
     [abi.EFORCE_AIRFOIL, abi.EFORCE_ORBIT, abi.EFORCE_POISON,
      abi.EFORCE_SPHERICAL_DENSITY_SUPPORT]),
    ("walls:zY", [abi.EFORCE_WALLS_Z, abi.EFORCE_WALLS_Y]),
    ("walls:xyzx", [abi.EFORCE_WALLS_X, abi.EFORCE_WALLS_Y, abi.EFORCE_WALLS_Z]),
])
def test_external_force_select(lib, spec, codes):
    """external_force::select's grammar (eforce.h:359-434): comma-separated
    terms in order, case-insensitive, at most three wall axes per term."""
    lib.fsph_params_set_external_force.argtypes = [C.POINTER(abi.Params), C.c_char_p]
    p = abi.Params.defaults()
    assert lib.fsph_params_set_external_force(C.byref(p), spec.encode()) == 0
    assert p.forces() == codes


@pytest.mark.parametrize("spec", ["gravity, poison", "walls:q", "walls", "wall",
                                  "gravity,gravity,gravity,gravity,gravity,gravity,gravity,gravity,gravity"])
def test_external_force_select_rejects(lib, spec):
    lib.fsph_params_set_external_force.argtypes = [C.POINTER(abi.Params), C.c_char_p]
    p = abi.Params.defaults()
    assert lib.fsph_params_set_external_force(C.byref(p), spec.encode()) == 1
