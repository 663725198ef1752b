"""The public headers compile on their own with strict warnings: `fsph.h` and
`fsph_work.h` as C99 (a caller binding the C ABI from C, cgo or another
FFI sees exactly this), `fsph_body_system.hpp` as C++17 (the drop-in for the
reference's body_system)."""
import os
import shutil
import subprocess

import pytest

INC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def _compile(tool, std, name, src, tmp_path):
    exe = shutil.which(tool)
    if exe is None:
        pytest.skip(f"no {tool}")
    f = tmp_path / name
    f.write_text(src)
    r = subprocess.run([exe, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", INC,
                        "-c", str(f), "-o", str(tmp_path / (name + ".o"))],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_headers_are_strict_c99(tmp_path):
    _compile("gcc", "-std=c99", "use_c.c",
             '#include "fsph.h"\n#include "fsph_work.h"\nint main(void) { return 0; }\n',
             tmp_path)


def test_body_system_header_is_strict_cxx17(tmp_path):
    _compile("g++", "-std=c++17", "use_cxx.cc",
             '#include "fsph_body_system.hpp"\nint main() { return 0; }\n', tmp_path)
