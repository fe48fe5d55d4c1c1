"""The C-ABI library loads and exports every symbol declared in include/ag2.h
(no GPU calls)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(REPO, "include", "ag2.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ag2_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import build

    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    assert "ag2_forces" in names and "ag2_build_tree" in names and len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_symbol():
    import ag2

    assert sorted(ag2.EXPORTS) == declared()


def test_default_params(lib):
    import ag2

    p = ag2.Params()
    ag2.load().ag2_default_params(ctypes.byref(p))
    assert p.G == 1.0 and p.theta == 0.5 and p.split_threshold == 100 and p.precision == ag2.PREC_FP32


def test_host_io_layout_matches_header(tmp_path):
    """ag2.py's ctypes mirror of ag2_host_io has the C struct's size and field
    offsets (gcc on the header, no GPU)."""
    import shutil
    import subprocess

    import ag2

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in ag2._HostIO._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "ag2.h"\nint main(void) {\n'
                   '    printf("%zu\\n", sizeof(ag2_host_io));\n' +
                   "".join(f'    printf("%zu\\n", offsetof(ag2_host_io, {f}));\n' for f in fields) +
                   "    return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I" + os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got[0] == ctypes.sizeof(ag2._HostIO)
    assert got[1:] == [getattr(ag2._HostIO, f).offset for f in fields]
