"""The C-ABI library loads and exports every symbol the public header
declares (no device calls: this runs without a GPU)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "mrfmap_gb300.h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(mrf_[a-z0-9_]+)\s*\(", txt))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("mrf_create", "mrf_add_view", "mrf_infer", "mrf_likelihood", "mrf_read_bricks",
                 "mrf_destroy", "mrf_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(native_lib):
    from mrfmap_gb300 import lib
    for name in sorted(declared_symbols()):
        assert hasattr(native_lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert declared_symbols() <= exported
    assert set(lib.EXPORTS) == declared_symbols()


def test_create_rejects_bad_params(native_lib):
    """Argument validation happens before any device call."""
    import ctypes as C

    from mrfmap_gb300 import lib
    from mrfmap_gb300.params import MapParams
    p = MapParams(res=0.05, dims=(2.0, 2.0, 2.0), rows=4, cols=4, fx=4, fy=4, cx=2, cy=2)
    s, keep = lib.make_params(p)
    s.res = -1.0
    h = C.c_void_p()
    assert native_lib.mrf_create(C.byref(s), C.byref(h)) == 1
    assert b"invalid" in native_lib.mrf_last_error()
    assert native_lib.mrf_infer(None, None, 0, 1, 0) == 1


def test_ctypes_structs_match_the_header(tmp_path):
    """lib.py's ctypes mirrors of mrf_params and mrf_stats have the header's
    layout: a C compiler reports every field's offset and each struct's
    size, which must equal ctypes' (a field added to one side only moves an
    offset or the size)."""
    import ctypes as C

    from mrfmap_gb300 import lib
    structs = (("mrf_params", lib.mrf_params), ("mrf_stats", lib.mrf_stats))
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "mrfmap_gb300.h"', "int main(void) {"]
    for cname, cls in structs:
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, fname, v = line.split()
        got[(cname, fname)] = int(v)
    for cname, cls in structs:
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, f"{cname}.{fname}"
