"""The public header is plain C, and the Python mirrors of its structs have its
layout.  A small C program compiled against include/nrgb300.h (gcc, C99,
warnings as errors) prints the size of every struct and the offset of every
field; each ctypes mirror must give the same numbers.  No GPU and no library
call: this pins the boundary a C, Go or Python caller binds."""
import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


def mirrors():
    from newrecon_gb300.geometry import NrBatchCase, NrGeom, NrOstrParams, NrSartParams
    from newrecon_gb300.warmstart import NrCnnDims

    return {"nr_geom": NrGeom, "nr_ostr_params": NrOstrParams, "nr_sart_params": NrSartParams,
            "nr_batch_case": NrBatchCase, "nr_cnn_dims": NrCnnDims}


# ctypes field names that differ from the C ones (Python keywords)
C_NAME = {"lam": "lambda"}


def c_program():
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "nrgb300.h"',
             "int main(void) {"]
    for cname, cls in mirrors().items():
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            c = C_NAME.get(fname, fname)
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {c}));')
    lines += ["    return 0;", "}"]
    return "\n".join(lines) + "\n"


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text(c_program())
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", INCLUDE, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    table = {}
    for ln in out.splitlines():
        struct, field, value = ln.split()
        table[(struct, field)] = int(value)
    return table


def test_header_compiles_as_c99_and_cxx(tmp_path):
    """The header alone, as C99 and as C++17 (no torch or CUDA types in it)."""
    for cc, std, ext in (("gcc", "-std=c99", "c"), ("g++", "-std=c++17", "cpp")):
        exe = shutil.which(cc)
        if exe is None:
            pytest.skip(f"no {cc}")
        src = tmp_path / f"h.{ext}"
        src.write_text('#include "nrgb300.h"\nint main(void) { return NR_OK; }\n')
        r = subprocess.run([exe, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", INCLUDE,
                            "-fsyntax-only", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, (cc, r.stderr)


@pytest.mark.parametrize("cname", ["nr_geom", "nr_ostr_params", "nr_sart_params",
                                   "nr_batch_case", "nr_cnn_dims"])
def test_ctypes_mirror_matches_the_c_layout(c_layout, cname):
    cls = mirrors()[cname]
    assert ctypes.sizeof(cls) == c_layout[(cname, "sizeof")], cname
    for fname, _ in cls._fields_:
        assert getattr(cls, fname).offset == c_layout[(cname, fname)], (cname, fname)
