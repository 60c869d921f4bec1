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


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "nrgb300.h"

/* A C caller of the boundary: geometry validation and workspace sizing run
 * on the host, so this needs no GPU. */
int main(void) {
    nr_geom g;
    nr_ostr_params p;
    size_t bytes = 0;
    memset(&g, 0, sizeof g);
    memset(&p, 0, sizeof p);
    g.nx = 256; g.ny = 128; g.nz = 24;
    g.vx = 0.4f; g.vy = 0.4f; g.vz = 1.0f;
    g.x_p0 = -51.2f; g.y_p0 = -51.2f; g.z_p0 = 0.0f;
    g.nbx = 320; g.nby = 160; g.bx = 0.4f; g.by = 0.4f;
    g.x_d0 = -64.0f; g.y_d0 = -64.0f;
    g.detectorR = 20.0f; g.sourceR = 640.0f; g.sourceY = 0.0f;
    g.n_angles = 9;
    p.subset_num = 9; p.potential = NR_POT_HYPERBOLA; p.beta = 50.0f; p.delta = 0.002f;
    printf("version %s\n", nr_version());
    printf("valid %d\n", (int)nr_validate_geometry(&g, 9));
    printf("bad_subsets %d\n", (int)nr_validate_geometry(&g, 4));
    printf("ws_status %d\n", (int)nr_ostr_workspace_size(&g, &p, &bytes));
    printf("ws_bytes %zu\n", bytes);
    p.upd_tile = NR_TILE_2;
    printf("ws_tile2 %d\n", (int)nr_ostr_workspace_size(&g, &p, &bytes));
    return 0;
}
"""


def test_a_c_program_links_and_calls_the_library(tmp_path, native_lib_path):
    """Compiled with gcc against the header and linked to libnrgb300.so: the
    host-side entry points answer as they do through ctypes."""
    from newrecon_gb300.geometry import Geometry, NrOstrParams

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no gcc")
    src, exe = tmp_path / "caller.c", tmp_path / "caller"
    src.write_text(C_CALLER)
    libdir = os.path.dirname(native_lib_path)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", INCLUDE, str(src), "-o", str(exe),
                        "-L", libdir, "-lnrgb300", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    vals = dict(ln.split(" ", 1) for ln in out.splitlines())
    assert "sm_103a" in vals["version"]
    assert vals["valid"] == "0" and vals["bad_subsets"] != "0"
    assert vals["ws_status"] == "0" and vals["ws_tile2"] == "0"
    # the same size through the Python binding
    from newrecon_gb300 import native

    g = Geometry(256, 128, 24, 0.4, 0.4, 1.0, -51.2, -51.2, 0.0, 320, 160, 0.4, 0.4, -64.0,
                 -64.0, 20.0, 640.0, 0.0, 9)
    gc = g.to_c()
    p = NrOstrParams(9, 2, 0, 0, 50.0, 0.002)
    size = ctypes.c_size_t(0)
    assert native.load(native_lib_path).nr_ostr_workspace_size(
        ctypes.byref(gc), ctypes.byref(p), ctypes.byref(size)) == 0
    assert int(vals["ws_bytes"]) == size.value
