"""The C ABI used from C and C++ directly (no Python in between): the header compiles as C99,
a C++ client links against libprgpu.so, and (on the GPU) the client's checks pass."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(REPO, "include")
PKG = os.path.join(REPO, "poissonrecon_gpu_gb300")
CLIENT = os.path.join(REPO, "tests", "cpp", "api_client.cpp")


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "use.c"
    src.write_text('#include "prgpu.h"\n'
                   'int use(void* ctx) {\n'
                   '    prgpu_params p; prgpu_mesh m; prgpu_node_arrays na;\n'
                   '    prgpu_params_default(&p); (void)m; (void)na;\n'
                   '    return prgpu_solve_depth(ctx, 0, PRGPU_SOLVE_REFERENCE);\n'
                   '}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", INC, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_python_params_layout_matches_header(tmp_path):
    """The ctypes mirror of prgpu_params has the C struct's size and field offsets."""
    import ctypes
    from poissonrecon_gpu_gb300 import Params
    fields = [f[0] for f in Params._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "prgpu.h"\n'
                   'int main(void) {\n    printf("%zu\\n", sizeof(prgpu_params));\n' +
                   "".join('    printf("%%zu\\n", offsetof(prgpu_params, %s));\n' % f for f in fields) +
                   '    return 0;\n}\n')
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", INC, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert got[0] == ctypes.sizeof(Params)
    assert got[1:] == [getattr(Params, f).offset for f in fields]


def _build_client(lib_built, out):
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-Wall", "-I", INC, CLIENT, "-o", str(out), "-L", PKG, "-lprgpu",
                        "-Wl,-rpath," + PKG], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_client_links(lib_built, tmp_path):
    assert os.path.exists(_build_client(lib_built, tmp_path / "api_client"))


@pytest.mark.gpu
def test_cpp_client_runs(lib_built, tmp_path):
    exe = _build_client(lib_built, tmp_path / "api_client")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
