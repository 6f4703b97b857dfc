"""CPU tests of the C-ABI library: it builds, loads without a GPU, and exports
every function ``include/gde.h`` declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

from gde import _build
from gde import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gde.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(gde_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return L.load(build_if_missing=False)


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("gde_ctx_create", "gde_graph_upload", "gde_solve", "gde_feature_push", "gde_feature_update",
                 "gde_plain_ppr_local", "gde_hk_estimate_n"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert set(declared_functions()) == set(L.SIGNATURES)


def test_status_strings_and_host_only_entry_points(lib):
    assert lib.gde_status_str(L.GDE_OK) == b"ok"
    assert lib.gde_status_str(L.GDE_EITERCAP) == b"round cap reached"
    assert lib.gde_version() >= 1
    # estimate_n is host arithmetic (hk_solver.py:28-48): compare with the oracle
    from oracle import oracle as O
    for t, e in [(1.0, 1e-3), (3.0, 1e-6), (5.0, 1e-4), (5.0, 0.5e-8), (10.0, 1e-7)]:
        assert lib.gde_hk_estimate_n(t, e) == O.hk_estimate_n(t, e)
    assert lib.gde_hk_estimate_n(0.5, 1e-3) == -1  # tau < 1 is refused (hk_solver.py:35)


def test_null_arguments_are_rejected_without_a_gpu(lib):
    out = ctypes.c_void_p()
    assert lib.gde_graph_upload(None, 10, 0, None, None, None, None, ctypes.byref(out)) == L.GDE_EINVAL
    assert lib.gde_ctx_destroy(None) == L.GDE_EINVAL
    assert lib.gde_graph_free(None) == L.GDE_EINVAL


def _struct_fields(name):
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", src).group(1)
    return re.findall(r"([a-z_0-9]+)\s*;", body)


@pytest.mark.parametrize("cname,py", [("gde_params", L.Params), ("gde_stats", L.Stats)])
def test_ctypes_structs_mirror_the_header(cname, py, tmp_path):
    """Field names, order, offsets and size of the ctypes mirrors equal the C layout (gcc)."""
    names = _struct_fields(cname)
    assert names == [f for f, _ in py._fields_]
    prog = tmp_path / "layout.c"
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gde.h"', "int main(void) {",
             f'  printf("%zu\\n", sizeof({cname}));']
    lines += [f'  printf("%zu\\n", offsetof({cname}, {f}));' for f in names]
    prog.write_text("\n".join(lines + ["  return 0;", "}"]) + "\n")
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(prog), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got[0] == ctypes.sizeof(py)
    assert got[1:] == [getattr(py, f).offset for f in names]
