"""The C-ABI libraries load and export every entry point their headers declare (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(eqd_\w+)\s*\(", text, flags=re.M)))


def _exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@pytest.fixture(scope="module")
def gpu_lib_path():
    from eqdyna_gb300 import build
    return build.build_gpu()[0]


def test_gpu_header_symbols_exported(gpu_lib_path):
    decl = _declared("eqdyna_gb300.h")
    assert {"eqd_gpu_init", "eqd_gpu_step", "eqd_gpu_fetch", "eqd_gpu_finalize"} <= set(decl)
    missing = set(decl) - _exported(gpu_lib_path)
    assert not missing, missing
    C.CDLL(gpu_lib_path)  # loads (links against libcudart only)


def test_case_header_symbols_exported():
    from eqdyna_gb300 import build
    lib = build.build_case()
    decl = _declared("eqdyna_case.h")
    assert len(decl) >= 6
    missing = set(decl) - _exported(lib)
    assert not missing, missing


def test_status_strings(gpu_lib_path):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    for code in range(0, 9):
        assert lib.eqd_gpu_status_string(code)
    assert lib.eqd_gpu_status_string(0) == b"ok"


def test_init_rejects_bad_input_without_touching_a_device(gpu_lib_path):
    from eqdyna_gb300 import _native as N
    lib = N.gpu_lib()
    h = C.c_void_p()
    # NULL scalars / arrays are rejected by validation before any CUDA call
    assert lib.eqd_gpu_init(None, None, None, C.byref(h)) == 1
    assert not h.value
    # step/fetch on a NULL context report "call out of order"
    assert lib.eqd_gpu_step(None, 1, 1) == 8
    assert lib.eqd_gpu_fetch(None, None) == 8
    assert lib.eqd_gpu_finalize(None) == 0


def test_product_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "eqdyna_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "liboracle" not in src or f == "build.py", f
