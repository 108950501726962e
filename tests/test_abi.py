"""CPU checks of the C ABI: the built library loads and exports every function
declared in include/fhist.h, and the Python binding covers them all.  No
compute call is made (no GPU here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(REPO, "include", "fhist.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fh_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from theses_code_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_functions():
    names = declared_functions()
    assert "fh_history_sum" in names and "fh_tg_step" in names and len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from theses_code_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.declared_symbols())


def test_version_callable_without_gpu(lib):
    lib.fh_version.restype = ctypes.c_int
    assert lib.fh_version() >= 10000


def test_ctx_create_fails_cleanly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from theses_code_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.fh_ctx_create(0, ctypes.byref(h))
    assert rc == _lib.FH_ECUDA and not h.value
    assert b"device" in L.fh_last_error(None)


def test_host_classes_compile_and_link(lib, tmp_path):
    """include/fhist.hpp compiles against the C header and the C++ host parity
    program links against the library and the oracle (it runs on a GPU in
    tests/test_gpu_host_classes.py)."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from oracle import oracle as O
    O.build()
    pkg = os.path.join(REPO, "theses_code_gb300")
    orc = os.path.join(REPO, "oracle", "_build")
    out = str(tmp_path / "host_parity")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", os.path.join(REPO, "tests", "cpp", "host_parity.cpp"),
           "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "oracle"),
           "-I", "/usr/local/cuda/include", "-L", pkg, "-lfhist", "-L", orc, "-lfh_oracle", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
