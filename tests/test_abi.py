"""CPU tests of the drop-in boundary: the C-ABI library builds, loads without a GPU and
exports every entry point include/chefsi.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "chefsi.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(chefsi_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from dftfe_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    assert "chefsi_solve" in syms and "chefsi_hx" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_lists_every_export():
    from dftfe_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.EXPORTS)


def test_host_only_entry_points(lib):
    from dftfe_gb300 import _lib
    l = _lib.load()
    assert b"sm_103a" in l.chefsi_version()
    assert l.chefsi_chebyshev_order(400.0) == 24
    assert l.chefsi_chebyshev_order(1.0e9) == 1250
    # null handles are rejected with a status, not a crash
    assert l.chefsi_operator_create(None, None) == _lib.CHEFSI_ERR_INVALID
    assert b"null" in l.chefsi_last_error()


@pytest.mark.parametrize("compiler,flags", [("gcc", ["-std=c99", "-x", "c"]),
                                            ("g++", ["-std=c++17", "-x", "c++"])])
def test_header_compiles_and_links_from_c_and_cpp(lib, tmp_path, compiler, flags):
    """include/chefsi.h from a C99 and a C++17 consumer (tests/abi/consumer.c): compiled with
    -Wall -Werror, linked against the library, and run for its host-side calls."""
    import shutil
    import subprocess
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not installed")
    libdir = os.path.dirname(lib._name)
    exe = tmp_path / f"consumer_{compiler}"
    cmd = [compiler, *flags, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi", "consumer.c"), "-x", "none", "-o", str(exe),
           "-L", libdir, "-lchefsi_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    ver, m, rejected, _ = out.strip().split("|")
    assert "sm_103a" in ver and m == "24" and rejected == "1"


def test_cpp_host_layer_compiles_links_and_runs(lib, tmp_path):
    """include/chefsi.hpp (the C++ host layer shaped like DFT-FE's operator and solver classes)
    from a C++17 consumer: -Wall -Wextra -Werror, linked against the library, host logic run."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not installed")
    libdir = os.path.dirname(lib._name)
    exe = tmp_path / "consumer_cpp"
    cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi", "consumer.cpp"), "-o", str(exe),
           "-L", libdir, "-lchefsi_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert "empty operator" in out and "failures=0" in out
