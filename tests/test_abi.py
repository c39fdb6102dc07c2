"""The C ABI library loads on a CPU-only host and exports every entry point include/awigner.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "awigner.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(aw_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from accuratewigner_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "aw_create" in names and "aw_propagate" in names and len(names) >= 30


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(lib):
    from accuratewigner_gb300 import _lib

    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(_declared()) <= bound, sorted(set(_declared()) - bound)


def test_version_and_error_channel(lib):
    assert lib.aw_version() >= 1
    # a null config is rejected without touching the GPU
    import ctypes

    h = ctypes.c_void_p()
    assert lib.aw_create(None, ctypes.byref(h)) == -1
    assert b"null" in lib.aw_last_error()


def test_classes_reject_bad_arguments_like_the_reference():
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    with pytest.raises(AttributeError, match="X_gridDIM"):
        WignerMoyalCUDA1D(P_gridDIM=64, X_amplitude=1.0, P_amplitude=1.0, V="X", K="P", dt=0.1)
    with pytest.raises(AssertionError, match="power of two"):
        WignerMoyalCUDA1D(X_gridDIM=100, P_gridDIM=64, X_amplitude=1.0, P_amplitude=1.0, V="X", K="P", dt=0.1)
    with pytest.raises(AttributeError, match="dt"):
        WignerMoyalCUDA1D(X_gridDIM=64, P_gridDIM=64, X_amplitude=1.0, P_amplitude=1.0, V="X", K="P")


def test_header_compiles_as_c_and_the_library_serves_a_c_caller(lib, tmp_path):
    """tests/c_abi_check.c: a C99 program against include/awigner.h, linked to libawigner.so."""
    import shutil
    import subprocess

    from accuratewigner_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "c_abi_check")
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_abi_check.c"), "-o", exe, "-L" + libdir, "-l:libawigner.so",
                    "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    assert "valid configuration: 0" in r.stdout


def test_noalloc_argument_checks_need_no_device(lib):
    """aw_reduce_noalloc rejects bad arguments before any CUDA call: an oversized input, an unknown
    mode and a trace whose last index (n - 1) * stride overflows 64 bits."""
    import ctypes

    from accuratewigner_gb300 import _lib

    p = ctypes.c_void_p(16)  # never dereferenced: every call below fails its argument checks
    assert lib.aw_reduce_noalloc(p, 16, 67108864 + 1, 0, 0, p, None) == _lib.AW_E_ARG
    assert b"67108864" in lib.aw_last_error()
    assert lib.aw_reduce_noalloc(p, 16, 8, 0, 4, p, None) == _lib.AW_E_ARG
    assert lib.aw_reduce_noalloc(p, 12, 8, 0, 0, p, None) == _lib.AW_E_ARG
    assert lib.aw_reduce_noalloc(p, 16, 3, 2 ** 62, 3, p, None) == _lib.AW_E_ARG
    assert b"overflows" in lib.aw_last_error()
    assert lib.aw_reduce_noalloc(p, 16, 3, 0, 3, p, None) == _lib.AW_E_ARG
