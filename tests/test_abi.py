"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/edward_gb300.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "edward_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(edg_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from edward_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    assert "edg_hmc_glm_run" in names and "edg_klqp_glm_step" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from edward_gb300 import _lib
    assert set(declared()) <= set(_lib.exported_symbols())


def test_abi_version_and_null_checks(lib):
    lib.edg_abi_version.restype = ctypes.c_int
    assert lib.edg_abi_version() == 1
    lib.edg_last_error_string.restype = ctypes.c_char_p
    lib.edg_glm_logjoint_grad.restype = ctypes.c_int
    rc = lib.edg_glm_logjoint_grad(None, None, 1, 1, ctypes.c_float(1.0), None, None, None,
                                   ctypes.c_size_t(0), None)
    assert rc == -1  # EDG_E_NULL, raised before any CUDA call
    assert b"NULL" in lib.edg_last_error_string()


def test_library_targets_sm103a():
    """The build uses exactly one -gencode, for sm_103a."""
    from edward_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
