"""CPU checks of the C ABI: the library loads without a GPU and exports
every entry point declared in include/porescale.h (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "porescale.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(ps_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from porescale_gb300 import _build
    _build.build_gpu()
    return ctypes.CDLL(os.path.join(ROOT, "porescale_gb300", "libporescale_gpu.so"))


def test_header_declares_entry_points():
    names = _declared()
    for must in ("ps_lbm_create", "ps_lbm_step", "ps_lbm_observables", "ps_lsm_create", "ps_lsm_solve",
                 "ps_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_without_gpu(lib):
    lib.ps_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.ps_version()
    buf = ctypes.create_string_buffer(64)
    assert lib.ps_last_error(buf, 64) == 0


def test_python_bindings_cover_header():
    from porescale_gb300 import _lib, gray, springs  # noqa: F401  (these register their signatures)
    missing = [n for n in _declared() if n not in _lib.SIGNATURES]
    assert not missing, missing
