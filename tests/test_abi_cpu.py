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


def test_fortran_module_binds_every_entry_point():
    """The ISO_C_BINDING module (no Fortran compiler on this machine, so read
    as text) binds exactly the entry points the header declares, each under
    its own name, in lines within the free-form limit of 132 characters."""
    src = open(os.path.join(ROOT, "fortran", "porescale_gpu.f90")).read()
    bound = re.findall(r"function\s+(ps_\w+)\s*\([^)]*\)\s*&?\s*bind\(c,\s*name='(ps_\w+)'\)", src)
    assert all(f == c for f, c in bound), [b for b in bound if b[0] != b[1]]
    assert sorted(c for _, c in bound) == _declared()
    assert max(len(line) for line in src.splitlines()) <= 132


def _c_structs():
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "porescale.h")).read(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(ps_\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in filter(None, (d.strip() for d in body.split(";"))):
            ctype, rest = decl.split(None, 1)
            for v in rest.split(","):
                m = re.fullmatch(r"\s*(\w+)\s*(?:\[(\d+)\])?\s*", v)
                fields.append((ctype, m.group(1).lower(), int(m.group(2) or 1)))
        out[name] = fields
    return out


def _fortran_types():
    src = open(os.path.join(ROOT, "fortran", "porescale_gpu.f90")).read()
    kinds = {"c_double": "double", "c_int32_t": "int32_t", "c_int64_t": "int64_t"}
    out = {}
    for name, body in re.findall(r"type, bind\(c\) :: (ps_\w+)\n(.*?)\n\s*end type", src, flags=re.S):
        fields = []
        for line in body.splitlines():
            m = re.fullmatch(r"\s*(?:real|integer)\((\w+)\) :: (.*)", line)
            for v in re.findall(r"(\w+)(?:\((\d+)\))?", m.group(2)):
                fields.append((kinds[m.group(1)], v[0].lower(), int(v[1] or 1)))
        out[name] = fields
    return out


def test_fortran_types_match_c_structs():
    """Every bind(c) derived type of the Fortran module lists the fields of
    the header's struct of the same name: same order, types and extents, so
    the two layouts agree byte for byte."""
    c, f = _c_structs(), _fortran_types()
    assert sorted(f) == sorted(c)
    for name in c:
        assert f[name] == c[name], name


def test_version_and_error_without_gpu(lib):
    lib.ps_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.ps_version()
    buf = ctypes.create_string_buffer(64)
    assert lib.ps_last_error(buf, 64) == 0


def test_python_bindings_cover_header():
    from porescale_gb300 import _lib, gray, springs  # noqa: F401  (these register their signatures)
    missing = [n for n in _declared() if n not in _lib.SIGNATURES]
    assert not missing, missing
    # and with the header's parameter count
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "porescale.h")).read(), flags=re.S)
    for name, params in re.findall(r"\b(ps_\w+)\s*\(([^)]*)\)\s*;", src):
        count = 0 if params.strip() in ("", "void") else params.count(",") + 1
        assert len(_lib.SIGNATURES[name][1]) == count, name


def test_argument_errors_and_missing_device(lib):
    """Entry points validate their arguments before touching the device and
    fail with a code and a message (never a CPU fallback): bad boxes and
    precisions are PS_ERR_ARG; on a machine without a GPU a valid lattice
    request is PS_ERR_NODEVICE."""
    import numpy as np
    from porescale_gb300 import _lib
    from porescale_gb300.lattice import make_params

    for name, (res, args) in _lib.SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    p = make_params(vir=0.1, vib=0.1, wet=0.5)
    h = ctypes.c_void_p()
    ind = np.ones((4, 4, 4), np.int32)
    ip = ind.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    assert lib.ps_lbm_create(ctypes.byref(p), ip, 1025, 4, 4, 0, ctypes.byref(h)) == 1
    assert lib.ps_lbm_create(ctypes.byref(p), ip, 4, 4, 4, 7, ctypes.byref(h)) == 1
    assert lib.ps_lbm_create(ctypes.byref(p), ip, 0, 4, 4, 0, ctypes.byref(h)) == 1
    assert lib.ps_lbm_create(None, ip, 4, 4, 4, 0, ctypes.byref(h)) == 1
    assert lib.ps_batch_create(None, 0, ctypes.byref(h)) == 1
    assert lib.ps_lbm_step(None, 1) == 1
    buf = ctypes.create_string_buffer(256)
    lib.ps_last_error(buf, 256)
    assert b"null" in buf.value
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert lib.ps_lbm_create(ctypes.byref(p), ip, 4, 4, 4, 0, ctypes.byref(h)) == 6  # PS_ERR_NODEVICE
        lib.ps_last_error(buf, 256)
        assert b"device" in buf.value
