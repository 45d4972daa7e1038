"""Gray partial-bounce-back lattice and its adjoint (ctypes side of the
ps_gray_* entry points of include/porescale.h).

Single-phase D3Q19 TRT on a dense periodic box whose voxels carry a solid
fraction s in [0, 1] (partial bounce-back, Walsh, Burwinkle & Saar 2009);
``GrayLattice.gradient`` returns the permeability and its derivative with
respect to every voxel's s by the discrete adjoint with checkpointing.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr


class GrayParams(C.Structure):
    _fields_ = [("tau", C.c_double), ("magic", C.c_double), ("F", C.c_double * 3), ("idir", C.c_int32),
                ("nsteps", C.c_int32), ("segment", C.c_int32), ("reserved", C.c_int32)]


_SIGS = {
    "ps_gray_create": (C.c_int, [C.POINTER(GrayParams), C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "ps_gray_destroy": (C.c_int, [C.c_void_p]),
    "ps_gray_set_field": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ps_gray_permeability": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ps_gray_gradient": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ps_gray_get_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
}
_lib.SIGNATURES.update(_SIGS)


def gray_params(tau=1.0, magic=3.0 / 16.0, F=(1e-6, 0.0, 0.0), idir=1, nsteps=4000, segment=200) -> GrayParams:
    return GrayParams(tau, magic, (C.c_double * 3)(*F), idir, nsteps, segment, 0)


class GrayLattice:
    """Gray lattice of shape (nz, ny, nx) on the current CUDA device."""

    def __init__(self, params: GrayParams, shape):
        lib = _lib.library()
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        nz, ny, nx = shape
        h = C.c_void_p()
        check(lib.ps_gray_create(C.byref(params), nx, ny, nz, C.byref(h)))
        self._lib, self._h, self.params, self.shape = lib, h, params, (nz, ny, nx)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ps_gray_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_field(self, s: np.ndarray) -> None:
        s = np.ascontiguousarray(s, np.float64)
        assert s.shape == self.shape
        check(self._lib.ps_gray_set_field(self._h, dptr(s)))

    def permeability(self) -> float:
        k = C.c_double()
        check(self._lib.ps_gray_permeability(self._h, C.byref(k)))
        return k.value

    def gradient(self):
        """(k, dk/ds shaped (nz, ny, nx))."""
        k = C.c_double()
        g = np.zeros(self.shape)
        check(self._lib.ps_gray_gradient(self._h, C.byref(k), dptr(g)))
        return k.value, g

    def state(self) -> np.ndarray:
        f = np.zeros((int(np.prod(self.shape)), 19))
        check(self._lib.ps_gray_get_state(self._h, dptr(f)))
        return f

