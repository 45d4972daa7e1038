"""The lattice-spring static solve behind the C ABI (ps_lsm_*).

Mirrors the standalone drivers LSM2S/Cxxxx/XX_P.f (x stretch, Cxxxx) and
LSM2S/Cyzyz/YZ_P.f (yz shear, Cyzyz): build the two-solid spring network from
``ind`` (0 solid phase 1, 3 solid phase 2), impose the tied-face jump 2g,
solve for static equilibrium and report the effective modulus of
calc_stress.  The reference relaxes with damped Verlet dynamics; this solves
the same linear system by conjugate gradients.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr

LOAD_XSTRETCH, LOAD_YZSHEAR, LOAD_NONE = 0, 1, 2
LSM_F64, LSM_MIXED = 0, 1


class LsmParams(C.Structure):
    _fields_ = [("alf1", C.c_double), ("bet1", C.c_double), ("alf2", C.c_double), ("bet2", C.c_double),
                ("gstrain", C.c_double), ("load", C.c_int32), ("precision", C.c_int32)]


class LsmInfo(C.Structure):
    _fields_ = [("nnode", C.c_int64), ("ncube", C.c_int64), ("nvox", C.c_int64), ("nx", C.c_int32),
                ("ny", C.c_int32), ("nz", C.c_int32), ("load", C.c_int32), ("precision", C.c_int32),
                ("reserved", C.c_int32), ("device_bytes", C.c_int64)]


class LsmResult(C.Structure):
    _fields_ = [("modulus", C.c_double), ("sigma", C.c_double * 9), ("strain", C.c_double),
                ("relres", C.c_double), ("iterations", C.c_int64), ("inner_iterations", C.c_int64),
                ("nnode", C.c_int64), ("ncube", C.c_int64), ("refinements", C.c_int32), ("converged", C.c_int32)]


_SIGS = {
    "ps_lsm_create": (C.c_int, [C.POINTER(LsmParams), C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.c_int32,
                                C.POINTER(C.c_void_p)]),
    "ps_lsm_destroy": (C.c_int, [C.c_void_p]),
    "ps_lsm_get_info": (C.c_int, [C.c_void_p, C.POINTER(LsmInfo)]),
    "ps_lsm_solve": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.POINTER(LsmResult)]),
    "ps_lsm_get_disp": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ps_lsm_stream": (C.c_void_p, [C.c_void_p]),
    "ps_lsm_stress_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "ps_lsm_dyn_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double]),
    "ps_lsm_set_dyn_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "ps_lsm_get_dyn_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "ps_lsm_gradients": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ps_lsm_batch_solve": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_double, C.c_int32, C.POINTER(LsmResult)]),
    "ps_lsm_set_wall_load": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double]),
    "ps_lsm_alpha_beta": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.c_double,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}
_lib.SIGNATURES.update(_SIGS)


def spring_constants(Em: float, nu: float, dl: float = 1.0):
    """alpha, beta of the alpha-beta model (XX_P.f:411-414)."""
    alf = dl * Em / (5.0 - 10.0 * nu)
    bet = dl ** 3 * Em * (4 * nu - 1) / (20.0 * (2 * nu * nu + nu - 1))
    return alf, bet


class SpringNetwork:
    """Two-solid lattice-spring network on the current CUDA device."""

    def __init__(self, ind: np.ndarray, alf1, bet1, alf2, bet2, gstrain, load=LOAD_XSTRETCH, precision=LSM_F64):
        lib = _lib.library()
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        ind = np.ascontiguousarray(ind, np.int32)
        nz, ny, nx = ind.shape
        p = LsmParams(alf1, bet1, alf2, bet2, gstrain, load, precision)
        h = C.c_void_p()
        check(lib.ps_lsm_create(C.byref(p), iptr(ind), nx, ny, nz, C.byref(h)))
        self._lib, self._h, self.params = lib, h, p
        info = LsmInfo()
        check(lib.ps_lsm_get_info(h, C.byref(info)))
        self.info = info

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ps_lsm_destroy(self._h)
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

    def solve(self, rtol=1e-10, maxit=200000) -> LsmResult:
        r = LsmResult()
        rc = self._lib.ps_lsm_solve(self._h, float(rtol), int(maxit), C.byref(r))
        check(rc)
        return r

    def displacements(self, ns: int) -> np.ndarray:
        """(ns, 3) displacements in the reference node order (LSM_displ_field)."""
        u = np.zeros((ns, 3))
        check(self._lib.ps_lsm_get_disp(self._h, dptr(u)))
        return u

    def dyn_step(self, nsteps: int, dt: float = 1.0, rsi: float = 1.0, damp: float = 0.25) -> None:
        """nsteps of the coupled driver's damped spring dynamics (lsm_step,
        S1:1721-1903) under the wall load set by set_wall_load."""
        check(self._lib.ps_lsm_dyn_step(self._h, int(nsteps), float(dt), float(rsi), float(damp)))

    def set_dyn_state(self, r=None, v=None, a=None) -> None:
        """(ns, 3) arrays in the reference node order; None = zero."""
        arrs = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (r, v, a)]
        check(self._lib.ps_lsm_set_dyn_state(self._h, *[None if x is None else dptr(x) for x in arrs]))

    def dyn_state(self, ns: int):
        """(r, v, a), each (ns, 3) in the reference node order."""
        out = [np.zeros((ns, 3)) for _ in range(3)]
        check(self._lib.ps_lsm_get_dyn_state(self._h, *[dptr(x) for x in out]))
        return tuple(out)

    def gradients(self) -> np.ndarray:
        """d modulus / d(alf1, bet1, alf2, bet2) at the last converged
        solution, then the energy form of the modulus (5 values)."""
        g = np.zeros(5)
        check(self._lib.ps_lsm_gradients(self._h, dptr(g)))
        return g

    def set_wall_load(self, lattice, rsi: float = 1.0) -> None:
        """Applies the wall load of `lattice` (a Lattice on the same box) in
        the following solves; None removes it."""
        check(self._lib.ps_lsm_set_wall_load(self._h, lattice._h if lattice is not None else None, float(rsi)))

    def alpha_beta(self, lab: np.ndarray, npores: int, iipore: int, pres: float):
        """calc_ab on the last solution: (alpha[3,3], beta[npores])."""
        lab = np.ascontiguousarray(lab, np.int32)
        a = np.zeros(9)
        b = np.zeros(max(npores, 1))
        check(self._lib.ps_lsm_alpha_beta(self._h, iptr(lab), int(npores), int(iipore), float(pres), dptr(a), dptr(b)))
        return a.reshape(3, 3), b[:npores]

    @property
    def stream(self) -> int:
        return int(self._lib.ps_lsm_stream(self._h) or 0)


def batch_solve(networks, rtol=1e-10, maxit=200000):
    """Solves several SpringNetworks together (ps_lsm_batch_solve); returns
    their LsmResults in order."""
    lib = networks[0]._lib
    arr = (C.c_void_p * len(networks))(*[N._h.value for N in networks])
    res = (LsmResult * len(networks))()
    check(lib.ps_lsm_batch_solve(arr, len(networks), float(rtol), int(maxit), res))
    return list(res)
