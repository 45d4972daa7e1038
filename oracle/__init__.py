"""ctypes wrapper of the CPU FP64 oracle (libps_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, never by the porescale_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libps_oracle.so")


class OrLbmParams(C.Structure):
    _fields_ = [("cr2", C.c_double), ("rr0", C.c_double), ("rb0", C.c_double), ("B", C.c_double),
                ("sig", C.c_double), ("vir", C.c_double), ("vib", C.c_double), ("wet", C.c_double),
                ("ee", C.c_double), ("dt", C.c_double), ("bfr", C.c_double * 3), ("bfb", C.c_double * 3),
                ("idir", C.c_int32), ("iipore", C.c_int32)]


_lib = None
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
_LP = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from porescale_gb300 import _build
            _build.build_oracle()
        L = C.CDLL(LIB_PATH)
        sig = {
            "or_lbm_create": (C.c_void_p, [C.POINTER(OrLbmParams), _IP, C.c_int, C.c_int, C.c_int]),
            "or_lbm_destroy": (None, [C.c_void_p]),
            "or_lbm_sizes": (None, [C.c_void_p, _LP]),
            "or_lbm_tables": (None, [C.c_void_p, _IP, _IP, _IP, _IP, _IP, _IP]),
            "or_lbm_init_random": (None, [C.c_void_p, C.c_double]),
            "or_lbm_set_state": (None, [C.c_void_p, _DP, _DP]),
            "or_lbm_get_state": (None, [C.c_void_p, _DP, _DP]),
            "or_lbm_fields": (None, [C.c_void_p, _DP, _DP, _DP]),
            "or_lbm_run": (None, [C.c_void_p, C.c_int, C.c_int]),
            "or_lbm_observables": (None, [C.c_void_p, _DP]),
            "or_lbm_wall_load": (None, [C.c_void_p, C.c_double, _DP]),
            "or_collision": (None, [C.c_double, C.c_double, C.c_double, _DP, _DP, C.c_double, _DP, _DP, _DP,
                                    C.c_double, C.c_double, C.c_double]),
            "or_collmatr_trt": (None, [C.c_double, _DP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_DP)


def _i(a):
    return a.ctypes.data_as(_IP)


OBS_NAMES = ["tmr", "tmb", "tm", "Cpr", "Cpb", "nr", "nb", "Qr0", "Qr1", "Qr2", "Qb0", "Qb1", "Qb2", "um0", "um1",
             "um2", "umr0", "umr1", "umr2", "umb0", "umb1", "umb2", "tfr0", "tfr1", "tfr2", "tfb0", "tfb1", "tfb2",
             "bmt0", "bmt1", "bmt2", "rmt0", "rmt1", "rmt2", "isneg", "nneg_rr", "nneg_rb", "permr", "permb",
             "nr_cf", "nb_cf"]


class OracleLattice:
    """FP64 CPU restatement of the reference LBM (see ps_oracle.h)."""

    def __init__(self, params, ind: np.ndarray):
        p = OrLbmParams()
        for name, _ in OrLbmParams._fields_:
            v = getattr(params, name)
            if name in ("bfr", "bfb"):
                for i in range(3):
                    getattr(p, name)[i] = v[i]
            else:
                setattr(p, name, v)
        ind = np.ascontiguousarray(ind, np.int32)
        nz, ny, nx = ind.shape
        self.shape = (nz, ny, nx)
        self._h = C.c_void_p(lib().or_lbm_create(C.byref(p), _i(ind), nx, ny, nz))
        s = np.zeros(6, np.int64)
        lib().or_lbm_sizes(self._h, s.ctypes.data_as(_LP))
        self.nl, self.nps, self.npb2, self.npb4, self.ns, self.n_overflow = (int(v) for v in s)

    def close(self):
        if self._h:
            lib().or_lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tables(self):
        nz, ny, nx = self.shape
        icor = np.zeros((self.nl, 3), np.int32)
        ips = np.zeros((self.nps, 3), np.int32)
        ipb2 = np.zeros((self.npb2, 4), np.int32)
        ipb4 = np.zeros((self.npb4, 6), np.int32)
        mijk = np.zeros((nz, ny, nx), np.int32)
        mijks = np.zeros((nz, ny, nx), np.int32)
        lib().or_lbm_tables(self._h, _i(icor), _i(ips), _i(ipb2), _i(ipb4), _i(mijk), _i(mijks))
        return icor, ips, ipb2, ipb4, mijk, mijks

    def init_random(self, sat):
        lib().or_lbm_init_random(self._h, sat)

    def set_state(self, fr, fb):
        fr = np.ascontiguousarray(fr, np.float64)
        fb = np.ascontiguousarray(fb, np.float64)
        lib().or_lbm_set_state(self._h, _d(fr), _d(fb))

    def get_state(self):
        fr, fb = np.empty((self.nl, 19)), np.empty((self.nl, 19))
        lib().or_lbm_get_state(self._h, _d(fr), _d(fb))
        return fr, fb

    def fields(self):
        rr, rb, cf = np.empty(self.nl), np.empty(self.nl), np.empty(self.nl)
        lib().or_lbm_fields(self._h, _d(rr), _d(rb), _d(cf))
        return rr, rb, cf

    def run(self, nsteps, nthreads=1):
        lib().or_lbm_run(self._h, int(nsteps), int(nthreads))

    def wall_load(self, rsi):
        """afdat as (ns, 3) after at least one step (S1:3849-3882)."""
        out = np.zeros((self.ns, 3))
        lib().or_lbm_wall_load(self._h, float(rsi), _d(out))
        return out

    def observables(self) -> dict:
        out = np.zeros(41)
        lib().or_lbm_observables(self._h, _d(out))
        return dict(zip(OBS_NAMES, out.tolist()))


class OrGrayParams(C.Structure):
    _fields_ = [("tau", C.c_double), ("magic", C.c_double), ("F", C.c_double * 3), ("idir", C.c_int32),
                ("nsteps", C.c_int32), ("segment", C.c_int32), ("reserved", C.c_int32)]


def _gray_sigs(L):
    L.or_gray_forward.restype = C.c_double
    L.or_gray_forward.argtypes = [C.POINTER(OrGrayParams), C.c_int, C.c_int, C.c_int, _DP, _DP]
    L.or_gray_gradient.restype = C.c_double
    L.or_gray_gradient.argtypes = [C.POINTER(OrGrayParams), C.c_int, C.c_int, C.c_int, _DP, _DP]


def gray_params(tau, magic, F, idir, nsteps, segment=1):
    return OrGrayParams(tau, magic, (C.c_double * 3)(*F), idir, nsteps, segment, 0)


def gray_forward(p, s: np.ndarray, want_state=False):
    """(k, f(n, 19) or None) of the gray lattice, s shaped (nz, ny, nx)."""
    L = lib()
    _gray_sigs(L)
    s = np.ascontiguousarray(s, np.float64)
    nz, ny, nx = s.shape
    f = np.zeros((s.size, 19)) if want_state else None
    k = L.or_gray_forward(C.byref(p), nx, ny, nz, _d(s), _d(f) if f is not None else None)
    return k, f


def gray_gradient(p, s: np.ndarray):
    """(k, dk/ds shaped like s) by the oracle's adjoint."""
    L = lib()
    _gray_sigs(L)
    s = np.ascontiguousarray(s, np.float64)
    nz, ny, nx = s.shape
    dk = np.zeros_like(s)
    k = L.or_gray_gradient(C.byref(p), nx, ny, nz, _d(s), _d(dk))
    return k, dk


def _lsm_sigs(L):
    sig = {
        "or_lsm_create": (C.c_void_p, [_IP, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_int]),
        "or_lsm_destroy": (None, [C.c_void_p]),
        "or_lsm_sizes": (None, [C.c_void_p, _LP]),
        "or_lsm_tables": (None, [C.c_void_p, _IP, _IP, _DP, _IP, _DP]),
        "or_lsm_forces": (None, [C.c_void_p, _DP, _DP]),
        "or_lsm_relax": (C.c_int64, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double]),
        "or_lsm_cg": (C.c_int64, [C.c_void_p, C.c_double, C.c_int64, _DP]),
        "or_lsm_cg_par": (C.c_int64, [C.c_void_p, C.c_double, C.c_int64, _DP, C.c_int]),
        "or_lsm_relax_par": (C.c_int64, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_double,
                                         C.c_int]),
        "or_lsm_dyn_step": (None, [C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int]),
        "or_lsm_get_dyn": (None, [C.c_void_p, _DP, _DP, _DP]),
        "or_lsm_set_load": (None, [C.c_void_p, _DP]),
        "or_lsm_get_disp": (None, [C.c_void_p, _DP]),
        "or_lsm_set_disp": (None, [C.c_void_p, _DP]),
        "or_lsm_stress": (None, [C.c_void_p, _DP]),
        "or_lsm_anf": (None, [_DP]),
        "or_lsm_cube_tables": (None, [_IP, _DP, _IP, _DP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


class OracleSprings:
    """FP64 CPU restatement of the two-solid lattice-spring model
    (load 0 = x-stretch as XX_P.f, 1 = yz-shear as YZ_P.f)."""

    def __init__(self, ind: np.ndarray, alf1, bet1, alf2, bet2, gstrain, load=0):
        L = lib()
        if not getattr(L, "_lsm_ready", False):
            _lsm_sigs(L)
            L._lsm_ready = True
        ind = np.ascontiguousarray(ind, np.int32)
        nz, ny, nx = ind.shape
        self.shape = (nz, ny, nx)
        self._h = C.c_void_p(L.or_lsm_create(_i(ind), nx, ny, nz, alf1, bet1, alf2, bet2, gstrain, load))
        s = np.zeros(4, np.int64)
        L.or_lsm_sizes(self._h, s.ctypes.data_as(_LP))
        self.ns, self.nbo, self.nna, self.nunique = (int(v) for v in s)

    def close(self):
        if self._h:
            lib().or_lsm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tables(self):
        icors = np.zeros((self.ns, 3), np.int32)
        bon = np.zeros((self.nbo, 3), np.int32)
        sbond = np.zeros(self.nbo)
        ang = np.zeros((self.nna, 6), np.int32)
        abond = np.zeros(self.nna)
        lib().or_lsm_tables(self._h, _i(icors), _i(bon), _d(sbond), _i(ang), _d(abond))
        return icors, bon, sbond, ang, abond

    def forces(self, u):
        u = np.ascontiguousarray(u, np.float64)
        a = np.zeros_like(u)
        lib().or_lsm_forces(self._h, _d(u), _d(a))
        return a

    def relax(self, dt, rs, damp, maxsteps, ftol, nthreads=1):
        """XX:1377-1545's damped Verlet relaxation until the largest nodal
        force is below ftol or maxsteps; returns the steps done."""
        if nthreads > 1:
            return int(lib().or_lsm_relax_par(self._h, dt, rs, damp, int(maxsteps), ftol, int(nthreads)))
        return int(lib().or_lsm_relax(self._h, dt, rs, damp, int(maxsteps), ftol))

    def cg(self, rtol=1e-10, maxit=100000, nthreads=1):
        rel = C.c_double()
        if nthreads > 1:
            it = int(lib().or_lsm_cg_par(self._h, rtol, int(maxit), C.byref(rel), int(nthreads)))
        else:
            it = int(lib().or_lsm_cg(self._h, rtol, int(maxit), C.byref(rel)))
        return it, rel.value

    def dyn_step(self, nsteps, dt, rsi, damp, nthreads=1):
        """The coupled driver's spring dynamics (lsm_step, S1:1721-1903)
        with the external load (set_load) as afdat."""
        lib().or_lsm_dyn_step(self._h, int(nsteps), dt, rsi, damp, int(nthreads))

    def dyn_state(self):
        """(r, v, a), each (ns, 3) in node order."""
        out = [np.zeros((self.ns, 3)) for _ in range(3)]
        lib().or_lsm_get_dyn(self._h, *[_d(x) for x in out])
        return tuple(out)

    def set_load(self, f):
        """external nodal load (ns, 3) in node order for the next cg(); None removes it"""
        if f is None:
            lib().or_lsm_set_load(self._h, None)
        else:
            f = np.ascontiguousarray(f, np.float64)
            lib().or_lsm_set_load(self._h, _d(f))

    def disp(self):
        u = np.zeros((self.ns, 3))
        lib().or_lsm_get_disp(self._h, _d(u))
        return u

    def set_disp(self, u):
        u = np.ascontiguousarray(u, np.float64)
        lib().or_lsm_set_disp(self._h, _d(u))

    def stress(self):
        out = np.zeros(12)
        lib().or_lsm_stress(self._h, _d(out))
        return {"sigma": out[:9].reshape(3, 3), "modulus": out[9], "strain": out[10], "ncube": int(out[11])}


def lsm_constant_tables():
    """(anf[48,9], cube bonds[24,3], sbond[24], cube angles[72,6], abond[72])
    as derived / generated by the oracle (1-based corner and direction ids)."""
    L = lib()
    if not getattr(L, "_lsm_ready", False):
        _lsm_sigs(L)
        L._lsm_ready = True
    anf = np.zeros((48, 9))
    b = np.zeros((24, 3), np.int32)
    sb = np.zeros(24)
    a = np.zeros((72, 6), np.int32)
    ab = np.zeros(72)
    L.or_lsm_anf(_d(anf))
    L.or_lsm_cube_tables(_i(b), _d(sb), _i(a), _d(ab))
    return anf, b, sb, a, ab
