"""The colour-gradient D3Q19 lattice behind the C ABI (ps_lbm_*).

Mirrors the reference driver's use of its LBM (``majorityrule`` in
LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f): build the tables from the
``ind`` voxel field, initialise the populations (``initdistr``), advance
``itw`` steps, then read ``check_state`` observables and the state for the
``iteration2`` checkpoint.  Arrays use the reference layouts: ``ind`` as a
numpy array indexed ``[z, y, x]`` (x fastest in memory, the Fortran
ind(ncx,ncy,ncz)), populations as ``fr[nl, 19]`` (Fortran fr(19,nl)).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import LbmInfo, LbmObs, LbmParams, check, dptr, iptr


def make_params(cr2=1.0 / 3.0, rr0=1.0, rb0=1.0, B=0.7, sig=1e-3, vir=1.0 / 6.0, vib=1.0 / 6.0, wet=0.0, ee=0.0,
                dt=1.0, bfr=(0.0, 0.0, 0.0), bfb=(0.0, 0.0, 0.0), idir=1, iipore=1) -> LbmParams:
    """ps_lbm_params from INPUT_PARAMETERS values (S1:435-469 names)."""
    p = LbmParams()
    p.cr2, p.rr0, p.rb0, p.B, p.sig = cr2, rr0, rb0, B, sig
    p.vir, p.vib, p.wet, p.ee, p.dt = vir, vib, wet, ee, dt
    for i in range(3):
        p.bfr[i] = bfr[i]
        p.bfb[i] = bfb[i]
    p.idir, p.iipore = idir, iipore
    return p


class Lattice:
    """One two-phase lattice on the current CUDA device.

    Parameters
    ----------
    params : LbmParams (see :func:`make_params`)
    ind : int array [nz, ny, nx] with the reference's ``ind`` values
    precision : PREC_F64 / PREC_F32 / PREC_F16 / PREC_BF16
    """

    def __init__(self, params: LbmParams, ind: np.ndarray, precision: int = _lib.PREC_F64):
        lib = _lib.library()
        ind = np.ascontiguousarray(ind, dtype=np.int32)
        if ind.ndim != 3:
            raise ValueError("ind must be a 3-D array [nz, ny, nx]")
        nz, ny, nx = ind.shape
        self._lib = lib
        self.params = params
        self.precision = precision
        self.shape = (nz, ny, nx)
        h = C.c_void_p()
        check(lib.ps_lbm_create(C.byref(params), iptr(ind), nx, ny, nz, precision, C.byref(h)))
        self._h = h
        self.info = self.get_info()
        self.nl = int(self.info.nl)

    # -- lifetime --
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ps_lbm_destroy(self._h)
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

    # -- queries --
    def get_info(self) -> LbmInfo:
        info = LbmInfo()
        check(self._lib.ps_lbm_get_info(self._h, C.byref(info)))
        return info

    def tables(self):
        """(icor[nl,3], ips[nps,3], ipb2[npb2,4], ipb4[npb4,6]), 1-based as in S1."""
        i = self.info
        icor = np.zeros((i.nl, 3), np.int32)
        ips = np.zeros((i.nps, 3), np.int32)
        ipb2 = np.zeros((i.npb2, 4), np.int32)
        ipb4 = np.zeros((i.npb4, 6), np.int32)
        check(self._lib.ps_lbm_tables(self._h, iptr(icor), iptr(ips), iptr(ipb2), iptr(ipb4)))
        return icor, ips, ipb2, ipb4

    # -- state --
    def set_state(self, fr: np.ndarray, fb: np.ndarray) -> None:
        fr = np.ascontiguousarray(fr, np.float64).reshape(self.nl, 19)
        fb = np.ascontiguousarray(fb, np.float64).reshape(self.nl, 19)
        check(self._lib.ps_lbm_set_state(self._h, dptr(fr), dptr(fb)))

    def get_state(self, out=None):
        if out is None:
            out = (np.empty((self.nl, 19)), np.empty((self.nl, 19)))
        check(self._lib.ps_lbm_get_state(self._h, dptr(out[0]), dptr(out[1])))
        return out

    def init_random(self, sat: float) -> None:
        """initdistr (S1:2800-2843): blue with probability `sat` per node."""
        check(self._lib.ps_lbm_init_random(self._h, float(sat)))

    # -- stepping --
    def step(self, nsteps: int = 1) -> None:
        check(self._lib.ps_lbm_step(self._h, int(nsteps)))

    def sync(self) -> None:
        check(self._lib.ps_lbm_sync(self._h))

    @property
    def stream(self) -> int:
        """cudaStream_t (as an int) that this lattice launches on."""
        return int(self._lib.ps_lbm_stream(self._h) or 0)

    def set_tile(self, tx: int, ty: int, occ: int = 0) -> None:
        """Step-kernel configuration (collide CTA size, density CTA size,
        minimum collide CTAs per SM)."""
        check(self._lib.ps_lbm_set_tile(self._h, tx, ty, occ))
        self.info = self.get_info()

    def set_fused(self, planes: int, ahead: int = 1) -> None:
        """Fused one-launch step over z-slabs of `planes` planes (0: two-pass)."""
        check(self._lib.ps_lbm_set_fused(self._h, planes, ahead))

    def set_march(self, rows: int, planes: int = 0, producers: int = 4, sort: bool = True) -> None:
        """Marching one-launch step over items of `rows` y-rows and `planes`
        z-planes (0: about three per SM), `producers` density warps per CTA
        (4, 8 or 12),
        bulk nodes collided before interface nodes when sort; rows 0 turns
        it off."""
        check(self._lib.ps_lbm_set_march(self._h, rows, planes, producers, int(bool(sort))))
        self.info = self.get_info()

    def set_sort(self, on: bool) -> None:
        """Two-pass collide: bulk nodes before interface nodes in each CTA."""
        check(self._lib.ps_lbm_set_sort(self._h, int(bool(on))))

    def set_rounding_seed(self, seed: int) -> None:
        """Seed of the stochastic rounding of 16-bit stores (default 0)."""
        check(self._lib.ps_lbm_set_rounding_seed(self._h, int(seed) & 0xFFFFFFFF))

    def set_wait_limit(self, polls: int) -> None:
        """Polls before a fused- or marching-step wait gives up (0: the
        default 2^22)."""
        check(self._lib.ps_lbm_set_wait_limit(self._h, polls))

    def set_wave(self, planes: int, window: int = 0) -> None:
        """Wavefront schedule: 8-step graphs of z-slab launches of `planes`
        planes ordered by their data dependencies (0: off)."""
        check(self._lib.ps_lbm_set_wave(self._h, planes, window))

    def autotune(self, steps: int = 4):
        tx, ty, zc = C.c_int32(), C.c_int32(), C.c_int32()
        check(self._lib.ps_lbm_autotune(self._h, steps, C.byref(tx), C.byref(ty), C.byref(zc)))
        self.info = self.get_info()
        return tx.value, ty.value, zc.value

    # -- outputs --
    def observables(self) -> LbmObs:
        o = LbmObs()
        check(self._lib.ps_lbm_observables(self._h, C.byref(o)))
        return o

    def fields(self):
        rr, rb, cf = np.empty(self.nl), np.empty(self.nl), np.empty(self.nl)
        check(self._lib.ps_lbm_fields(self._h, dptr(rr), dptr(rb), dptr(cf)))
        return rr, rb, cf

    def wall_load(self, rsi: float = 1.0) -> np.ndarray:
        """afdat as (ns, 3): the fluid's wall load on the LSM nodes in the
        reference's node order (S1:3849-3882)."""
        out = np.zeros((self.info.ns, 3))
        check(self._lib.ps_lbm_wall_load(self._h, float(rsi), dptr(out)))
        return out


class LatticeBatch:
    """Many lattices (same precision and parameters) advanced by shared
    persistent launches replayed from a CUDA graph (ps_batch_*).  The
    lattices remain usable on their own and must outlive the batch."""

    def __init__(self, lattices):
        self.lattices = list(lattices)
        self._lib = self.lattices[0]._lib
        arr = (C.c_void_p * len(self.lattices))(*[L._h.value for L in self.lattices])
        h = C.c_void_p()
        check(self._lib.ps_batch_create(arr, len(self.lattices), C.byref(h)))
        self._h = h
        self.nodes = sum(L.nl for L in self.lattices)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ps_batch_destroy(self._h)
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

    def step(self, n: int = 1) -> None:
        check(self._lib.ps_batch_step(self._h, int(n)))

    def set_tile(self, tx: int, ty: int, occ: int = 0) -> None:
        check(self._lib.ps_batch_set_tile(self._h, tx, ty, occ))

    def autotune(self, steps: int = 6):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(self._lib.ps_batch_autotune(self._h, steps, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    @property
    def stream(self) -> int:
        return int(self._lib.ps_batch_stream(self._h) or 0)
