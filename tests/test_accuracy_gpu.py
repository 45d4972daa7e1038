"""Relative-permeability accuracy of the 32- and 16-bit storage forms
against the FP64 lattice, which reproduces the FP64 oracle bit for bit.

k_r of a phase is its flux-based permeability of check_state (permr /
permb, S1:3181-3182) over k_abs, the same k_abs for every precision, so its
relative error is that of permr / permb.  The error is taken on the time
average over the second half of the run, the quantity k_r measures once the
flux has developed.  In a porous two-phase flow the trajectory is chaotic:
runs that differ by rounding drift apart, and the time-averaged error then
carries the statistical floor of the averaging window.  This test uses a
flow without that floor, so that the bound measures the storage itself: two
fluid layers stacked along z in a periodic box and driven in opposite
directions along x by equal and opposite body forces (the viscosity ratio
of the 256^3 workload), which settles to a steady counter-current layered
flow with flat interfaces.  In a steady flow every population takes the
same value step after step, so a rounding that is not zero-mean biases the
flux: this is the case the stochastic rounding of the 16-bit stores is for.
Bounds: 1e-3 (the headline metric's error bound) for FP16 storage, 2e-4
for FP32."""
import numpy as np
import pytest

from porescale_gb300 import PREC_BF16, PREC_F16, PREC_F32, PREC_F64, Lattice
from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params

pytestmark = pytest.mark.gpu

STEPS, EVERY = 12000, 100


def _layers():
    nz, ny, nx = 32, 4, 8
    ind = np.ones((nz, ny, nx), np.int32)
    col = np.zeros(ind.shape)
    col[:16] = 1.0  # red layer z < 16, blue above (periodic: two interfaces)
    fr, fb = geo.colour_state(ind, col)
    p = make_params(B=0.7, sig=1e-3, vir=(0.8 - 0.5) / 3, vib=(1.5 - 0.5) / 3, wet=0.0,
                    bfr=(1e-5, 0, 0), bfb=(-1e-5, 0, 0))
    return ind, p, fr, fb


def _history(prec):
    ind, p, fr, fb = _layers()
    out = []
    with Lattice(p, ind, prec) as L:
        L.set_state(fr, fb)
        for _ in range(STEPS // EVERY):
            L.step(EVERY)
            o = L.observables()
            out.append((o.permr, o.permb))
    return np.array(out)


def test_kr_error_of_storage_forms(gpu):
    ref = _history(PREC_F64)
    h0 = len(ref) // 2
    mean_ref = ref[h0:].mean(0)
    assert (mean_ref > 0).all()
    # the flow has settled: the second half's first and last samples agree
    assert np.abs(ref[-1] - ref[h0]).max() <= 1e-2 * mean_ref.max()
    err = {}
    for prec in (PREC_F32, PREC_F16, PREC_BF16):
        mean = _history(prec)[h0:].mean(0)
        err[prec] = np.abs(mean - mean_ref) / mean_ref
    assert err[PREC_F32].max() <= 2e-4, err
    assert err[PREC_F16].max() <= 1e-3, err
    # BF16 keeps 8 mantissa bits: reported, bounded only loosely
    assert err[PREC_BF16].max() <= 5e-2, err
