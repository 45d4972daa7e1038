"""Parity on the reference's own inputs: 40^3 crops of the two `ind` files
the reference ships (LBM-LSM: pore / solid; LBM-LSM2S: pore / matrix /
phase-2 solid), committed as tests/golden/shipped_crops.npz by
tests/golden/make_golden.py together with the oracle's table sizes for
them."""
import json
import os

import numpy as np
import pytest

from porescale_gb300 import PREC_F16, PREC_F64
from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import Lattice, make_params

HERE = os.path.dirname(os.path.abspath(__file__))


def _crops():
    d = np.load(os.path.join(HERE, "golden", "shipped_crops.npz"))
    return {k: d[k].astype(np.int32) for k in d.files}


def _recorded():
    with open(os.path.join(HERE, "golden", "reference_tables.json")) as f:
        return json.load(f)["shipped_crop_tables"]


def _params():
    return make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.7071067811865476, bfr=(1e-5, 0, 0),
                       bfb=(1e-5, 0, 0))


def test_crop_fixture_tables_cpu(oracle_lib):
    """The oracle still builds the table sizes recorded for the crops."""
    rec = _recorded()
    for key, ind in _crops().items():
        assert ind.shape == (40, 40, 40)
        assert sorted(int(v) for v in np.unique(ind)) == rec[key]["values"]
        o = oracle_lib.OracleLattice(_params(), ind)
        got = {"nl": o.nl, "nps": o.nps, "npb2": o.npb2, "npb4": o.npb4, "ns": o.ns}
        o.close()
        assert got == {k: rec[key][k] for k in got}, key


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["lbm_lsm_40", "lbm_lsm2s_40"])
def test_shipped_crop_lattice_bit_exact(gpu, oracle_lib, key):
    """Tables and 12 FP64 steps on a crop of a shipped geometry equal the
    oracle's bit for bit; 16-bit storage stays within its rounding."""
    ind = _crops()[key]
    p = _params()
    o = oracle_lib.OracleLattice(p, ind)
    oic, ops, opb2, opb4 = o.tables()[:4]
    o.init_random(0.5)
    o.run(12, 4)
    fr, fb = o.get_state()
    with Lattice(p, ind, PREC_F64) as L:
        ic, ps, pb2, pb4 = L.tables()
        assert np.array_equal(ic, oic) and np.array_equal(ps, ops)
        assert np.array_equal(pb2, opb2) and np.array_equal(pb4, opb4)
        L.init_random(0.5)
        L.step(12)
        gr, gb = L.get_state()
    assert np.array_equal(gr, fr) and np.array_equal(gb, fb)
    with Lattice(p, ind, PREC_F16) as L:
        L.init_random(0.5)
        L.step(12)
        hr, hb = L.get_state()
    assert max(np.abs(hr - fr).max(), np.abs(hb - fb).max()) <= 5e-4


@pytest.mark.gpu
def test_shipped_crop_spring_moduli(gpu, oracle_lib):
    """Cxxxx and Cyzyz of the two-material network of a 24^3 crop of the
    shipped LBM-LSM2S geometry (matrix and phase-2 solid, solid clusters not
    face-joined to the largest made pore): FP64 within 1e-9 and mixed
    precision within 1e-6 of the oracle's CG."""
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork
    ind = geo.spanning_solid(_crops()["lbm_lsm2s_40"][:24, :24, :24])
    g = 1e-3 * 24 / 2
    for load in (LOAD_XSTRETCH, LOAD_YZSHEAR):
        osp = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, load)
        osp.cg(1e-12, 200000)
        want = osp.stress()["modulus"]
        osp.close()
        for prec, tol in ((LSM_F64, 1e-9), (LSM_MIXED, 1e-6)):
            with SpringNetwork(ind, 1.0, 0.4, 0.3, 0.1, g, load, prec) as S:
                got = S.solve(1e-11, 200000).modulus
            assert got == pytest.approx(want, rel=tol), (load, prec)
