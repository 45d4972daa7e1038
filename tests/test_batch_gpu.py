"""Batched lattices (many subvolumes per persistent launch, CUDA-graph
replays): every lattice of a batch ends bit-identical to the same lattice
stepped on its own, whatever the mix of step counts, graph replays and
individual steps; the autotuner restores the states it times on."""
import numpy as np
import pytest

from porescale_gb300 import PREC_BF16, PREC_F16, PREC_F32, PREC_F64, Lattice, LatticeBatch
from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params

pytestmark = pytest.mark.gpu

SHAPES = [(12, 16, 20), (16, 20, 24), (22, 18, 14)]


def _params():
    return make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))


def _lattices(prec):
    out = []
    for k, shp in enumerate(SHAPES):
        ind = geo.sphere_pack(shp, 0.4 + 0.03 * k, 2.5 + k, seed=31 + k)
        L = Lattice(_params(), ind, prec)
        L.init_random(0.3 + 0.2 * k)
        out.append(L)
    return out


@pytest.mark.parametrize("prec", [PREC_F64, PREC_F32, PREC_F16, PREC_BF16])
def test_batch_matches_individual_lattices(gpu, prec):
    solo, grouped = _lattices(prec), _lattices(prec)
    with LatticeBatch(grouped) as B:
        B.step(7)          # direct launches
        grouped[1].step(1)  # one lattice alone: mixed buffer parities
        B.step(45)         # two graph replays of 20 steps + 5 direct
    for L in solo:
        L.step(52)
    solo[1].step(1)
    for a, b in zip(solo, grouped):
        fa, fb = a.get_state(), b.get_state()
        assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])
    for L in solo + grouped:
        L.close()


def test_batch_autotune_restores_states(gpu):
    lat = _lattices(PREC_F16)
    before = [L.get_state() for L in lat]
    with LatticeBatch(lat) as B:
        cfg = B.autotune(4)
        assert len(cfg) == 3
        for L, s in zip(lat, before):
            now = L.get_state()
            assert np.array_equal(now[0], s[0]) and np.array_equal(now[1], s[1])
        B.step(3)
    ref = _lattices(PREC_F16)
    for L in ref:
        L.set_tile(*cfg)
        L.step(3)
    for a, b in zip(ref, lat):
        fa, fb = a.get_state(), b.get_state()
        assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])


def test_batch_rejects_mixed_precision(gpu):
    from porescale_gb300._lib import PorescaleError
    a = _lattices(PREC_F32)[0]
    b = _lattices(PREC_F16)[0]
    with pytest.raises(PorescaleError):
        LatticeBatch([a, b])
