"""GPU parity on the full-size 64^3 two-solid lattice-spring cube that
bench.py times (matrix alpha 1.0 / beta 0.4, radius-5 inclusions at volume
fraction 0.25 with alpha 0.3 / beta 0.1, strain 1e-3).

A converged oracle CG at this size takes about a minute on one host core,
so the GPU solution is checked through properties the oracle evaluates in a
second: the GPU displacement field is an equilibrium of the oracle's own
spring network (the oracle's spring forces, with the duplicate planes tied
as XX_P.f:1511-1520 does, vanish at it to the CG tolerance), and the
oracle's calc_stress (XX_P.f:1628-1997) at that field gives the GPU's
modulus.
"""
import numpy as np
import pytest

from porescale_gb300 import geometry as geo
from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork

pytestmark = pytest.mark.gpu

A1, B1 = 1.0, 0.4     # phase 1 (matrix)
A2, B2 = 0.3, 0.1     # phase 2 (inclusions)


@pytest.fixture(scope="module")
def cube64():
    return geo.inclusions(64, 0.25, 5.0, 20240601)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_full_size_solution_is_oracle_equilibrium(gpu, oracle_lib, cube64, load):
    n = cube64.shape[0]
    g = 1e-3 * n / 2
    o = oracle_lib.OracleSprings(cube64, A1, B1, A2, B2, g, load)
    # residual forces of the starting field (the jump alone) set the scale
    a0 = np.linalg.norm(o.forces(o.disp()))
    with SpringNetwork(cube64, A1, B1, A2, B2, g, load, LSM_F64) as S:
        r64 = S.solve(1e-10, 100000)
        assert r64.converged and r64.relres <= 1e-10
        assert r64.nnode == o.nunique
        u = S.displacements(o.ns)
    with SpringNetwork(cube64, A1, B1, A2, B2, g, load, LSM_MIXED) as S:
        rm = S.solve(1e-10, 100000)
        assert rm.converged and rm.relres <= 1e-10
    # CG stops at |b - A x| <= 1e-10 |b|; the tied rows count twice in the
    # oracle's force vector, hence the margin
    assert np.linalg.norm(o.forces(u)) <= 1e-9 * a0
    o.set_disp(u)
    ref = o.stress()["modulus"]
    assert r64.modulus == pytest.approx(ref, rel=1e-9)
    assert rm.modulus == pytest.approx(ref, rel=1e-6)
