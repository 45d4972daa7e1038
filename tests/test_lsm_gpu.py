"""GPU parity of the lattice-spring static solve against the FP64 oracle.

The oracle restates the reference's bond/angle tables and calc_stress and
solves the same network by FP64 CG (and by the reference's damped Verlet
relaxation on small boxes).  Tolerances: FP64 GPU moduli within 1e-9
relative of the oracle; mixed precision (FP32 CG in FP64 refinement) within
1e-6 relative, the stated bound for moduli.
"""
import numpy as np
import pytest

from porescale_gb300 import geometry as geo
from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork, spring_constants

pytestmark = pytest.mark.gpu

A1, B1 = 1.0, 0.4     # phase 1 (matrix)
A2, B2 = 0.3, 0.1     # phase 2 (inclusions)


def _two_phase(n=12, seed=5, r=2.5, frac=0.25):
    return geo.inclusions(n, frac, r, seed)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_homogeneous_matches_analytic(gpu, load):
    """The reference's own known answer: for one homogeneous solid the
    simulated modulus equals C_xxxx = Em(nu-1)/(2nu^2+nu-1) or
    C_xyxy = Em/(2(1+nu)) printed next to it (XX_P.f:1686-1688)."""
    Em, nu = 18.369, 0.35065
    a, b = spring_constants(Em, nu)
    ind = np.zeros((8, 8, 8), np.int32)
    with SpringNetwork(ind, a, b, a, b, 0.004, load, LSM_F64) as S:
        r = S.solve(1e-12, 10000)
    want = Em * (nu - 1) / (2 * nu * nu + nu - 1) if load == LOAD_XSTRETCH else Em / (2 * (1 + nu))
    assert r.modulus == pytest.approx(want, rel=1e-10)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_two_phase_modulus_vs_oracle(gpu, oracle_lib, load):
    ind = _two_phase()
    n = ind.shape[0]
    g = 1e-3 * n / 2
    o = oracle_lib.OracleSprings(ind, A1, B1, A2, B2, g, load)
    it, rel = o.cg(1e-12, 100000)
    ref = o.stress()["modulus"]
    with SpringNetwork(ind, A1, B1, A2, B2, g, load, LSM_F64) as S:
        r64 = S.solve(1e-10, 100000)
        assert r64.converged and r64.relres <= 1e-10
        assert r64.nnode == o.nunique
        u = S.displacements(o.ns)
    assert r64.modulus == pytest.approx(ref, rel=1e-9)
    # displacement field in the reference node order, up to a rigid translation
    uo = o.disp()
    du = (u - u.mean(0)) - (uo - uo.mean(0))
    assert np.abs(du).max() <= 1e-8 * max(1e-30, np.abs(uo - uo.mean(0)).max())
    with SpringNetwork(ind, A1, B1, A2, B2, g, load, LSM_MIXED) as S:
        rm = S.solve(1e-10, 100000)
    assert rm.converged and rm.relres <= 1e-10
    assert rm.modulus == pytest.approx(ref, rel=1e-6)


def test_relaxation_reaches_cg_solution(gpu, oracle_lib):
    """The reference's damped Verlet relaxation converges to the state the
    GPU CG solves for (small box, oracle DR run to a small residual force)."""
    ind = _two_phase(n=6, seed=3, r=1.5)
    g = 0.003
    o = oracle_lib.OracleSprings(ind, A1, B1, A2, B2, g, LOAD_XSTRETCH)
    o.relax(0.1, 1.0, 0.5, 400000, 1e-13)
    dr = o.stress()["modulus"]
    with SpringNetwork(ind, A1, B1, A2, B2, g, LOAD_XSTRETCH, LSM_F64) as S:
        r = S.solve(1e-12, 100000)
    assert r.modulus == pytest.approx(dr, rel=1e-7)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_modulus_gradients_vs_central_differences(gpu, load):
    """d modulus / d(alf1, bet1, alf2, bet2) from the spring energies at the
    converged displacement against FP64 central finite differences of the
    modulus itself (h = 1e-4 relative), within 1e-4 relative; the energy
    form of the modulus equals the stress form at equilibrium."""
    ind = _two_phase(n=12, seed=9, r=3.0)
    k0 = np.array([A1, B1, A2, B2])
    g = 1e-3 * 12 / 2
    with SpringNetwork(ind, *k0, g, load, LSM_F64) as S:
        r = S.solve(1e-12, 100000)
        grad = S.gradients()
    assert grad[4] == pytest.approx(r.modulus, rel=1e-9)
    for k in range(4):
        h = 1e-4 * k0[k]
        mods = []
        for sgn in (1, -1):
            kk = k0.copy()
            kk[k] += sgn * h
            with SpringNetwork(ind, *kk, g, load, LSM_F64) as S:
                mods.append(S.solve(1e-13, 100000).modulus)
        fd = (mods[0] - mods[1]) / (2 * h)
        assert grad[k] == pytest.approx(fd, rel=1e-4), (k, grad[k], fd)
    # homogeneous-limit identity: modulus = sum_k k dC/dk (C is homogeneous
    # of degree 1 in the spring constants)
    assert float(np.dot(k0, grad[:4])) == pytest.approx(r.modulus, rel=1e-9)


def test_modulus_gradients_mixed_precision(gpu):
    """The mixed-precision solution gives the same gradients within 1e-6."""
    ind = _two_phase(n=12, seed=9, r=3.0)
    g = 1e-3 * 6
    out = []
    for prec in (LSM_F64, LSM_MIXED):
        with SpringNetwork(ind, A1, B1, A2, B2, g, LOAD_XSTRETCH, prec) as S:
            S.solve(1e-11, 100000)
            out.append(S.gradients())
    assert np.allclose(out[1], out[0], rtol=1e-6, atol=0)


@pytest.mark.parametrize("prec", [LSM_F64, LSM_MIXED])
def test_batch_solve_matches_individual(gpu, prec):
    """ps_lsm_batch_solve: three networks of different boxes and loads
    solved by shared launches give the moduli of their individual solves."""
    from porescale_gb300.springs import batch_solve
    cases = [(geo.inclusions(10, 0.25, 2.5, 3), LOAD_XSTRETCH), (geo.inclusions((12, 8, 14), 0.2, 2.0, 4), LOAD_YZSHEAR),
             (geo.inclusions(16, 0.3, 3.0, 5), LOAD_XSTRETCH)]
    nets = [SpringNetwork(ind, A1, B1, A2, B2, 0.002 * ind.shape[2], load, prec) for ind, load in cases]
    try:
        got = batch_solve(nets, 1e-11, 200000)
        for N, r in zip(nets, got):
            alone = N.solve(1e-11, 200000)
            assert r.converged == 1
            assert r.modulus == pytest.approx(alone.modulus, rel=1e-12 if prec == LSM_F64 else 1e-9)
            assert np.allclose(r.sigma[:], alone.sigma[:], rtol=1e-9, atol=1e-12 * max(abs(v) for v in alone.sigma))
    finally:
        for N in nets:
            N.close()


def test_batch_solve_with_a_network_above_the_group_budget(gpu):
    """ps_lsm_batch_solve (mixed precision) groups networks by CG working
    set: a 100^3 network (48 MB of FP32 CG vectors, above the 40 MB group
    budget) runs the individual refinement in a group of its own, the small
    ones share batched launches; every network's modulus and inner
    iteration count equal its individual solve's exactly."""
    from porescale_gb300.springs import batch_solve
    inds = [geo.inclusions(100, 0.25, 5.0, 11), geo.inclusions(12, 0.25, 2.5, 12), geo.inclusions(14, 0.2, 3.0, 13),
            geo.inclusions((10, 12, 16), 0.3, 2.0, 14)]
    nets = [SpringNetwork(ind, A1, B1, A2, B2, 0.002 * ind.shape[2], LOAD_XSTRETCH, LSM_MIXED) for ind in inds]
    try:
        got = batch_solve(nets, 1e-10, 200000)
        for N, r in zip(nets, got):
            alone = N.solve(1e-10, 200000)
            assert r.converged == 1
            assert r.modulus == alone.modulus
            assert r.inner_iterations == alone.inner_iterations
            assert r.refinements == alone.refinements
    finally:
        for N in nets:
            N.close()
