"""The coupled driver's damped spring dynamics (lsm_step, S1:1721-1903)
through ps_lsm_dyn_step against the oracle's restatement of it.

The GPU applies the static solve's linear spring operator (per-cube
matrices, forces gathered per node); the oracle follows the reference's
bond and angle loops, summing in another order, and its bond term keeps the
equilibrium vector rn, (rt . xn) xn - rn, which cancels only up to rounding
(~1e-16 per diagonal bond and step).  Both trajectories are damped and
linear, so they stay within rounding of each other: under the fluid load
1e-11 of each state vector's largest entry.  In the standalone relaxation
the displacements grow from the imposed jump while the rn residue
accumulates like a constant force, t^2/2 ~ 1e-16 x 200 steps^2: there the
bound is 1e-8."""
import numpy as np
import pytest

from porescale_gb300 import PREC_F64, Lattice
from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params
from porescale_gb300.springs import LOAD_NONE, LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork

pytestmark = pytest.mark.gpu

SHAPE = (16, 14, 18)  # (nz, ny, nx)


def _params():
    return make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))


def _s1_corners(ind):
    """(x, y, z) of the coupled driver's LSM nodes in their number order
    (corner dilation with periodic wrap, k-j-i, S1:541-602)."""
    solid = (ind == 0) | (ind == 3)
    nz, ny, nx = ind.shape
    out = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if any(solid[(k - dk) % nz, (j - dj) % ny, (i - di) % nx]
                       for dk in (0, 1) for dj in (0, 1) for di in (0, 1)):
                    out.append((i, j, k))
    return np.array(out)


def _oracle_index(osp, ind, pa):
    """For each S1 node (in S1 order) the oracle network's node: plane 1 of
    the tied axis, or its duplicate plane N+1 when plane 1 has no node."""
    icors = osp.tables()[0]
    where = {tuple(c): n for n, c in enumerate(icors)}
    N = ind.shape[::-1]
    idx = []
    for x, y, z in _s1_corners(ind):
        c = [x + 1, y + 1, z + 1]
        if tuple(c) not in where and c[pa] == 1:
            c[pa] = N[pa] + 1
        idx.append(where[tuple(c)])
    return np.array(idx)


def _close(got, want, tol):
    scale = max(np.abs(want).max(), 1e-300)
    return np.abs(got - want).max() <= tol * scale


@pytest.mark.parametrize("prec", [LSM_F64, LSM_MIXED])
def test_coupled_dynamics_under_wall_load(gpu, oracle_lib, prec):
    """50 coupled steps (dt 0.5, rsi 0.37, damping 0.25) under the fluid's
    wall load from rest: r, v, a equal the oracle's, in the reference node
    order of the network (the dynamics run in FP64 in either precision)."""
    ind = geo.sphere_pack(SHAPE, 0.45, 3.0, seed=7)
    rsi, dt = 0.37, 0.5
    with Lattice(_params(), ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(20)
        afdat = L.wall_load(rsi)
        osp = oracle_lib.OracleSprings(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH)
        with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH, prec) as S:
            S.set_wall_load(L, rsi)
            S.dyn_step(30, dt, rsi, 0.25)
            S.dyn_step(20, dt, rsi, 0.25)
            got = S.dyn_state(osp.ns)
    idx = _oracle_index(osp, ind, 0)
    f = np.zeros((osp.ns, 3))
    f[idx] = afdat
    osp.set_load(f)
    osp.dyn_step(50, dt, rsi, 0.25)
    want = osp.dyn_state()
    assert np.abs(want[0]).max() > 0
    for g, w in zip(got, want):
        assert _close(g, w, 1e-11)


def test_periodic_network_in_s1_order(gpu, oracle_lib):
    """PS_LOAD_NONE: the coupled driver's periodic network in its own node
    order (no duplicate plane), the order of ps_lbm_wall_load's afdat; a
    restart through set_dyn_state continues the trajectory exactly."""
    ind = geo.sphere_pack(SHAPE, 0.45, 3.0, seed=7)
    rsi, dt = 0.37, 0.5
    with Lattice(_params(), ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(20)
        afdat = L.wall_load(rsi)
        ns = L.info.ns
        with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_NONE, LSM_F64) as S:
            S.set_wall_load(L, rsi)
            S.dyn_step(40, dt, rsi, 0.25)
            got = S.dyn_state(ns)
            S.dyn_step(10, dt, rsi, 0.25)
            cont = S.dyn_state(ns)
        with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_NONE, LSM_F64) as S2:
            S2.set_wall_load(L, rsi)
            S2.set_dyn_state(*got)
            S2.dyn_step(10, dt, rsi, 0.25)
            restarted = S2.dyn_state(ns)
    for g, w in zip(restarted, cont):
        assert np.array_equal(g, w)
    osp = oracle_lib.OracleSprings(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH)
    idx = _oracle_index(osp, ind, 0)
    assert len(idx) == ns
    f = np.zeros((osp.ns, 3))
    f[idx] = afdat
    osp.set_load(f)
    osp.dyn_step(40, dt, rsi, 0.25)
    want = osp.dyn_state()
    for g, w in zip(got, want):
        assert _close(g, w[idx], 1e-11)


@pytest.mark.parametrize("case", ["two-solid", "pore-space"])
def test_spring_forces_of_a_random_state(gpu, oracle_lib, case):
    """One undamped step (dt 1) from rest at a random displacement, with no
    load, leaves r in place and sets a = F(r) (and v = a / 2, the closing
    half kick): the operator's bulk stencil (nodes
    whose 8 cubes share one material) and its per-cube gather (surface and
    interface nodes) against the oracle's bond and angle loops, at 1e-12 of
    the largest force.  The periodic network is compared through the
    oracle's tied layout (a duplicate-plane node carries its partner's
    displacement, and the tied forces are the periodic ones)."""
    if case == "two-solid":
        ind = geo.inclusions((10, 12, 14), 0.3, 2.5, seed=3)
        consts = (1.0, 0.4, 0.3, 0.1)
    else:
        ind = geo.sphere_pack(SHAPE, 0.45, 3.0, seed=7)
        consts = (0.8, 0.3, 0.8, 0.3)
    osp = oracle_lib.OracleSprings(ind, *consts, 0.0, LOAD_XSTRETCH)
    idx = _oracle_index(osp, ind, 0)
    ns = len(idx)
    r = np.random.default_rng(11).standard_normal((ns, 3))
    with SpringNetwork(ind, *consts, 0.0, LOAD_NONE, LSM_F64) as S:
        S.set_dyn_state(r)
        S.dyn_step(1, 1.0, 1.0, 0.0)
        got_r, got_v, got_a = S.dyn_state(ns)
    assert np.array_equal(got_r, r) and np.array_equal(got_v, 0.5 * got_a)
    icors = osp.tables()[0]
    where = {tuple(c): n for n, c in enumerate(icors)}
    u = np.zeros((osp.ns, 3))
    u[idx] = r
    nx = ind.shape[2]
    for n, c in enumerate(icors):
        if c[0] == nx + 1 and (1, c[1], c[2]) in where:
            u[n] = u[where[(1, c[1], c[2])]]
    want = osp.forces(u)[idx]
    assert _close(got_a, want, 1e-12)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_relaxation_with_imposed_jump(gpu, oracle_lib, load):
    """The standalone relaxation XX:1377-1545 (damping 0.5, no fluid load)
    through the same entry point: from the reference's starting field (tied
    planes at -g / +g), 200 steps agree with the oracle's, the jump staying
    on the duplicate plane."""
    ind = geo.inclusions(10, 0.25, 2.0, seed=4)
    g, dt = 0.005, 0.1
    osp = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, load)
    r0 = osp.dyn_state()[0]
    osp.dyn_step(200, dt, 1.0, 0.5)
    want = osp.dyn_state()
    with SpringNetwork(ind, 1.0, 0.4, 0.3, 0.1, g, load, LSM_F64) as S:
        S.set_dyn_state(r0)
        S.dyn_step(200, dt, 1.0, 0.5)
        got = S.dyn_state(osp.ns)
    assert np.abs(want[1]).max() > 0
    for a, b in zip(got, want):
        assert _close(a, b, 1e-8)
