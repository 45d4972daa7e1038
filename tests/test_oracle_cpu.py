"""CPU tests of the FP64 oracle (the parity reference of the GPU kernels).

The reference ships no golden outputs, so the oracle is pinned by the
reference's own known answers and by physics: the homogeneous-solid moduli
printed by calc_stress, the Park-Miller recurrence of initdistr, exact mass
conservation, the TRT magic parameter, Poiseuille-type flow, and the damped
Verlet relaxation of the reference reaching the CG solution.
"""
import math
import os

import numpy as np
import pytest

from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params
from porescale_gb300.springs import spring_constants


def test_trt_magic(oracle_lib):
    """collmatrTRT: (1/s_nu - 1/2)(1/s_q - 1/2) = 3/16 (S1:2858-2893)."""
    S = np.zeros(19)
    for sv in (0.6, 1.0, 1.0 / 1.3, 1.9):
        oracle_lib.lib().or_collmatr_trt(sv, S.ctypes.data_as(oracle_lib._DP))
        assert (1 / S[1] - 0.5) * (1 / S[4] - 0.5) == pytest.approx(3 / 16, rel=1e-14)
        assert S[0] == S[3] == S[5] == S[7] == 0.0


def test_collision_conserves_mass_and_momentum(oracle_lib):
    rng = np.random.default_rng(3)
    t = (1 - 2 / 3, 1 / 18, 1 / 36)
    w = np.array([t[0]] + [t[1]] * 6 + [t[2]] * 12)
    S = np.zeros(19)
    oracle_lib.lib().or_collmatr_trt(1.2, S.ctypes.data_as(oracle_lib._DP))
    cv = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0],
                   [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1], [0, 1, 1],
                   [0, -1, 1], [0, 1, -1], [0, -1, -1]], float)
    for _ in range(20):
        f = w * (1 + 0.05 * rng.standard_normal(19))
        r = f.sum()
        f0 = f.copy()
        pcf = np.zeros(19)
        bf = np.zeros(3)
        Fp = np.zeros(19)
        oracle_lib.lib().or_collision(t[0], t[1], t[2], f.ctypes.data_as(oracle_lib._DP),
                                      pcf.ctypes.data_as(oracle_lib._DP), r, bf.ctypes.data_as(oracle_lib._DP),
                                      Fp.ctypes.data_as(oracle_lib._DP), S.ctypes.data_as(oracle_lib._DP), 1.0, 1.0,
                                      1.0)
        post = np.concatenate([[f[0]], pcf[1:]])
        assert post.sum() == pytest.approx(r, rel=1e-14)
        assert np.allclose(post @ cv, f0 @ cv, atol=1e-15)


def test_park_miller_sequence(oracle_lib):
    """initdistr's generator: seed <- mod(16807 seed, 2^31-1) from 13.081984,
    node blue when seed/2^31 <= sat (S1:2828-2843)."""
    ind = np.ones((5, 4, 3), np.int32)
    p = make_params()
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.37)
    fr, fb = o.get_state()
    seed, expect = 13.081984, []
    for _ in range(o.nl):
        seed = math.fmod(16807.0 * seed, 2147483647.0)
        expect.append(seed / 2147483648.0 <= 0.37)
    blue = fb[:, 0] > 0
    assert blue.tolist() == expect


def test_tables_consistent(oracle_lib):
    ind = geo.sphere_pack((14, 10, 12), 0.45, 2.5, 9)
    o = oracle_lib.OracleLattice(make_params(), ind)
    icor, ips, ipb2, ipb4, mijk, mijks = o.tables()
    assert o.nps + o.npb2 + o.npb4 == 18 * o.nl
    # every (node, incoming direction) is written exactly once per step
    opp = [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]
    hit = np.zeros((o.nl, 19), int)
    np.add.at(hit, (ips[:, 1] - 1, ips[:, 2] - 1), 1)
    np.add.at(hit, (ipb2[:, 0] - 1, ipb2[:, 1] - 1), 1)
    np.add.at(hit, (ipb4[:, 0] - 1, ipb4[:, 1] - 1), 1)
    assert (hit[:, 1:] == 1).all()
    # wall links point at LSM nodes
    assert (ipb2[:, 2:] > 0).all() and (ipb4[:, 2:] > 0).all()
    assert o.n_overflow == 0


def test_mass_conserved_two_phase(oracle_lib):
    ind = geo.sphere_pack((12, 12, 12), 0.5, 2.5, 4)
    p = make_params(B=0.7, sig=1e-3, wet=0.3, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    fr, fb = o.get_state()
    m0r, m0b = fr.sum(), fb.sum()
    o.run(30, 2)
    fr, fb = o.get_state()
    assert fr.sum() == pytest.approx(m0r, rel=1e-12)
    assert fb.sum() == pytest.approx(m0b, rel=1e-12)


def test_single_phase_channel_flow(oracle_lib):
    """Body-force-driven flow between two walls (plane Poiseuille): with
    half-way bounce-back and TRT magic 3/16 the parabola is exact at the
    nodes, so the node-averaged velocity is F (H^2/12 + 1/24) / nu (the mean
    of u(z) = F z (H - z) / (2 nu) over z = 1/2, 3/2, ...)."""
    H, nu, F = 8, 1 / 6, 1e-5
    ind = np.ones((H + 2, 4, 4), np.int32)  # [z, y, x]; z = 0 and z = H+1 are walls
    ind[0] = 0
    ind[H + 1] = 0
    p = make_params(vir=nu, vib=nu, bfr=(F, 0, 0), bfb=(F, 0, 0), sig=0.0, B=0.0)
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.0)  # sat = 0: all red, single phase
    o.run(6000, 2)
    ob = o.observables()
    ux_mean = ob["Qr0"] * (ind.size) / (H * 16)  # Q is per unit cell volume
    assert ux_mean == pytest.approx(F * (H * H / 12 + 1 / 24) / nu, rel=1e-6)


@pytest.mark.parametrize("load", [0, 1])
def test_homogeneous_moduli_match_reference_analytic(oracle_lib, load):
    """calc_stress prints C_xxxx and C_xyxy next to the simulated moduli
    (XX_P.f:1686-1688); for one homogeneous solid they agree."""
    Em, nu = 94.529, 0.0742
    a, b = spring_constants(Em, nu)
    o = oracle_lib.OracleSprings(np.zeros((6, 6, 6), np.int32), a, b, a, b, 0.003, load)
    o.cg(1e-13, 1000)
    want = Em * (nu - 1) / (2 * nu * nu + nu - 1) if load == 0 else Em / (2 * (1 + nu))
    assert o.stress()["modulus"] == pytest.approx(want, rel=1e-11)


def test_relaxation_equals_cg(oracle_lib):
    """The reference's damped Verlet relaxation (XX:1377-1545) and the CG
    solve of the same network reach the same modulus."""
    ind = geo.inclusions(6, 0.25, 1.5, 3)
    o1 = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, 0.003, 0)
    o1.relax(0.1, 1.0, 0.5, 200000, 1e-13)
    o2 = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, 0.003, 0)
    o2.cg(1e-13, 100000)
    assert o1.stress()["modulus"] == pytest.approx(o2.stress()["modulus"], rel=1e-10)


def test_lsm_bond_table_counts(oracle_lib):
    """All-solid cube: 9 bonds and 48 angles per node (XX:626-1261), the
    tied plane duplicated."""
    n = 5
    o = oracle_lib.OracleSprings(np.zeros((n, n, n), np.int32), 1, 0.1, 1, 0.1, 0.001, 0)
    assert o.ns == (n + 1) * n * n and o.nunique == n ** 3
    icors, bon, sbond, ang, abond = o.tables()
    # interior bonds carry the full constants (4 x 1/4, 2 x 1/2); bonds in the
    # tied planes see only the cubes on their side: half of those
    assert set(np.round(sbond, 12)) <= {0.125, 0.25, 0.5, 1.0}
    assert np.isclose(sbond, 1.0).sum() + np.isclose(sbond, 0.5).sum() > 0
    # per unique node 9 bonds, plus the in-plane bonds of the duplicate
    # plane (y, z edges and the yz face diagonals: 4 per node)
    assert len(bon) == 9 * n ** 3 + 4 * n * n


def _golden():
    import json
    import os
    return json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tables.json")))


def test_angle_table_matches_reference(oracle_lib):
    """Our derivation of anf (n = c_j x c_k / |.|, f_j = n x c_j / |c_j|^2,
    f_k = -n x c_k / |c_k|^2) equals the literal table of the reference
    (S1:264-432) row by row up to the orientation of the plane normal: the
    reference orients its xz-plane angles against the right-hand rule
    (normal +y), which negates n, f_j and f_k together and leaves every
    force and stress unchanged (they are bilinear in the row)."""
    g = np.array(_golden()["anf"])
    anf, *_ = oracle_lib.lsm_constant_tables()
    for i in range(48):
        assert np.allclose(anf[i], g[i], atol=1e-15) or np.allclose(anf[i], -g[i], atol=1e-15), i + 1
    flipped = [i + 1 for i in range(48) if not np.allclose(anf[i], g[i], atol=1e-15)]
    assert flipped == list(range(9, 17))  # exactly the eight xz-plane angles


def test_cube_tables_match_reference(oracle_lib):
    """The 24 cube bonds and 72 cube angles we generate from geometry are the
    reference's cube_bon / cube_ang sets with the same unit constants."""
    g = _golden()
    _, b, sb, a, ab = oracle_lib.lsm_constant_tables()
    bonds = sorted([int(x[0]), int(x[1]), int(x[2]), float(s)] for x, s in zip(b, sb))
    angles = sorted([*map(int, x), float(s)] for x, s in zip(a, ab))
    assert bonds == [list(r) for r in g["cube_bonds"]]
    assert angles == [list(r) for r in g["cube_angles"]]


def test_wall_load_of_fluid_at_rest_has_no_net_force(oracle_lib):
    """S1:3849-3882 on a fluid at rest at uniform density (no body force):
    every wall link carries 0.01 of its rest population (ppp = 0.99), and
    the loads of a periodic pack sum to zero (open links pair up, so the
    closed ones balance), while single nodes see a nonzero pressure load."""
    ind = geo.sphere_pack((12, 10, 14), 0.45, 2.5, seed=2)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=1 / 6, wet=0.5, bfr=(0, 0, 0), bfb=(0, 0, 0))
    o = oracle_lib.OracleLattice(p, ind)
    t = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    fr = np.tile(t, (o.nl, 1))
    o.set_state(fr, np.zeros_like(fr))
    o.run(1)
    a = o.wall_load(1.0)
    assert np.abs(a).max() > 1e-4
    assert np.abs(a.sum(0)).max() < 1e-13
    # a face link gives -2 (0.01/18) c / 4 per node, an edge link -2 (0.01/36)
    # c / 2: both 0.01/36 per component, so every nodal load is a multiple
    k = a * 3600.0
    assert np.abs(k - np.round(k)).max() < 1e-9


def test_gray_adjoint_matches_central_differences(oracle_lib):
    """The oracle's discrete adjoint of the gray partial-bounce-back lattice
    against central finite differences of its own forward (h = 1e-5)."""
    rng = np.random.default_rng(1)
    s = rng.uniform(0, 1, (6, 5, 7)) ** 3
    p = oracle_lib.gray_params(0.8, 3 / 16, (1e-5, 0, 0), 1, 60)
    k, dk = oracle_lib.gray_gradient(p, s)
    assert k == oracle_lib.gray_forward(p, s)[0]
    h = 1e-5
    for v in [(0, 0, 0), (3, 2, 4), (5, 4, 6), (1, 1, 1), (2, 3, 0)]:
        kk = []
        for sg in (1, -1):
            sp = s.copy()
            sp[v] += sg * h
            kk.append(oracle_lib.gray_forward(p, sp)[0])
        fd = (kk[0] - kk[1]) / (2 * h)
        assert dk[v] == pytest.approx(fd, rel=1e-5)


def test_gray_open_channel_permeability(oracle_lib):
    """s = 0 everywhere: no resistance, the body force accelerates the fluid
    uniformly (momentum gains F per step and node), so k = nu (T + 1/2)."""
    s = np.zeros((4, 4, 4))
    T = 40
    p = oracle_lib.gray_params(0.9, 3 / 16, (1e-6, 0, 0), 1, T)
    k, _ = oracle_lib.gray_forward(p, s)
    nu = (0.9 - 0.5) / 3
    assert k == pytest.approx(nu * (T + 0.5), rel=1e-10)


def test_generated_cube_constants_are_current(tmp_path):
    """lsm_cube_const.h (the cube matrices as literals for the FP32 matvec)
    is the output of its generator on the current lsm_cube.h."""
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "porescale_gb300", "csrc")
    exe = str(tmp_path / "gen")
    subprocess.run([cxx, "-O2", "-I" + csrc, os.path.join(csrc, "gen_cube_const.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert out == open(os.path.join(csrc, "lsm_cube_const.h")).read()


def test_threaded_spring_forces_match_serial(oracle_lib):
    """The OpenMP force evaluation (odd/even slab chunks, as the reference
    schedules its force loops) gives the serial CG's iterations and modulus
    up to summation order, and the same dynamics trajectory."""
    ind = geo.inclusions(12, 0.25, 2.5, seed=5)
    g = 0.006
    a = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    b = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    ia, ra = a.cg(1e-10, 10000)
    ib, rb = b.cg(1e-10, 10000, nthreads=4)
    assert ia == ib
    assert b.stress()["modulus"] == pytest.approx(a.stress()["modulus"], rel=1e-12)
    c = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    d = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    c.dyn_step(30, 0.1, 1.0, 0.5)
    d.dyn_step(30, 0.1, 1.0, 0.5, nthreads=4)
    rc, rd = c.dyn_state()[0], d.dyn_state()[0]
    assert np.abs(rc - rd).max() <= 1e-12 * np.abs(rc).max()


def test_dynamics_without_load_is_the_relaxation(oracle_lib):
    """lsm_step's Verlet scheme (S1:1721-1903) with no fluid load and the
    standalone damping 0.5 is the relaxation of XX:1377-1545, step for step."""
    ind = geo.inclusions(8, 0.25, 2.0, seed=3)
    a = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, 0.004, 0)
    b = oracle_lib.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, 0.004, 0)
    assert a.relax(0.1, 1.0, 0.5, 40, 0.0) == 40
    b.dyn_step(40, 0.1, 1.0, 0.5)
    assert np.array_equal(a.disp(), b.dyn_state()[0])
