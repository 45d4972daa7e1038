"""Fluid -> solid coupling on the GPU against the FP64 oracle: the wall load
afdat of S1:3849-3882, the static lattice-spring solve under that load, and
calc_ab's alpha / beta (S1:4008-4468)."""
import numpy as np
import pytest

from porescale_gb300 import PREC_BF16, PREC_F16, PREC_F32, PREC_F64, Lattice
from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params
from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork

pytestmark = pytest.mark.gpu

SHAPE = (16, 14, 18)  # (nz, ny, nx)
RSI = 0.37


def _params():
    return make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))


def _geometry(seed=3):
    return geo.sphere_pack(SHAPE, 0.45, 3.0, seed=seed)


def test_wall_load_f64_bit_exact(gpu, oracle_lib):
    ind = _geometry()
    o = oracle_lib.OracleLattice(_params(), ind)
    o.init_random(0.5)
    fr, fb = o.get_state()
    o.run(7, 4)
    want = o.wall_load(RSI)
    with Lattice(_params(), ind, PREC_F64) as L:
        L.set_state(fr, fb)
        L.step(7)
        got = L.wall_load(RSI)
    assert got.shape == want.shape == (o.ns, 3)
    assert np.abs(want).max() > 0
    assert np.array_equal(got, want)


@pytest.mark.parametrize("prec,rtol", [(PREC_F32, 1e-4), (PREC_F16, 2e-2), (PREC_BF16, 1e-1)])
def test_wall_load_low_precision(gpu, oracle_lib, prec, rtol):
    """One step from the same state: the load of the 32/16-bit forms within
    rtol of the largest nodal load.  q = f - 0.99 fq is a difference of two
    near-equal numbers: an FP32 population near 1/18 carries 3.7e-9 of
    rounding, x2 per link and up to a dozen links per node, ~4e-8 against
    loads of ~1e-3; the 16-bit storage error shows at ~1e-2."""
    ind = _geometry()
    o = oracle_lib.OracleLattice(_params(), ind)
    o.init_random(0.5)
    fr, fb = o.get_state()
    o.run(1)
    want = o.wall_load(RSI)
    with Lattice(_params(), ind, prec) as L:
        L.set_state(fr, fb)
        L.step(1)
        got = L.wall_load(RSI)
    assert np.abs(got - want).max() <= rtol * np.abs(want).max()


def _s1_corners(ind):
    """0-based (x, y, z) of the reference's LSM nodes in their number order
    (corner dilation with periodic wrap, k-j-i loops, S1:541-602)."""
    solid = ind == 0
    nz, ny, nx = ind.shape
    out = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if any(solid[(k - dk) % nz, (j - dj) % ny, (i - di) % nx]
                       for dk in (0, 1) for dj in (0, 1) for di in (0, 1)):
                    out.append((i, j, k))
    return np.array(out)


def _oracle_load(osp, ind, afdat, pa):
    """afdat (S1 node order) -> the oracle network's node order.  A corner
    on the tied plane (coordinate 0 along the loaded axis pa) is the
    network's plane-1 node, or its duplicate plane N+1 when only the cube
    on the far side of the tie is solid (the tie then carries it)."""
    icors = osp.tables()[0]
    where = {tuple(c): n for n, c in enumerate(icors)}
    N = ind.shape[::-1]
    f = np.zeros((osp.ns, 3))
    for (x, y, z), v in zip(_s1_corners(ind), afdat):
        c = [x + 1, y + 1, z + 1]
        if tuple(c) not in where and c[pa] == 1:
            c[pa] = N[pa] + 1
        f[where[tuple(c)]] = v
    return f


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_spring_solve_under_wall_load_vs_oracle(gpu, oracle_lib, load):
    """The static solve under imposed strain plus the fluid's wall load:
    summed cube stress within 1e-9 of the oracle's CG under the same load,
    and linear (strain alone + load alone = both)."""
    ind = _geometry(seed=5)
    a1, b1 = 1.0, 0.4
    g = 1e-3 * SHAPE[2] / 2
    with Lattice(_params(), ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(20)
        afdat = L.wall_load(1.0)
        sig = {}
        for gs, with_load in ((g, True), (g, False), (0.0, True)):
            with SpringNetwork(ind, a1, b1, a1, b1, gs, load, LSM_F64) as S:
                if with_load:
                    S.set_wall_load(L, 1.0)
                r = S.solve(1e-12, 200000)
                sig[(gs, with_load)] = np.array(r.sigma[:]).reshape(3, 3)
    osp = oracle_lib.OracleSprings(ind, a1, b1, a1, b1, g, load)
    osp.set_load(_oracle_load(osp, ind, afdat, 0 if load == LOAD_XSTRETCH else 1))
    osp.cg(1e-12, 200000)
    want = osp.stress()["sigma"]
    scale = np.abs(want).max()
    assert np.allclose(sig[(g, True)], want, rtol=0, atol=1e-9 * scale)
    both = sig[(g, False)] + sig[(0.0, True)]
    assert np.allclose(sig[(g, True)], both, rtol=0, atol=1e-9 * scale)


def _calc_ab_beta(lab, u_box, npores, vcell, pres):
    """S1:4262-4439 restated in numpy on the periodic corner box u_box
    (nz, ny, nx, 3)."""
    nz, ny, nx = lab.shape
    beta = np.zeros(npores)
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                p = lab[k, j, i]
                if p < 1 or p > npores:
                    continue
                for c in dirs:
                    if lab[(k + c[2]) % nz, (j + c[1]) % ny, (i + c[0]) % nx] != 0:
                        continue
                    ax = int(np.nonzero(c)[0][0])
                    base = [i, j, k]
                    base[ax] += (c[ax] + 1) // 2
                    others = [a for a in range(3) if a != ax]
                    up = np.zeros(3)
                    for q in range(4):
                        pt = list(base)
                        pt[others[0]] += q & 1
                        pt[others[1]] += q >> 1
                        up += u_box[pt[2] % nz, pt[1] % ny, pt[0] % nx]
                    up *= 0.25
                    beta[p - 1] -= up[0] * c[0] + up[1] * c[1] + up[2] * c[2]
    return beta / vcell / pres


def test_alpha_beta_under_wall_load(gpu, oracle_lib):
    """calc_ab after the static solve under the wall load alone (no imposed
    strain): alpha from the summed stress, beta per pore from the face
    displacements, against the same formulas on the oracle's solution."""
    ind = _geometry(seed=7)
    nz, ny, nx = ind.shape
    # two pore labels: split the pore space at the x midplane
    lab = np.where(ind == 0, 0, np.where(np.arange(nx)[None, None, :] < nx // 2, 1, 2)).astype(np.int32)
    pres = 0.01 * 1.0 / 3.0
    with Lattice(_params(), ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(20)
        afdat = L.wall_load(1.0)
        for prec in (LSM_F64, LSM_MIXED):
            with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH, prec) as S:
                S.set_wall_load(L, 1.0)
                S.solve(1e-12, 200000)
                alpha, beta = S.alpha_beta(lab, 2, 1, pres)
            if prec == LSM_F64:
                ref_alpha, ref_beta = alpha, beta
            else:
                assert np.allclose(alpha, ref_alpha, rtol=1e-6, atol=1e-6 * np.abs(ref_alpha).max())
                assert np.allclose(beta, ref_beta, rtol=1e-6, atol=1e-6 * np.abs(ref_beta).max())
    osp = oracle_lib.OracleSprings(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH)
    osp.set_load(_oracle_load(osp, ind, afdat, 0))
    osp.cg(1e-12, 200000)
    st = osp.stress()
    vcell = float(ind.size)
    epsi = float((lab == 1).sum()) / vcell
    want_alpha = -epsi * np.eye(3) + st["sigma"] / vcell / pres
    assert np.allclose(ref_alpha, want_alpha, rtol=0, atol=1e-9 * np.abs(want_alpha).max())
    # the oracle's displacements on the periodic corner box (first plane of
    # each tied pair; the network's solution is unique up to a translation,
    # which beta's surface sums over closed pore walls do not see)
    icors = osp.tables()[0]
    u = osp.disp()
    u_box = np.zeros((nz, ny, nx, 3))
    for (i, j, k), v in zip(icors, u):  # the tied duplicate plane folds onto plane 1 (no jump: g = 0)
        u_box[(k - 1) % nz, (j - 1) % ny, (i - 1) % nx] = v
    want_beta = _calc_ab_beta(lab, u_box, 2, vcell, pres)
    assert np.allclose(ref_beta, want_beta, rtol=1e-8, atol=1e-9 * np.abs(want_beta).max())
