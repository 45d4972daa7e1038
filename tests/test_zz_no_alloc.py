"""The allocation-free stress entry point (ps_lsm_stress_noalloc) against
ps_lsm_solve's own stress result.

ps_lsm_stress_noalloc serves callers that cannot allocate device memory
when they need the moduli (an application whose own pool has already
reserved the device's memory, a driver stepping several streams where
freeing device memory would stall the others); its partial sums live in a
static device array of the library.  This file runs last (pytest collects
it after the others) and also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from porescale_gb300 import geometry as geo
from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, SpringNetwork, spring_constants

pytestmark = pytest.mark.gpu

# the tolerance of the FP64 modulus checks in test_lsm_gpu.py
RTOL = 1e-9


def _reference_nodes(ind, pa):
    """Coordinates of the reference's solid nodes in its node order: k-j-i
    over the padded grid, the loaded axis having node planes 0..N (plane N
    duplicates plane 0); a node exists when one of its cubes is solid, with
    no cubes beyond the ends of the loaded axis."""
    nz, ny, nx = ind.shape
    N = np.array([nx, ny, nz])
    M = N.copy()
    M[pa] += 1
    solid = (ind == 0) | (ind == 3)
    zz, yy, xx = np.meshgrid(np.arange(M[2]), np.arange(M[1]), np.arange(M[0]), indexing="ij")
    coords = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1)
    exists = np.zeros(len(coords), bool)
    for e in range(8):
        c = coords - np.array([e & 1, (e >> 1) & 1, (e >> 2) & 1])
        ok = (c[:, pa] >= 0) & (c[:, pa] < N[pa])
        for d in range(3):
            c[:, d] = np.clip(c[:, d], 0, N[d] - 1) if d == pa else c[:, d] % N[d]
        exists |= ok & solid[c[:, 2], c[:, 1], c[:, 0]]
    return coords[exists], N


def _unique_field(u_ref, nodes, N, pa, jc, g):
    """Reference-order displacements -> the layout ps_lsm_stress_noalloc
    reads: 3 planes of nx*ny*nz unique nodes, without the jump."""
    vals = u_ref.copy()
    vals[nodes[:, pa] == N[pa], jc] -= 2 * g
    uniq = nodes % N
    U = np.zeros((3, N[2], N[1], N[0]))
    U[:, uniq[:, 2], uniq[:, 1], uniq[:, 0]] = vals.T
    return np.ascontiguousarray(U)


@pytest.mark.parametrize("load", [LOAD_XSTRETCH, LOAD_YZSHEAR])
def test_stress_noalloc_matches_solve(gpu, load):
    import torch

    n = 16
    ind = geo.inclusions(n, 0.25, 3.0, seed=21)
    g = 1e-3 * n / 2
    pa, jc = (0, 0) if load == LOAD_XSTRETCH else (1, 2)
    nodes, N = _reference_nodes(ind, pa)
    with SpringNetwork(ind, 1.0, 0.4, 0.3, 0.1, g, load, LSM_F64) as S:
        r = S.solve(1e-11, 100000)
        u_ref = S.displacements(len(nodes))
        d_u = torch.from_numpy(_unique_field(u_ref, nodes, N, pa, jc, g)).cuda()
        torch.cuda.synchronize()
        sig_ref = np.array(r.sigma[:])
        for call in range(2):  # two calls in a row on the same static scratch
            out = (C.c_double * 10)()
            rc = S._lib.ps_lsm_stress_noalloc(S._h, C.c_void_p(d_u.data_ptr()), out)
            assert rc == 0, call
            sig = np.array(out[:9])
            assert np.allclose(sig, sig_ref, rtol=RTOL, atol=RTOL * np.abs(sig_ref).max()), call
            assert out[9] == pytest.approx(r.modulus, rel=RTOL), call


def _noalloc(S, d_u):
    out = (C.c_double * 10)()
    rc = S._lib.ps_lsm_stress_noalloc(S._h, C.c_void_p(d_u.data_ptr()), out)
    assert rc == 0
    return np.array(out[:])


def test_stress_noalloc_wall_load_only(gpu):
    """A handle with no imposed strain (gstrain 0) that carries only the
    fluid's wall load: the summed stress equals the solve's, and the modulus
    is 0 as ps_lsm_solve reports it (no division by the zero strain)."""
    import torch

    from porescale_gb300 import PREC_F64
    from porescale_gb300.lattice import Lattice, make_params

    ind = geo.sphere_pack((16, 14, 18), 0.45, 3.0, seed=7)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    nodes, N = _reference_nodes(ind, 0)
    with Lattice(p, ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(20)
        with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.0, LOAD_XSTRETCH, LSM_F64) as S:
            S.set_wall_load(L, 1.0)
            r = S.solve(1e-12, 200000)
            assert r.modulus == 0.0
            d_u = torch.from_numpy(_unique_field(S.displacements(len(nodes)), nodes, N, 0, 0, 0.0)).cuda()
            torch.cuda.synchronize()
            sig_ref = np.array(r.sigma[:])
            assert np.abs(sig_ref).max() > 0
            for call in range(2):
                out = _noalloc(S, d_u)
                assert np.allclose(out[:9], sig_ref, rtol=RTOL, atol=RTOL * np.abs(sig_ref).max()), call
                assert out[9] == 0.0, call


def test_stress_noalloc_at_max_cubes(gpu):
    """A box of exactly PS_LSM_NOALLOC_MAX_CUBES (128^3) cubes, which fills
    every partial-sum slot of the static array: a homogeneous solid under
    the affine x stretch u_x = e x is in equilibrium, and its modulus is the
    reference's analytic C_xxxx = Em(nu-1)/(2nu^2+nu-1) (XX_P.f:1686-1688)."""
    import torch

    n = 128
    Em, nu = 18.369, 0.35065
    a, b = spring_constants(Em, nu)
    e = 1e-3
    ind = np.zeros((n, n, n), np.int32)
    U = np.zeros((3, n, n, n))
    U[0] = e * np.arange(n)[None, None, :]
    with SpringNetwork(ind, a, b, a, b, e * n / 2, LOAD_XSTRETCH, LSM_F64) as S:
        d_u = torch.from_numpy(U).cuda()
        torch.cuda.synchronize()
        want = Em * (nu - 1) / (2 * nu * nu + nu - 1)
        for call in range(2):
            out = _noalloc(S, d_u)
            assert out[9] == pytest.approx(want, rel=1e-9), call
            assert out[0] == pytest.approx(want * e * n ** 3, rel=1e-9), call


def test_stress_noalloc_rejects_oversized_box(gpu):
    """Boxes above PS_LSM_NOALLOC_MAX_CUBES (128^3) are refused with PS_ERR_ARG."""
    import torch

    from porescale_gb300._lib import last_error

    ind = np.zeros((128, 128, 136), np.int32)  # 2,228,224 cubes
    with SpringNetwork(ind, 1.0, 0.4, 1.0, 0.4, 0.01, LOAD_XSTRETCH, LSM_F64) as S:
        d_u = torch.zeros(3 * ind.size, dtype=torch.float64, device="cuda")
        out = (C.c_double * 10)()
        rc = S._lib.ps_lsm_stress_noalloc(S._h, C.c_void_p(d_u.data_ptr()), out)
        assert rc == 1
        assert "maximum" in last_error()
