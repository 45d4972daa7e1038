"""Seeded synthetic porous geometries in the reference's ``ind`` convention.

The reference reads its geometry from an ``ind`` file (1 pore, 0 solid; the
two-solid codes also use 3 for the second solid, XX_P.f:446-523).  It ships
no benchmark geometries, so the workloads here are generated:

* :func:`sphere_pack` -- periodic union of solid spheres of radius r with
  centres uniform in the box, added until the porosity reaches the target;
* :func:`inclusions` -- an all-solid cube (value 0) with spherical phase-2
  inclusions (value 3) added until their volume fraction reaches the target;
* :func:`blob_colours` -- red/blue assignment of the pore voxels in random
  cubic blobs, used for the 256^3 two-phase workload;
* :func:`gray_field` -- smoothed-noise gray solid fraction in [0, 1].

Randomness comes from SplitMix64 so that a (seed, sizes) pair gives the same
geometry on every machine and numpy version.
"""
from __future__ import annotations

import numpy as np

_M64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 generator (Steele, Lea, Flood 2014) returning doubles in [0,1)."""

    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))


def _ball_offsets(r: float):
    ri = int(np.ceil(r))
    g = np.arange(-ri, ri + 1)
    dz, dy, dx = np.meshgrid(g, g, g, indexing="ij")
    keep = dx * dx + dy * dy + dz * dz <= r * r
    return dz[keep], dy[keep], dx[keep]


def _place_spheres(field: np.ndarray, value: int, background: int, radius, target_count: int, seed: int,
                   max_spheres: int = 10_000_000) -> int:
    """Paints balls of `value` over `background` voxels (periodic) until at
    least `target_count` voxels carry `value`.  radius is a float or a
    (rmin, rmax) pair drawn uniformly per sphere.  Returns spheres placed."""
    nz, ny, nx = field.shape
    rng = SplitMix64(seed)
    count = int(np.count_nonzero(field == value))
    n = 0
    cache = {}
    while count < target_count and n < max_spheres:
        cx, cy, cz = rng.uniform() * nx, rng.uniform() * ny, rng.uniform() * nz
        if isinstance(radius, tuple):
            r = radius[0] + (radius[1] - radius[0]) * rng.uniform()
        else:
            r = float(radius)
        key = round(r, 6)
        if key not in cache:
            cache[key] = _ball_offsets(r)
        dz, dy, dx = cache[key]
        iz = (dz + int(np.floor(cz))) % nz
        iy = (dy + int(np.floor(cy))) % ny
        ix = (dx + int(np.floor(cx))) % nx
        sel = field[iz, iy, ix]
        fresh = sel == background
        if fresh.any():
            field[iz[fresh], iy[fresh], ix[fresh]] = value
            count += int(fresh.sum())
        n += 1
    return n


def sphere_pack(n, porosity: float, radius, seed: int) -> np.ndarray:
    """ind[nz,ny,nx] (int32): 1 pore, 0 solid; solid = union of spheres."""
    nz, ny, nx = (n, n, n) if np.isscalar(n) else n
    ind = np.ones((nz, ny, nx), np.int32)
    target_solid = int(np.ceil((1.0 - porosity) * ind.size))
    _place_spheres(ind, 0, 1, radius, target_solid, seed)
    return ind


def inclusions(n, fraction: float, radius, seed: int) -> np.ndarray:
    """ind[nz,ny,nx]: 0 = solid phase 1 (matrix), 3 = spherical phase-2 inclusions."""
    nz, ny, nx = (n, n, n) if np.isscalar(n) else n
    ind = np.zeros((nz, ny, nx), np.int32)
    _place_spheres(ind, 3, 0, radius, int(np.ceil(fraction * ind.size)), seed)
    return ind


def blob_colours(ind: np.ndarray, red_fraction: float, blob: int, seed: int, iipore: int = 1) -> np.ndarray:
    """Per-voxel colour (1.0 red, 0.0 blue) on pore voxels: the box is cut in
    blob^3 cubes, each red with probability `red_fraction`."""
    nz, ny, nx = ind.shape
    bz, by, bx = -(-nz // blob), -(-ny // blob), -(-nx // blob)
    rng = SplitMix64(seed)
    red = np.array([1.0 if rng.uniform() < red_fraction else 0.0 for _ in range(bz * by * bx)]).reshape(bz, by, bx)
    col = np.repeat(np.repeat(np.repeat(red, blob, 0), blob, 1), blob, 2)[:nz, :ny, :nx]
    return np.where(ind == iipore, col, 0.0)


def colour_state(ind: np.ndarray, colour: np.ndarray, cr2=1.0 / 3.0, cb2=1.0 / 3.0, rr0=1.0, rb0=1.0,
                 dt=1.0, iipore: int = 1):
    """Rest-equilibrium populations fr, fb [nl,19] in the reference's fluid
    order (i outer, k inner: x slowest, z fastest) for a colour field, the
    same construction as initdistr (S1:2834-2841)."""
    def w(c2):
        t1 = 1.0 - 2.0 * c2 * dt * dt
        t2 = c2 * dt * dt * (1.0 / 6.0)
        t3 = c2 * dt * dt * (1.0 / 12.0)
        return np.array([t1] + [t2] * 6 + [t3] * 12)
    tr, tb = w(cr2), w(cb2)
    # reference order: loop x (outer), y, z (inner) over ind[z,y,x]
    sel = np.transpose(ind, (2, 1, 0)) == iipore
    c = np.transpose(colour, (2, 1, 0))[sel]
    fr = tr[None, :] * c[:, None] * rr0
    fb = tb[None, :] * (1.0 - c)[:, None] * rb0
    return np.ascontiguousarray(fr), np.ascontiguousarray(fb)


def gray_field(n, sigma: float, slope: float, quantile: float, seed: int) -> np.ndarray:
    """Gray solid fraction s in [0,1]: seeded Gaussian noise, periodic
    Gaussian smoothing of width sigma, then a sigmoid of the given slope
    centred at the given quantile."""
    nz, ny, nx = (n, n, n) if np.isscalar(n) else n
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.standard_normal((nz, ny, nx))
    k = [np.fft.fftfreq(m) for m in (nz, ny, nx)]
    kz, ky, kx = np.meshgrid(*k, indexing="ij")
    filt = np.exp(-2.0 * (np.pi * sigma) ** 2 * (kx * kx + ky * ky + kz * kz))
    sm = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    sm = (sm - sm.mean()) / sm.std()
    c = np.quantile(sm, quantile)
    return 1.0 / (1.0 + np.exp(-slope * (sm - c)))


def spanning_solid(ind: np.ndarray) -> np.ndarray:
    """ind with every solid cluster except the largest turned into pore (1).

    Solid voxels (0 and 3) belong to one cluster when they share a face,
    periodic in every axis.  The lattice-spring network couples cubes that
    share only a corner or an edge through no angular spring, so such a
    joint is a hinge, and a cluster not face-joined to the largest one is a
    free body or a mechanism: under a fluid wall load it has no static
    equilibrium."""
    from scipy import ndimage
    solid = (ind == 0) | (ind == 3)
    pad = np.pad(solid, 1, mode="wrap")
    lab, n = ndimage.label(pad, structure=ndimage.generate_binary_structure(3, 1))
    parent = np.arange(n + 1)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    # every padded voxel is a copy of an interior one: join their labels
    core = lab[1:-1, 1:-1, 1:-1]
    nz, ny, nx = solid.shape
    zi = (np.arange(nz + 2) - 1) % nz
    yi = (np.arange(ny + 2) - 1) % ny
    xi = (np.arange(nx + 2) - 1) % nx
    ref = core[np.ix_(zi, yi, xi)]
    shell = np.ones(pad.shape, bool)
    shell[1:-1, 1:-1, 1:-1] = False
    for a, b in zip(lab[shell & pad], ref[shell & pad]):
        ra, rb = find(int(a)), find(int(b))
        if ra != rb:
            parent[ra] = rb
    roots = np.array([find(int(c)) if c else 0 for c in range(n + 1)])
    comp = roots[core]
    if not solid.any():
        return ind.copy()
    counts = np.bincount(comp[solid])
    counts[0] = 0
    keep = int(np.argmax(counts))
    out = ind.copy()
    out[solid & (comp != keep)] = 1
    return out
