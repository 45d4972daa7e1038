"""GPU parity of the colour-gradient D3Q19 lattice against the FP64 oracle.

The FP64 lattice is compiled without FMA contraction and keeps the
reference's operation order, so after any number of steps its populations
must equal the oracle's bit for bit.  The FP32 and 16-bit storage forms are
compared against the FP64 oracle with the tolerances written in each test.
"""
import numpy as np
import pytest

from porescale_gb300 import PREC_BF16, PREC_F16, PREC_F32, PREC_F64
from porescale_gb300 import geometry as geo
from porescale_gb300._lib import PorescaleError
from porescale_gb300.lattice import Lattice, make_params

pytestmark = pytest.mark.gpu


def _case(n=(20, 18, 24), porosity=0.45, radius=4, seed=7, wet=0.7071067811865476, bf=1e-5, vir=1 / 6, vib=1 / 6,
          B=0.7, sig=1e-3):
    ind = geo.sphere_pack(n, porosity, radius, seed)
    p = make_params(B=B, sig=sig, vir=vir, vib=vib, wet=wet, bfr=(bf, 0, 0), bfb=(bf, 0, 0))
    return ind, p


def test_tables_bit_exact(gpu, oracle_lib):
    for n, seed in (((20, 18, 24), 7), ((16, 16, 16), 3), ((9, 13, 11), 5)):
        ind, p = _case(n=n, seed=seed)
        o = oracle_lib.OracleLattice(p, ind)
        with Lattice(p, ind, PREC_F64) as L:
            i = L.info
            assert (i.nl, i.nps, i.npb2, i.npb4, i.ns) == (o.nl, o.nps, o.npb2, o.npb4, o.ns)
            icor, ips, ipb2, ipb4 = L.tables()
            oicor, oips, oipb2, oipb4, _, _ = o.tables()
            assert np.array_equal(icor, oicor)
            assert np.array_equal(ips, oips)
            assert np.array_equal(ipb2, oipb2)
            assert np.array_equal(ipb4, oipb4)


def test_state_roundtrip(gpu, oracle_lib):
    """set_state/get_state is the identity for every storage precision on FP64 inputs
    within the storage rounding (exact for FP64)."""
    ind, p = _case()
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    o.run(3)
    fr, fb = o.get_state()
    for prec, tol in ((PREC_F64, 0.0), (PREC_F32, 1e-7), (PREC_F16, 2e-5), (PREC_BF16, 2e-4)):
        with Lattice(p, ind, prec) as L:
            L.set_state(fr, fb)
            gr, gb = L.get_state()
            assert np.max(np.abs(gr - fr)) <= tol
            assert np.max(np.abs(gb - fb)) <= tol


@pytest.mark.parametrize("steps", [1, 7, 40])
def test_f64_bit_exact_vs_oracle(gpu, oracle_lib, steps):
    ind, p = _case()
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    with Lattice(p, ind, PREC_F64) as L:
        L.init_random(0.5)
        a, b = L.get_state()
        fr0, fb0 = o.get_state()
        assert np.array_equal(a, fr0) and np.array_equal(b, fb0)
        L.step(steps)
        o.run(steps, 4)
        gr, gb = L.get_state()
        fr, fb = o.get_state()
        nd = int(np.sum(gr != fr) + np.sum(gb != fb))
        assert nd == 0, f"{nd} populations differ; max |d| = {max(np.abs(gr - fr).max(), np.abs(gb - fb).max())}"
        rr, rb, cf = L.fields()
        orr, orb, ocf = o.fields()
        assert np.array_equal(rr, orr) and np.array_equal(rb, orb) and np.array_equal(cf, ocf)


def test_f64_observables_vs_oracle(gpu, oracle_lib):
    ind, p = _case()
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    o.run(25, 4)
    with Lattice(p, ind, PREC_F64) as L:
        L.init_random(0.5)
        L.step(25)
        g = L.observables().as_dict()
    ob = o.observables()
    rel = 1e-11
    for k in ("tmr", "tmb", "tm", "Cpr", "Cpb", "permr", "permb"):
        if np.isnan(ob[k]):  # e.g. Cpr = cr2*0/0 when no node has cf > 0.99
            assert np.isnan(g[k]), k
            continue
        assert g[k] == pytest.approx(ob[k], rel=rel, abs=1e-14), k
    for d in range(3):
        assert g["Qr"][d] == pytest.approx(ob[f"Qr{d}"], rel=rel, abs=1e-16)
        assert g["Qb"][d] == pytest.approx(ob[f"Qb{d}"], rel=rel, abs=1e-16)
        assert g["bmt"][d] == pytest.approx(ob[f"bmt{d}"], rel=rel, abs=1e-12)
        assert g["rmt"][d] == pytest.approx(ob[f"rmt{d}"], rel=rel, abs=1e-12)
    assert (g["nr"], g["nb"], g["nr_cf"], g["nb_cf"]) == (ob["nr"], ob["nb"], ob["nr_cf"], ob["nb_cf"])
    assert g["isneg"] == int(ob["isneg"])


@pytest.mark.parametrize("prec,tol", [(PREC_F32, 2e-5), (PREC_F16, 5e-4), (PREC_BF16, 3e-3)])
def test_low_precision_close_to_oracle(gpu, oracle_lib, prec, tol):
    """Population max-abs error after 20 steps, relative to the rest weight
    scale (populations are O(0.05)): FP32 2e-5, FP16 5e-4, BF16 3e-3."""
    ind, p = _case()
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    o.run(20, 4)
    fr, fb = o.get_state()
    with Lattice(p, ind, prec) as L:
        L.init_random(0.5)
        L.step(20)
        gr, gb = L.get_state()
    err = max(np.abs(gr - fr).max(), np.abs(gb - fb).max())
    assert err <= tol, err


@pytest.mark.parametrize("prec", [PREC_F64, PREC_F32, PREC_F16])
def test_step_configurations_agree(gpu, prec):
    """Every compiled (collide, density) CTA-size pair gives the same state."""
    ind, p = _case(n=(11, 13, 40))
    ref = None
    for tx, ty, zc in ((128, 256, 0), (256, 256, 0), (128, 128, 0), (128, 256, 6), (128, 256, 7), (128, 256, 8),
                       (256, 256, 3)):
        with Lattice(p, ind, prec) as L:
            L.set_tile(tx, ty, zc)
            L.init_random(0.4)
            L.step(6)
            st = L.get_state()
        if ref is None:
            ref = st
        assert np.array_equal(st[0], ref[0]) and np.array_equal(st[1], ref[1]), (tx, ty, zc)


def test_plain_two_phase_64_workload(gpu, oracle_lib):
    """The plain FP64 two-phase configuration: 64^3 periodic union of
    radius-6 spheres down to porosity 0.40, each pore voxel red or blue with
    p = 0.5 (initdistr), tau = 1 (nu = 1/6), A = 1e-3, beta = 0.7, contact
    angle 45 degrees (wetting colour cos 45), body force 1e-5 along x.  The
    GPU FP64 lattice equals the oracle bit for bit after the 2 init steps
    plus 48 steps, and the check_state observables agree to 1e-11."""
    import math
    ind = geo.sphere_pack(64, 0.40, 6, seed=20240530)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=1 / 6, wet=math.cos(math.radians(45.0)), bfr=(1e-5, 0, 0),
                    bfb=(1e-5, 0, 0))
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    o.run(50, 8)
    with Lattice(p, ind, PREC_F64) as L:
        assert L.nl == o.nl and L.info.nps == o.nps
        L.init_random(0.5)
        L.step(50)
        gr, gb = L.get_state()
        g = L.observables().as_dict()
    fr, fb = o.get_state()
    assert np.array_equal(gr, fr) and np.array_equal(gb, fb)
    ob = o.observables()
    for k in ("permr", "permb", "tmr", "tmb"):
        assert g[k] == pytest.approx(ob[k], rel=1e-11), k
    assert (g["nr"], g["nb"]) == (ob["nr"], ob["nb"])


@pytest.mark.parametrize("prec", [0, 1, 2, 3])
@pytest.mark.parametrize("planes,ahead,tile", [(1, 1, (128, 256, 0)), (3, 2, (256, 256, 0)), (4, 1, (128, 256, 8))])
def test_fused_step_matches_two_pass(gpu, prec, planes, ahead, tile):
    """The fused one-launch step (density and collide tiles of z-slabs from
    one work list) gives the two-pass step's state bit for bit."""
    ind = geo.sphere_pack((22, 18, 20), 0.45, 3.0, seed=17)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    out = []
    for fused in (False, True):
        with Lattice(p, ind, prec) as L:
            L.init_random(0.5)
            L.set_tile(*tile)
            if fused:
                L.set_fused(planes, ahead)
                assert L.get_info().schedule == planes + 256 * ahead
            L.step(9)
            out.append(L.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("prec", [0, 1, 2, 3])
@pytest.mark.parametrize("planes,window,tile", [(1, 0, (128, 256, 0)), (2, 3, (128, 256, 6)),
                                                (7, 0, (256, 256, 0)), (32, 0, (128, 256, 8))])
def test_wave_schedule_matches_two_pass(gpu, prec, planes, window, tile):
    """The wavefront schedule (8-step graphs of z-slab launches ordered by
    their data dependencies) gives the two-pass step's state bit for bit,
    also with solid-only slabs (empty launches), a single slab and a step
    count that ends with two-pass steps."""
    ind = geo.sphere_pack((22, 18, 20), 0.45, 3.0, seed=17)
    ind[:, :, 8:10] = 1  # two solid planes: slabs without fluid nodes
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    out = []
    for wave in (False, True):
        with Lattice(p, ind, prec) as L:
            L.init_random(0.5)
            L.set_tile(*tile)
            if wave:
                L.set_wave(planes, window)
                assert L.get_info().wave == planes + 256 * window
            L.step(19)
            L.step(8)
            out.append(L.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("prec,tol", [(PREC_F16, 1e-4), (PREC_BF16, 1e-3)])
def test_restart_16bit(gpu, prec, tol):
    """A 16-bit lattice continued directly and one restarted from its
    get_state (stored against each node's own densities, then read so by
    the first step) stay within the storage rounding of each other."""
    ind, p = _case()
    with Lattice(p, ind, prec) as A, Lattice(p, ind, prec) as B:
        A.init_random(0.5)
        A.step(10)
        fr, fb = A.get_state()
        B.set_state(fr, fb)
        A.step(10)
        B.step(10)
        ar, ab = A.get_state()
        br, bb = B.get_state()
    assert max(np.abs(ar - br).max(), np.abs(ab - bb).max()) <= tol


def test_wave_schedule_without_fluid(gpu):
    """A lattice with no fluid node: every slab launch is an empty graph node."""
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, np.zeros((6, 5, 4), np.int32), PREC_F16) as L:
        L.set_wave(1)
        L.init_random(0.5)
        L.step(16)
        o = L.observables()
        assert o.tmr == 0.0 and o.tmb == 0.0


def test_wave_and_fused_exclusive(gpu):
    ind = geo.sphere_pack((12, 12, 12), 0.45, 3.0, seed=3)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, ind, 2) as L:
        L.set_wave(2)
        L.set_fused(2, 1)
        i = L.get_info()
        assert i.wave == 0 and i.schedule == 2 + 256
        L.set_wave(3, 2)
        i = L.get_info()
        assert i.wave == 3 + 512 and i.schedule == 0
        with pytest.raises(PorescaleError):
            L.set_wave(2, 1)


@pytest.mark.parametrize("prec", [0, 2])
def test_edge_geometries(gpu, oracle_lib, prec):
    """No fluid at all (every call succeeds, observables of an empty lattice),
    no solid at all (periodic box: FP64 still bit-exact), and a 2x3x2 box
    (every neighbour is a periodic image)."""
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, np.zeros((6, 5, 4), np.int32), prec) as L:
        assert L.nl == 0
        L.init_random(0.5)
        L.step(3)
        o = L.observables()
        assert o.tmr == 0.0 and o.tmb == 0.0
    for ind in (np.ones((6, 5, 4), np.int32), np.ones((2, 3, 2), np.int32)):
        o = oracle_lib.OracleLattice(p, ind)
        o.init_random(0.5)
        fr, fb = o.get_state()
        o.run(6)
        with Lattice(p, ind, prec) as L:
            L.set_state(fr, fb)
            L.step(6)
            gr, gb = L.get_state()
        want_r, want_b = o.get_state()
        if prec == 0:
            assert np.array_equal(gr, want_r) and np.array_equal(gb, want_b)
        else:
            assert max(np.abs(gr - want_r).max(), np.abs(gb - want_b).max()) < 5e-4


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("prec", [PREC_F64, PREC_F32, PREC_F16, PREC_BF16])
def test_state_io_through_pinned_buffers(gpu, prec):
    """Page-locked caller buffers (direct DMA by the copy engines) give the
    same state as pageable ones bit for bit, in both directions."""
    ind, p = _case()
    with Lattice(p, ind, PREC_F64) as S:
        S.init_random(0.5)
        S.step(5)
        fr, fb = S.get_state()
    nl = fr.shape[0]
    hr, hb = _pinned((nl, 19)), _pinned((nl, 19))
    hr[:], hb[:] = fr, fb
    with Lattice(p, ind, prec) as A, Lattice(p, ind, prec) as B:
        A.set_state(fr, fb)    # pageable
        B.set_state(hr, hb)    # page-locked
        A.step(7)
        B.step(7)
        ar, ab = A.get_state()
        br, bb = B.get_state((_pinned((nl, 19)), _pinned((nl, 19))))
        cr, cb = B.get_state()
    assert np.array_equal(ar, br) and np.array_equal(ab, bb)
    assert np.array_equal(br, cr) and np.array_equal(bb, cb)


def test_fused_wait_gives_up_and_recovers(gpu):
    """The fused schedule's bounded device wait, run out on purpose: with a
    limit of one poll the first collide tiles find their density tiles
    unfinished, give up, and the next synchronising call returns
    PS_ERR_TIMEOUT (the wait returns rather than spins, and every index the
    collide uses comes from the geometry, so nothing leaves the lattice's
    arrays).  After ps_lbm_set_state the same lattice, back on the default
    limit, steps exactly as a fresh one."""
    ind = geo.sphere_pack((48, 40, 40), 0.45, 3.0, seed=19)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, ind, PREC_F32) as L:
        L.init_random(0.5)
        fr0, fb0 = L.get_state()
        L.set_tile(128, 256, 0)
        L.set_fused(2, 1)
        L.set_wait_limit(1)
        timed_out = False
        for _ in range(20):
            L.step(1)
            try:
                L.sync()
            except PorescaleError as exc:
                assert exc.code == 4  # PS_ERR_TIMEOUT
                timed_out = True
                break
        assert timed_out
        L.sync()  # the flag is cleared once reported
        L.set_wait_limit(0)
        L.set_state(fr0, fb0)
        L.step(6)
        L.sync()
        got = L.get_state()
    with Lattice(p, ind, PREC_F32) as R:
        R.set_state(fr0, fb0)
        R.step(6)
        want = R.get_state()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("prec", [1, 2, 3])
@pytest.mark.parametrize("rows,planes,producers,sort", [(4, 0, 4, True), (1, 1, 4, True), (5, 7, 8, True),
                                                        (18, 3, 4, False), (64, 64, 8, True), (3, 2, 4, True),
                                                        (6, 5, 12, True)])
def test_march_schedule_matches_two_pass(gpu, prec, rows, planes, producers, sort):
    """The marching one-launch step (items of `rows` rows by `planes`
    planes walked by producer and consumer warps, halo rows recomputed)
    gives the two-pass step's state bit for bit: partial last band and
    chunk, one-row bands, one band or one chunk over the whole box, several
    items per CTA, solid planes, sorted and natural collide order, and the
    restart step that reads a state set from outside."""
    ind = geo.sphere_pack((22, 18, 20), 0.45, 3.0, seed=17)
    ind[:, :, 8:10] = 1  # two solid planes
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    out = []
    for march in (False, True):
        with Lattice(p, ind, prec) as L:
            L.init_random(0.5)
            if march:
                L.set_march(rows, planes, producers, sort)
                m = L.get_info().march
                assert m & 4095 == min(rows, 18) and (m >> 12) & 0x1FFF >= 1
                assert ((m >> 25) & 3) * 4 == producers and bool((m >> 30) & 1) == (not sort)
            L.step(13)
            fr, fb = L.get_state()
            L.set_state(fr, fb)
            L.step(4)
            L.sync()
            out.append(L.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_march_argument_errors(gpu):
    ind = geo.sphere_pack((12, 12, 12), 0.45, 3.0, seed=3)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, ind, PREC_F64) as L:
        with pytest.raises(PorescaleError):
            L.set_march(4, 0)  # FP64 has no marching form
    with Lattice(p, ind, PREC_F16) as L:
        with pytest.raises(PorescaleError):
            L.set_march(4, 0, producers=6)  # 4 or 8 producer warps
        L.set_march(4, 0)
        L.set_wave(4)
        assert L.get_info().march == 0
        L.set_march(2, 3)
        assert L.get_info().wave == 0 and L.get_info().march & 0x1FFFFFF == 2 + 4096 * 3


def test_march_wait_gives_up_and_recovers(gpu):
    """The marching step's bounded mbarrier waits, run out on purpose: with
    one poll the colliding warps find their planes unwritten, give up, and
    the next synchronising call returns PS_ERR_TIMEOUT; the launch ends
    (every wait returns, every thread arrives on every barrier, every index
    comes from the geometry).  After ps_lbm_set_state the lattice, back on
    the default limit, steps as a fresh one."""
    ind = geo.sphere_pack((48, 40, 40), 0.45, 3.0, seed=19)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    with Lattice(p, ind, PREC_F16) as L:
        L.init_random(0.5)
        fr0, fb0 = L.get_state()
        L.set_march(4, 0)
        L.set_wait_limit(1)
        timed_out = False
        for _ in range(20):
            L.step(1)
            try:
                L.sync()
            except PorescaleError as exc:
                assert exc.code == 4  # PS_ERR_TIMEOUT
                timed_out = True
                break
        assert timed_out
        L.sync()
        L.set_wait_limit(0)
        L.set_state(fr0, fb0)
        L.step(6)
        L.sync()
        got = L.get_state()
    with Lattice(p, ind, PREC_F16) as R:
        R.set_state(fr0, fb0)
        R.step(6)
        want = R.get_state()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_sorted_collide_matches_natural_order(gpu, prec):
    """The two-pass collide with each CTA's bulk nodes taken before its
    interface nodes gives the same state bit for bit, directly and in the
    wavefront graphs."""
    ind = geo.sphere_pack((22, 18, 20), 0.45, 3.0, seed=17)
    p = make_params(B=0.7, sig=1e-3, vir=1 / 6, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    out = []
    for sort in (False, True):
        with Lattice(p, ind, prec) as L:
            L.init_random(0.5)
            L.set_sort(sort)
            L.step(5)
            L.set_wave(4)
            L.step(16)
            out.append(L.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_rounding_seed(gpu):
    """16-bit stores: the same rounding seed reproduces a run exactly,
    another seed gives another sample within the storage rounding."""
    ind, p = _case()
    out = []
    for seed in (0, 0, 7):
        with Lattice(p, ind, PREC_F16) as L:
            L.init_random(0.5)
            L.set_rounding_seed(seed)
            L.step(10)
            out.append(L.get_state()[0])
    assert np.array_equal(out[0], out[1])
    assert not np.array_equal(out[0], out[2])
    assert np.abs(out[0] - out[2]).max() <= 1e-4
