"""porescale_run, the reference driver's LBM loop on the C ABI, run in a
directory laid out like the reference's (INPUT_PARAMETERS, ind,
velocities19): its output.m rows must match the FP64 oracle after the same
number of steps, and a restart from iteration2 must continue the run
exactly."""
import os
import subprocess

import numpy as np
import pytest

from porescale_gb300 import geometry as geo
from porescale_gb300.lattice import make_params

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
VEL19 = [[0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
         [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
         [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]]


def _write_case(d, ind, itm, itw, icon=0, sat=0.5, wet=0.5):
    nz, ny, nx = ind.shape
    lines = ["0.3333333333333333D0  cr2", "1.D0  rr0", "1.D0  rb0", "0.7D0  B", "0.001D0  sig", "0.1666666666666667D0 vir",
             "0.1D0  vib", f"{wet}D0  wet", "1  idir", f"{itm}  itm", f"{itw}  itw", "1  its", "-0.0000001D0 eps",
             "0  mtype", f"{icon}  icon", f"{sat}D0  sat", "1  iipore", "1  npores", "0.D0  ee", "20.D0  lsize",
             "1.D-5 0.D0 0.D0   bfr", "1.D-5 0.D0 0.D0   bfb", f"{nx}  ncx", f"{ny}  ncy", f"{nz}  ncz",
             "94.5D0  Em", "0.0742d0  nu", "2.65d0  rs", "1.d0  dt", "1.d0  dl"]
    open(os.path.join(d, "INPUT_PARAMETERS"), "w").write("\n".join(lines) + "\n")
    with open(os.path.join(d, "ind"), "w") as f:
        for k in range(nz):
            for j in range(ny):
                f.write(" " + "".join(str(v) for v in ind[k, j]) + "\n")
    with open(os.path.join(d, "velocities19"), "w") as f:
        for row in VEL19:
            f.write("".join(f"{v:3d}" for v in row) + "\n")


def _rows(d):
    rows = []
    for ln in open(os.path.join(d, "output.m")):
        ln = ln.strip()
        if ln and ln[0].isdigit():
            rows.append([float(t) for t in ln.rstrip(";").split()])
    return np.array(rows)


def _run(d, *args):
    exe = os.path.join(ROOT, "porescale_gb300", "porescale_run")
    r = subprocess.run([exe, "-d", d, "-q", *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_matches_oracle(gpu, oracle_lib, tmp_path):
    from porescale_gb300 import _build
    _build.build_driver()
    ind = geo.sphere_pack((20, 16, 12), 0.45, 3.0, seed=4)
    d = str(tmp_path)
    _write_case(d, ind, itm=3, itw=5)
    _run(d)
    rows = _rows(d)
    assert rows.shape == (3, 12)
    p = make_params(B=0.7, sig=1e-3, vir=0.1666666666666667, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    o = oracle_lib.OracleLattice(p, ind)
    o.init_random(0.5)
    o.run(2)  # the initialisation pass
    for it1 in range(1, 4):
        o.run(5, 4)
        ob = o.observables()
        assert rows[it1 - 1, 0] == it1 * 5
        # E15.8 keeps 8 significant digits
        assert rows[it1 - 1, 1] == pytest.approx(ob["permr"], rel=1e-7)
        assert rows[it1 - 1, 2] == pytest.approx(ob["permb"], rel=1e-7)
        assert rows[it1 - 1, 10] == pytest.approx(ob["nr"] / o.nl, rel=1e-7)
    # the last checkpoint is the oracle's state
    toks = open(os.path.join(d, "iteration2")).read().split()
    assert int(toks[0]) == 3
    vals = np.array([float(t) for t in toks[1:]])
    fr, fb = o.get_state()
    assert np.array_equal(vals[: fr.size], fr.ravel()) and np.array_equal(vals[fr.size:], fb.ravel())


def _read_checkpoint(d, nl):
    toks = open(os.path.join(d, "iteration2")).read().split()
    vals = np.array([float(t) for t in toks[1:]])
    assert vals.size == 2 * 19 * nl
    return int(toks[0]), vals[: 19 * nl].reshape(nl, 19), vals[19 * nl:].reshape(nl, 19)


def test_driver_restart_continues_exactly(gpu, oracle_lib, tmp_path):
    """icon = 1 restarts from iteration2: the initialisation pass runs again
    (majorityrule always runs it) and the blocks continue from it1 + 1."""
    from porescale_gb300 import _build
    _build.build_driver()
    ind = geo.sphere_pack((16, 12, 14), 0.45, 3.0, seed=6)
    d = str(tmp_path)
    _write_case(d, ind, itm=2, itw=3)
    _run(d)
    p = make_params(B=0.7, sig=1e-3, vir=0.1666666666666667, vib=0.1, wet=0.5, bfr=(1e-5, 0, 0), bfb=(1e-5, 0, 0))
    o = oracle_lib.OracleLattice(p, ind)
    it1, fr, fb = _read_checkpoint(d, o.nl)
    assert it1 == 2
    _write_case(d, ind, itm=4, itw=3, icon=1)
    _run(d)
    rows = _rows(d)
    assert rows.shape == (4, 12) and list(rows[:, 0]) == [3, 6, 9, 12]
    o.set_state(fr, fb)
    o.run(2)
    for it1 in (3, 4):
        o.run(3, 4)
        ob = o.observables()
        assert rows[it1 - 1, 1] == pytest.approx(ob["permr"], rel=1e-7)
        assert rows[it1 - 1, 11] == pytest.approx(ob["nb"] / o.nl, rel=1e-7)
    it1, fr2, fb2 = _read_checkpoint(d, o.nl)
    gr, gb = o.get_state()
    assert it1 == 4 and np.array_equal(fr2, gr) and np.array_equal(fb2, gb)
    assert not os.path.exists(os.path.join(d, "iteration"))


def _write_lsm_case(d, ind, Em1, nu1, Em2, nu2, g):
    nz, ny, nx = ind.shape
    vals = [nx, ny, nz, Em1, nu1, Em2, nu2, 2.65, 1.0, 1.0, 1, 1, g, 1, 0]
    open(os.path.join(d, "INPUT_PARAMETERS"), "w").write("\n".join(f"{v}" for v in vals) + "\n")
    with open(os.path.join(d, "ind"), "w") as f:
        for k in range(nz):
            for j in range(ny):
                f.write(" " + "".join(str(v) for v in ind[k, j]) + "\n")


@pytest.mark.parametrize("mode", ["xx", "yz"])
def test_driver_lsm_mode_matches_api(gpu, tmp_path, mode):
    """porescale_run -m xx|yz: the reference program's INPUT_PARAMETERS in,
    stress_tensor and LSM_displ_field out, equal to the C ABI's solve."""
    from porescale_gb300 import _build
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, SpringNetwork, spring_constants
    _build.build_driver()
    ind = geo.inclusions(10, 0.25, 2.5, seed=8)
    d = str(tmp_path)
    g = 0.004
    _write_lsm_case(d, ind, 18.0, 0.3, 6.0, 0.25, g)
    _run(d, "-m", mode)
    txt = open(os.path.join(d, "stress_tensor")).read()
    key = "Exxxx" if mode == "xx" else "Eyzyz"
    got = float(txt.split(key + " =")[1].split()[0])
    a1, b1 = spring_constants(18.0, 0.3)
    a2, b2 = spring_constants(6.0, 0.25)
    load = LOAD_XSTRETCH if mode == "xx" else LOAD_YZSHEAR
    with SpringNetwork(ind, a1, b1, a2, b2, g, load, LSM_F64) as S:
        r = S.solve(1e-10, 200000)
    assert got == pytest.approx(r.modulus, rel=1e-12)
    disp = np.loadtxt(os.path.join(d, "LSM_displ_field"))
    assert disp.shape == (ind.size, 3) and np.abs(disp).max() > 0
    assert os.path.exists(os.path.join(d, "iteration2")) and os.path.exists(os.path.join(d, "lsm_settings"))
