"""Writes tests/golden/reference_tables.json from the reference sources.

Usage: python tests/golden/make_golden.py <porescale checkout>, or with the
checkout's path in $PORESCALE_REF.  It extracts the lattice-spring constant tables
the reference ships or spells out literally, so the tests can check our own
derivations of them without the reference present:

* `anf` -- the 48 x 9 angle table (plane normal, force directions on the two
  arm ends) written literally in LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f;
* `nta` -- the 48 angle arm-direction pairs of the same file;
* the cube-local tables cube_bon / cube_sbond / cube_ang / cube_abond of
  LSM2S/Cxxxx (as canonical sorted sets: their row order is irrelevant);
* the table sizes the oracle builds for the two shipped `ind` geometries;
* 40^3 crops of those two geometries (shipped_crops.npz: the corner
  [0:40, 0:40, 0:40] of each, values as shipped) with the oracle's table
  sizes for them, so GPU parity runs on the reference's own inputs.
"""
import json
import math
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = None  # the porescale checkout, set by main()


def parse_anf(src):
    consts = {"0.d0": 0.0, "1.d0": 1.0, "c1d2": 0.5, "c1ds3": 1 / math.sqrt(3.0), "c1d2s3": 1 / (2 * math.sqrt(3.0)),
              "c1ds2": 1 / math.sqrt(2.0)}
    text = re.sub(r"\n\s*&", "", src)
    anf = np.zeros((48, 9))
    for j, body in re.findall(r"anf\(1:9,(\d+)\)=\(/([^/]*)/\)", text):
        toks = [t.strip() for t in body.split(",")]
        vals = []
        for t in toks:
            sgn = -1.0 if t.startswith("-") else 1.0
            vals.append(sgn * consts[t.lstrip("-")])
        anf[int(j) - 1] = vals
    nta = np.zeros((48, 2), int)
    for j, a, b in re.findall(r"nta\(1:2,(\d+)\)=\(/(\d+),(\d+)/\)", text):
        nta[int(j) - 1] = (int(a), int(b))
    return anf, nta


def read_ind(path, nx, ny, nz):
    lines = open(path).read().split("\n")
    ind = np.zeros((nz, ny, nx), np.int32)
    k = 0
    for z in range(nz):
        for y in range(ny):
            row = lines[k].strip()
            k += 1
            ind[z, y] = [int(c) for c in row[:nx]]
    return ind


def main():
    src = open(os.path.join(REF, "LBM-LSM", "lsm_lbm_static_alpha_beta_multipore.f")).read()
    anf, nta = parse_anf(src)
    d = os.path.join(REF, "LSM2S", "Cxxxx")
    bon = np.loadtxt(os.path.join(d, "cube_bon"), dtype=int).reshape(-1, 3)
    sb = np.loadtxt(os.path.join(d, "cube_sbond"))
    ang = np.loadtxt(os.path.join(d, "cube_ang"), dtype=int).reshape(-1, 6)
    ab = np.loadtxt(os.path.join(d, "cube_abond"))
    cube_bonds = sorted([int(b[0]), int(b[1]), int(b[2]), float(s)] for b, s in zip(bon, sb))
    cube_angles = sorted([*map(int, a), float(s)] for a, s in zip(ang, ab))
    out = {"anf": anf.tolist(), "nta": nta.tolist(), "cube_bonds": cube_bonds, "cube_angles": cube_angles}
    # table sizes of the shipped geometries through the oracle
    sys.path.insert(0, ROOT)
    import oracle
    from porescale_gb300.lattice import make_params
    sizes = {}
    for name, dims in (("LBM-LSM", (120, 120, 120)), ("LBM-LSM2S", (150, 150, 54))):
        ind = read_ind(os.path.join(REF, name, "ind"), *dims)
        o = oracle.OracleLattice(make_params(), ind)
        sizes[name] = {"nl": o.nl, "nps": o.nps, "npb2": o.npb2, "npb4": o.npb4, "ns": o.ns,
                       "n_overflow": o.n_overflow, "solid": int((ind == 0).sum()), "phase2": int((ind == 3).sum())}
    out["shipped_geometry_tables"] = sizes
    crops, crop_sizes = {}, {}
    for key, name, dims in (("lbm_lsm_40", "LBM-LSM", (120, 120, 120)), ("lbm_lsm2s_40", "LBM-LSM2S", (150, 150, 54))):
        c = read_ind(os.path.join(REF, name, "ind"), *dims)[:40, :40, :40].astype(np.uint8)
        crops[key] = c
        o = oracle.OracleLattice(make_params(), c.astype(np.int32))
        crop_sizes[key] = {"nl": o.nl, "nps": o.nps, "npb2": o.npb2, "npb4": o.npb4, "ns": o.ns,
                           "values": sorted(int(v) for v in np.unique(c))}
    np.savez_compressed(os.path.join(HERE, "shipped_crops.npz"), **crops)
    out["shipped_crop_tables"] = crop_sizes
    with open(os.path.join(HERE, "reference_tables.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_tables.json"))


if __name__ == "__main__":
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PORESCALE_REF")
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py <porescale checkout>  (or set PORESCALE_REF)")
    main()
