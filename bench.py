"""Benchmark of the colour-gradient D3Q19 two-phase step on GB300.

Workload (the precision-form two-phase configuration): 256^3 periodic box,
solid = union of radius-10 spheres (seeded centres) down to porosity 0.35,
red saturation 0.5 in random 8^3 blobs, tau_red 0.8 / tau_blue 1.5 (TRT,
magic 3/16), surface tension 1e-3, recolouring beta 0.7, contact angle 30
degrees (wetting colour cos 30), body force 1e-6 along x.  The reference
ships no benchmark geometry; seeded synthetic inputs with these sizes stand
in for it.

A step is one full lattice update (one launch of the fused step kernel).
`value` is MLUPS (fluid-node updates per second, all ranks) of the headline
precision (FP16 deviation storage, FP32 arithmetic) with the state resident
in HBM; `e2e` is the same metric through the C ABI with host buffers (state
uploaded from pinned host memory, `itw` steps, observables and state read
back, every e2e step).  FP64 (plain) and FP32 legs run on the same box.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes per fluid-node update: 2 components x 19 populations x
# (1 read + 1 write) x storage size + the per-node density field (1 write +
# 1 read per component)
ALGO_BYTES = {"f64": 640, "f32": 320, "f16": 168, "bf16": 168}
PREC_ID = {"f64": 0, "f32": 1, "f16": 2, "bf16": 3}


def workload_config(size: int):
    tau_r, tau_b = 0.8, 1.5
    return {
        "workload": f"two-phase colour-gradient D3Q19, {size}^3 sphere pack (r=10, porosity 0.35), "
                    f"S_r0=0.5 in 8^3 blobs",
        "size": size, "radius": 10, "porosity": 0.35, "seed": 20240531, "blob": 8, "red_fraction": 0.5,
        "tau_red": tau_r, "tau_blue": tau_b, "vir": (tau_r - 0.5) / 3.0, "vib": (tau_b - 0.5) / 3.0,
        "sig": 1e-3, "B": 0.7, "wet": math.cos(math.radians(30.0)), "bf": 1e-6,
    }


def march_fields(m: int):
    """(rows, planes, producer warps, sorted) of ps_lbm_info.march."""
    return m & 4095, (m >> 12) & 0x1FFF, ((m >> 25) & 3) * 4, not (m >> 30) & 1  # producer warps 4, 8, 12


def bench_config(cfg, nl):
    """The `config` object of both bench arms (identical for the same
    workload): the workload, its size, seed and fluid-node count.  The state
    of every precision is larger than the 129 MB L2, so no flush is needed
    between timed steps."""
    return {"workload": cfg["workload"], "size": cfg["size"], "seed": cfg["seed"], "fluid_nodes": int(nl),
            "l2": "state > L2 (no flush needed)"}


def make_workload(cfg):
    from porescale_gb300 import geometry
    from porescale_gb300.lattice import make_params
    n = cfg["size"]
    ind = geometry.sphere_pack(n, cfg["porosity"], cfg["radius"], cfg["seed"])
    col = geometry.blob_colours(ind, cfg["red_fraction"], cfg["blob"], cfg["seed"] + 1)
    fr, fb = geometry.colour_state(ind, col)
    p = make_params(B=cfg["B"], sig=cfg["sig"], vir=cfg["vir"], vib=cfg["vib"], wet=cfg["wet"],
                    bfr=(cfg["bf"], 0, 0), bfb=(cfg["bf"], 0, 0))
    return ind, p, fr, fb


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_accuracy(prec: str, cfg):
    """The k_r errors of storage precision `prec` against FP64 from the
    committed 20,000-step record of this workload (profiles/accuracy_256.json,
    written by --accuracy-steps 20000 --accuracy-every 100), or None.  For
    stochastically rounded storage the mean over the recorded rounding
    seeds, with the largest and the error of the seed ensemble."""
    path = os.path.join(ROOT, "profiles", "accuracy_256.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    if d.get("workload") != cfg["workload"] or prec not in d.get("kr_err", {}):
        return None
    k = d["kr_err"]
    out = {"kr_err_red": k[prec]["red"], "kr_err_blue": k[prec]["blue"], "definition": k["definition"],
           "window": k["window"], "samples": k["samples"], "steps": d["steps"],
           "floor_f64_one_ulp": [k["f64p"]["red"], k["f64p"]["blue"]],
           "max_sample_rel_err": [d["rel_err_vs_f64"][prec]["permr"], d["rel_err_vs_f64"][prec]["permb"]],
           "source": "profiles/accuracy_256.json"}
    if "f64n" in k:
        out["floor_f64_perturbed_1e-7"] = [k["f64n"]["red"], k["f64n"]["blue"]]
    seeds = k.get(prec + "_over_seeds")
    if seeds:
        out.update({"kr_err_red": seeds["red_mean"], "kr_err_blue": seeds["blue_mean"],
                    "kr_err_max_over_seeds": [seeds["red_max"], seeds["blue_max"]],
                    "kr_err_of_seed_ensemble": [seeds["ensemble_mean_error"]["red"],
                                                seeds["ensemble_mean_error"]["blue"]],
                    "rounding_seeds": seeds["seeds"]})
    return out


def load_traffic(prec: str, nl: int, kind: str = "two-pass"):
    """DRAM bytes of one step from the committed ncu summary (scaled to this
    workload's fluid-node count; key "<prec>" for the two-pass step,
    "<prec>_fused" / "<prec>_wave" for the other schedules, the two-pass
    figure standing for the wavefront where it has none), or None."""
    path = os.path.join(ROOT, "profiles", "lbm_step_dram.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    e = d.get(prec + ("" if kind == "two-pass" else "_" + kind))
    if not e and kind == "wave":  # measured to move the two-pass step's bytes
        e = d.get(prec)
    if not e:
        return None
    return float(e["dram_bytes_per_fluid_node"]) * nl


def max_over_ranks(t: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time (the whole job's time): all-reduce MAX over
    the process group; the value itself with one rank."""
    if world <= 1:
        return t
    import torch
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def job_rate(units_per_rank: float, t_max: float, world: int) -> float:
    """Whole-job throughput of a weak-scaled run: every rank processes the
    same units (its own replica) and the job takes the slowest rank's time."""
    return units_per_rank * world / t_max


def time_steps(L, steps, warmup, torch):
    """Device time of `steps` step launches on the lattice's stream (CUDA events).
    Under the wavefront schedule the warm-up is whole 8-step graphs, so the
    graph of the timed steps' starting buffer is built before the timing."""
    stream = torch.cuda.ExternalStream(L.stream)
    if int(L.get_info().wave):
        warmup = max(8, -(-warmup // 8) * 8)
    L.step(warmup)
    L.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    L.step(steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0


def cpu_oracle_mlups(ind, p, fr, fb, threads: int, budget_s: float):
    """Times the CPU restatement (OpenMP, `threads` threads) on the workload:
    whole-lattice steps until `budget_s` seconds are used."""
    import oracle
    o = oracle.OracleLattice(p, ind)
    o.set_state(fr, fb)
    t = time.perf_counter()
    o.run(1, threads)
    one = time.perf_counter() - t
    n = max(1, int(budget_s / max(one, 1e-6)))
    t = time.perf_counter()
    o.run(n, threads)
    dt = time.perf_counter() - t
    nl = o.nl
    o.close()
    return nl * n / dt / 1e6, n, dt


def lsm_leg(size=64, seed=20240601, cpu_budget=0.0):
    """Lattice-spring static solve on the two-solid cube (matrix alpha 1.0,
    beta 0.4; radius-5 inclusions at volume fraction 0.25, alpha 0.3, beta
    0.1; strain 1e-3): Cxxxx and Cyzyz by FP64 CG and by FP32 CG in FP64
    refinement, CG iterations per second and the inner iteration's
    bandwidth (133 algorithmic bytes per node per FP32 iteration, 265 for
    FP64).  cpu_budget > 0 also times the oracle on all host cores, about
    cpu_budget seconds for each of the two CPU algorithms (lsm_cpu_baseline)."""
    from porescale_gb300 import geometry
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, LSM_MIXED, SpringNetwork
    ind = geometry.inclusions(size, 0.25, 5.0, seed)
    g = 1e-3 * size / 2
    out = {"workload": f"two-solid lattice-spring cube {size}^3, radius-5 inclusions (fraction 0.25)",
           "rtol": 1e-10}
    peak, _ = load_peaks()
    for load, name in ((LOAD_XSTRETCH, "Cxxxx"), (LOAD_YZSHEAR, "Cyzyz")):
        for prec, pname, bpn in ((LSM_F64, "f64", 265), (LSM_MIXED, "mixed", 133)):
            with SpringNetwork(ind, 1.0, 0.4, 0.3, 0.1, g, load, prec) as S:
                S.solve(1e-10, 200000)  # warm-up (kernel loading, caches)
                t = time.perf_counter()
                r = S.solve(1e-10, 200000)
                dt = time.perf_counter() - t
                its = r.inner_iterations
                out[f"{name}_{pname}"] = {"modulus": r.modulus, "relres": r.relres, "iterations": its,
                                          "refinements": r.refinements, "seconds": dt,
                                          "cg_iters_per_s": its / dt,
                                          "achieved_gbs": its * r.nnode * bpn / dt / 1e9,
                                          "frac": its * r.nnode * bpn / dt / 1e9 / peak}
        out[f"{name}_rel_diff_mixed_vs_f64"] = abs(out[f"{name}_mixed"]["modulus"] - out[f"{name}_f64"]["modulus"]) / \
            abs(out[f"{name}_f64"]["modulus"])
    if cpu_budget > 0:
        out["cpu_baseline"] = lsm_cpu_baseline(ind, g, cpu_budget, out["Cxxxx_f64"])
    return out


# the standalone relaxation's parameters in the reference's shipped input
# (LSM2S/Cxxxx/INPUT_PARAMETERS: dt 0.01, rs 1; damping 0.5 at XX:1533)
DR_DT, DR_RS, DR_DAMP = 0.01, 1.0, 0.5


def lsm_cpu_baseline(ind, g, budget, gpu_f64):
    """The spring solve's CPU baselines on all host cores (OpenMP, the
    reference's odd/even slab scheduling of its force loops): the oracle's
    FP64 CG (iterations/s; the solve needs the GPU FP64 CG's iteration
    count) and the reference's own algorithm, the damped Verlet relaxation
    XX:1377-1545 at its shipped dt 0.01 (steps/s; the steps it needs to
    reach the CG's residual come from the committed GPU run of the same
    dynamics, profiles/lsm_dr_64.json).  Each is a bounded sample of about
    `budget` seconds on the Cxxxx system."""
    import oracle
    threads = os.cpu_count() or 1
    out = {}
    o = oracle.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    t = time.perf_counter()
    o.cg(1e-10, 3, nthreads=threads)
    per = max((time.perf_counter() - t) / 3, 1e-6)
    o.close()
    o = oracle.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    t = time.perf_counter()
    its, _ = o.cg(1e-10, max(3, int(budget / per)), nthreads=threads)
    dt = time.perf_counter() - t
    o.close()
    rate = its / dt
    out["cg"] = {"value": rate, "unit": "CG iterations/s", "cores": threads, "kind": "port", "algorithm": "CG",
                 "sample": f"first {its} FP64 CG iterations of the Cxxxx system ({dt:.1f} s, C restatement of the "
                           f"spring forces, {threads} threads)",
                 "seconds_to_solution": gpu_f64["iterations"] / rate,
                 "gpu_f64_speedup": (gpu_f64["iterations"] / rate) / gpu_f64["seconds"]}
    o = oracle.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, 0)
    t = time.perf_counter()
    o.relax(DR_DT, DR_RS, DR_DAMP, 5, 0.0, nthreads=threads)
    per = max((time.perf_counter() - t) / 5, 1e-6)
    t = time.perf_counter()
    steps = o.relax(DR_DT, DR_RS, DR_DAMP, max(5, int(budget / per)), 0.0, nthreads=threads)
    dt = time.perf_counter() - t
    o.close()
    rate = steps / dt
    dr = {"value": rate, "unit": "DR steps/s", "cores": threads, "kind": "port",
          "algorithm": "damped Verlet relaxation (XX:1377-1545)",
          "sample": f"{steps} relaxation steps of the Cxxxx system (dt {DR_DT}, damping {DR_DAMP}; {dt:.1f} s, "
                    f"{threads} threads)"}
    rec = os.path.join(ROOT, "profiles", "lsm_dr_64.json")
    if os.path.exists(rec):
        with open(rec) as f:
            need = json.load(f)["Cxxxx"]["steps"]
        dr["steps_to_cg_residual"] = need
        dr["seconds_to_solution"] = need / rate
        dr["gpu_f64_cg_speedup"] = (need / rate) / gpu_f64["seconds"]
    out["dr"] = dr
    return out


def lsm_dr_mode(args):
    """The reference's relaxation (XX:1377-1545, YZ likewise) run on the GPU
    to the static solve's residual: ps_lsm_dyn_step with dt 0.01, rs 1,
    damping 0.5 and no fluid load, from the reference's starting field (tied
    planes at -g / +g), until |F| <= 1e-10 |F_1| (F the spring forces, F_1
    those after the first step), checked every `check` steps.  Gives the
    step count the CPU relaxation baseline is scaled by."""
    import oracle
    from porescale_gb300 import geometry
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, SpringNetwork
    size = args.lsm_size
    ind = geometry.inclusions(size, 0.25, 5.0, 20240601)
    g = 1e-3 * size / 2
    out = {"mode": "lsm_dr", "size": size, "dt": DR_DT, "rs": DR_RS, "damping": DR_DAMP, "rtol": 1e-10}
    for load, name in ((LOAD_XSTRETCH, "Cxxxx"), (LOAD_YZSHEAR, "Cyzyz")):
        osp = oracle.OracleSprings(ind, 1.0, 0.4, 0.3, 0.1, g, load)
        r0 = osp.dyn_state()[0]
        ns = osp.ns
        osp.close()
        with SpringNetwork(ind, 1.0, 0.4, 0.3, 0.1, g, load, LSM_F64) as S:
            cg = S.solve(1e-10, 200000)
            S.set_dyn_state(r0)

            def fnorm():
                _, v, a = S.dyn_state(ns)
                return float(np.linalg.norm((a + DR_DAMP * v) * DR_RS))

            S.dyn_step(1, DR_DT, 1.0 / DR_RS, DR_DAMP)
            f0 = fnorm()
            steps, rel = 1, 1.0
            t = time.perf_counter()
            while rel > 1e-10 and steps < args.lsm_dr_max:
                S.dyn_step(args.lsm_dr_check, DR_DT, 1.0 / DR_RS, DR_DAMP)
                steps += args.lsm_dr_check
                rel = fnorm() / f0
            dt = time.perf_counter() - t
        out[name] = {"steps": steps, "rel_force": rel, "gpu_seconds": dt, "cg_iterations": int(cg.iterations),
                     "cg_modulus": cg.modulus}
    print(json.dumps(out))


def accuracy(args, cfg):
    """Relative-permeability, saturation and mass errors of the FP32 and
    16-bit forms against the FP64 lattice (which reproduces the FP64 oracle
    bit for bit) after the same number of steps on the same workload.

    "f64p" is the FP64 lattice started from the same state with every
    nonzero population moved by one unit in the last place: its distance from
    "f64" is the flow's own sensitivity to rounding, the floor that no
    storage precision can go below.  Errors are reported per sample (max
    over the run) and for the mean over the second half of the run."""
    from porescale_gb300.lattice import Lattice
    ind, p, fr, fb = make_workload(cfg)
    every = args.accuracy_every or args.accuracy_steps
    hist = {}
    t_run = {}
    legs = ("f64", "f64p", "f32", "f16", "bf16") if not args.accuracy_legs else ("f64",) + tuple(
        args.accuracy_legs.split(","))
    ref_hist = None
    if args.accuracy_ref:  # the FP64 run is deterministic: reuse a saved one
        with open(args.accuracy_ref) as f:
            saved = json.loads(f.read().strip().splitlines()[-1])
        if saved["steps"] == args.accuracy_steps and saved["workload"] == cfg["workload"]:
            ref_hist, t_run["f64"] = saved["history"]["f64"], saved["seconds"]["f64"]
    for q in legs:
        expected = sorted(set(list(range(every, args.accuracy_steps + 1, every)) + [args.accuracy_steps]))
        if q == "f64" and ref_hist is not None and [r["step"] for r in ref_hist] == expected:
            hist[q] = ref_hist
            continue
        L = Lattice(p, ind, PREC_ID["f64" if q in ("f64p", "f64n") else q.split(":")[0]])
        if ":" in q:  # "f16:k": the same storage with rounding seed k
            L.set_rounding_seed(int(q.split(":")[1]))
        if q == "f64n":
            # a perturbation of the size of FP32 rounding (1e-7 relative,
            # seeded): an FP64 run that diverges from the unperturbed one as
            # early as the low-precision runs do, so that its time-averaged
            # difference is the realisation floor of the metric
            rng = np.random.Generator(np.random.PCG64(20241204))
            L.set_state(fr * (1 + 1e-7 * rng.uniform(-1, 1, fr.shape)), fb * (1 + 1e-7 * rng.uniform(-1, 1, fb.shape)))
        elif q == "f64p":
            # exact zeros (the absent component of bulk nodes) stay zero: a
            # denormal there would turn every bulk node into an interface node
            L.set_state(np.where(fr != 0, np.nextafter(fr, np.inf), fr), np.where(fb != 0, np.nextafter(fb, np.inf), fb))
        else:
            L.set_state(fr, fb)
        rows = []
        t0 = time.perf_counter()
        done = 0
        while done < args.accuracy_steps:
            n = min(every, args.accuracy_steps - done)
            L.step(n)
            done += n
            o = L.observables()
            rows.append({"step": done, "permr": o.permr, "permb": o.permb, "sat_r": o.sat_r, "sat_b": o.sat_b,
                         "tmr": o.tmr, "tmb": o.tmb})
        t_run[q] = time.perf_counter() - t0
        hist[q] = rows
        L.close()
    out = accuracy_summary(hist, legs, cfg["workload"], args.accuracy_steps, t_run)
    out["size"] = cfg["size"]
    if args.accuracy_out:
        with open(args.accuracy_out, "w") as f:
            f.write(json.dumps(out) + "\n")
    print(json.dumps(out))


def accuracy_summary(hist, legs, workload, steps, t_run):
    """Errors of each leg's observables against the FP64 leg's.

    The relative-permeability error is defined on the time average: k_r of
    a phase is its flux-based permeability (check_state's permr / permb,
    S1:3181-3182; k_r = perm / k_abs with the same k_abs for every
    precision, so the relative error of perm is that of k_r) averaged over
    the samples of the second half of the run, and the error is
    |mean_q - mean_f64| / |mean_f64|.  The flow is chaotic: instantaneous
    samples of two runs that differ by rounding drift apart (the FP64 run
    started one ulp off, leg "f64p", shows that floor), while the time
    average over the developed window is the quantity k_r measures.  The
    per-sample maxima are reported beside it."""
    ref = hist["f64"]
    out = {"mode": "accuracy", "workload": workload, "steps": steps, "seconds": t_run,
           "final": {q: hist[q][-1] for q in hist}, "rel_err_vs_f64": {}, "rel_err_mean_2nd_half_vs_f64": {}}
    h0 = len(ref) // 2
    for q in legs[1:]:
        e, m = {}, {}
        for k in ("permr", "permb", "sat_r", "sat_b", "tmr", "tmb"):
            e[k] = max(abs(a[k] - b[k]) / max(abs(b[k]), 1e-300) for a, b in zip(hist[q], ref))
            ma = sum(a[k] for a in hist[q][h0:]) / len(hist[q][h0:])
            mb = sum(b[k] for b in ref[h0:]) / len(ref[h0:])
            m[k] = abs(ma - mb) / max(abs(mb), 1e-300)
        out["rel_err_vs_f64"][q] = e
        out["rel_err_mean_2nd_half_vs_f64"][q] = m
    out["kr_err"] = {"definition": "relative error of the time-averaged k_r (permr, permb) over the samples of the "
                                   "second half of the run, against the FP64 run",
                     "window": [ref[h0]["step"], ref[-1]["step"]], "samples": len(ref) - h0,
                     **{q: {"red": out["rel_err_mean_2nd_half_vs_f64"][q]["permr"],
                            "blue": out["rel_err_mean_2nd_half_vs_f64"][q]["permb"]} for q in legs[1:]}}
    out["history"] = hist
    return out


def differentiation(args):
    """The differentiation workloads.  (a) Gray partial-bounce-back TRT on a
    size^3 box (s: seeded Gaussian noise smoothed with sigma 3, sigmoid of
    slope 8 at the 0.35 quantile), body force 1e-6 along x, `steps` steps:
    dk/ds by the checkpointed adjoint (checkpoint every 200 steps) against
    FP64 central differences (h = 1e-4, and 2h for the Richardson value) at
    16 seeded voxels among those where |dk/ds| is at least 1e-2 of its
    largest value.  (b) Two-solid
    lattice-spring cube (radius-10 inclusions, fraction 0.25): d modulus /
    d(alf1, bet1, alf2, bet2) from the spring energies against central
    differences (h = 1e-4 relative), Cxxxx and Cyzyz."""
    from porescale_gb300 import geometry
    from porescale_gb300.gray import GrayLattice, gray_params
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_F64, SpringNetwork
    n, T = args.adjoint_size, args.adjoint_steps
    s = geometry.gray_field(n, sigma=3.0, slope=8.0, quantile=0.35, seed=20240604)
    p = gray_params(tau=1.0, F=(1e-6, 0, 0), idir=1, nsteps=T, segment=200)
    out = {"mode": "differentiation", "gray": {"size": n, "steps": T, "segment": 200, "h": 1e-4}}
    with GrayLattice(p, s.shape) as G:
        G.set_field(s)
        G.permeability()  # warm-up
        t0 = time.perf_counter()
        k = G.permeability()
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        k2, grad = G.gradient()
        t_grad = time.perf_counter() - t0
        rng = np.random.Generator(np.random.PCG64(20240605))
        h = 1e-4
        # seeded voxels where k responds to s (|dk/ds| >= 1e-2 of its largest
        # value): elsewhere the k difference of a central pair, 2h |dk/ds|,
        # sinks below the FP64 rounding noise of k itself
        gmax = float(np.abs(grad).max())
        cand = np.argwhere((s > 4 * h) & (s < 1 - 4 * h) & (np.abs(grad) >= 1e-2 * gmax))
        picks = cand[rng.choice(len(cand), 16, replace=False)]
        errs = []

        def central(v, hh):
            kk = []
            for sg in (1, -1):
                sp = s.copy()
                sp[v] += sg * hh
                G.set_field(sp)
                kk.append(G.permeability())
            return (kk[0] - kk[1]) / (2 * hh)

        for v in map(tuple, picks):
            fd, fd2 = central(v, h), central(v, 2 * h)
            rich = (4 * fd - fd2) / 3  # removes the O(h^2) truncation term
            errs.append({"voxel": [int(c) for c in v], "s": float(s[v]), "adjoint": float(grad[v]), "fd": fd,
                         "fd_2h": fd2, "rel_err": abs(grad[v] - fd) / abs(fd),
                         "rel_err_richardson": abs(grad[v] - rich) / abs(rich),
                         "err_over_max_gradient": abs(grad[v] - fd) / gmax})
    out["gray"].update({"k": k, "k_gradient_run": k2, "forward_s": t_fwd, "gradient_s": t_grad,
                        "forward_mlups": s.size * T / t_fwd / 1e6, "gradient_over_forward": t_grad / t_fwd,
                        "max_rel_err": max(e["rel_err"] for e in errs),
                        "max_rel_err_richardson": max(e["rel_err_richardson"] for e in errs),
                        "max_err_over_max_gradient": max(e["err_over_max_gradient"] for e in errs),
                        "max_abs_gradient": gmax, "checks": errs})
    m = args.adjoint_lsm_size
    ind = geometry.inclusions(m, 0.25, 10.0, 20240606)
    g = 1e-3 * m / 2
    k0 = np.array([1.0, 0.4, 0.3, 0.1])
    lsm = {"size": m, "h_rel": 1e-4}
    for load, name in ((LOAD_XSTRETCH, "Cxxxx"), (LOAD_YZSHEAR, "Cyzyz")):
        t0 = time.perf_counter()
        with SpringNetwork(ind, *k0, g, load, LSM_F64) as S:
            r = S.solve(1e-12, 400000)
            gr = S.gradients()
        t_solve = time.perf_counter() - t0
        fds = []
        for i in range(4):
            hh = 1e-4 * k0[i]
            mods = []
            for sg in (1, -1):
                kk = k0.copy()
                kk[i] += sg * hh
                with SpringNetwork(ind, *kk, g, load, LSM_F64) as S:
                    mods.append(S.solve(1e-12, 400000).modulus)
            fds.append((mods[0] - mods[1]) / (2 * hh))
        lsm[name] = {"modulus": r.modulus, "energy_modulus": gr[4], "gradient": gr[:4].tolist(), "fd": fds,
                     "max_rel_err": max(abs(a - b) / abs(b) for a, b in zip(gr[:4], fds)), "solve_s": t_solve}
    out["lsm"] = lsm
    print(json.dumps(out))


def batch_workload(nvol, seed):
    """Subvolume specs of the batched coupled workload: edge from {48, 64,
    96, 128}, porosity U[0.2, 0.45], sphere radius U[4, 10], initial red
    saturation U[0.3, 0.7], all from one seeded generator."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for v in range(nvol):
        specs.append({"edge": int(rng.choice([48, 64, 96, 128])), "porosity": float(rng.uniform(0.2, 0.45)),
                      "radius": float(rng.uniform(4.0, 10.0)), "sat": float(rng.uniform(0.3, 0.7)),
                      "seed": int(seed * 1000 + v)})
    return specs


def batch_mode(args):
    """The batched coupled workload: nvol subvolumes stepped together (one
    persistent launch per kernel and step, CUDA-graph replays, autotuned
    configuration), then per subvolume the fluid wall load applied to a
    two-solid lattice-spring network of the same voxels (matrix alpha 1.0,
    beta 0.4; radius-3 inclusions at fraction 0.25 of the solid, alpha 0.3,
    beta 0.1) solved for Cxxxx and Cyzyz.  A few subvolumes are also run on
    the plain FP64 path for the speed and error comparison.  Solid clusters
    not joined to the largest one (free bodies under a wall load) are made
    pore in both models."""
    import concurrent.futures as cf
    import torch
    from porescale_gb300 import geometry
    from porescale_gb300._lib import PorescaleError
    from porescale_gb300.lattice import Lattice, LatticeBatch, make_params
    from porescale_gb300.springs import LOAD_XSTRETCH, LOAD_YZSHEAR, LSM_MIXED, SpringNetwork
    specs = batch_workload(args.batch_volumes, 20240607)
    p = make_params(B=0.7, sig=1e-3, vir=(0.8 - 0.5) / 3, vib=(1.5 - 0.5) / 3, wet=np.cos(np.radians(30.0)),
                    bfr=(1e-6, 0, 0), bfb=(1e-6, 0, 0))
    prec = PREC_ID[args.prec]
    inds, lats = [], []
    for sp in specs:
        # solid clusters not joined to the skeleton are free bodies with no
        # static equilibrium under a wall load: they become pore in both models
        ind = geometry.spanning_solid(geometry.sphere_pack(sp["edge"], sp["porosity"], sp["radius"], sp["seed"]))
        L = Lattice(p, ind, prec)
        L.init_random(sp["sat"])
        inds.append(ind)
        lats.append(L)
    nodes = sum(L.nl for L in lats)
    T = args.batch_steps
    peak, peak_kind = load_peaks()
    bpn = ALGO_BYTES[args.prec]
    with LatticeBatch(lats) as B:
        tile = B.autotune(4)
        stream = torch.cuda.ExternalStream(B.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        B.step(T)
        e1.record(stream)
        e1.synchronize()
        t_lbm = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
    mlups = nodes * T / (ms * 1e-3) / 1e6

    # the spring networks of every subvolume and load case, built on 8 host
    # threads (geometry, node tables, wall load); the solves below start
    # from x = 0 each time, so both solve paths use the same networks
    from porescale_gb300.springs import batch_solve
    cases = ((LOAD_XSTRETCH, "Cxxxx"), (LOAD_YZSHEAR, "Cyzyz"))

    def build_nets(v):
        ind = inds[v]
        incl = geometry.inclusions(ind.shape, 0.25, 3.0, specs[v]["seed"] + 7)
        ind_s = np.where(ind == 0, np.where(incl == 3, 3, 0), 1).astype(np.int32)
        nets = []
        for load, _ in cases:
            N = SpringNetwork(ind_s, 1.0, 0.4, 0.3, 0.1, 1e-3 * ind.shape[2] / 2, load, LSM_MIXED)
            N.set_wall_load(lats[v], 1.0)
            nets.append(N)
        return nets

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(8) as ex:
        nets = list(ex.map(build_nets, range(len(lats))))
    t_lsm_setup = time.perf_counter() - t0

    # all networks of a load case in one batched solve (shared launches)
    t0 = time.perf_counter()
    moduli = [{} for _ in lats]
    for c, (_, name) in enumerate(cases):
        try:
            for v, r in enumerate(batch_solve([n[c] for n in nets], 1e-8, 400000)):
                moduli[v][name] = r.modulus
                moduli[v][name + "_inner"] = int(r.inner_iterations)
        except PorescaleError as exc:
            for v in range(len(lats)):
                moduli[v][name + "_error"] = str(exc)
    t_lsm = time.perf_counter() - t0

    # the same solves one network at a time on 8 host threads, for comparison
    def lsm_job(v):
        out = {}
        for c, (_, name) in enumerate(cases):
            try:
                r = nets[v][c].solve(1e-8, 400000)
                out[name] = r.modulus
                out[name + "_inner"] = int(r.inner_iterations)
            except PorescaleError as exc:
                out[name] = None
                out[name + "_error"] = str(exc)
        return out

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(8) as ex:
        moduli_ind = list(ex.map(lsm_job, range(len(lats))))
    t_lsm_ind = time.perf_counter() - t0
    for n in nets:
        for N in n:
            N.close()
    agree = max((abs(a[k] - b[k]) / abs(b[k]) for a, b in zip(moduli, moduli_ind) for k in ("Cxxxx", "Cyzyz")
                 if a.get(k) and b.get(k)), default=None)
    # plain per-volume FP64 path on the first few subvolumes: time and errors
    nref = min(args.batch_reference, len(lats))
    ref = []
    t_f64 = 0.0
    for v in range(nref):
        L64 = Lattice(p, inds[v], PREC_ID["f64"])
        L64.init_random(specs[v]["sat"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L64.step(T)
        L64.sync()
        t_f64 += time.perf_counter() - t0
        o64, o = L64.observables(), lats[v].observables()
        ref.append({"edge": specs[v]["edge"], "nodes": L64.nl, "permr_f64": o64.permr, "permr": o.permr,
                    "rel_err_permr": abs(o.permr - o64.permr) / abs(o64.permr),
                    "rel_err_permb": abs(o.permb - o64.permb) / abs(o64.permb),
                    "rel_err_sat_r": abs(o.sat_r - o64.sat_r) / abs(o64.sat_r)})
        L64.close()
    ref_nodes = sum(r["nodes"] for r in ref)
    f64_mlups = ref_nodes * T / t_f64 / 1e6 if t_f64 > 0 else None
    out = {"mode": "batch", "volumes": len(lats), "steps": T, "precision": args.prec, "fluid_nodes": nodes,
           "tile": list(tile), "lbm_seconds": ms * 1e-3, "lbm_wall_seconds": t_lbm, "mlups": mlups,
           "achieved_gbs": mlups * 1e6 * bpn / 1e9, "frac": mlups * 1e6 * bpn / 1e9 / peak, "peak_kind": peak_kind,
           "lsm_setup_seconds": t_lsm_setup, "lsm_seconds": t_lsm, "lsm_individual_seconds": t_lsm_ind, "lsm_batch_vs_individual_max_rel": agree,
           "lsm_inner_iterations_batched": sum(m.get(k, 0) for m in moduli for k in ("Cxxxx_inner", "Cyzyz_inner")),
           "lsm_inner_iterations_individual": sum(m.get(k, 0) for m in moduli_ind for k in ("Cxxxx_inner", "Cyzyz_inner")),
           "subvolumes_per_s": len(lats) / (ms * 1e-3 + t_lsm_setup + min(t_lsm, t_lsm_ind)),
           "lbm_subvolumes_per_s": len(lats) / (ms * 1e-3),
           "f64_plain_mlups": f64_mlups,
           "f64_plain_subvolumes_per_s_estimate": (f64_mlups * 1e6 / (nodes * T / len(lats))) if f64_mlups else None,
           "lsm_failures": sum(1 for m in moduli for k in m if k.endswith("_error")),
           "reference_volumes": ref, "moduli": moduli, "specs": specs}
    for L in lats:
        L.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--prec", default=None, choices=list(PREC_ID),
                    help="population storage (default f16; f32 for --batch, whose transient subvolume flows FP16's "
                         "rounding noise moves by several percent)")
    ap.add_argument("--itw", type=int, default=100, help="steps per e2e step (check_state cadence)")
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-legs", action="store_true", help="skip the FP64/FP32 comparison legs")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of timing: run this many steps in every precision and report the errors of "
                         "permeabilities, saturation and masses against FP64")
    ap.add_argument("--accuracy-every", type=int, default=0, help="observable cadence of the accuracy run")
    ap.add_argument("--batch", action="store_true",
                    help="instead of the 256^3 step: the batched coupled workload (subvolumes in shared persistent "
                         "launches, then wall-loaded lattice-spring solves)")
    ap.add_argument("--batch-volumes", type=int, default=48)
    ap.add_argument("--batch-steps", type=int, default=3000)
    ap.add_argument("--batch-reference", type=int, default=3, help="subvolumes also run on the plain FP64 path")
    ap.add_argument("--adjoint", action="store_true",
                    help="instead of timing the step: the differentiation workloads (gray-lattice adjoint and "
                         "spring-constant gradients against central differences)")
    ap.add_argument("--adjoint-size", type=int, default=128)
    ap.add_argument("--adjoint-steps", type=int, default=4000)
    ap.add_argument("--adjoint-lsm-size", type=int, default=128)
    ap.add_argument("--accuracy-ref", default="", help="a previous accuracy JSON whose FP64 history is reused")
    ap.add_argument("--accuracy-legs", default="", help="comma list of legs besides f64 (default f64p,f32,f16,bf16)")
    ap.add_argument("--accuracy-out", default="", help="also write the accuracy JSON to this file")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default step configuration")
    ap.add_argument("--tile", default="", help="tx,ty,occ: pin the step configuration instead of autotuning")
    ap.add_argument("--wave", default="", help="planes,window: with --tile, pin the wavefront schedule")
    ap.add_argument("--march", default="", help="rows,planes,producers,sort: with --tile, pin the marching step")
    ap.add_argument("--sort", type=int, default=-1, help="with --tile: 1/0 pins the sorted collide order")
    ap.add_argument("--no-lsm", action="store_true", help="skip the lattice-spring leg")
    ap.add_argument("--lsm-cpu-budget", type=float, default=10.0,
                    help="seconds of each CPU spring-solve baseline (CG, relaxation)")
    ap.add_argument("--lsm-dr", action="store_true",
                    help="instead of timing the step: the reference's relaxation on the GPU to the CG residual")
    ap.add_argument("--lsm-size", type=int, default=64)
    ap.add_argument("--lsm-dr-check", type=int, default=2000)
    ap.add_argument("--lsm-dr-max", type=int, default=1000000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.prec is None:
        args.prec = "f32" if args.batch else "f16"

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    cfg = workload_config(args.size)
    metric = "D3Q19 two-phase MLUPS"

    if args.impl == "reference":
        # the reference is Fortran and no Fortran compiler exists on either
        # build host: its CPU path is timed through the C restatement
        if rank != 0:
            return
        from porescale_gb300 import _build
        _build.build_oracle()
        ind, p, fr, fb = make_workload(cfg)
        threads = os.cpu_count() or 1
        import oracle
        o = oracle.OracleLattice(p, ind)
        o.set_state(fr, fb)
        o.run(args.warmup, threads)
        t = time.perf_counter()
        o.run(args.steps, threads)
        dt = time.perf_counter() - t
        v = o.nl * args.steps / dt / 1e6
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "MLUPS", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": bench_config(cfg, o.nl),
                "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": threads, "kind": "port",
                                 "sample": f"{args.steps} full-lattice steps of the {args.size}^3 workload"},
                "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from porescale_gb300 import _build
    _build.build_all()
    from porescale_gb300.lattice import Lattice
    if args.accuracy_steps > 0:
        accuracy(args, cfg)
        return
    if args.adjoint:
        differentiation(args)
        return
    if args.batch:
        batch_mode(args)
        return
    if args.lsm_dr:
        lsm_dr_mode(args)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local_rank)

    ind, p, fr, fb = make_workload(cfg)
    peak, peak_kind = load_peaks()
    res = {}
    legs = [args.prec] if args.no_legs else [args.prec] + [q for q in ("f64", "f32") if q != args.prec]
    clocks = None
    nl = None
    for q in legs:
        L = Lattice(p, ind, PREC_ID[q])
        nl = L.nl
        L.set_state(fr, fb)
        if args.tile:
            L.set_tile(*[int(v) for v in args.tile.split(",")])
            if args.wave:
                L.set_wave(*[int(v) for v in args.wave.split(",")])
            if args.march:
                L.set_march(*[int(v) for v in args.march.split(",")])
            if args.sort >= 0:
                L.set_sort(bool(args.sort))
            L.info = L.get_info()
        elif not args.no_autotune:
            L.autotune(4 if q != "f64" else 2)
            L.set_state(fr, fb)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        steps = args.steps if q == args.prec else max(3, args.steps // 5 if q == "f64" else args.steps)
        sampler = ClockSampler(local_rank) if q == args.prec else None
        if sampler:
            sampler.start()
        t = time_steps(L, steps, args.warmup, torch)
        if sampler:
            clocks = sampler.stop()
        t = max_over_ranks(t, world)
        mlups = job_rate(nl * steps, t, world) / 1e6
        launch_s = t / steps
        achieved = nl * ALGO_BYTES[q] / launch_s / 1e9
        if q != "f64" and not args.no_autotune and not args.tile:
            # the step schedules side by side on this workload (fused: slab
            # planes x look-ahead), each from the same state
            study = {}
            tile = (L.info.tile_x, L.info.tile_y, L.info.occupancy, int(L.info.schedule), int(L.info.wave),
                    int(L.info.march))
            for planes, ahead in ((0, 1), (1, 1), (2, 1), (4, 1), (8, 1), (2, 2), (4, 2)):
                try:
                    L.set_wave(0)
                    L.set_march(0)
                    L.set_fused(0, 1)
                    L.set_tile(128, 256, 0)
                    L.set_fused(planes, ahead)
                except Exception as exc:  # configuration without a fused form
                    study[f"{planes}/{ahead}"] = str(exc)
                    continue
                L.set_state(fr, fb)
                study[f"{planes}/{ahead}"] = nl * 20 / time_steps(L, 20, 3, torch) / 1e6
            # wavefront graphs (slab planes / window) on the collide tile 128 x 6
            L.set_fused(0, 1)
            L.set_tile(128, 256, 6)
            for planes, window in ((2, 0), (4, 0), (8, 0), (16, 0), (32, 0), (64, 0), (128, 0), (4, 3), (8, 3)):
                L.set_wave(planes, window)
                L.set_state(fr, fb)
                study[f"w{planes}/{window}"] = nl * 48 / time_steps(L, 48, 8, torch) / 1e6
            # marching one-launch steps (band rows, producer warps, sorted order)
            for rows, pw, srt in ((8, 4, True), (8, 8, True), (16, 8, True), (8, 12, True), (16, 12, True),
                                  (8, 8, False)):
                L.set_wave(0)
                L.set_march(rows, 0, pw, srt)
                L.set_state(fr, fb)
                study[f"m{rows}p{pw}{'' if srt else 'u'}"] = nl * 20 / time_steps(L, 20, 3, torch) / 1e6
                L.set_march(0)
            L.set_wave(0)
            L.set_tile(*tile[:3])
            if tile[5]:
                L.set_march(*march_fields(tile[5]))
            if tile[3]:
                L.set_fused(tile[3] % 256, tile[3] // 256)
            if tile[4]:
                L.set_wave(tile[4] % 256, tile[4] // 256)
            L.set_state(fr, fb)
            L.info = L.get_info()
            res[q + "_schedules_mlups"] = study
        sched, wave, march = int(L.info.schedule), int(L.info.wave), int(L.info.march)
        if march:
            rows, planes, pw, srt = march_fields(march)
            schedule = {"kind": "march", "band_rows": rows, "chunk_planes": planes, "producer_warps": pw,
                        "consumer_warps": 24 - pw, "sorted": srt}
            kps = 1
        elif sched:
            schedule, kps = {"kind": "fused", "slab_planes": sched % 256, "lookahead": sched // 256}, 1
        elif wave:
            nslab = -(-int(L.info.nz) // (wave % 256))
            schedule = {"kind": "wave", "slab_planes": wave % 256, "window": wave // 256, "steps_per_graph": 8,
                        "slabs": nslab}
            kps = 2 * nslab
        else:
            schedule, kps = {"kind": "two-pass"}, 2
        res[q] = {"mlups": mlups, "ms_per_step": launch_s * 1e3, "steps": steps, "achieved_gbs": achieved,
                  "frac": achieved / peak, "tile": [L.info.tile_x, L.info.tile_y, L.info.occupancy],
                  "schedule": schedule, "kernels_per_step": kps}
        if q == args.prec:
            # e2e through the C ABI with host buffers (pinned)
            hfr = torch.empty((nl, 19), dtype=torch.float64, pin_memory=True).numpy()
            hfb = torch.empty((nl, 19), dtype=torch.float64, pin_memory=True).numpy()
            hfr[:] = fr
            hfb[:] = fb
            ofr = torch.empty((nl, 19), dtype=torch.float64, pin_memory=True).numpy()
            ofb = torch.empty((nl, 19), dtype=torch.float64, pin_memory=True).numpy()
            L.set_state(hfr, hfb)
            L.step(args.itw)
            L.observables()
            L.get_state((ofr, ofb))
            if world > 1:
                torch.distributed.barrier()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                L.set_state(hfr, hfb)
                L.step(args.itw)
                obs = L.observables()
                L.get_state((ofr, ofb))
            te = time.perf_counter() - t0
            te = max_over_ranks(te, world)
            res["e2e"] = {"value": job_rate(nl * args.itw * args.e2e_steps, te, world) / 1e6, "unit": "MLUPS",
                          "h2d_bytes_per_step": 2 * 19 * nl * 8, "d2h_bytes_per_step": 2 * 19 * nl * 8 + 8 * 40,
                          "steps_per_e2e_step": args.itw, "e2e_steps": args.e2e_steps,
                          "permr": obs.permr, "permb": obs.permb}
        L.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, dt = cpu_oracle_mlups(ind, p, fr, fb, threads, args.cpu_budget)
        cpu = {"value": v, "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": f"{n} full-lattice steps of the {args.size}^3 workload ({dt:.1f} s, FP64 C restatement)"}

    lsm = None
    if rank == 0 and not args.no_lsm:
        lsm = lsm_leg(cpu_budget=0.0 if args.no_cpu_baseline else args.lsm_cpu_budget)
        # the same solve at 128^3 (the differentiation workload's size), where
        # the CG vectors no longer fit in L2
        big = lsm_leg(size=128)
        lsm["size128"] = {k: v for k, v in big.items() if k != "cpu_baseline"}
    h = res[args.prec]
    traffic = load_traffic(args.prec, nl, h["schedule"]["kind"])
    line = {
        "metric": metric, "value": h["mlups"], "unit": "MLUPS", "n_gpus": world, "steps": h["steps"],
        "warmup": args.warmup, "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.prec, "data": "synthetic",
        "config": bench_config(cfg, nl),
        "kernel_config": {"precision": args.prec, "tile": h["tile"], "schedule": h["schedule"]},
        "roofline": {"bound": "hbm", "achieved": h["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": h["frac"], "traffic": traffic, "peak_kind": peak_kind,
                     "algo_bytes_per_node": ALGO_BYTES[args.prec]},
        "e2e": res.get("e2e"),
        "accuracy": load_accuracy(args.prec, cfg) if args.size == 256 else None,
        "cpu_baseline": cpu,
        "gpu_launches": (h["steps"] // 8 * 8 * h["kernels_per_step"] + h["steps"] % 8 * 2
                         if h["schedule"]["kind"] == "wave" else h["steps"] * h["kernels_per_step"]),
        "clocks": clocks,
        "legs": {q: res[q] for q in legs},
        "schedules_mlups": {k[:-len("_schedules_mlups")]: v for k, v in res.items() if k.endswith("_schedules_mlups")},
        "lsm": lsm,
    }
    if "f64" in res:
        line["mixed_vs_f64"] = h["mlups"] / res["f64"]["mlups"]
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
