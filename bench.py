"""Benchmark: particle-steps/s of the SPH step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]
                    [--n1d 128] [--precision mixed|fp64]
                    [--workload sedov|kh|polytrope|ensemble]

Workload: the 3D Sedov blast, 128^3 = 2,097,152 particles on a 1%-jittered
lattice (seeded), Wendland C6, ideal gas gamma 5/3, thermokinetic energy,
adaptive dt -- one "step" is one full leapfrog iteration of the hydro
driver loop (kick/drift, keys, sort, tree, neighbour lists, density/EOS,
signal speed, acceleration, de/dt with the pressure predictor, dt
reduction).  Inputs are resident in HBM when the timed region starts; the
particle state (~0.5 GB) and neighbour lists (~0.8 GB) exceed the 129 MB L2,
so no explicit flush is needed between steps.

`value` is measured with CUDA events on the library's stream around K
steps; `e2e` repeats the measurement through the C ABI with host buffers,
copying each step's inputs from pinned host memory and its results back
(fsph_step_io, which overlaps those copies with the step where the data
dependences allow).
Other workloads (not the default line): `kh` -- Kelvin-Helmholtz in the
periodic box, 256^3 by default, with the energy and momentum drift of the
timed steps in both precisions; `polytrope` -- the n=1 polytrope with tree
gravity (quadrupole, theta 0.5), 4M particles by default, with the gravity
error of 64 sampled blocks of sinks against direct FP64 summation over all
sources on the host cores; `ensemble` -- 256 independent 2D problems (Sod and
Noh, log-uniform sizes 2k-200k, about 12.4M particles) stepped as CUDA
graphs with the lane count and walk-group size chosen by
fsph_ensemble_tune_shape, against the same members stepped one by one.

`--impl reference` times the reference algorithm on the host cores instead
(the CPU oracle: the reference compiled from its sources where those exist
on this machine, otherwise the plain-C restatement) on the same 128^3
problem with every host thread, and reports the single-core rate of a 64^3
sample beside it.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic work per particle and timer phase: the constants of
# include/fsph_work.h (the one table both this file and the design notes
# use), parsed from the header.
HBM_PEAK = 6815.2  # GB/s, MEASURED_PEAKS.json hbm_gbs
# ncu dram__bytes_read.sum + dram__bytes_write.sum per particle of the
# dominant kernel of a phase, from 96^3 Sedov captures (884,736 particles;
# lists and records well above L2): the walk (459.4 MB,
# profiles/k_neighbors_uni_sedov3d_96.md); the float-float
# density and acceleration passes and the de/dt pass of the warm-up
# iteration (567.6, 569.2 and 597.8 MB,
# profiles/k_density_ff_accel_ff_dedt_ahyd_sedov3d_96.md)
MEASURED_TRAFFIC_PER_PARTICLE = {"neighbors": 519.3, "density": 641.6, "accel": 643.3,
                                 "energy": 675.7}


def read_work_header(path=os.path.join(ROOT, "include", "fsph_work.h")):
    """{name without the FSPH_ prefix: value} of the #defines in fsph_work.h."""
    import re
    out = {}
    for line in open(path):
        m = re.match(r"\s*#define\s+FSPH_(\w+)\s+([0-9.]+)", line)
        if m:
            out[m.group(1)] = float(m.group(2))
    return out


WORK = read_work_header()


def work_model(phase, nb, mixed, thermokinetic=True):
    """Algorithmic work per particle of a timer phase: {"flop": F, "byte": B}
    (either may be 0), or None for phases the table does not model (gravity,
    periodic copies).  nb is the mean neighbour count including self."""
    W = WORK
    lst = W["BYTES_PAIR_LIST"] * nb  # the list read by a pair pass
    energy_flops = W["FLOPS_PAIR_DEDT"] if thermokinetic else W["FLOPS_PAIR_DUDT"]
    table = {
        "range_keys": (0.0, W["BYTES_RANGE_KEYS"]),
        "sort": (0.0, W["BYTES_SORT"]),
        "tree": (0.0, W["BYTES_TREE"]),
        "neighbors": (0.0, W["BYTES_NEIGHBORS"] + lst),
        "density": (W["FLOPS_PAIR_DENSITY"] * nb, W["BYTES_DENSITY"] + lst),
        "vsig": (W["FLOPS_PAIR_VSIG"] * nb, lst),
        # the mixed path evaluates the signal speed in the acceleration loop
        "accel": ((W["FLOPS_PAIR_ACCEL"] + (W["FLOPS_PAIR_VSIG"] if mixed else 0.0)) * nb,
                  W["BYTES_ACCEL"] + lst),
        # de/dt (du/dt) with the pressure predictor that follows it
        "energy": (energy_flops * nb, W["BYTES_DEDT"] + W["BYTES_RECOMPUTE_P"] + lst),
        "integrate": (0.0, W["BYTES_INTEGRATE"]),
        "dt": (0.0, W["BYTES_DT"]),
    }
    if phase not in table:
        return None
    f, b = table[phase]
    return {"flop": f, "byte": b}


def phase_roofline(work, n, seconds, peak_flop, flop_kind, peak_hbm=HBM_PEAK):
    """Roofline of one launch of a phase over n particles taking `seconds`:
    the bound is the larger of F / peak_flop and B / peak_hbm; `achieved`
    and `frac` are in that bound's unit."""
    t_f = n * work["flop"] / (peak_flop * 1e12) if work["flop"] else 0.0
    t_b = n * work["byte"] / (peak_hbm * 1e9) if work["byte"] else 0.0
    if t_f >= t_b:
        ach = n * work["flop"] / seconds / 1e12
        return {"bound": flop_kind, "achieved": ach, "peak": peak_flop,
                "unit": "TFLOP/s", "frac": ach / peak_flop,
                "t_roof_ms": 1e3 * t_f}
    ach = n * work["byte"] / seconds / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": peak_hbm, "unit": "GB/s",
            "frac": ach / peak_hbm, "t_roof_ms": 1e3 * t_b}


def step_roofline(per_phase, phase_ms, ms_per_step):
    """Step-level roofline of the work model: t_roof = sum over the modelled
    phases of work / peak (= frac x measured time, frac as in
    `roofline_all`), against the measured step.  Phases without a work model
    (gravity, periodic copies) count as measured time with no roofline
    time, and are listed."""
    t_roof = sum(per_phase[k]["frac"] * phase_ms[k] for k in per_phase if k in phase_ms)
    unmodelled = {k: v for k, v in phase_ms.items() if k not in per_phase}
    return {"t_roof_ms": t_roof, "t_step_ms": ms_per_step,
            "frac": t_roof / ms_per_step if ms_per_step > 0 else None,
            "unmodelled_ms": unmodelled,
            "model": "sum_k max(F_k / peak_flop, B_k / peak_hbm) over the timer "
                     "phases, one bound per phase as in roofline_all"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--workload", default="sedov",
                    choices=["sedov", "kh", "polytrope", "ensemble"])
    ap.add_argument("--n1d", type=int, default=None,
                    help="lattice size (sedov 128, kh 256)")
    ap.add_argument("--n", type=int, default=None, help="particles (polytrope 4M)")
    ap.add_argument("--problems", type=int, default=256, help="ensemble members")
    ap.add_argument("--precision", default="auto", choices=["auto", "mixed", "fp64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the polytrope's direct-summation gravity check")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # start the region once the sampler is writing (nvidia-smi takes a
        # moment to come up; a short region would otherwise see no sample)
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < 3.0:
            try:
                if os.path.getsize(self.f.name) > 0:
                    break
            except OSError:
                break
            time.sleep(0.01)
        self.t_start = time.time()
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines()]
        except OSError:
            return out
        rows = [[x.strip() for x in r] for r in rows if len(r) >= 8]
        if not rows:
            return out
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[4 + k].lower() == "active":
                    reasons.add(nm)
        out.update(sm_mhz=statistics.median(sm) if sm else None,
                   sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        os.unlink(self.f.name)
        return out


def run_cpu_oracle(n1d, steps, threads, min_seconds=10.0, max_steps=None, warmup=0):
    """Time the reference algorithm on the host cores on the Sedov problem
    (`warmup` untimed iterations after the initial one, then `max_steps`
    timed ones, or as many as fill `min_seconds`)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from flecsph_gb300 import setups
    kind = "reference" if pyoracle.have_ref(3) else "port"
    if kind == "port":
        pyoracle.build_port()
    s, p, meta = setups.sedov3d(n1d)
    o = pyoracle.Oracle(kind, p, threads=threads)
    o.upload(s)
    o.step()  # initial iteration (not timed)
    for _ in range(warmup):
        o.step()
    done = 0
    t0 = time.perf_counter()
    while True:
        o.step()
        done += 1
        el = time.perf_counter() - t0
        if max_steps is not None and done >= max_steps:
            break
        if max_steps is None and el >= min_seconds:
            break
    el = time.perf_counter() - t0
    return dict(value=meta["n"] * done / el, unit="particle-steps/s",
                cores=threads if kind == "port" else 1, kind=kind,
                sample=f"Sedov 3D {n1d}^3 = {meta['n']} particles, {done} leapfrog "
                       f"iterations after the initial one, {el:.1f} s",
                seconds=el, steps=done)


def reference_arm(args):
    """The reference algorithm on the host cores (all threads), on the same
    workload as the GPU line: the oracle built from the reference's sources
    where those exist, else the plain-C restatement.  Beside it, the
    single-core rate on a 64^3 sample of the same problem (one iteration)."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n1d = args.n1d or 128
    steps, warm = args.steps, args.warmup
    r = run_cpu_oracle(n1d, steps, threads, max_steps=steps, warmup=warm)
    one = run_cpu_oracle(64, 1, 1, max_steps=1)
    line = {
        "metric": "particle-steps/s", "value": r["value"], "unit": "particle-steps/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": 1e3 * r["seconds"] / r["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"sedov3d_{n1d}^3", "n_particles": n1d ** 3,
                   "kernel": "wendland_c6", "threads": r["cores"]},
        "cpu_baseline": {"value": r["value"], "unit": "particle-steps/s",
                         "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]},
        "single_core": {"value": one["value"], "unit": "particle-steps/s", "cores": 1,
                        "kind": one["kind"], "sample": one["sample"]},
        "e2e": {"value": r["value"], "unit": "particle-steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# fields a host driver hands over per step (what the leapfrog step reads) and
# takes back (what it writes)
IN_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "gax", "gay", "gaz",
             "m", "h", "cs", "u", "e", "dedt", "K"]
OUT_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "vhx", "vhy", "vhz", "ax", "ay", "az",
              "gax", "gay", "gaz", "gpot", "rho", "P", "cs", "u", "e", "dedt", "vsig",
              "dt", "h"]


def drift(c0, c1, s, s1=None):
    """Relative change of the conserved sums over the timed steps: energy
    against |E0|, momentum against sum m|v| (the larger of the input's and
    the final state's, for problems that start at rest)."""
    def mv(t):
        return float((t["m"] * np.sqrt(t["vx"] ** 2 + t["vy"] ** 2 + t["vz"] ** 2)).sum())
    scale_p = max(mv(s), mv(s1) if s1 is not None else 0.0)
    dp = np.array(c1["momentum"]) - np.array(c0["momentum"])
    return {"energy": abs(c1["energy"] - c0["energy"]) / abs(c0["energy"]),
            "momentum": float(np.linalg.norm(dp)) / max(scale_p, 1e-300),
            "mass": abs(c1["mass"] - c0["mass"]) / c0["mass"]}


def per_field_errors(ref, test, p):
    """Per-field error of `test` against `ref` (both downloaded states of
    the same particles, matched by id): normwise max|d| / max|ref| and the
    median, 99th percentile and maximum per particle.  Scalars with a
    positive scale (rho, P, c_s) use |d| / |ref|; signed or vanishing fields
    (a, de/dt or du/dt, g_acc) use |d| / max(|ref|, 1e-3 rms|ref|)."""
    o_r = np.argsort(ref["id"])
    o_t = np.argsort(test["id"])

    def stats(err, normwise):
        return {"normwise": float(normwise), "median": float(np.median(err)),
                "p99": float(np.percentile(err, 99)), "max": float(err.max())}

    out = {}
    for f in ("rho", "P", "cs"):
        r, t = ref[f][o_r], test[f][o_t]
        if not np.any(r):
            continue
        err = np.abs(t - r) / np.maximum(np.abs(r), 1e-300)
        out[f] = stats(err, np.abs(t - r).max() / np.abs(r).max())
    vec = {"a": ("ax", "ay", "az")}
    if p.enable_fmm:
        vec["g_acc"] = ("gax", "gay", "gaz")
    for name, ks in vec.items():
        R = np.stack([ref[k][o_r] for k in ks], 1)
        T = np.stack([test[k][o_t] for k in ks], 1)
        mag = np.linalg.norm(R, axis=1)
        rms = np.sqrt((mag ** 2).mean())
        err = np.linalg.norm(T - R, axis=1) / np.maximum(mag, 1e-3 * rms)
        out[name] = stats(err, np.abs(T - R).max() / max(np.abs(R).max(), 1e-300))
    f = "dedt" if p.thermokinetic_formulation else "dudt"
    r, t = ref[f][o_r], test[f][o_t]
    rms = np.sqrt((r ** 2).mean())
    err = np.abs(t - r) / np.maximum(np.abs(r), max(1e-3 * rms, 1e-300))
    out[f] = stats(err, np.abs(t - r).max() / max(np.abs(r).max(), 1e-300))
    return out


def gravity_check(bs, p, blocks=64, block=1024, seed=7):
    """Tree gravity of the current state against direct FP64 summation over
    all sources (the oracle, on every host core) for `blocks` blocks of
    `block` consecutive sinks at seeded offsets of the sorted order."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build_port()
    st = bs.download()
    n = len(st["x"])
    o = pyoracle.Oracle("port", p, threads=os.cpu_count() or 1)
    o.upload(st)
    rng = np.random.Generator(np.random.PCG64(seed))
    starts = np.sort(rng.choice(max(1, n // block), size=min(blocks, n // block),
                                replace=False)) * block
    t0 = time.perf_counter()
    for a in starts:
        o.gravity_direct(int(a), int(min(n, a + block)))
    el = time.perf_counter() - t0
    ref = o.download()
    o.close()
    idx = np.concatenate([np.arange(a, min(n, a + block)) for a in starts])
    G = np.stack([st[k][idx] for k in ("gax", "gay", "gaz")], 1)
    R = np.stack([ref[k][idx] for k in ("gax", "gay", "gaz")], 1)
    mag = np.linalg.norm(R, axis=1)
    rms = np.sqrt((mag ** 2).mean())
    err = np.linalg.norm(G - R, axis=1) / np.maximum(mag, 1e-3 * rms)
    pot = np.abs(st["gpot"][idx] - ref["gpot"][idx]) / np.abs(ref["gpot"][idx])
    return {"sinks": int(len(idx)), "sources": n, "theta": p.fmm_macangle,
            "order": p.gravity_order, "accel_rel_err_median": float(np.median(err)),
            "accel_rel_err_p99": float(np.percentile(err, 99)),
            "accel_rel_err_max": float(err.max()),
            "potential_rel_err_median": float(np.median(pot)),
            "direct_sum_seconds": el}


def ensemble_arm(args):
    """Config 4: independent 2D problems stepped together as CUDA graphs,
    against the same members stepped one by one (graphs off)."""
    rank, world, local = dist_info()
    dist = init_dist(world)
    from flecsph_gb300 import build, setups
    if rank == 0:
        build.build()
    barrier(dist)
    from flecsph_gb300 import sph
    probs = setups.ensemble2d(args.problems)
    ntot = sum(m["n"] for _, _, m in probs)
    ens = sph.Ensemble(device=local)
    members = [ens.add(p, m["n"]) for s, p, m in probs]
    for mb, (s, p, m) in zip(members, probs):
        mb.read_bodies(s)
    ens.step(1 + args.warmup)
    ens.sync()
    res = {}
    gsize = 32
    for mode in ("one_by_one", "graphs"):
        if mode == "graphs":
            lanes, gsize, _ = ens.tune_shape(2)
        else:
            ens.set_lanes(0)
            lanes = 0
        ens.step(2)
        ens.sync()
        l0 = sum(mb.launch_count() for mb in members)
        barrier(dist)
        with Clocks(local) as clk:
            t0 = time.perf_counter()
            ens.step(args.steps)
            ens.sync()
            el = time.perf_counter() - t0
        el = max_over_ranks(dist, el)
        res[mode] = dict(seconds=el, lanes=lanes, clocks=clk.summary(),
                         launches=sum(mb.launch_count() for mb in members) - l0)
    ens.close()
    if rank != 0:
        return
    K = args.steps
    g = res["graphs"]
    sizes = [m["n"] for _, _, m in probs]
    line = {
        "metric": "particle-steps/s", "value": world * ntot * K / g["seconds"],
        "unit": "particle-steps/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": 1e3 * g["seconds"] / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"ensemble2d_{len(probs)}_sod_noh",
                   "problems": len(probs), "n_particles_total": ntot,
                   "n_min": min(sizes), "n_max": max(sizes), "precision": "mixed",
                   "lanes": g["lanes"], "group_size": gsize,
                   "timing": "host wall clock around K steps "
                   "with a device sync on both sides (many streams)"},
        "one_by_one": {"value": world * ntot * K / res["one_by_one"]["seconds"],
                       "ms_per_step": 1e3 * res["one_by_one"]["seconds"] / K},
        "gpu_launches": g["launches"],
        "clocks": g["clocks"],
    }
    print(json.dumps(line), flush=True)


def link_gbs(nbytes=256 << 20, reps=4):
    """Host<->device copy rate of this machine right after the e2e loop: one
    256 MiB pinned buffer copied `reps` times each way (CUDA events), so that
    the e2e figure can be read against the link it ran on."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    out = {}
    with torch.cuda.stream(s):
        for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
            dst.copy_(src, non_blocking=True)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(s)
            e1.synchronize()
            out[name] = round(reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    del h, d
    return out


def one_pass(bs, state, p):
    """One pass of every physics callback from `state`: density, pressure,
    sound speed, acceleration, the energy rate and gravity."""
    bs.read_bodies(state)
    bs.update_iteration()
    bs.eos_init()
    if p.thermokinetic_formulation:
        bs.set_total_energy()
    bs.density_pressure_soundspeed()
    bs.save_velocityhalf()
    bs.acceleration()
    if p.thermokinetic_formulation:
        bs.dedt()
    else:
        bs.dudt()
    if p.enable_fmm:
        bs.gravitation()
    return bs.download(fields=["ax", "ay", "az", "gax", "gay", "gaz", "rho", "P", "cs",
                               "dedt", "dudt", "id"])


def gpu_arm(args):
    rank, world, local = dist_info()
    dist = init_dist(world)
    from flecsph_gb300 import build, setups
    from flecsph_gb300.abi import PRECISION_FP64, PRECISION_MIXED, make_view
    if rank == 0:
        build.build()
    barrier(dist)
    from flecsph_gb300 import sph

    if args.workload == "kh":
        n1d = args.n1d or 256
        s, p, meta = setups.kh3d(n1d)
        wname = f"kh3d_{n1d}^3_periodic"
    elif args.workload == "polytrope":
        npart = args.n or (1 << 22)
        s, p, meta = setups.polytrope3d(npart, rho_floor=1e-2)
        p.max_neighbors = 512
        wname = f"polytrope3d_{npart}_gravity_quadrupole_theta0.5"
    else:
        n1d = args.n1d or 128
        s, p, meta = setups.sedov3d(n1d)
        wname = f"sedov3d_{n1d}^3"
    n = meta["n"]
    cap = sph.capacity_for(p, n, s)
    mixed_ok = sph.mixed_available() if hasattr(sph, "mixed_available") else False
    prec = args.precision
    if prec == "auto":
        prec = "mixed" if mixed_ok else "fp64"
    results = {}
    modes = ["fp64"] + (["mixed"] if mixed_ok else [])
    if args.precision == "fp64":
        modes = ["fp64"]
    elif args.precision == "mixed":
        modes = ["mixed"]
    cmp_state = None
    for mode in modes:
        p.precision_mode = PRECISION_MIXED if mode == "mixed" else PRECISION_FP64
        bs = sph.BodySystem(p, cap, device=local)
        bs.read_bodies(s)
        bs.step()  # initial iteration
        for _ in range(args.warmup):
            bs.step()
        bs.sync()
        ntot = bs.count()[0]
        off = np.zeros(ntot + 1, np.int64)
        bs.lib.fsph_get_neighbors(bs.ctx, off.ctypes.data, None, 0)
        nb_mean = float(off[-1]) / ntot
        cons0 = bs.conserved()
        bs.timers_reset()
        launches0 = bs.launch_count()
        barrier(dist)
        with Clocks(local) as clk:
            bs.mark(0)
            for _ in range(args.steps):
                bs.step()
            bs.mark(1)
            ms = bs.elapsed_ms(0, 1)
        bs.sync()
        launches = bs.launch_count() - launches0
        ms = max_over_ranks(dist, ms)
        timers = bs.timers()
        cons1 = bs.conserved()
        state = bs.download(fields=["m", "vx", "vy", "vz", "id"])
        results[mode] = dict(ms=ms, timers=timers, launches=launches, nb_mean=nb_mean,
                             clocks=clk.summary(), ntot=ntot,
                             drift=drift(cons0, cons1, s, state))
        # one pass of each precision from one common state: the FP64 run's
        # state after its timed steps (velocities and the blast or shear
        # developed, so the energy rates are not trivially zero), real
        # particles only (periodic copies carry ids >= n)
        if cmp_state is None:
            full = bs.download()
            real = full["id"] < n
            cmp_state = {f: np.ascontiguousarray(full[f][real]) for f in s}
        results[mode]["same_state"] = one_pass(bs, cmp_state, p)
        if len(modes) == 2 and p.sph_viscosity == 0:
            # the same pass without artificial viscosity: how much of the
            # acceleration error is the FP32 viscosity's
            visc = (p.sph_viscosity_alpha, p.sph_viscosity_beta)
            p.sph_viscosity_alpha = p.sph_viscosity_beta = 0.0
            b2 = sph.BodySystem(p, cap, device=local)
            results[mode]["no_visc"] = one_pass(b2, cmp_state, p)
            b2.close()
            p.sph_viscosity_alpha, p.sph_viscosity_beta = visc
        if (args.workload == "polytrope" and rank == 0 and mode == modes[-1]
                and not args.no_check):
            results[mode]["gravity_check"] = gravity_check(bs, p)
        # end to end through the C ABI with pinned host buffers
        if not args.no_e2e:
            # page-locked host buffers (cudaHostAlloc through torch's pinned
            # allocator), filled with the current state
            import torch
            host = bs.download()
            pinned = []
            for f in set(IN_FIELDS + OUT_FIELDS) | {"id", "key"}:
                if f not in host:
                    continue
                src = np.ascontiguousarray(host[f])
                buf = torch.empty(src.nbytes, dtype=torch.uint8, pin_memory=True)
                arr = buf.numpy().view(src.dtype)
                arr[:] = src
                pinned.append(buf)
                host[f] = arr
            vin = make_view(host, fields=set(IN_FIELDS) | {"id"})
            vout = make_view(host, fields=set(OUT_FIELDS) | {"id", "key"})
            h2d = 8 * ntot * (len(IN_FIELDS) + 1)
            d2h = 8 * ntot * (len(OUT_FIELDS) + 2)
            barrier(dist)
            t0 = time.perf_counter()
            bs.mark(2)
            for _ in range(args.steps):
                # inputs in, one iteration, results out (fsph_step_io:
                # the copies overlap the step where the data allow)
                bs.step_io(vin, vout)
            bs.mark(3)
            e2e_ms = bs.elapsed_ms(2, 3)
            wall = time.perf_counter() - t0
            e2e_ms = max_over_ranks(dist, e2e_ms)
            # the same pinned host buffers copied alone, once each way
            bs.mark(4)
            bs.upload_fields(vin)
            bs.mark(5)
            bs.download_into(vout)
            bs.mark(6)
            copy_gbs = {"h2d": round(h2d / (bs.elapsed_ms(4, 5) * 1e-3) / 1e9, 1),
                        "d2h": round(d2h / (bs.elapsed_ms(5, 6) * 1e-3) / 1e9, 1)}
            del pinned
            results[mode]["e2e"] = dict(ms=e2e_ms, wall_s=wall, h2d=h2d, d2h=d2h,
                                        link_gbs=link_gbs(), copy_gbs=copy_gbs)
        bs.close()

    if rank != 0:
        return
    head = results["mixed" if "mixed" in results else "fp64"]
    K = args.steps
    value = world * n * K / (head["ms"] * 1e-3)
    # dominant kernel and its roofline; every phase's fraction beside it
    t = head["timers"]
    mixed_run = "mixed" in results
    fp64_peak = sph.measure_peak(0, local)
    fp32_peak = sph.measure_peak(1, local)
    pk_flop = fp32_peak if mixed_run else fp64_peak
    per_phase = {}
    for ph, (ms_tot, calls) in t.items():
        if not calls:
            continue
        work = work_model(ph, head["nb_mean"], mixed_run, bool(p.thermokinetic_formulation))
        if work is None:
            continue
        per_launch_s = ms_tot / calls * 1e-3
        per_phase[ph] = phase_roofline(work, head["ntot"], per_launch_s, pk_flop,
                                       "fp32" if mixed_run else "fp64")
    top = max((k for k in t if t[k][1] > 0), key=lambda k: t[k][0])
    roof = dict(per_phase.get(top, {"bound": "hbm", "achieved": None,
                                    "peak": HBM_PEAK, "unit": "GB/s", "frac": None}))
    roof["kernel"] = top
    tpp = MEASURED_TRAFFIC_PER_PARTICLE.get(top)
    roof["traffic"] = tpp * head["ntot"] if (tpp and mixed_run) else None
    if roof["traffic"] is not None:
        roof["traffic_source"] = ("ncu dram bytes of a 96^3 capture, per particle, "
                                  "scaled to this launch")
    roof["peak_source"] = ("MEASURED_PEAKS.json hbm_gbs" if roof.get("bound") == "hbm" else
                           "in-repo FMA-chain probe (fsph_measure_peak), measured this run")
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": head["ms"] / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if "mixed" in results else "f64",
        "data": "synthetic",
        "config": {"workload": wname, "n_particles": n,
                   "n_with_periodic_copies": head["ntot"],
                   "kernel": "wendland_c6", "gamma": p.poly_gamma, "eta": p.sph_eta,
                   "mean_neighbors": head["nb_mean"], "parallelism": f"replicas{world}",
                   "l2": "inputs exceed L2 (state ~0.5 GB, lists ~0.8 GB); no flush",
                   "precision": "mixed" if "mixed" in results else "fp64"},
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
        "roofline": roof,
        "roofline_all": per_phase,
        "per_kernel_ms_per_step": {k: v[0] / K for k, v in t.items() if v[1]},
    }
    line["roofline_step"] = step_roofline(per_phase, line["per_kernel_ms_per_step"],
                                          line["ms_per_step"])
    if "fp64" in results:
        line["fp64"] = {"value": world * n * K / (results["fp64"]["ms"] * 1e-3),
                        "ms_per_step": results["fp64"]["ms"] / K}
    if "mixed" in results and "fp64" in results:
        # one pass of each precision from the same state (after K steps the
        # two runs have drifted apart, which says nothing about one pass)
        a64 = results["fp64"]["same_state"]
        am = results["mixed"]["same_state"]
        pf = per_field_errors(a64, am, p)
        line["mixed_vs_fp64"] = {"speedup": results["fp64"]["ms"] / results["mixed"]["ms"],
                                 "accel_rel_err_max": pf["a"]["max"],
                                 "accel_rel_err_median": pf["a"]["median"],
                                 "accel_normwise": pf["a"]["normwise"],
                                 "per_field": pf,
                                 "measured_on": "one pass of each precision from the "
                                                "FP64 run's state after its timed steps "
                                                "(density, acceleration, energy rate, "
                                                "gravity); per particle "
                                                "|d|/|ref| for rho, P, c_s and "
                                                "|d|/max(|ref|, 1e-3 rms|ref|) for a, "
                                                "de/dt (du/dt), g_acc"}
        if "no_visc" in results["mixed"]:
            pv = per_field_errors(results["fp64"]["no_visc"], results["mixed"]["no_visc"], p)
            line["mixed_vs_fp64"]["accel_without_viscosity"] = pv["a"]
        if p.enable_fmm:
            line["mixed_vs_fp64"]["gravity_rel_err_max"] = pf["g_acc"]["max"]
            line["mixed_vs_fp64"]["gravity_rel_err_median"] = pf["g_acc"]["median"]
    if "e2e" in head:
        e = head["e2e"]
        line["e2e"] = {"value": world * n * K / (e["ms"] * 1e-3), "unit": "particle-steps/s",
                       "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"],
                       "ms_per_step": e["ms"] / K,
                       "wall_ms_per_step": 1e3 * e["wall_s"] / K,
                       "copy_gbs": e["copy_gbs"], "link_gbs": e["link_gbs"],
                       "host": {"cpus": len(os.sched_getaffinity(0)),
                                "loadavg_1min": os.getloadavg()[0]}}
    if args.workload == "kh":
        line["drift"] = {m: results[m]["drift"] for m in results}
    if args.workload == "polytrope":
        line["gravity_check"] = head.get("gravity_check")
        line["drift"] = {m: results[m]["drift"] for m in results}
    if not args.no_cpu and args.workload == "sedov":
        cpu = run_cpu_oracle(n1d, None, os.cpu_count() or 1, min_seconds=10.0)
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line["peaks_measured"] = {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "ensemble":
        ensemble_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
