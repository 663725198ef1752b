"""Generate the golden fixtures from the reference itself.

Runs the laristra/flecsph hot path compiled here (oracle/_ref, built from the
reference sources by oracle/Makefile) on small seeded inputs and stores
inputs and outputs as compressed .npz files next to this script:

    python tests/golden/make_golden.py [REFERENCE_ROOT] [--only NAME ...]

Each fixture holds: the input state (in a shuffled order), the parameter
block, and after update_iteration the Morton keys, sorted ids, range and
neighbour lists (CSR, in the reference's own order) plus the processing
order of apply_in_smoothinglength; then the full state and (dt, time,
iteration) after each of `steps` driver iterations.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from flecsph_gb300 import setups  # noqa: E402
from flecsph_gb300.abi import (DOUBLE_FIELDS, EOS_NO_EOS, EOS_PPT, EOS_WD,  # noqa: E402
                               KERNEL_QUINTIC_SPLINE, KERNEL_SUPER_GAUSSIAN,
                               KERNEL_WENDLAND_C4, VISC_CULLEN)
import pyoracle  # noqa: E402


def cases():
    s, p, m = setups.sod3d(40, 10, 10)
    yield "sod3d_4000", setups.shuffled(s, 1), p, 3
    s, p, m = setups.sod3d(40, 10, 10)
    p.thermokinetic_formulation = 0
    yield "sod3d_dudt_4000", setups.shuffled(s, 2), p, 2
    s, p, m = setups.sedov3d(16, eta=1.44)
    yield "sedov3d_4096", setups.shuffled(s, 3), p, 2
    s, p, m = setups.polytrope3d(3000)
    p.enable_fmm = 0
    p.sph_variable_h = 1
    p.thermokinetic_formulation = 1
    yield "polytrope3d_varh_3000", s, p, 2
    s, p, m = setups.sod3d(40, 10, 10)
    p.sph_kernel = KERNEL_WENDLAND_C4
    yield "sod3d_c4_4000", setups.shuffled(s, 4), p, 2
    s, p, m = setups.sod2d(100, 10)
    yield "sod2d_1000", setups.shuffled(s, 5), p, 2
    s, p, m = setups.noh2d(40)
    yield "noh2d_1264", setups.shuffled(s, 6), p, 2
    # Cullen & Dehnen adaptive viscosity
    s, p, m = setups.sod3d(40, 10, 10)
    p.sph_viscosity = VISC_CULLEN
    yield "sod3d_cullen_4000", setups.shuffled(s, 9), p, 3
    # the kernels of kernel width 3
    s, p, m = setups.sod2d(100, 10)
    p.sph_kernel = KERNEL_SUPER_GAUSSIAN
    yield "sod2d_supergauss_1000", setups.shuffled(s, 10), p, 2
    s, p, m = setups.sod3d(40, 10, 10)
    p.sph_kernel = KERNEL_QUINTIC_SPLINE
    p.sph_variable_h = 1
    yield "sod3d_quintic_varh_4000", setups.shuffled(s, 11), p, 2
    # the other equations of state
    for name, seed, s, p in eos_cases():
        yield name, setups.shuffled(s, seed), p, 2
    # external forces and particle relaxation
    for k, name in enumerate(setups.EXTERNAL_FORCE_PROBLEMS):
        s, p = setups.external_force_problem(name)
        yield "eforce_" + name, setups.shuffled(s, 20 + k), p, 2
    # periodic boundaries: copies regenerated at every update_iteration;
    # a few particles start outside the box and are teleported back
    s, p, m = setups.kh2d(40)
    yield "kh2d_periodic_1600", setups.shuffled(_outside(s), 7), p, 2
    s, p, m = setups.kh3d(12)
    p.periodic_boundary_y = p.periodic_boundary_z = 0
    yield "kh3d_periodic_x_1728", setups.shuffled(_outside(s), 8), p, 2
    # the driver's energy branches (hydro/main_driver.cc:145-171,214-240):
    # two pressure updates per step, and no energy evolution
    s, p, m = setups.sod3d(40, 10, 10)
    p.pressure_updates_number = 2
    yield "sod3d_pu2_4000", setups.shuffled(s, 30), p, 2
    s, p, m = setups.sod3d(40, 10, 10)
    p.thermokinetic_formulation = 0
    p.pressure_updates_number = 2
    yield "sod3d_dudt_pu2_4000", setups.shuffled(s, 31), p, 2
    s, p, m = setups.sod3d(40, 10, 10)
    p.evolve_internal_energy = 0
    yield "sod3d_noevolve_4000", setups.shuffled(s, 32), p, 2
    s, p, m = setups.sod2d(100, 10)
    p.thermokinetic_formulation = 0
    p.evolve_internal_energy = 0
    yield "sod2d_noevolve_dudt_1000", setups.shuffled(s, 33), p, 2


def eos_cases():
    """Sod tubes under the piecewise polytrope (threshold between the two
    states), the white-dwarf EOS (densities 1e7 and 1.25e6 g/cc, Ye = 0.5)
    and no EOS (pressure and sound speed frozen at their inputs)."""
    s, p, m = setups.sod3d(40, 10, 10)
    p.eos_type = EOS_PPT
    p.poly_gamma2 = 2.5
    p.ppt_density_thr = 0.5
    yield "sod3d_ppt_4000", 12, s, p
    s, p, m = setups.sod3d(40, 10, 10)
    p.eos_type = EOS_WD
    s["m"] *= 1.0e7
    s["rho"] *= 1.0e7
    s["Ye"][:] = 0.5
    yield "sod3d_wd_4000", 13, s, p
    s, p, m = setups.sod2d(100, 10)
    p.eos_type = EOS_NO_EOS
    s["cs"][:] = np.sqrt(p.poly_gamma * s["P"] / s["rho"])
    yield "sod2d_noeos_1000", 14, s, p


def _outside(s):
    """Move a few particles out of the box, off the lattice."""
    s = {k: v.copy() for k, v in s.items()}
    s["x"][:5] += 0.6137
    s["x"][5:8] -= 0.5419
    return s


def main():
    args = sys.argv[1:]
    only = None
    if "--only" in args:
        k = args.index("--only")
        only = set(args[k + 1:])
        args = args[:k]
    ref_root = args[0] if args else pyoracle.reference_root()
    if not ref_root or not pyoracle.build_ref(ref_root):
        sys.exit(f"reference sources not found at {ref_root}")
    for name, state, params, steps in cases():
        if only is not None and name not in only:
            continue
        o = pyoracle.Oracle("reference", params)
        o.upload(state)
        out = {}
        for f in DOUBLE_FIELDS + ["id"]:
            out["in_" + f] = state[f]
        o.update_iteration()
        upd = o.download()
        out["upd_key"] = upd["key"]
        out["upd_id"] = upd["id"]
        out["upd_range"] = o.range()
        off, idx = o.neighbors()
        out["nb_offsets"] = off.astype(np.int64)
        out["nb_indices"] = idx.astype(np.int32)
        out["order"] = o.order().astype(np.int32)
        # restart from the input so the steps start at the initial iteration
        o.close()
        o = pyoracle.Oracle("reference", params)
        o.upload(state)
        for k in range(steps):
            o.step()
            st = o.download()
            for f in DOUBLE_FIELDS + ["id"]:
                out[f"s{k}_{f}"] = st[f]
            out[f"s{k}_time"] = np.array(o.time()[:2])
            out[f"s{k}_iteration"] = np.array(o.time()[2])
        out["params_json"] = np.array(json.dumps(params.as_dict()))
        out["steps"] = np.array(steps)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        o.close()
        print(f"{name}: n={len(state['x'])} steps={steps} -> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
