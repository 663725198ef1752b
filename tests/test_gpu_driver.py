"""The C++ hydro driver, written call by call against the body_system mirror
(include/fsph_body_system.hpp) the way app/drivers/hydro/main_driver.cc
calls the reference, gives exactly the state of the fused fsph_step."""
import os
import subprocess

import numpy as np
import pytest

from flecsph_gb300 import build, setups, snapshot
from flecsph_gb300.abi import DOUBLE_FIELDS

pytestmark = pytest.mark.gpu


def test_cpp_driver_matches_fused_step(tmp_path):
    build.build()
    from flecsph_gb300.sph import BodySystem
    s, p, meta = setups.sod3d(40, 10, 10)
    s = setups.shuffled(s, 21)
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    snapshot.write(src, s, 3)
    args = [build.DRIVER, str(src), str(dst), "4", "sph_kernel=4", "poly_gamma=1.4",
            "sph_eta=1.5", "adaptive_timestep=1", "initial_dt=1e-12"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, dim = snapshot.read(dst)
    bs = BodySystem(p, meta["n"])
    bs.read_bodies(s)
    for _ in range(4):
        bs.step()
    ref = bs.download()
    assert np.array_equal(out["id"], ref["id"])
    for f in DOUBLE_FIELDS:
        assert np.array_equal(out[f], ref[f]), f
    dt, t, it = bs.time()
    assert f"iteration {it} " in r.stdout


def test_cpp_driver_relaxation_and_external_force(tmp_path):
    """The driver's relaxation branch (drag, repulsion, drag terms in the
    energy equation) for two iterations and then two regular ones, with a
    spherical wall named by its external_force_type string."""
    build.build()
    from flecsph_gb300.sph import BodySystem, set_external_force
    s, p = setups.external_force_problem("relaxation_3d")
    p.relaxation_steps = 2
    p.sphere_radius, p.extforce_wall_steepness, p.extforce_wall_powerindex = 0.45, 1e3, 3.0
    set_external_force(p, "spherical wall")
    s = setups.shuffled(s, 22)
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    snapshot.write(src, s, 3)
    args = [build.DRIVER, str(src), str(dst), "4", f"sph_kernel={p.sph_kernel}",
            f"poly_gamma={p.poly_gamma!r}", f"sph_eta={p.sph_eta!r}",
            f"adaptive_timestep={p.adaptive_timestep}", f"initial_dt={p.initial_dt!r}",
            f"timestep_cfl_factor={p.timestep_cfl_factor!r}",
            "relaxation_steps=2", f"relaxation_beta={p.relaxation_beta!r}",
            f"relaxation_gamma={p.relaxation_gamma!r}",
            f"relaxation_repulsion_radius={p.relaxation_repulsion_radius!r}",
            f"relaxation_repulsion_gamma={p.relaxation_repulsion_gamma!r}",
            "external_force_type=spherical wall", "sphere_radius=0.45",
            "extforce_wall_steepness=1000", "extforce_wall_powerindex=3"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, dim = snapshot.read(dst)
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    for _ in range(4):
        bs.step()
    ref = bs.download()
    assert np.array_equal(out["id"], ref["id"])
    for f in DOUBLE_FIELDS:
        assert np.array_equal(out[f], ref[f]), f


def _driver_args(p, extra=()):
    return [f"sph_kernel={p.sph_kernel}", f"poly_gamma={p.poly_gamma!r}",
            f"sph_eta={p.sph_eta!r}", f"adaptive_timestep={p.adaptive_timestep}",
            f"initial_dt={p.initial_dt!r}",
            f"thermokinetic_formulation={p.thermokinetic_formulation}",
            f"evolve_internal_energy={p.evolve_internal_energy}",
            f"pressure_updates_number={p.pressure_updates_number}", *extra]


@pytest.mark.parametrize("thermo,evolve,updates", [(1, 1, 2), (0, 1, 2), (1, 0, 1),
                                                   (0, 0, 1)])
def test_cpp_driver_energy_branches(tmp_path, thermo, evolve, updates):
    """The driver's energy branches (hydro/main_driver.cc:145-171,214-240):
    two pressure updates per step, or no energy evolution, in both energy
    formulations, equal to the fused step bit for bit (which the golden
    fixtures sod3d_pu2, sod3d_dudt_pu2, sod3d_noevolve and
    sod2d_noevolve_dudt pin against the reference)."""
    build.build()
    from flecsph_gb300.sph import BodySystem
    s, p, meta = setups.sod3d(40, 10, 10)
    p.adaptive_timestep, p.initial_dt = 1, 1e-12
    p.thermokinetic_formulation, p.evolve_internal_energy = thermo, evolve
    p.pressure_updates_number = updates
    s = setups.shuffled(s, 24)
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    snapshot.write(src, s, 3)
    r = subprocess.run([build.DRIVER, str(src), str(dst), "3", *_driver_args(p)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, dim = snapshot.read(dst)
    bs = BodySystem(p, meta["n"])
    bs.read_bodies(s)
    for _ in range(3):
        bs.step()
    ref = bs.download()
    bs.close()
    assert np.array_equal(out["id"], ref["id"])
    for f in DOUBLE_FIELDS:
        assert np.array_equal(out[f], ref[f]), f


def test_cpp_driver_restart(tmp_path):
    """A run split in two: the first part's snapshot carries (iteration, dt,
    time); the second part restarts from it at that iteration with the
    driver's initial-iteration branch and the restored dt and time, as the
    reference's read_bodies(..., initial_iteration) does
    (mpisph/io.h:523-586,818-836).  The restarted run equals the same
    restart of the oracle to 1e-12, and of the fused step bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))), "oracle"))
    import pyoracle
    build.build()
    pyoracle.build_port()
    from flecsph_gb300.sph import BodySystem
    s, p, meta = setups.sod3d(40, 10, 10)
    p.adaptive_timestep, p.initial_dt = 1, 1e-12
    s = setups.shuffled(s, 25)
    src, mid, dst = tmp_path / "in.bin", tmp_path / "mid.bin", tmp_path / "out.bin"
    snapshot.write(src, s, 3)
    r = subprocess.run([build.DRIVER, str(src), str(mid), "2", *_driver_args(p)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    st_mid, dim, tm = snapshot.read(mid, with_time=True)
    assert tm[0] == 2 and tm[1] > 0 and tm[2] > 0
    # a mismatching initial_iteration is refused, as the reference stops
    # when no snapshot holds that iteration
    r = subprocess.run([build.DRIVER, str(mid), str(dst), "3",
                        *_driver_args(p, ["initial_iteration=7"])],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 2 and "initial_iteration" in r.stderr
    r = subprocess.run([build.DRIVER, str(mid), str(dst), "3",
                        *_driver_args(p, ["initial_iteration=2"])],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, dim, tm_out = snapshot.read(dst, with_time=True)
    assert tm_out[0] == 5
    # the same restart through the fused step and through the oracle
    p.initial_iteration = 2
    bs = BodySystem(p, meta["n"])
    bs.read_bodies(st_mid)
    bs.set_time(tm[1], tm[2], tm[0])
    for _ in range(3):
        bs.step()
    ref = bs.download()
    dt, t, it = bs.time()
    bs.close()
    assert (it, dt, t) == tm_out
    assert np.array_equal(out["id"], ref["id"])
    for f in DOUBLE_FIELDS:
        assert np.array_equal(out[f], ref[f]), f
    o = pyoracle.Oracle("port", p, threads=4)
    o.upload(st_mid)
    o.set_time(tm[1], tm[2], tm[0])
    for _ in range(3):
        o.step()
    oref = o.download()
    o.close()
    assert np.array_equal(out["id"], oref["id"])
    for f in DOUBLE_FIELDS:
        scale = max(np.abs(oref[f]).max(), 1e-300)
        assert np.abs(out[f] - oref[f]).max() <= 1e-12 * scale, f


@pytest.mark.parametrize("thermo,updates", [(1, 1), (0, 1), (1, 2), (0, 2)])
def test_cpp_driver_matches_fused_step_mixed(tmp_path, thermo, updates):
    """The mixed-precision path, Wendland C6: the driver's call-by-call
    sequence (acceleration, kick, energy rate, pressure update, energy kick
    as separate calls) gives the state of the fused step, which skips
    repacking records that its own passes left current.  The fused step
    takes the signal speed inside the acceleration pass (FP32, its own
    geometry), the call-by-call sequence in a pass of its own, so dt and
    with it the state may differ in the last bits; a stale record (v - v_half
    of the previous step) would differ at the size of the kick."""
    build.build()
    from flecsph_gb300.abi import PRECISION_MIXED
    from flecsph_gb300.sph import BodySystem
    s, p, meta = setups.sod3d(40, 10, 10)
    p.adaptive_timestep, p.initial_dt = 1, 1e-12
    p.thermokinetic_formulation, p.pressure_updates_number = thermo, updates
    p.precision_mode = PRECISION_MIXED
    s = setups.shuffled(s, 25)
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    snapshot.write(src, s, 3)
    r = subprocess.run([build.DRIVER, str(src), str(dst), "4",
                        *_driver_args(p, (f"precision_mode={PRECISION_MIXED}",))],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, dim = snapshot.read(dst)
    bs = BodySystem(p, meta["n"])
    bs.read_bodies(s)
    for _ in range(4):
        bs.step()
    ref = bs.download()
    bs.close()
    assert np.array_equal(out["id"], ref["id"])
    worst = {f: float(np.abs(out[f] - ref[f]).max() / max(np.abs(ref[f]).max(), 1e-300))
             for f in DOUBLE_FIELDS}
    print("mixed driver vs fused step, largest field difference:",
          max(worst.items(), key=lambda kv: kv[1]))
    for f in DOUBLE_FIELDS:
        assert worst[f] <= 1e-9, (f, worst[f])
