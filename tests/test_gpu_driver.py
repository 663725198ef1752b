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
