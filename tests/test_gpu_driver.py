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
