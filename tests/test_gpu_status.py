"""Device-detected failures come back as C-ABI status codes, replacing the
reference's assert()/abort (default_physics.h:215-226, 918-979).  All
faults are planted on the host side (bad inputs, tiny capacities): nothing
here faults or hangs the GPU."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import FsphError

pytestmark = pytest.mark.gpu


def _bs(params, n):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    return BodySystem(params, n)


def _expect(bs, call, code):
    with pytest.raises(FsphError) as ei:
        call()
        bs.sync()
    assert ei.value.status == code


def test_negative_mass_gives_negative_density():
    s, p, m = setups.sod3d(20, 5, 5)
    s["m"][:] = -s["m"]
    bs = _bs(p, m["n"])
    bs.read_bodies(s)
    bs.update_iteration()
    _expect(bs, bs.density_pressure_soundspeed, 4)


def test_nonpositive_internal_energy():
    s, p, m = setups.sod3d(20, 5, 5)
    bs = _bs(p, m["n"])
    s["e"][:] = -1.0
    bs.read_bodies(s)
    bs.update_iteration()
    _expect(bs, bs.density_pressure_soundspeed, 5)


def test_duplicate_positions_rejected():
    s, p, m = setups.sod3d(20, 5, 5)
    s["x"][1], s["y"][1], s["z"][1] = s["x"][0], s["y"][0], s["z"][0]
    bs = _bs(p, m["n"])
    bs.read_bodies(s)
    _expect(bs, bs.update_iteration, 10)


def test_list_overflow_reported():
    s, p, m = setups.sod3d(20, 5, 5)
    p.max_neighbors = 16
    bs = _bs(p, m["n"])
    bs.read_bodies(s)
    _expect(bs, bs.update_iteration, 7)


def test_nan_detected():
    s, p, m = setups.sod3d(20, 5, 5)
    bs = _bs(p, m["n"])
    s["vx"][5] = np.nan
    bs.read_bodies(s)
    _expect(bs, bs.check_nans, 3)


def test_context_usable_after_error():
    s, p, m = setups.sod3d(20, 5, 5)
    bs = _bs(p, m["n"])
    s2 = dict(s)
    s2["e"] = np.full_like(s["e"], -1.0)
    bs.read_bodies(s2)
    bs.update_iteration()
    _expect(bs, bs.density_pressure_soundspeed, 5)
    bs.read_bodies(s)
    bs.step()
    bs.step()
    bs.sync()
