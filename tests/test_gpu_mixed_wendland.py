"""The float-float density and acceleration passes for each Wendland kernel
(C2, C4, C6) in 2D and 3D, against the FP64 path from the same state: the
polynomials in t = 1 - q and their constants are checked here.  Bars:
density 1e-10 relative, acceleration 1e-5 per particle
(|da| / max(|a|, 1e-3 rms|a|)), de/dt (through the pressure-only
acceleration) 1e-5 normwise."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import (KERNEL_WENDLAND_C2, KERNEL_WENDLAND_C4, KERNEL_WENDLAND_C6,
                               PRECISION_FP64, PRECISION_MIXED)

pytestmark = pytest.mark.gpu


def _problem(dim, kernel):
    if dim == 3:
        s, p, m = setups.sedov3d(20, eta=1.5)
    else:
        s, p, m = setups.sod2d(80, 16)
    p.sph_kernel = kernel
    s = setups.shuffled(s, 7)
    rng = np.random.Generator(np.random.PCG64(3))
    # a smooth flow and a slightly irregular lattice
    for k in ("x", "y", "z")[:dim]:
        s[k] = s[k] + 0.02 * (rng.random(len(s[k])) - 0.5) * (s["h"] / 3.0)
    s["vx"][:] = 0.05 * np.sin(2 * np.pi * s["y"])
    s["vy"][:] = 0.05 * np.sin(2 * np.pi * s["x"])
    return s, p


def _one_pass(s, p, mode):
    from flecsph_gb300 import build
    build.build()
    from flecsph_gb300.sph import BodySystem
    p.precision_mode = mode
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    bs.update_iteration()
    bs.eos_init()
    bs.set_total_energy()
    bs.density_pressure_soundspeed()
    bs.save_velocityhalf()
    bs.acceleration()
    bs.dedt()
    out = bs.download()
    bs.close()
    o = np.argsort(out["id"])
    return {k: v[o] for k, v in out.items()}


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", [KERNEL_WENDLAND_C2, KERNEL_WENDLAND_C4,
                                    KERNEL_WENDLAND_C6])
def test_float_float_wendland(dim, kernel):
    s, p = _problem(dim, kernel)
    a = _one_pass(s, p, PRECISION_FP64)
    b = _one_pass(s, p, PRECISION_MIXED)
    rho = np.abs(b["rho"] - a["rho"]) / a["rho"]
    ks = ("ax", "ay", "az")[:dim]
    A = np.stack([a[k] for k in ks], 1)
    B = np.stack([b[k] for k in ks], 1)
    mag = np.linalg.norm(A, axis=1)
    e = np.linalg.norm(B - A, axis=1) / np.maximum(mag, 1e-3 * np.sqrt((mag ** 2).mean()))
    de = np.abs(b["dedt"] - a["dedt"]).max() / np.abs(a["dedt"]).max()
    print(dim, kernel, "rho", rho.max(), "accel", e.max(), np.median(e), "dedt", de)
    assert rho.max() <= 1e-10, rho.max()
    assert e.max() <= 1e-5, e.max()
    assert de <= 1e-5, de
