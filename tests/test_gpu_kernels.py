"""The quintic spline, Gaussian, super-Gaussian and sinc kernels on the GPU: FP64
mode against the CPU oracle to 1e-12 over full driver iterations, and the
mixed path's one-pass accelerations against FP64 from the same state."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import (DOUBLE_FIELDS, KERNEL_GAUSSIAN, KERNEL_QUINTIC_SPLINE,
                               KERNEL_SINC, KERNEL_SUPER_GAUSSIAN, PRECISION_FP64,
                               PRECISION_MIXED)

pytestmark = pytest.mark.gpu
KERNELS = [KERNEL_QUINTIC_SPLINE, KERNEL_GAUSSIAN, KERNEL_SUPER_GAUSSIAN, KERNEL_SINC]


def normwise(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())


def _problem(kernel):
    s, p, m = setups.sedov3d(20, eta=1.44)
    p.sph_kernel = kernel
    s = setups.shuffled(s, 61)
    two_pi = 2 * np.pi
    s["vx"][:] = 0.05 * np.sin(two_pi * s["y"])
    s["vy"][:] = 0.05 * np.sin(two_pi * s["z"])
    return s, p


@pytest.mark.parametrize("kernel", KERNELS)
def test_fp64_vs_oracle(oracle_port, kernel):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _problem(kernel)
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    o = oracle_port.Oracle("port", p, threads=8)
    o.upload(s)
    for k in range(3):
        bs.step()
        o.step()
        g, r = bs.download(), o.download()
        assert np.array_equal(g["id"], r["id"])
        for f in DOUBLE_FIELDS:
            assert normwise(g[f], r[f]) <= 1e-12, (k, f)
    bs.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_mixed_vs_fp64(kernel):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _problem(kernel)
    out = {}
    for mode in (PRECISION_FP64, PRECISION_MIXED):
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
        out[mode] = bs.download()
        bs.close()
    a, b = out[PRECISION_FP64], out[PRECISION_MIXED]
    assert np.abs(b["rho"] - a["rho"]).max() / np.abs(a["rho"]).max() <= 1e-6
    A = np.stack([a[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([b[k] for k in ("ax", "ay", "az")], 1)
    assert np.abs(A - B).max() / np.abs(A).max() <= 1e-5
    assert normwise(b["dedt"], a["dedt"]) <= 1e-5
