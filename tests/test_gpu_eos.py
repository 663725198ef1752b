"""The piecewise polytrope, white-dwarf and no-EOS equations of state on the
GPU: FP64 mode against the CPU oracle to 1e-12 over full driver iterations
at the full Sod size (80x20x20), and the mixed path's one-pass accelerations
against FP64 from the same state (relative 1e-5).  The golden fixtures
sod3d_ppt_4000, sod3d_wd_4000 and sod2d_noeos_1000 hold the reference's own
outputs for the same three."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import (DOUBLE_FIELDS, EOS_NO_EOS, EOS_PPT, EOS_WD, PRECISION_FP64,
                               PRECISION_MIXED)

pytestmark = pytest.mark.gpu


def normwise(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())


def _problem(eos):
    s, p, m = setups.sod3d()
    p.eos_type = eos
    if eos == EOS_PPT:
        p.poly_gamma2 = 2.5
        p.ppt_density_thr = 0.5
    elif eos == EOS_WD:
        s["m"] *= 1.0e7
        s["rho"] *= 1.0e7
        s["Ye"][:] = 0.5
    else:
        s["cs"][:] = np.sqrt(p.poly_gamma * s["P"] / s["rho"])
    return setups.shuffled(s, 71 + eos), p


@pytest.mark.parametrize("eos", [EOS_PPT, EOS_WD, EOS_NO_EOS])
def test_fp64_vs_oracle(oracle_port, eos):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _problem(eos)
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
        assert bs.time()[2] == o.time()[2]
    bs.close()


@pytest.mark.parametrize("eos", [EOS_PPT, EOS_WD, EOS_NO_EOS])
def test_mixed_vs_fp64(eos):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _problem(eos)
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
    for f in ("rho", "P", "cs"):
        assert normwise(b[f], a[f]) <= 1e-6, f
    A = np.stack([a[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([b[k] for k in ("ax", "ay", "az")], 1)
    assert np.abs(A - B).max() / np.abs(A).max() <= 1e-5
    assert normwise(b["dedt"], a["dedt"]) <= 1e-5
