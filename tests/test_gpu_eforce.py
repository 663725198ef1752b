"""External forces (include/physics/eforce.h) and the particle relaxation
terms on the GPU: FP64 mode against the CPU oracle to 1e-12 over four
driver iterations for every problem of setups.external_force_problem, the
mixed path against FP64 (one pass from the same state), and the relaxation
entry points called one by one against the oracle.  The golden fixtures
eforce_* hold the reference's own outputs for the same problems."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import DOUBLE_FIELDS, PRECISION_FP64, PRECISION_MIXED

pytestmark = pytest.mark.gpu


def normwise(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())


@pytest.mark.parametrize("case", setups.EXTERNAL_FORCE_PROBLEMS)
def test_fp64_vs_oracle(oracle_port, case):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = setups.external_force_problem(case)
    s = setups.shuffled(s, 93)
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    o = oracle_port.Oracle("port", p, threads=8)
    o.upload(s)
    for k in range(4):
        bs.step()
        o.step()
        g, r = bs.download(), o.download()
        assert np.array_equal(g["id"], r["id"])
        for f in DOUBLE_FIELDS:
            assert normwise(g[f], r[f]) <= 1e-12, (k, f, normwise(g[f], r[f]))
        gt, rt = bs.time(), o.time()
        assert gt[2] == rt[2] and abs(gt[0] - rt[0]) <= 1e-12 * rt[0]
    bs.close()


@pytest.mark.parametrize("case", setups.EXTERNAL_FORCE_PROBLEMS)
def test_mixed_vs_fp64(case):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = setups.external_force_problem(case)
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
        if p.relaxation_steps:
            bs.add_drag_acceleration()
            bs.add_short_range_repulsion()
        if p.thermokinetic_formulation:
            bs.dedt()
        else:
            bs.dudt()
        out[mode] = bs.download()
        bs.close()
    a, b = out[PRECISION_FP64], out[PRECISION_MIXED]
    A = np.stack([a[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([b[k] for k in ("ax", "ay", "az")], 1)
    assert np.abs(A - B).max() / np.abs(A).max() <= 1e-5
    assert normwise(b["u"], a["u"]) <= 1e-6
    de = "dedt" if p.thermokinetic_formulation else "dudt"
    assert normwise(b[de], a[de]) <= 1e-5


def test_relaxation_calls_vs_oracle(oracle_port):
    """fsph_add_drag_acceleration, fsph_add_short_range_repulsion,
    fsph_add_drag_dedt and fsph_add_drag_dudt one by one against the oracle."""
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = setups.external_force_problem("relaxation_3d")
    s = setups.shuffled(s, 94)
    bs = BodySystem(p, len(s["x"]))
    o = oracle_port.Oracle("port", p, threads=8)
    for x in (bs, o):
        x.read_bodies(s) if x is bs else x.upload(s)
        x.update_iteration()
        x.eos_init()
        x.set_total_energy()
        x.density_pressure_soundspeed()
        x.save_velocityhalf()
        x.acceleration()
        x.add_drag_acceleration()
        x.add_short_range_repulsion()
        x.dedt()
        x.add_drag_dedt()
        x.dudt()
        x.add_drag_dudt()
    g, r = bs.download(), o.download()
    for f in ("ax", "ay", "az", "dedt", "dudt"):
        assert normwise(g[f], r[f]) <= 1e-12, f
    bs.close()
