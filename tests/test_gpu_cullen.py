"""Cullen & Dehnen adaptive viscosity on the GPU (FP64 mode) against the CPU
oracle beyond the golden fixture: a Noh implosion in 2D and a Sedov blast
with du/dt, every field within 1e-12 after several full iterations; and the
mixed path against FP64 (one pass from the same state, and four full
iterations)."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import DOUBLE_FIELDS, PRECISION_FP64, PRECISION_MIXED, VISC_CULLEN

pytestmark = pytest.mark.gpu


def normwise(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())


@pytest.mark.parametrize("case", ["noh2d", "sedov3d_dudt", "sod3d_thermo"])
def test_cullen_vs_oracle(oracle_port, case):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    if case == "noh2d":
        s, p, m = setups.noh2d(60)
    elif case == "sedov3d_dudt":
        s, p, m = setups.sedov3d(24, eta=1.44)
        p.thermokinetic_formulation = 0
    else:
        s, p, m = setups.sod3d(60, 12, 12)
    p.sph_viscosity = VISC_CULLEN
    s = setups.shuffled(s, 41)
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    o = oracle_port.Oracle("port", p, threads=8)
    o.upload(s)
    worst = {}
    for k in range(4):
        bs.step()
        o.step()
        g, r = bs.download(), o.download()
        assert np.array_equal(g["id"], r["id"])
        for f in DOUBLE_FIELDS:
            e = normwise(g[f], r[f])
            worst[f] = max(worst.get(f, 0.0), e)
            assert e <= 1e-12, (k, f, e)
        assert bs.time()[2] == o.time()[2]
    print(case, {f: v for f, v in worst.items() if v})
    bs.close()


def _mixed_problem(case, one_pass=False):
    if case == "noh2d":
        s, p, m = setups.noh2d(80)
    else:
        s, p, m = setups.sod3d()
    p.sph_viscosity = VISC_CULLEN
    if one_pass:
        # a wave on top of the problem's own velocities, so that the
        # trigger -d(div v)/dt fires where the flow converges
        two_pi = 2 * np.pi
        s["vx"] += 0.05 * np.sin(two_pi * s["x"])
        s["vy"] += 0.05 * np.sin(two_pi * s["y"])
    return setups.shuffled(s, 43), p


def _both_modes(s, p, calls):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    out = {}
    for mode in (PRECISION_FP64, PRECISION_MIXED):
        p.precision_mode = mode
        bs = BodySystem(p, len(s["x"]))
        bs.read_bodies(s)
        bs.set_time(1e-4, 0.0, 0)
        bs.update_iteration()
        for c in calls:
            getattr(bs, c)()
        out[mode] = bs.download()
        bs.close()
    return out[PRECISION_FP64], out[PRECISION_MIXED]


def _smooth_fields(s):
    """Smooth, sign-changing div v, d(div v)/dt and alpha fields of the
    particles' positions, and sound speeds from the problem's state."""
    two_pi = 2 * np.pi
    x, y = s["x"], s["y"]
    s = {k: v.copy() for k, v in s.items()}
    s["divv"][:] = np.sin(two_pi * x) * np.cos(3 * y)
    s["ddivvdt"][:] = -2.0e4 * np.cos(two_pi * x) * np.sin(5 * y + 0.3)
    s["alpha"][:] = 0.5 + 0.4 * np.sin(7 * x + 2 * y)
    s["cs"][:] = np.sqrt(1.4 * s["P"] / s["rho"])
    return s


@pytest.mark.parametrize("case", ["noh2d", "sod3d"])
def test_mixed_cullen_divergence(case):
    """Density pass with div v and d(div v)/dt, mixed against FP64."""
    s, p = _mixed_problem(case, one_pass=True)
    s["divv"][:] = 0.3
    a, b = _both_modes(s, p, ["eos_init", "set_total_energy",
                              "density_pressure_soundspeed"])
    errs = {f: normwise(b[f], a[f]) for f in ("rho", "divv", "ddivvdt")}
    print(case, errs)
    assert errs["rho"] <= 1e-6
    assert errs["divv"] <= 1e-6 and errs["ddivvdt"] <= 1e-6


@pytest.mark.parametrize("case", ["noh2d", "sod3d"])
def test_mixed_cullen_alpha(case):
    """The alpha pass from identical inputs (density, sound speeds, div v,
    its rate and the previous alpha uploaded): both branches of the update
    (growth to the local alpha, exponential decay) occur."""
    s, p = _mixed_problem(case, one_pass=True)
    s = _smooth_fields(s)
    a, b = _both_modes(s, p, ["compute_alpha"])
    alpha_in = np.empty(len(s["x"]))
    alpha_in[s["id"]] = s["alpha"]
    grew = a["alpha"] > alpha_in[a["id"]]
    e = normwise(b["alpha"], a["alpha"])
    print(case, "alpha", e, "grew:", int(grew.sum()), "of", len(grew))
    assert 0 < grew.sum() < len(grew)
    assert e <= 1e-5


@pytest.mark.parametrize("case", ["noh2d", "sod3d"])
def test_mixed_cullen_forces(case):
    """Acceleration and de/dt with a per-particle alpha field, mixed against
    FP64 (relative 1e-5)."""
    s, p = _mixed_problem(case, one_pass=True)
    s = _smooth_fields(s)
    a, b = _both_modes(s, p, ["eos_init", "set_total_energy",
                              "density_pressure_soundspeed", "save_velocityhalf",
                              "acceleration", "dedt"])
    A = np.stack([a[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([b[k] for k in ("ax", "ay", "az")], 1)
    acc = float(np.abs(A - B).max() / np.abs(A).max())
    de = normwise(b["dedt"], a["dedt"])
    print(case, "acc", acc, "dedt", de)
    assert acc <= 1e-5 and de <= 1e-5


@pytest.mark.parametrize("case", ["noh2d", "sod3d"])
def test_mixed_cullen_steps(case):
    """Four full driver iterations in each mode: alpha, accelerations and
    the time step stay within 1e-4 of the FP64 run."""
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _mixed_problem(case)
    out, times = {}, {}
    for mode in (PRECISION_FP64, PRECISION_MIXED):
        p.precision_mode = mode
        bs = BodySystem(p, len(s["x"]))
        bs.read_bodies(s)
        for _ in range(4):
            bs.step()
        out[mode] = bs.download()
        times[mode] = bs.time()
        bs.close()
    a, b = out[PRECISION_FP64], out[PRECISION_MIXED]
    assert np.array_equal(a["id"], b["id"])
    assert abs(times[PRECISION_MIXED][0] - times[PRECISION_FP64][0]) <= 1e-4 * times[PRECISION_FP64][0]
    errs = {f: normwise(b[f], a[f]) for f in ("alpha", "divv", "u", "vx")}
    A = np.stack([a[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([b[k] for k in ("ax", "ay", "az")], 1)
    errs["acc"] = float(np.abs(A - B).max() / np.abs(A).max())
    print(case, errs)
    for f, e in errs.items():
        assert e <= 1e-4, (f, e)


def test_mixed_cullen_periodic_kh2d():
    """Cullen & Dehnen in the periodic Kelvin-Helmholtz box: the mixed path
    against FP64 over four iterations (copies regenerated every step).

    The shear layers move over a uniform lattice, where the reference's
    div v = v_a . sum m_b grad W_ab is FP64 rounding noise whose sign follows
    the summation order; R_a counts those signs for the particles next to
    the interfaces, so alpha there differs at the 0.1 level between any two
    summation orders.  Density, div v, u and v stay at the FP32 level; alpha
    and the accelerations get the bound that sensitivity allows."""
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem, capacity_for
    build.build()
    s, p, m = setups.kh2d(48)
    p.sph_viscosity = VISC_CULLEN
    s = setups.shuffled(s, 44)
    out = {}
    for mode in (PRECISION_FP64, PRECISION_MIXED):
        p.precision_mode = mode
        bs = BodySystem(p, capacity_for(p, len(s["x"]), s))
        bs.read_bodies(s)
        for _ in range(4):
            bs.step()
        out[mode] = bs.download()
        bs.close()
    a, b = out[PRECISION_FP64], out[PRECISION_MIXED]
    assert np.array_equal(a["id"], b["id"])
    A = np.stack([a[k] for k in ("ax", "ay")], 1)
    B = np.stack([b[k] for k in ("ax", "ay")], 1)
    acc = float(np.abs(A - B).max() / np.abs(A).max())
    errs = {f: normwise(b[f], a[f]) for f in ("alpha", "divv", "u", "vx")}
    print("kh2d cullen", acc, errs)
    assert errs["divv"] <= 1e-5 and errs["u"] <= 1e-5 and errs["vx"] <= 1e-5
    assert errs["alpha"] <= 0.2 and acc <= 1e-3
