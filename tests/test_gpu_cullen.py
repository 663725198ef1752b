"""Cullen & Dehnen adaptive viscosity on the GPU (FP64 mode) against the CPU
oracle beyond the golden fixture: a Noh implosion in 2D and a Sedov blast
with du/dt, every field within 1e-12 after several full iterations; and the
mixed path refuses visc_cullen with a message."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import DOUBLE_FIELDS, FsphError, PRECISION_MIXED, VISC_CULLEN

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


def test_mixed_refuses_cullen():
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p, m = setups.sod3d(20, 5, 5)
    p.sph_viscosity = VISC_CULLEN
    p.precision_mode = PRECISION_MIXED
    with pytest.raises(FsphError):
        BodySystem(p, len(s["x"]))
