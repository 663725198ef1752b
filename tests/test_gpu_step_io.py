"""fsph_step_io (copies overlapped with the step) gives exactly what
fsph_upload_fields + fsph_step + fsph_download give, in every formulation
whose fields finish at different stages of the step."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import (DOUBLE_FIELDS, PRECISION_MIXED, VISC_CULLEN, make_view,
                               new_state)

pytestmark = pytest.mark.gpu


def _problem(case):
    if case == "sod3d_thermo":
        s, p, m = setups.sod3d(40, 10, 10)
    elif case == "sod3d_dudt_mixed":
        s, p, m = setups.sod3d(40, 10, 10)
        p.thermokinetic_formulation = 0
        p.precision_mode = PRECISION_MIXED
    elif case == "sedov_varh_mixed":
        s, p, m = setups.sedov3d(20, eta=1.44)
        p.sph_variable_h = 1
        p.precision_mode = PRECISION_MIXED
        p.max_neighbors = 512
    elif case == "noh2d_cullen":
        s, p, m = setups.noh2d(50)
        p.sph_viscosity = VISC_CULLEN
    else:
        s, p = setups.external_force_problem("relaxation_3d")
        p.relaxation_steps = 3
    return setups.shuffled(s, 17), p


@pytest.mark.parametrize("case", ["sod3d_thermo", "sod3d_dudt_mixed", "sedov_varh_mixed",
                                  "noh2d_cullen", "relaxation"])
def test_step_io_matches_separate_calls(case):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem
    build.build()
    s, p = _problem(case)
    n = len(s["x"])
    runs = []
    for use_io in (False, True):
        bs = BodySystem(p, n)
        bs.read_bodies(s)
        host = {k: v.copy() for k, v in s.items()}
        outs = []
        for k in range(6):
            vin = make_view(host, fields=set(DOUBLE_FIELDS) | {"id"}) if k else None
            out = new_state(n)
            vout = make_view(out)
            if use_io:
                bs.step_io(vin, vout)
            else:
                if vin is not None:
                    bs.upload_fields(vin)
                bs.step()
                bs.download_into(vout)
            outs.append(out)
            host = {f: out[f].copy() for f in out}
        runs.append(outs)
        bs.close()
    for k, (a, b) in enumerate(zip(*runs)):
        assert np.array_equal(a["id"], b["id"]), k
        assert np.array_equal(a["key"], b["key"]), k
        for f in DOUBLE_FIELDS:
            assert np.array_equal(a[f], b[f]), (k, f)
