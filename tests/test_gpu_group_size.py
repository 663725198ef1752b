"""The walk-group size (fsph_params.group_size: particles per warp of the
neighbour and gravity walks) is a launch-shape parameter only: the lists
(in the reference's order, FP64 mode) and every field after full driver
iterations are identical for 8, 16 and 32, and the ensemble tuner that
searches it leaves the members' results unchanged.  (On the mixed path the
lists are sets whose order follows the walk, so there the sums round
differently.)"""
import numpy as np
import pytest

import _golden
from flecsph_gb300.abi import DOUBLE_FIELDS

pytestmark = pytest.mark.gpu


def _run(name, group_size, steps=2):
    from flecsph_gb300 import build
    build.build()
    from flecsph_gb300.sph import BodySystem
    d, params, state = _golden.load(name)
    params.group_size = group_size
    bs = BodySystem(params, len(state["x"]))
    bs.read_bodies(state)
    bs.update_iteration()
    lists = bs.neighbors()
    bs.read_bodies(state)
    for _ in range(steps):
        bs.step()
    out = bs.download()
    bs.close()
    return lists, out


@pytest.mark.parametrize("name", ["sod3d_4000", "polytrope3d_varh_3000"])
def test_group_size_changes_nothing(name):
    l32, o32 = _run(name, 32)
    for g in (8, 16):
        lg, og = _run(name, g)
        assert np.array_equal(lg[0], l32[0]) and np.array_equal(lg[1], l32[1]), g
        assert np.array_equal(og["id"], o32["id"]), g
        for f in DOUBLE_FIELDS:
            assert np.array_equal(og[f], o32[f]), (g, f)


def test_ensemble_tune_shape():
    from flecsph_gb300 import build, setups
    build.build()
    from flecsph_gb300.sph import BodySystem, Ensemble
    probs = setups.ensemble2d(6, nmin=1500, nmax=6000, seed=5)
    # FP64 members: their lists come in the reference's order whatever the
    # walk's group size, so stepping alone must agree bit for bit
    for s, p, m in probs:
        p.precision_mode = 0
    ens = Ensemble()
    members = [ens.add(p, m["n"]) for s, p, m in probs]
    for mb, (s, p, m) in zip(members, probs):
        mb.read_bodies(s)
    ens.step(2)
    lanes, gsize, ms = ens.tune_shape(1)
    assert gsize in (8, 16, 32) and lanes >= 1 and ms > 0
    ens.step(2)
    ens.sync()
    # every member equals the same problem stepped alone
    for mb, (s, p, m) in zip(members, probs):
        it = mb.time()[2]
        p.group_size = gsize
        alone = BodySystem(p, m["n"])
        alone.read_bodies(s)
        for _ in range(it):
            alone.step()
        a, b = alone.download(), mb.download()
        alone.close()
        assert np.array_equal(a["id"], b["id"])
        for f in ("x", "y", "vx", "vy", "rho", "e"):
            assert np.array_equal(a[f], b[f]), f
    ens.close()
