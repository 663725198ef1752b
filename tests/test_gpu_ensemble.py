"""Ensembles: many independent problems stepped together as CUDA graphs
must give, member by member, exactly what stepping each problem on its own
gives."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import DOUBLE_FIELDS, FsphError

pytestmark = pytest.mark.gpu


def _lib():
    from flecsph_gb300 import build
    build.build()
    from flecsph_gb300 import sph
    return sph


def _problems(k=10, seed=5):
    return setups.ensemble2d(k, nmin=1500, nmax=20000, seed=seed)


def _alone(sph, s, p, steps):
    bs = sph.BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    for _ in range(steps):
        bs.step()
    out = bs.download(), bs.time()
    bs.close()
    return out


def _assert_same(a, b):
    (sa, ta), (sb, tb) = a, b
    assert ta == tb
    assert np.array_equal(sa["id"], sb["id"])
    for f in DOUBLE_FIELDS:
        assert np.array_equal(sa[f], sb[f]), f


def test_graph_steps_match_single_problems():
    sph = _lib()
    probs = _problems()
    ens = sph.Ensemble()
    members = [ens.add(p, len(s["x"])) for s, p, m in probs]
    for mb, (s, p, m) in zip(members, probs):
        mb.read_bodies(s)
    ens.set_lanes(3)
    steps = 7          # 2 eager, then graphs from both parities
    ens.step(3)
    ens.step(steps - 3)
    ens.sync()
    for mb, (s, p, m) in zip(members, probs):
        _assert_same((mb.download(), mb.time()), _alone(sph, s, p, steps))
    assert all(mb.time()[2] == steps for mb in members)
    ens.close()


def test_member_reupload_recaptures():
    sph = _lib()
    probs = _problems(6, seed=9)
    ens = sph.Ensemble()
    members = [ens.add(p, len(s["x"])) for s, p, m in probs]
    for mb, (s, p, m) in zip(members, probs):
        mb.read_bodies(s)
    ens.step(5)
    # restart member 2 from its input: every member steps eagerly until it is
    # level again, then the graphs are captured anew
    s2, p2, _ = probs[2]
    members[2].read_bodies(s2)
    ens.step(4)
    ens.sync()
    _assert_same((members[2].download(), members[2].time()), _alone(sph, s2, p2, 4))
    s0, p0, _ = probs[0]
    _assert_same((members[0].download(), members[0].time()), _alone(sph, s0, p0, 9))
    ens.close()


def test_tune_and_member_error_reported():
    sph = _lib()
    probs = _problems(8, seed=3)
    ens = sph.Ensemble()
    members = [ens.add(p, len(s["x"])) for s, p, m in probs]
    for mb, (s, p, m) in zip(members, probs):
        mb.read_bodies(s)
    ens.step(2)
    lanes, ms = ens.tune(2)
    assert lanes in (1, 2, 4, 8) and ms > 0
    ens.sync()
    ens.close()
    # a member whose lists cannot hold its neighbours reports at sync
    ens = sph.Ensemble()
    for k, (s, p, m) in enumerate(probs[:3]):
        if k == 1:
            p.max_neighbors = 8
        mb = ens.add(p, len(s["x"]))
        mb.read_bodies(s)
    with pytest.raises(FsphError) as e:
        ens.step(3)
        ens.sync()
    assert "LIST_OVERFLOW" in str(e.value)
    ens.close()


def test_mixed_physics_members():
    """Members with Cullen & Dehnen viscosity, external forces, relaxation
    iterations (stepped eagerly: their passes depend on the iteration
    number) and the other equations of state, in both precisions, next to
    plain members: each equals its problem stepped alone."""
    sph = _lib()
    from flecsph_gb300.abi import EOS_PPT, PRECISION_MIXED, VISC_CULLEN
    probs = []
    s, p, m = setups.noh2d(40)
    p.sph_viscosity = VISC_CULLEN
    probs.append((s, p))
    s, p, m = setups.noh2d(40)
    p.sph_viscosity = VISC_CULLEN
    p.precision_mode = PRECISION_MIXED
    probs.append((s, p))
    s, p = setups.external_force_problem("gravity_walls_2d")
    probs.append((s, p))
    s, p = setups.external_force_problem("relaxation_dudt_2d")
    p.relaxation_steps = 4
    probs.append((s, p))
    s, p = setups.external_force_problem("airfoil_2d")
    p.precision_mode = PRECISION_MIXED
    probs.append((s, p))
    s, p, m = setups.sod2d(100, 10)
    p.eos_type = EOS_PPT
    p.poly_gamma2, p.ppt_density_thr = 2.5, 0.5
    probs.append((s, p))
    probs = [(setups.shuffled(s, 30 + k), p) for k, (s, p) in enumerate(probs)]
    ens = sph.Ensemble()
    members = [ens.add(p, len(s["x"])) for s, p in probs]
    for mb, (s, p) in zip(members, probs):
        mb.read_bodies(s)
    ens.set_lanes(2)
    steps = 8
    ens.step(steps)
    ens.sync()
    for mb, (s, p) in zip(members, probs):
        _assert_same((mb.download(), mb.time()), _alone(sph, s, p, steps))
    ens.close()
