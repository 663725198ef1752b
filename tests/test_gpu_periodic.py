"""Periodic boundaries on the GPU (boundary.h:45-248 via
bodies_system.h:160-169) against the CPU oracle: the copies appended at each
update_iteration bit-exact (count, order, positions, ids, keys), the lists
over them, and full driver iterations within the FP64 bar."""
import numpy as np
import pytest

from flecsph_gb300 import setups
from flecsph_gb300.abi import DOUBLE_FIELDS, FsphError, PRECISION_MIXED

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def _bs(params, n, cap=None):
    from flecsph_gb300 import build
    from flecsph_gb300.sph import BodySystem, capacity_for
    build.build()
    return BodySystem(params, cap if cap is not None else capacity_for(params, n))


def _kh(n1d=24):
    s, p, m = setups.kh3d(n1d)
    s = {k: v.copy() for k, v in s.items()}
    s["x"][:7] += 0.6137     # outside the box, off the lattice
    s["z"][7:11] -= 0.5531
    return setups.shuffled(s, 21), p


def normwise(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())


def test_copies_bit_exact_and_steps(oracle_port):
    s, p = _kh()
    n = len(s["x"])
    bs = _bs(p, n)
    bs.read_bodies(s)
    o = oracle_port.Oracle("port", p, threads=8)
    o.upload(s)
    bs.update_iteration()
    o.update_iteration()
    assert bs.count() == o.count()
    total, real = bs.count()
    assert real == n and total > n
    g, r = bs.download(), o.download()
    for f in ("x", "y", "z", "id", "key"):
        assert np.array_equal(g[f], r[f]), f
    go, gi = bs.neighbors()
    ro, ri = o.neighbors()
    assert np.array_equal(go, ro) and np.array_equal(gi, ri)
    # full iterations from the input
    bs.read_bodies(s)
    o.upload(s)
    for k in range(3):
        bs.step()
        o.step()
        assert bs.count() == o.count()
        g, r = bs.download(), o.download()
        assert np.array_equal(g["id"], r["id"])
        for f in DOUBLE_FIELDS:
            assert normwise(g[f], r[f]) <= FP64_TOL, (k, f)
        assert bs.time()[2] == o.time()[2]
    bs.close()


def test_conserved_sums_skip_copies():
    s, p = _kh(16)
    bs = _bs(p, len(s["x"]))
    bs.read_bodies(s)
    bs.update_iteration()
    assert bs.count()[0] > len(s["x"])
    c = bs.conserved()
    assert abs(c["mass"] - s["m"].sum()) <= 1e-13 * s["m"].sum()
    mom = (s["m"] * s["vx"]).sum()
    assert abs(c["momentum"][0] - mom) <= 1e-12 * np.abs(s["m"] * s["vx"]).sum()
    bs.close()


def test_capacity_too_small_is_an_error():
    s, p = _kh(12)
    n = len(s["x"])
    bs = _bs(p, n, cap=n + 10)
    bs.read_bodies(s)
    with pytest.raises(FsphError) as e:
        bs.update_iteration()
    assert "capacity" in str(e.value)
    bs.close()


def test_ids_must_be_dense():
    s, p = _kh(12)
    s["id"][0] = len(s["x"]) + 5
    bs = _bs(p, len(s["x"]))
    with pytest.raises(FsphError):
        bs.read_bodies(s)
    bs.close()


def test_mixed_periodic_2d_steps_stay_close():
    s, p, m = setups.kh2d(64)
    out = {}
    for mode in (0, PRECISION_MIXED):
        p.precision_mode = mode
        bs = _bs(p, m["n"])
        bs.read_bodies(s)
        for _ in range(4):
            bs.step()
        out[mode] = (bs.download(), bs.time(), bs.count())
        bs.close()
    (a, ta, ca), (b, tb, cb) = out[0], out[PRECISION_MIXED]
    assert ca == cb and ta[2] == tb[2]
    assert np.array_equal(a["id"], b["id"])
    for f in ("x", "y", "rho", "P", "u"):
        assert np.abs(a[f] - b[f]).max() <= 1e-6 * np.abs(a[f]).max(), f
