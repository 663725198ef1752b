"""The gravity oracle (orc_gravity_direct, the accuracy reference of the GPU
tree walk) against an independent numpy direct sum of the reference's
unsoftened pair kernel, fmm::gravitation_p2p (fmm.h:37-46):
    phi_a += -G m_b / d,   g_a += -G m_b (x_a - x_b) / d^3,
over every source but the sink itself (fmm.h:136-137)."""
import numpy as np

from flecsph_gb300 import setups


def _numpy_direct(x, m, G):
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt((d * d).sum(-1))
    np.fill_diagonal(r, np.inf)
    pot = (-G * m[None, :] / r).sum(1)
    acc = (-G * m[None, :, None] / r[..., None] ** 3 * d).sum(1)
    return acc, pot


def test_direct_sum_matches_pair_kernel(oracle_port):
    s, p, _ = setups.polytrope3d(1500, seed=11)
    p.gravitational_constant = 0.7
    o = oracle_port.Oracle("port", p, threads=4)
    o.upload(s)
    o.gravity_direct()
    out = o.download()
    k = np.argsort(out["id"])
    x = np.stack([out["x"], out["y"], out["z"]], 1)[k]
    acc, pot = _numpy_direct(x, out["m"][k], 0.7)
    got = np.stack([out["gax"], out["gay"], out["gaz"]], 1)[k]
    assert np.abs(got - acc).max() <= 1e-12 * np.abs(acc).max()
    assert np.abs(out["gpot"][k] - pot).max() <= 1e-12 * np.abs(pot).max()


def test_sink_range_leaves_other_sinks(oracle_port):
    """orc_gravity_direct(s0, s1) writes sinks s0..s1-1 only."""
    s, p, _ = setups.polytrope3d(600, seed=12)
    o = oracle_port.Oracle("port", p, threads=2)
    o.upload(s)
    o.gravity_direct(100, 200)
    part = o.download()
    o.gravity_direct()
    full = o.download()
    sel = np.zeros(len(part["gax"]), bool)
    sel[100:200] = True
    assert np.array_equal(part["gax"][sel], full["gax"][sel])
    assert np.array_equal(part["gpot"][sel], full["gpot"][sel])
    assert not np.any(part["gax"][~sel] == full["gax"][~sel])
