"""The CPU oracle (plain-C restatement) against the golden vectors made by
running the reference's own code (tests/golden/make_golden.py).

Everything is bit-exact: keys, sort order, neighbour lists in the
reference's order, processing order, and every FP64 field after each driver
iteration, with the same (dt, time, iteration)."""
import numpy as np
import pytest

from flecsph_gb300.abi import DOUBLE_FIELDS

import _golden


@pytest.mark.parametrize("name", _golden.names())
def test_update_iteration_and_lists(oracle_port, name):
    d, params, state = _golden.load(name)
    o = oracle_port.Oracle("port", params)
    o.upload(state)
    o.update_iteration()
    out = o.download()
    assert np.array_equal(out["key"], d["upd_key"])
    assert np.array_equal(out["id"], d["upd_id"])
    assert np.array_equal(o.range(), d["upd_range"])
    off, idx = o.neighbors()
    assert np.array_equal(off, d["nb_offsets"])
    assert np.array_equal(idx, d["nb_indices"].astype(np.int64))
    assert np.array_equal(o.order(), d["order"].astype(np.int64))


@pytest.mark.parametrize("name", _golden.names())
def test_driver_steps_bit_exact(oracle_port, name):
    d, params, state = _golden.load(name)
    o = oracle_port.Oracle("port", params, threads=2)
    o.upload(state)
    for k in range(int(d["steps"])):
        o.step()
        st = o.download()
        dt, t, it = o.time()
        assert it == int(d[f"s{k}_iteration"])
        assert (dt, t) == tuple(d[f"s{k}_time"])
        for f in DOUBLE_FIELDS + ["id"]:
            assert np.array_equal(st[f], d[f"s{k}_{f}"]), (k, f)
