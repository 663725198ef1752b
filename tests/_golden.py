"""Helpers to read the golden fixtures made by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

from flecsph_gb300.abi import DOUBLE_FIELDS, Params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    params = Params.defaults(**json.loads(str(d["params_json"])))
    # room for the longest list of this fixture (the variable-h polytrope
    # has particles with several hundred neighbours)
    longest = int(np.diff(d["nb_offsets"]).max())
    want = longest + longest // 4 + 32
    if params.sph_variable_h:
        # h is recomputed every step (a kernel of width 3 makes it grow at
        # the first one): room for the lists of later iterations
        want = max(want, 8 * longest)
    params.max_neighbors = min(4096, max(params.max_neighbors, want))
    state = {f: np.ascontiguousarray(d["in_" + f]) for f in DOUBLE_FIELDS}
    state["id"] = np.ascontiguousarray(d["in_id"])
    state["key"] = np.zeros(len(state["x"]), np.uint64)
    return d, params, state


def csr_lists(off, idx):
    return [idx[off[i]:off[i + 1]] for i in range(len(off) - 1)]
