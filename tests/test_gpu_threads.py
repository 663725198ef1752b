"""Two host threads, each with its own context on one device, stepping at
once in a fresh process: the kernels' one-time launch attributes (the
ordered walk's and the gravity walk's shared-memory sizes, the sort
scatter's) are set under a lock before either thread's first launch, so
both runs succeed and give identical results."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = textwrap.dedent("""
    import sys, threading
    import numpy as np
    sys.path.insert(0, {root!r})
    from flecsph_gb300 import setups
    from flecsph_gb300.abi import PRECISION_FP64, PRECISION_MIXED
    from flecsph_gb300.sph import BodySystem
    out = {{}}
    errors = []
    gate = threading.Barrier(4)

    def run(tag, mode, gravity):
        try:
            if gravity:
                s, p, m = setups.polytrope3d(8000, seed=11)
                p.max_neighbors = 1024
                p.adaptive_timestep = 0
                p.initial_dt = 1e-5
            else:
                s, p, m = setups.sod3d(40, 10, 10)
            p.precision_mode = mode
            bs = BodySystem(p, m["n"])
            bs.read_bodies(s)
            gate.wait()
            for _ in range(3):
                bs.step()
            out[tag] = bs.download()
            bs.close()
        except Exception as e:  # reported below
            errors.append((tag, repr(e)))

    ts = [threading.Thread(target=run, args=(f"{{k}}{{j}}", mode, grav))
          for k, (mode, grav) in enumerate([(PRECISION_FP64, False),
                                           (PRECISION_MIXED, True)])
          for j in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for k in range(2):
        a, b = out[f"{{k}}0"], out[f"{{k}}1"]
        for f in a:
            assert np.array_equal(a[f], b[f]), (k, f)
    print("ok")
""")


def test_threads_share_a_device():
    from flecsph_gb300 import build
    build.build()
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert r.stdout.strip().endswith("ok")
