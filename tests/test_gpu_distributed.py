"""The key-range decomposition with the GPU library as each rank's engine:
two ranks as two processes sharing the one GPU (their kernels never wait on
each other; all exchange goes through gloo on the host) against the
one-rank GPU run.  Same bar as the host-side test: every field but the
order-dependent signal speed and dt to rounding, with a fixed timestep."""
import os
import socket

import numpy as np
import pytest

from flecsph_gb300.abi import DOUBLE_FIELDS

pytestmark = pytest.mark.gpu

from test_distributed import FIELDS, _problem  # noqa: E402


def _rank_main(rank, world, port, outdir, steps):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from flecsph_gb300.distributed import Comm, DistributedSystem, GpuEngine
    comm = Comm(dist)
    s, p = _problem()
    share = np.random.Generator(np.random.PCG64(5)).integers(0, world, len(s["x"]))
    local = {f: s[f][share == rank] for f in FIELDS}
    ds = DistributedSystem(GpuEngine(p, len(s["x"])), p, comm)
    ds.read_bodies(local)
    for _ in range(steps):
        ds.step()
    out = ds.own_state()
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), nghost=len(ds.ghost_ids),
             **{"s_" + f: out[f] for f in FIELDS})
    dist.destroy_process_group()


def test_two_ranks_on_one_gpu_match_one_rank(tmp_path):
    from flecsph_gb300 import build
    build.build()
    import torch.multiprocessing as mp
    from flecsph_gb300.sph import BodySystem
    steps = 3
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path), steps), nprocs=2,
                       join=True, start_method="spawn")
    ranks = [dict(np.load(os.path.join(tmp_path, f"rank{r}.npz"))) for r in range(2)]
    assert all(int(r["nghost"]) > 0 for r in ranks)
    s, p = _problem()
    bs = BodySystem(p, len(s["x"]))
    bs.read_bodies(s)
    for _ in range(steps):
        bs.step()
    ref = bs.download()
    bs.close()
    rk = np.argsort(ref["id"])
    got = {f: np.concatenate([r["s_" + f] for r in ranks]) for f in FIELDS}
    gk = np.argsort(got["id"])
    assert np.array_equal(got["id"][gk], ref["id"][rk])
    for f in DOUBLE_FIELDS:
        if f in ("vsig", "dt"):
            continue
        a, b = got[f][gk], ref[f][rk]
        scale = np.abs(b).max()
        e = float(np.abs(a - b).max() / scale) if scale else float(np.abs(a).max())
        assert e <= 1e-12, (f, e)
