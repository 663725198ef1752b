"""Key-range decomposition of one particle system over several ranks.

The reference spreads a run over MPI ranks (mpisph/bodies_system.h:152-229):
each update_iteration computes the global range (mpi_compute_range,
:231-268), Morton keys, and a distributed sort that leaves every rank a
contiguous range of (key, id) with equal particle counts (psort,
mpisph/psort.h:227-322); the tree then exchanges branches and ghost
particles so each rank's neighbour walks see everything within reach
(tree_topology.h:1142-1744), and reset_ghosts refreshes the ghosts' fields
between physics passes (bodies_system.h:273).  Global quantities (dt, the
conserved sums) are MPI reductions.

This module is that decomposition for one process per GPU over
torch.distributed (NCCL between GPUs, gloo on the host):

* ``global_range`` / ``morton_keys`` -- the reference's range and key
  formulas, on the host;
* ``partition`` -- sample sort by (key, id): every rank sends its sampled
  keys to all, the ranks agree on splitters at equal count quantiles, and
  particles move with one all-to-all;
* ``halo`` -- every rank publishes its particles' bounding box and largest
  h; a particle b goes to rank s as a ghost when its distance to s's box is
  at most max(h_b, h_max(s)) -- a superset of every pair the predicate
  d <= max(h_a, h_b) can accept, so the lists of the rank's own particles
  are complete;
* ``DistributedSystem`` -- the hydro driver loop of one rank over any
  engine with the body-system call surface (the GPU BodySystem here), with
  ghost refreshes after each neighbour pass and the timestep chosen from
  the minimum over all ranks' own particles (set_adaptive_timestep,
  default_physics.h:761-823, evaluated on the host).

Ghosts are full particle records: every elementwise update applied to them
is the one applied to their owner's copy, and each refresh replaces them
with the owner's values, so a ghost equals its owner whenever a neighbour
pass reads it.
"""
import numpy as np

from .abi import DOUBLE_FIELDS, new_state

FIELDS = DOUBLE_FIELDS + ["id"]


# --------------------------------------------------------------- transport --
class Comm:
    """torch.distributed collectives on host (CPU) tensors."""

    def __init__(self, dist=None):
        self.dist = dist
        if dist is None:
            self.rank, self.size = 0, 1
        else:
            self.rank, self.size = dist.get_rank(), dist.get_world_size()

    def _t(self, a):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a))

    def allreduce(self, values, op):
        a = np.atleast_1d(np.asarray(values, dtype=np.float64)).copy()
        if self.dist is None:
            return a
        t = self._t(a)
        ops = {"min": self.dist.ReduceOp.MIN, "max": self.dist.ReduceOp.MAX,
               "sum": self.dist.ReduceOp.SUM}
        self.dist.all_reduce(t, op=ops[op])
        return t.numpy().copy()

    def allgather(self, values):
        """Equal-length float64 vectors from every rank, stacked by rank."""
        a = np.atleast_1d(np.asarray(values, dtype=np.float64))
        if self.dist is None:
            return a[None, :].copy()
        import torch
        out = [torch.empty(len(a), dtype=torch.float64) for _ in range(self.size)]
        self.dist.all_gather(out, self._t(a))
        return np.stack([o.numpy() for o in out])

    def alltoallv(self, parts):
        """parts[s]: 1-D array for rank s (one dtype); returns the arrays
        received from every rank, concatenated in rank order."""
        if self.dist is None:
            return np.ascontiguousarray(parts[0])
        import torch
        dtype = parts[0].dtype
        counts = np.array([len(p) for p in parts], np.int64)
        rc = self._t(np.zeros(self.size, np.int64))
        self.dist.all_to_all_single(rc, self._t(counts))
        recv_counts = rc.numpy().astype(np.int64)
        send = np.concatenate(parts) if len(parts) else np.zeros(0, dtype)
        view = send.view(np.int64) if dtype.itemsize == 8 else send
        out = torch.empty(int(recv_counts.sum()), dtype=torch.int64)
        self.dist.all_to_all_single(out, self._t(view), recv_counts.tolist(),
                                    counts.tolist())
        return out.numpy().view(dtype).copy()


def exchange(comm, state, dest):
    """Move whole particles: particle i goes to rank dest[i]."""
    order = np.argsort(dest, kind="stable")
    bounds = np.searchsorted(dest[order], np.arange(comm.size + 1))
    out = {}
    for f in FIELDS:
        v = state[f][order]
        parts = [v[bounds[s]:bounds[s + 1]] for s in range(comm.size)]
        out[f] = comm.alltoallv(parts)
    return out


# ------------------------------------------------------ range, keys, order --
def global_range(comm, state, dim):
    """mpi_compute_range: [min(x - h), max(x + h)] over every rank."""
    lo = [np.min(state["xyz"[d]] - state["h"]) if len(state["h"]) else np.inf
          for d in range(dim)]
    hi = [np.max(state["xyz"[d]] + state["h"]) if len(state["h"]) else -np.inf
          for d in range(dim)]
    return comm.allreduce(lo, "min"), comm.allreduce(hi, "max")


def _spread3(v):
    v = v & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def _spread2(v):
    v = v & np.uint64(0x7FFFFFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x0000FFFF0000FFFF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF00FF00FF)
    v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F0F0F0F0F)
    v = (v | (v << np.uint64(2))) & np.uint64(0x3333333333333333)
    v = (v | (v << np.uint64(1))) & np.uint64(0x5555555555555555)
    return v


def morton_keys(state, lo, hi, dim):
    """morton_curve_u (filling_curve.h:503-525): bit 63/D*D marker, coordinate
    j truncated to 63/D bits, bit i of coordinate j at bit D*i + j."""
    bits = 63 // dim
    top = float(1 << bits)
    maxv = np.uint64((1 << bits) - 1)
    key = np.full(len(state["x"]), np.uint64(1) << np.uint64(bits * dim), np.uint64)
    spread = _spread3 if dim == 3 else _spread2
    for d in range(dim):
        q = ((state["xyz"[d]] - lo[d]) / (hi[d] - lo[d]) * top).astype(np.uint64)
        q = np.minimum(q, maxv)
        key |= spread(q) << np.uint64(d)
    return key


def _order_key(keys, ids):
    # (key, id) as one comparable record
    return np.rec.fromarrays([keys, ids.astype(np.int64)], names="k,i")


def partition(comm, keys, ids, oversample=64):
    """Destination rank of every particle: sample sort on (key, id) with
    splitters at equal quantiles of the gathered samples."""
    n = len(keys)
    if comm.size == 1:
        return np.zeros(n, np.int64)
    rec = _order_key(keys, ids)
    srt = np.sort(rec, order=("k", "i"))
    m = oversample * comm.size
    pick = np.linspace(0, n - 1, num=min(m, n)).astype(np.int64) if n else np.zeros(0, np.int64)
    samp = np.full((m, 2), -1.0)
    # keys travel as their bit patterns in float64 slots; -1 marks no sample
    samp[:len(pick), 0] = srt["k"][pick].view(np.float64)
    samp[:len(pick), 1] = srt["i"][pick].astype(np.float64)
    allv = comm.allgather(samp.ravel()).reshape(-1, 2)
    valid = allv[:, 1] >= 0
    sk = allv[valid, 0].copy().view(np.uint64)
    si = allv[valid, 1].astype(np.int64)
    srec = np.sort(_order_key(sk, si), order=("k", "i"))
    q = [srec[int(round(len(srec) * r / comm.size))] for r in range(1, comm.size)]
    dest = np.zeros(n, np.int64)
    for s, (k, i) in enumerate(q, start=1):
        beyond = (keys > k) | ((keys == k) & (ids >= i))
        dest[beyond] = s
    return dest


# --------------------------------------------------------------------- halo --
def halo_destinations(comm, state, dim):
    """For each rank s != own, the indices of particles that s needs as
    ghosts: distance to s's box <= max(h_b, h_max(s))."""
    n = len(state["x"])
    if n:
        lo = [state["xyz"[d]].min() for d in range(dim)]
        hi = [state["xyz"[d]].max() for d in range(dim)]
        hm = state["h"].max()
    else:
        lo, hi, hm = [np.inf] * dim, [-np.inf] * dim, 0.0
    info = comm.allgather(np.array(lo + hi + [hm, float(n)]))
    out = []
    for s in range(comm.size):
        if s == comm.rank or info[s, -1] == 0 or n == 0:
            out.append(np.zeros(0, np.int64))
            continue
        d2 = np.zeros(n)
        for d in range(dim):
            x = state["xyz"[d]]
            g = np.maximum(0.0, np.maximum(info[s, d] - x, x - info[s, dim + d]))
            d2 += g * g
        r = np.maximum(state["h"], info[s, 2 * dim])
        # a relative hair over the radius keeps rounding from dropping a pair
        out.append(np.nonzero(d2 <= (r * (1 + 1e-12)) ** 2)[0].astype(np.int64))
    return out


# ------------------------------------------------------------------ driver --
def _take(state, idx):
    return {f: state[f][idx] for f in FIELDS}


def _concat(a, b):
    return {f: np.concatenate([a[f], b[f]]) for f in FIELDS}


class DistributedSystem:
    """One rank of a key-range-decomposed particle system.

    `engine` has the body-system surface (read_bodies/upload, download,
    update_iteration, the physics passes and elementwise updates, set_time)
    plus ``refresh(state)``, which replaces the fields of the particles it
    holds (same order as its last download) without rebuilding its tree.
    The engine's own timestep reduction is not used: dt comes from the
    minimum over every rank's own particles."""

    def __init__(self, engine, params, comm):
        self.e = engine
        self.p = params
        self.comm = comm
        self.dim = params.dimension
        self.local = None
        self.nlocal = 0
        self.ghost_src = None   # per rank: local indices sent as ghosts
        self.ghost_ids = None
        # time (analysis::set_initial_time_iteration, analysis.h:221-249)
        self.dt = params.initial_dt
        self.totaltime = params.initial_time
        self.iteration = params.initial_iteration
        self.dt_saved = 0.0
        self.totaltime_next = 0.0
        self.t_out = [0.0, 0.0, 0.0]
        for k, step in enumerate((params.out_screen_dt, params.out_scalar_dt,
                                  params.out_h5data_dt)):
            if step > 0:
                t = step * int(self.totaltime / step)
                self.t_out[k] = max(t, self.totaltime)

    # -- data ---------------------------------------------------------------
    def read_bodies(self, local_state):
        self.local = {f: np.ascontiguousarray(local_state[f]) for f in FIELDS}
        self.nlocal = len(self.local["x"])

    def own_state(self):
        """This rank's own particles, current values."""
        st = self.e.download()
        own = np.isin(st["id"], self.own_ids)
        return {f: st[f][own] for f in FIELDS}

    # -- decomposition ------------------------------------------------------
    def update_iteration(self):
        if self.local is None:
            raise RuntimeError("read_bodies first")
        if self.e_has_state():
            self.local = self.own_state()
        lo, hi = global_range(self.comm, self.local, self.dim)
        keys = morton_keys(self.local, lo, hi, self.dim)
        dest = partition(self.comm, keys, self.local["id"])
        self.local = exchange(self.comm, self.local, dest)
        self.nlocal = len(self.local["x"])
        self.own_ids = self.local["id"].copy()
        self.ghost_src = halo_destinations(self.comm, self.local, self.dim)
        ghosts = exchange_parts(self.comm, self.local, self.ghost_src)
        self.ghost_ids = ghosts["id"].copy()
        full = _concat(self.local, ghosts)
        self.e.upload(full)
        self.e.set_time(self.dt, self.totaltime, self.iteration)
        self.e.update_iteration()
        self._uploaded = True

    def e_has_state(self):
        return getattr(self, "_uploaded", False)

    def refresh_ghosts(self):
        """reset_ghosts: every ghost takes its owner's current values."""
        st = self.e.download()
        pos = {int(i): k for k, i in enumerate(st["id"])}
        own_rows = np.array([pos[int(i)] for i in self.own_ids], np.int64)
        mine = {f: st[f][own_rows] for f in FIELDS}
        got = exchange_parts(self.comm, mine, self.ghost_src)
        rows = np.array([pos[int(i)] for i in got["id"]], np.int64)
        for f in DOUBLE_FIELDS:
            st[f][rows] = got[f]
        self.e.refresh(st)

    # -- time ---------------------------------------------------------------
    def _global_dt_min(self):
        st = self.e.download()
        own = np.isin(st["id"], self.own_ids)
        loc = st["dt"][own].min() if own.any() else 1e24
        return float(self.comm.allreduce([loc], "min")[0])

    def set_adaptive_timestep(self):
        """default_physics.h:761-823 with the minimum over every rank."""
        dtmin = self._global_dt_min()
        if dtmin < self.dt:
            self.dt = min(dtmin, self.dt / 2.0)
        if dtmin > 2.0 * self.dt:
            self.dt = self.dt * 2.0
        self.totaltime_next = self.totaltime + self.dt
        steps = (self.p.out_screen_dt, self.p.out_scalar_dt, self.p.out_h5data_dt)
        for k, step in enumerate(steps):
            if step <= 0:
                continue
            if self.totaltime == self.t_out[k]:
                if self.dt_saved > 0:
                    self.dt = self.dt_saved
                self.t_out[k] += step
            if self.totaltime + self.dt > self.t_out[k] - 0.1 * step:
                self.dt_saved = self.dt
                self.totaltime_next = (self.t_out[k] if k == 0
                                       else min(self.totaltime_next, self.t_out[k]))
        self.dt = self.totaltime_next - self.totaltime
        self.e.set_time(self.dt, self.totaltime, self.iteration)

    def advance_time(self):
        self.iteration += 1
        if self.p.adaptive_timestep:
            self.totaltime = self.totaltime_next
        else:
            self.totaltime = self.totaltime + self.dt
        self.e.set_time(self.dt, self.totaltime, self.iteration)

    # -- the driver loop ----------------------------------------------------
    def step(self):
        """One iteration of hydro/main_driver.cc:98-279 over the ranks."""
        p, e = self.p, self.e
        thermo = p.thermokinetic_formulation
        if self.iteration == p.initial_iteration:
            self.update_iteration()
            e.eos_init()
            if thermo:
                e.set_total_energy()
            e.density_pressure_soundspeed()
            e.save_velocityhalf()
            self.refresh_ghosts()
            e.acceleration()
            if p.adaptive_timestep:
                e.compute_dt()
                self.set_adaptive_timestep()
            if p.evolve_internal_energy:
                self._energy_updates(thermo)
        else:
            e.set_time(self.dt, self.totaltime, self.iteration)
            if p.evolve_internal_energy:
                (e.leapfrog_kick_e if thermo else e.leapfrog_kick_u)()
            e.leapfrog_kick_v()
            e.save_velocityhalf()
            e.leapfrog_drift()
            self.update_iteration()
            e.density_pressure_soundspeed()
            self.refresh_ghosts()
            e.acceleration()
            e.leapfrog_kick_v()
            self.refresh_ghosts()
            if p.evolve_internal_energy:
                self._energy_updates(thermo)
                (e.leapfrog_kick_e if thermo else e.leapfrog_kick_u)()
        if p.sph_variable_h:
            e.compute_smoothinglength()
        elif p.sph_update_uniform_h:
            raise NotImplementedError("sph_update_uniform_h over several ranks")
        e.check_nans()
        e.check_negativity()
        if p.adaptive_timestep:
            e.compute_dt()
            self.set_adaptive_timestep()
        self.advance_time()

    def _energy_updates(self, thermo):
        e = self.e
        for m in range(1, self.p.pressure_updates_number + 1):
            if thermo:
                e.dedt()
                e.recompute_pressure_soundspeed_thermokinetic()
            else:
                e.dudt()
                e.recompute_pressure_soundspeed()
            if m < self.p.pressure_updates_number:
                self.refresh_ghosts()


def exchange_parts(comm, state, idx_per_rank):
    """Send the particles state[idx_per_rank[s]] to rank s; returns what
    arrives from all ranks (rank order)."""
    out = {}
    for f in FIELDS:
        parts = [state[f][idx_per_rank[s]] for s in range(comm.size)]
        out[f] = comm.alltoallv(parts)
    return out


class GpuEngine:
    """The GPU BodySystem behind a DistributedSystem rank."""

    def __init__(self, params, capacity, device=0):
        from .sph import BodySystem
        self.bs = BodySystem(params, capacity, device=device)

    def upload(self, state):
        s = dict(state)
        s["key"] = np.zeros(len(s["x"]), np.uint64)
        self.bs.read_bodies(s)

    def refresh(self, state):
        from .abi import make_view
        keep = {f: np.ascontiguousarray(state[f]) for f in FIELDS}
        self._keep = keep
        self.bs.upload_fields(make_view(keep, fields=set(FIELDS)))

    def download(self):
        return self.bs.download()

    def __getattr__(self, name):
        return getattr(self.bs, name)
