"""Key-range decomposition of one particle system over several ranks.

The reference spreads a run over MPI ranks (mpisph/bodies_system.h:152-229):
each update_iteration computes the global range (mpi_compute_range,
:231-268), Morton keys, and a distributed sort that leaves every rank a
contiguous range of (key, id) with equal particle counts (psort,
mpisph/psort.h:227-322); the tree then exchanges branches and ghost
particles so each rank's neighbour walks see everything within reach
(tree_topology.h:1142-1744), and reset_ghosts refreshes the ghosts' fields
between physics passes (bodies_system.h:273).  Global quantities (dt, the
conserved sums) are MPI reductions; the newtonian driver's gravity walks
the whole tree over ranks (bodies_system.h:282-288).

This module is that decomposition for one process per GPU over
torch.distributed.  The data plane is torch tensors on the rank's device:
with NCCL the exchanges move device memory to device memory (no host
staging); with gloo (host collectives, the CPU tests) the same code runs on
host tensors, and device tensors are staged through host memory.

* ``global_range`` / ``morton_keys`` -- the reference's range and key
  formulas as tensor operations (keys as int64 bit patterns; every key has
  its depth marker bit set, so signed order is the unsigned order);
* ``partition`` -- sample sort by (key, id): every rank gathers the others'
  sampled keys, the ranks agree on splitters at equal count quantiles, and
  particles move with one all-to-all of packed records;
* ``halo_destinations`` -- every rank publishes its particles' bounding box
  and largest h; a particle b goes to rank s as a ghost when its distance
  to s's box is at most max(h_b, h_max(s)) -- a superset of every pair the
  predicate d <= max(h_a, h_b) can accept, so the lists of the rank's own
  particles are complete;
* ``DistributedSystem`` -- the hydro / newtonian driver loop of one rank
  over any engine with the body-system call surface (the GPU BodySystem
  behind ``GpuEngine``), with ghost refreshes after each neighbour pass, the
  timestep from the minimum over all ranks' own particles
  (set_adaptive_timestep, default_physics.h:761-823), and gravity as a
  locally essential tree: each rank's own particles in a gravity context,
  which walks its tree for them, exports far cells (multipoles) and the
  particles of near cells for every other rank's box, and adds what the
  other ranks export for its box (fsph_gravity_export / _import).

Ghosts are full particle records: every elementwise update applied to them
is the one applied to their owner's copy, and each refresh replaces them
with the owner's values, so a ghost equals its owner whenever a neighbour
pass reads it.
"""
import numpy as np

from .abi import DOUBLE_FIELDS

FIELDS = DOUBLE_FIELDS + ["id"]
NFD = len(DOUBLE_FIELDS)


def _torch():
    import torch
    return torch


# --------------------------------------------------------------- transport --
class Comm:
    """torch.distributed collectives on tensors of one device.

    `device` is where the rank's tensors live.  Under NCCL every collective
    takes them as they are; under gloo (host collectives) device tensors are
    staged through host memory."""

    def __init__(self, dist=None, device="cpu"):
        torch = _torch()
        self.dist = dist
        self.device = torch.device(device)
        if dist is None:
            self.rank, self.size = 0, 1
            self.staged = False
        else:
            self.rank, self.size = dist.get_rank(), dist.get_world_size()
            self.staged = (dist.get_backend() != "nccl" and self.device.type != "cpu")

    def _out(self, t):
        return t.cpu() if self.staged else t

    def _in(self, t):
        return t.to(self.device) if self.staged else t

    def allreduce(self, values, op):
        """Elementwise min / max / sum over ranks of a float64 vector."""
        torch = _torch()
        if not torch.is_tensor(values):
            values = np.atleast_1d(np.asarray(values, dtype=np.float64))
        t = torch.as_tensor(values, dtype=torch.float64,
                            device=self.device).reshape(-1).clone()
        if self.dist is None:
            return t
        ops = {"min": self.dist.ReduceOp.MIN, "max": self.dist.ReduceOp.MAX,
               "sum": self.dist.ReduceOp.SUM}
        s = self._out(t)
        self.dist.all_reduce(s, op=ops[op])
        return self._in(s)

    def allgather(self, t):
        """Equal-shape tensors from every rank, stacked by rank."""
        torch = _torch()
        if self.dist is None:
            return t.unsqueeze(0).clone()
        s = self._out(t.contiguous())
        out = [torch.empty_like(s) for _ in range(self.size)]
        self.dist.all_gather(out, s)
        return self._in(torch.stack(out))

    def alltoallv(self, send, counts):
        """send: [n, ...] rows grouped by destination rank, counts[s] rows for
        rank s; returns the rows every rank sent here, in rank order."""
        torch = _torch()
        if self.dist is None:
            return send.clone()
        counts = [int(c) for c in counts]
        cs = self._out(torch.tensor(counts, dtype=torch.int64, device=self.device))
        rcs = torch.empty_like(cs)
        self.dist.all_to_all_single(rcs, cs)
        recv_counts = [int(c) for c in rcs.tolist()]
        s = self._out(send.contiguous())
        out = torch.empty((sum(recv_counts),) + tuple(send.shape[1:]), dtype=send.dtype,
                          device=s.device)
        self.dist.all_to_all_single(out, s, recv_counts, counts)
        return self._in(out)


# --------------------------------------------------------- packed records --
def pack(batch):
    """[n, NF + 1] float64 rows: the FP64 fields and the id's bits."""
    torch = _torch()
    cols = [batch[f] for f in DOUBLE_FIELDS] + [batch["id"].view(torch.float64)]
    return torch.stack(cols, 1)


def unpack(rows):
    torch = _torch()
    out = {f: rows[:, k].contiguous() for k, f in enumerate(DOUBLE_FIELDS)}
    out["id"] = rows[:, NFD].contiguous().view(torch.int64)
    return out


def take(batch, idx):
    return {f: batch[f][idx].contiguous() for f in FIELDS}


def concat(a, b):
    torch = _torch()
    return {f: torch.cat([a[f], b[f]]) for f in FIELDS}


def to_tensors(state, device):
    """A numpy particle state as contiguous tensors on `device`."""
    torch = _torch()
    out = {}
    for f in FIELDS:
        a = np.ascontiguousarray(state[f], np.int64 if f == "id" else np.float64)
        out[f] = torch.from_numpy(a.copy()).to(device)
    return out


def to_numpy(batch):
    return {f: batch[f].detach().cpu().numpy() for f in batch}


def exchange(comm, batch, dest):
    """Move whole particles: particle i goes to rank dest[i]."""
    torch = _torch()
    order = torch.argsort(dest, stable=True)
    counts = torch.bincount(dest, minlength=comm.size).tolist()
    return unpack(comm.alltoallv(pack(batch)[order], counts))


def exchange_parts(comm, batch, idx_per_rank):
    """Send the particles batch[idx_per_rank[s]] to rank s; returns what
    arrives from all ranks (rank order)."""
    torch = _torch()
    rows = pack(batch)
    idx = torch.cat(idx_per_rank) if idx_per_rank else torch.zeros(0, dtype=torch.int64)
    return unpack(comm.alltoallv(rows[idx.to(rows.device)], [len(i) for i in idx_per_rank]))


# ------------------------------------------------------ range, keys, order --
def global_range(comm, batch, dim):
    """mpi_compute_range: [min(x - h), max(x + h)] over every rank."""
    torch = _torch()
    h = batch["h"]
    if h.numel():
        lo = torch.stack([torch.min(batch["xyz"[d]] - h) for d in range(dim)])
        hi = torch.stack([torch.max(batch["xyz"[d]] + h) for d in range(dim)])
    else:
        lo = torch.full((dim,), float("inf"), dtype=torch.float64, device=h.device)
        hi = torch.full((dim,), float("-inf"), dtype=torch.float64, device=h.device)
    return comm.allreduce(lo, "min"), comm.allreduce(hi, "max")


def _spread3(v):
    v = v & 0x1FFFFF
    v = (v | (v << 32)) & 0x1F00000000FFFF
    v = (v | (v << 16)) & 0x1F0000FF0000FF
    v = (v | (v << 8)) & 0x100F00F00F00F00F
    v = (v | (v << 4)) & 0x10C30C30C30C30C3
    v = (v | (v << 2)) & 0x1249249249249249
    return v


def _spread2(v):
    v = v & 0x7FFFFFFF
    v = (v | (v << 16)) & 0x0000FFFF0000FFFF
    v = (v | (v << 8)) & 0x00FF00FF00FF00FF
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0F
    v = (v | (v << 2)) & 0x3333333333333333
    v = (v | (v << 1)) & 0x5555555555555555
    return v


def morton_keys(batch, lo, hi, dim):
    """morton_curve_u (filling_curve.h:503-525) as int64 bit patterns: the
    depth marker at bit 63 (3D) or 62 (2D), coordinate j truncated to 63/D
    bits, bit i of coordinate j at bit D*i + j.  The same FP64 operations,
    in the same order, as the reference."""
    torch = _torch()
    bits = 63 // dim
    top = float(1 << bits)
    maxv = (1 << bits) - 1
    n = batch["x"].shape[0]
    marker = -(1 << 63) if bits * dim == 63 else (1 << (bits * dim))
    key = torch.full((n,), marker, dtype=torch.int64, device=batch["x"].device)
    spread = _spread3 if dim == 3 else _spread2
    for d in range(dim):
        q = ((batch["xyz"[d]] - lo[d]) / (hi[d] - lo[d]) * top).to(torch.int64)
        q = torch.clamp(q, max=maxv)
        key = key | (spread(q) << d)
    return key


def _lex_order(keys, ids):
    """Permutation sorting by (key, id)."""
    torch = _torch()
    o1 = torch.argsort(ids, stable=True)
    o2 = torch.argsort(keys[o1], stable=True)
    return o1[o2]


def partition(comm, keys, ids, oversample=64):
    """Destination rank of every particle: sample sort on (key, id) with
    splitters at equal quantiles of the gathered samples."""
    torch = _torch()
    n = keys.shape[0]
    dev = keys.device
    if comm.size == 1:
        return torch.zeros(n, dtype=torch.int64, device=dev)
    order = _lex_order(keys, ids)
    m = oversample * comm.size
    samp = torch.zeros((m, 3), dtype=torch.int64, device=dev)
    if n:
        pick = torch.linspace(0, n - 1, steps=min(m, n), device=dev,
                              dtype=torch.float64).to(torch.int64)
        sel = order[pick]
        samp[:len(pick), 0] = keys[sel]
        samp[:len(pick), 1] = ids[sel]
        samp[:len(pick), 2] = 1
    allv = comm.allgather(samp).reshape(-1, 3)
    allv = allv[allv[:, 2] == 1]
    so = _lex_order(allv[:, 0], allv[:, 1])
    sk, si = allv[so, 0], allv[so, 1]
    dest = torch.zeros(n, dtype=torch.int64, device=dev)
    for r in range(1, comm.size):
        q = int(round(len(sk) * r / comm.size))
        k, i = sk[q], si[q]
        dest += ((keys > k) | ((keys == k) & (ids >= i))).to(torch.int64)
    return dest


# --------------------------------------------------------------------- halo --
def halo_destinations(comm, batch, dim):
    """For each rank s, the indices of particles that s needs as ghosts
    (none for this rank itself): distance to s's box <= max(h_b, h_max(s))."""
    torch = _torch()
    x = [batch["xyz"[d]] for d in range(dim)]
    h = batch["h"]
    n = h.shape[0]
    dev = h.device
    if n:
        info = torch.cat([torch.stack([v.min() for v in x]), torch.stack([v.max() for v in x]),
                          h.max().reshape(1),
                          torch.tensor([float(n)], dtype=torch.float64, device=dev)])
    else:
        info = torch.tensor([np.inf] * dim + [-np.inf] * dim + [0.0, 0.0],
                            dtype=torch.float64, device=dev)
    info = comm.allgather(info)
    out = []
    for s in range(comm.size):
        if s == comm.rank or float(info[s, -1]) == 0 or n == 0:
            out.append(torch.zeros(0, dtype=torch.int64, device=dev))
            continue
        d2 = torch.zeros(n, dtype=torch.float64, device=dev)
        for d in range(dim):
            g = torch.clamp(torch.maximum(info[s, d] - x[d], x[d] - info[s, dim + d]), min=0.0)
            d2 = d2 + g * g
        r = torch.clamp(h, min=float(info[s, 2 * dim]))
        # a relative hair over the radius keeps rounding from dropping a pair
        out.append(torch.nonzero(d2 <= (r * (1 + 1e-12)) ** 2).reshape(-1))
    return out


def _rows_of(ids_held, ids_wanted):
    """Rows of ids_held holding each of ids_wanted (every one present)."""
    torch = _torch()
    order = torch.argsort(ids_held)
    pos = torch.searchsorted(ids_held[order], ids_wanted)
    return order[pos]


# ------------------------------------------------------------------ driver --
class DistributedSystem:
    """One rank of a key-range-decomposed particle system.

    `engine` has the body-system surface on tensors of the rank's device:
    upload(batch), download() -> batch, refresh(batch) (the fields of the
    particles it holds, in the order of its last download, without
    rebuilding its tree), set_time and the physics passes.  The engine's own
    timestep reduction is not used: dt comes from the minimum over every
    rank's own particles.  With enable_fmm, `gravity` is a second engine
    (own particles only) with upload/update_iteration/gravitation/
    gravity_export/gravity_import/download."""

    def __init__(self, engine, params, comm, gravity=None):
        self.e = engine
        self.p = params
        self.comm = comm
        self.g = gravity
        if params.enable_fmm and gravity is None:
            raise ValueError("enable_fmm needs a gravity engine")
        if params.periodic_boundary_x or params.periodic_boundary_y or \
           params.periodic_boundary_z:
            raise ValueError("periodic boundaries over several ranks are not supported")
        self.dim = params.dimension
        self.dev = comm.device
        self.local = None
        self.nlocal = 0
        self.ghost_src = None   # per rank: local indices sent as ghosts
        self.ghost_ids = None
        self.own_ids = None
        self.cells_received = 0
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
        self._uploaded = False

    # -- data ---------------------------------------------------------------
    def read_bodies(self, local_state):
        """This rank's initial particles: numpy arrays or tensors."""
        torch = _torch()
        if torch.is_tensor(local_state["x"]):
            self.local = {f: local_state[f].to(self.dev).contiguous() for f in FIELDS}
        else:
            self.local = to_tensors(local_state, self.dev)
        self.nlocal = int(self.local["x"].shape[0])

    def own_batch(self):
        """This rank's own particles, current values (tensors)."""
        st = self.e.download()
        return take(st, _rows_of(st["id"], self.own_ids))

    def own_state(self):
        """This rank's own particles as numpy arrays."""
        return to_numpy(self.own_batch())

    # -- decomposition ------------------------------------------------------
    def update_iteration(self):
        if self.local is None:
            raise RuntimeError("read_bodies first")
        if self._uploaded:
            self.local = self.own_batch()
        lo, hi = global_range(self.comm, self.local, self.dim)
        keys = morton_keys(self.local, lo, hi, self.dim)
        dest = partition(self.comm, keys, self.local["id"])
        self.local = exchange(self.comm, self.local, dest)
        self.nlocal = int(self.local["x"].shape[0])
        self.own_ids = self.local["id"].clone()
        self.ghost_src = halo_destinations(self.comm, self.local, self.dim)
        ghosts = exchange_parts(self.comm, self.local, self.ghost_src)
        self.ghost_ids = ghosts["id"].clone()
        self.e.upload(concat(self.local, ghosts))
        self.e.set_time(self.dt, self.totaltime, self.iteration)
        self.e.update_iteration()
        self._uploaded = True

    def refresh_ghosts(self):
        """reset_ghosts: every ghost takes its owner's current values."""
        st = self.e.download()
        mine = take(st, _rows_of(st["id"], self.own_ids))
        got = exchange_parts(self.comm, mine, self.ghost_src)
        if got["id"].numel():
            rows = _rows_of(st["id"], got["id"])
            for f in DOUBLE_FIELDS:
                st[f][rows] = got[f]
        self.e.refresh(st)

    # -- gravity over ranks -------------------------------------------------
    def gravitation(self):
        """gravitation_fmm over the ranks: the own particles' tree walk in
        the gravity engine, the cells the other ranks export for this rank's
        box, and the result into the engine's own particles."""
        torch = _torch()
        g = self.g
        own = self.own_batch()
        for f in ("gax", "gay", "gaz", "gpot"):
            own[f] = torch.zeros_like(own[f])
        g.upload(own)
        g.set_time(self.dt, self.totaltime, self.iteration)
        g.update_iteration()
        g.gravitation()
        # every rank's box of own particles
        x = [own["xyz"[d]] for d in range(self.dim)]
        n = own["x"].shape[0]
        box = torch.cat([torch.stack([v.min() for v in x]), torch.stack([v.max() for v in x]),
                         torch.tensor([float(n)], dtype=torch.float64, device=self.dev)])
        boxes = self.comm.allgather(box)
        parts = []
        for s in range(self.comm.size):
            if s == self.comm.rank or float(boxes[s, -1]) == 0:
                parts.append(torch.zeros((0, 10), dtype=torch.float64, device=self.dev))
                continue
            lo = boxes[s, :self.dim].cpu().numpy()
            hi = boxes[s, self.dim:2 * self.dim].cpu().numpy()
            parts.append(g.gravity_export(lo, hi, self.p.fmm_macangle).to(self.dev))
        cells = self.comm.alltoallv(torch.cat(parts), [len(c) for c in parts])
        if cells.shape[0]:
            g.gravity_import(cells)
        res = g.download()
        st = self.e.download()
        rows = _rows_of(st["id"], res["id"])
        for f in ("gax", "gay", "gaz", "gpot"):
            st[f][rows] = res[f]
        self.e.refresh(st)
        self.cells_received = int(cells.shape[0])

    # -- time ---------------------------------------------------------------
    def _global_dt_min(self):
        st = self.e.download()
        own = st["dt"][_rows_of(st["id"], self.own_ids)]
        loc = float(own.min()) if own.numel() else 1e24
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
        """One iteration of hydro/main_driver.cc:98-279 (newtonian/
        main_driver.cc:103-298 with enable_fmm) over the ranks."""
        p, e = self.p, self.e
        thermo = p.thermokinetic_formulation
        grav = p.enable_fmm
        if self.iteration == p.initial_iteration:
            self.update_iteration()
            e.eos_init()
            if thermo:
                e.set_total_energy()
            e.density_pressure_soundspeed()
            e.save_velocityhalf()
            self.refresh_ghosts()
            e.acceleration()
            if grav:
                self.gravitation()
                if thermo:
                    e.set_total_energy()
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
            if grav:
                self.gravitation()
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


class GpuEngine:
    """The GPU BodySystem behind a DistributedSystem rank: particles move
    in and out as device tensors (fsph_upload_device, fsph_download_device,
    fsph_upload_fields_device), never through host memory."""

    def __init__(self, params, capacity, device=0):
        import torch
        from .sph import BodySystem
        self.bs = BodySystem(params, capacity, device=device)
        self.device = torch.device("cuda", device)

    def upload(self, batch):
        self.bs.read_bodies_device(batch)

    def refresh(self, batch):
        self.bs.upload_fields_device({f: batch[f] for f in FIELDS})

    def download(self):
        return self.bs.download_device(fields=DOUBLE_FIELDS + ["id"], device=self.device)

    def gravity_export(self, box_lo, box_hi, theta):
        return self.bs.gravity_export(box_lo, box_hi, theta, device=self.device)

    def __getattr__(self, name):
        return getattr(self.bs, name)
