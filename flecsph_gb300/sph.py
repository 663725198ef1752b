"""Python host mirror of FleCSPH's body_system over libfsph_gb300.so.

``BodySystem`` exposes the calls the reference drivers make on
``body_system<double, D>`` (mpisph/bodies_system.h) and the physics modules
they pass to it, each forwarding to one C-ABI entry point of
include/fsph.h.  The reference's template-callback style
(``bs.apply_in_smoothinglength(physics::compute_acceleration)``) becomes an
explicit method per physics module, because the GPU library fuses the
traversal with the physics.

There is no CPU fallback: if the shared library or a CUDA device is missing
every call raises.
"""
import ctypes as C
import os

import numpy as np

from .abi import (Conserved, FsphError, Params, SoAView, TIMER_COUNT, TIMER_NAMES,
                  make_view, new_state)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfsph_gb300.so")

_lib = None

_STEP_FUNCS = [
    "update_iteration", "reset_ghosts", "density_pressure_soundspeed",
    "acceleration", "dudt", "dedt", "eos_init", "set_total_energy",
    "save_velocityhalf", "leapfrog_kick_v", "leapfrog_kick_u", "leapfrog_kick_e",
    "leapfrog_drift", "recompute_pressure_soundspeed",
    "recompute_pressure_soundspeed_thermokinetic", "compute_dt", "check_nans",
    "check_negativity", "set_adaptive_timestep", "compute_smoothinglength",
    "compute_average_smoothinglength", "gravitation", "advance_time", "step", "sync",
    "timers_reset", "compute_alpha", "initialize_alpha", "add_drag_acceleration",
    "add_short_range_repulsion", "add_drag_dedt", "add_drag_dudt",
]


def library():
    """Load libfsph_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run flecsph_gb300.build.build() first")
    lib = C.CDLL(LIB_PATH)
    lib.fsph_create.restype = C.c_void_p
    lib.fsph_create.argtypes = [C.POINTER(Params), C.c_int32, C.c_int64,
                                C.POINTER(C.c_int)]
    lib.fsph_destroy.argtypes = [C.c_void_p]
    lib.fsph_destroy.restype = None
    lib.fsph_params_default.argtypes = [C.POINTER(Params)]
    lib.fsph_params_set_external_force.argtypes = [C.POINTER(Params), C.c_char_p]
    lib.fsph_params_default.restype = None
    lib.fsph_abi_version.restype = C.c_int32
    lib.fsph_status_string.restype = C.c_char_p
    lib.fsph_status_string.argtypes = [C.c_int32]
    lib.fsph_last_error.restype = C.c_char_p
    lib.fsph_last_error.argtypes = [C.c_void_p]
    for f in _STEP_FUNCS:
        fn = getattr(lib, "fsph_" + f)
        fn.argtypes = [C.c_void_p]
        fn.restype = C.c_int
    lib.fsph_upload.argtypes = [C.c_void_p, C.POINTER(SoAView)]
    lib.fsph_download.argtypes = [C.c_void_p, C.POINTER(SoAView)]
    lib.fsph_get_time.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.fsph_set_time.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int64]
    lib.fsph_get_range.argtypes = [C.c_void_p, C.c_void_p]
    lib.fsph_get_neighbors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    lib.fsph_conserved_sums.argtypes = [C.c_void_p, C.POINTER(Conserved)]
    lib.fsph_timers.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    lib.fsph_launch_count.argtypes = [C.c_void_p]
    lib.fsph_launch_count.restype = C.c_int64
    lib.fsph_ensemble_create.restype = C.c_void_p
    lib.fsph_ensemble_create.argtypes = [C.c_int32, C.POINTER(C.c_int)]
    lib.fsph_ensemble_add.restype = C.c_void_p
    lib.fsph_ensemble_add.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int64,
                                      C.POINTER(C.c_int)]
    lib.fsph_ensemble_step.argtypes = [C.c_void_p, C.c_int32]
    lib.fsph_ensemble_sync.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    lib.fsph_ensemble_set_lanes.argtypes = [C.c_void_p, C.c_int32]
    lib.fsph_ensemble_tune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_double)]
    lib.fsph_ensemble_set_group_size.argtypes = [C.c_void_p, C.c_int32]
    lib.fsph_ensemble_tune_shape.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    lib.fsph_ensemble_last_error.restype = C.c_char_p
    lib.fsph_ensemble_last_error.argtypes = [C.c_void_p]
    lib.fsph_ensemble_destroy.argtypes = [C.c_void_p]
    lib.fsph_ensemble_destroy.restype = None
    lib.fsph_ensemble_size.argtypes = [C.c_void_p]
    lib.fsph_ensemble_member.restype = C.c_void_p
    lib.fsph_ensemble_member.argtypes = [C.c_void_p, C.c_int32]
    lib.fsph_particle_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]
    lib.fsph_upload_fields.argtypes = [C.c_void_p, C.POINTER(SoAView)]
    lib.fsph_step_io.argtypes = [C.c_void_p, C.POINTER(SoAView), C.POINTER(SoAView)]
    lib.fsph_host_register.argtypes = [C.c_void_p, C.c_int64]
    lib.fsph_host_unregister.argtypes = [C.c_void_p]
    lib.fsph_mark.argtypes = [C.c_void_p, C.c_int32]
    lib.fsph_mark_elapsed.argtypes = [C.c_void_p, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_double)]
    lib.fsph_measure_peak.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_double)]
    for f in ("fsph_upload_device", "fsph_download_device", "fsph_upload_fields_device"):
        getattr(lib, f).argtypes = [C.c_void_p, C.POINTER(SoAView)]
    lib.fsph_gravity_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                        C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    lib.fsph_gravity_import.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    _lib = lib
    return lib


class BodySystem:
    """One particle system on one GPU (mirror of body_system<double, D>)."""

    def __init__(self, params, capacity, device=0, _member_of=None):
        lib = library()
        self.params = params
        st = C.c_int(0)
        if _member_of is None:
            self.ctx = lib.fsph_create(C.byref(params), device, int(capacity),
                                       C.byref(st))
        else:
            self.ctx = lib.fsph_ensemble_add(_member_of, C.byref(params),
                                             int(capacity), C.byref(st))
        if not self.ctx:
            raise FsphError(st.value, "fsph_create")
        self.lib = lib
        self.capacity = capacity
        self._owned = _member_of is None

    def close(self):
        if getattr(self, "ctx", None):
            if self._owned:
                self.lib.fsph_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, where):
        if st:
            detail = self.lib.fsph_last_error(self.ctx).decode()
            raise FsphError(st, where, detail)

    def __getattr__(self, name):
        if name in _STEP_FUNCS:
            fn = getattr(self.lib, "fsph_" + name)

            def call():
                self._check(fn(self.ctx), name)
            call.__name__ = name
            return call
        raise AttributeError(name)

    # -- data movement ---------------------------------------------------
    @property
    def n(self):
        """Particles held, periodic copies included (what download returns)."""
        return self.count()[0]

    def count(self):
        """(total, real): total includes the periodic copies."""
        t, r = C.c_int64(), C.c_int64()
        self._check(self.lib.fsph_particle_count(self.ctx, C.byref(t), C.byref(r)),
                    "particle_count")
        return t.value, r.value

    def read_bodies(self, state):
        """Upload a particle state (dict of numpy arrays, FP64 SoA)."""
        keep = {k: np.ascontiguousarray(v) for k, v in state.items()}
        self._keep = keep
        v = make_view(keep)
        self._check(self.lib.fsph_upload(self.ctx, C.byref(v)), "upload")

    upload = read_bodies

    def download(self, fields=None):
        out = new_state(self.n)
        v = make_view(out, fields=fields)
        self._check(self.lib.fsph_download(self.ctx, C.byref(v)), "download")
        if fields is not None:
            out = {k: out[k] for k in fields}
        return out

    def upload_fields(self, view):
        """Copy the non-NULL fields of an fsph_soa_view (host pointers) into
        the current particle order without touching time or iteration."""
        self._check(self.lib.fsph_upload_fields(self.ctx, C.byref(view)), "upload_fields")

    def download_into(self, view):
        self._check(self.lib.fsph_download(self.ctx, C.byref(view)), "download")

    # -- device-resident data (torch tensors on this context's device) ------
    @staticmethod
    def _tensors_ready(batch):
        """The library's stream does not wait for torch's: finish the work
        that wrote these tensors before the library reads them."""
        import torch
        for t in batch.values() if isinstance(batch, dict) else [batch]:
            if torch.is_tensor(t) and t.is_cuda:
                torch.cuda.current_stream(t.device).synchronize()
                return

    def read_bodies_device(self, batch):
        """fsph_upload_device from a dict of device tensors (float64 fields,
        int64 id)."""
        from .abi import make_view_tensors
        self._tensors_ready(batch)
        self._check(self.lib.fsph_upload_device(self.ctx, C.byref(make_view_tensors(batch))),
                    "upload_device")

    def download_device(self, fields=None, device=None):
        """Current state as a dict of tensors on `device` (fsph_download_device)."""
        import torch
        from .abi import DOUBLE_FIELDS, make_view_tensors
        n = self.count()[0]
        keep = fields or (DOUBLE_FIELDS + ["id"])
        out = {f: torch.empty(n, dtype=torch.int64 if f in ("id", "key") else torch.float64,
                              device=device) for f in keep}
        self._check(self.lib.fsph_download_device(self.ctx, C.byref(make_view_tensors(out, n))),
                    "download_device")
        return out

    def upload_fields_device(self, batch):
        """fsph_upload_fields_device, then a sync so `batch` may be freed."""
        from .abi import make_view_tensors
        n = self.count()[0]
        self._tensors_ready(batch)
        self._check(self.lib.fsph_upload_fields_device(
            self.ctx, C.byref(make_view_tensors(batch, n))), "upload_fields_device")
        self.sync()

    def gravity_export(self, box_lo, box_hi, theta, device=None):
        """Cell records (tensor [k, 10] float64) of this context's tree for a
        remote box (fsph_gravity_export)."""
        import torch
        lo = np.ascontiguousarray(box_lo, np.float64)
        hi = np.ascontiguousarray(box_hi, np.float64)
        cnt = C.c_int64(0)
        self._check(self.lib.fsph_gravity_export(self.ctx, lo.ctypes.data, hi.ctypes.data,
                                                 float(theta), None, 0, C.byref(cnt)),
                    "gravity_export")
        out = torch.empty((cnt.value, 10), dtype=torch.float64, device=device)
        if cnt.value:
            self._check(self.lib.fsph_gravity_export(
                self.ctx, lo.ctypes.data, hi.ctypes.data, float(theta), out.data_ptr(),
                cnt.value, C.byref(cnt)), "gravity_export")
        return out

    def gravity_import(self, cells):
        """Add the field of cell records (tensor [k, 10] float64, host or
        device) to every particle held (fsph_gravity_import)."""
        cells = cells.contiguous()
        self._tensors_ready(cells)
        self._check(self.lib.fsph_gravity_import(self.ctx, cells.data_ptr(),
                                                 int(cells.shape[0])), "gravity_import")
        self.sync()

    def step_io(self, vin, vout):
        """One iteration with its host copies (fsph_step_io): the non-NULL
        fields of vin go in, those of vout come back; copies overlap the
        step in regular iterations."""
        self._check(self.lib.fsph_step_io(self.ctx, C.byref(vin) if vin is not None else None,
                                          C.byref(vout)), "step_io")

    def mark(self, slot):
        self._check(self.lib.fsph_mark(self.ctx, slot), "mark")

    def elapsed_ms(self, a, b):
        ms = C.c_double()
        self._check(self.lib.fsph_mark_elapsed(self.ctx, a, b, C.byref(ms)), "mark_elapsed")
        return ms.value

    def time(self):
        dt, t, it = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.lib.fsph_get_time(self.ctx, C.byref(dt), C.byref(t), C.byref(it)),
                    "get_time")
        return dt.value, t.value, it.value

    def set_time(self, dt, t, it):
        self._check(self.lib.fsph_set_time(self.ctx, dt, t, it), "set_time")

    def range(self):
        r = np.zeros(2 * self.params.dimension)
        self._check(self.lib.fsph_get_range(self.ctx, r.ctypes.data), "get_range")
        return r

    def neighbors(self):
        off = np.zeros(self.n + 1, np.int64)
        self._check(self.lib.fsph_get_neighbors(self.ctx, off.ctypes.data, None, 0),
                    "get_neighbors")
        idx = np.zeros(int(off[-1]), np.int64)
        self._check(self.lib.fsph_get_neighbors(self.ctx, off.ctypes.data,
                                                idx.ctypes.data, len(idx)),
                    "get_neighbors")
        return off, idx

    def conserved(self):
        c = Conserved()
        self._check(self.lib.fsph_conserved_sums(self.ctx, C.byref(c)), "conserved")
        return dict(mass=c.mass, energy=c.energy, momentum=list(c.momentum),
                    angular_momentum=list(c.angular_momentum))

    def timers(self):
        ms = np.zeros(TIMER_COUNT)
        calls = np.zeros(TIMER_COUNT, np.int64)
        self._check(self.lib.fsph_timers(self.ctx, ms.ctypes.data, TIMER_COUNT,
                                         calls.ctypes.data), "timers")
        return {TIMER_NAMES[k]: (ms[k], int(calls[k])) for k in range(len(TIMER_NAMES))}

    def launch_count(self):
        return int(self.lib.fsph_launch_count(self.ctx))

    # -- reference-style aliases ------------------------------------------
    def apply_in_smoothinglength(self, name):
        """apply_in_smoothinglength(f) for f in the physics modules the
        library implements ('compute_density_pressure_soundspeed',
        'compute_acceleration', 'compute_dudt', 'compute_dedt')."""
        table = {
            "compute_density_pressure_soundspeed": self.density_pressure_soundspeed,
            "compute_acceleration": self.acceleration,
            "compute_dudt": self.dudt,
            "compute_dedt": self.dedt,
        }
        table[name]()

    def gravitation_fmm(self):
        self.gravitation()


class Ensemble:
    """Many independent problems on one GPU, stepped together as CUDA graphs
    (fsph_ensemble_* of include/fsph.h).  Members are BodySystem objects
    owned by the ensemble."""

    def __init__(self, device=0):
        lib = library()
        st = C.c_int(0)
        self.ens = lib.fsph_ensemble_create(device, C.byref(st))
        if not self.ens:
            raise FsphError(st.value, "fsph_ensemble_create")
        self.lib = lib
        self.members = []

    def add(self, params, capacity):
        m = BodySystem(params, capacity, _member_of=self.ens)
        self.members.append(m)
        return m

    def _check(self, st, where):
        if st:
            raise FsphError(st, where, self.lib.fsph_ensemble_last_error(self.ens).decode())

    def step(self, nsteps=1):
        self._check(self.lib.fsph_ensemble_step(self.ens, nsteps), "ensemble_step")

    def sync(self):
        failed = C.c_int32(-1)
        self._check(self.lib.fsph_ensemble_sync(self.ens, C.byref(failed)), "ensemble_sync")

    def set_lanes(self, lanes):
        self._check(self.lib.fsph_ensemble_set_lanes(self.ens, lanes), "ensemble_set_lanes")

    def set_group_size(self, group_size):
        self._check(self.lib.fsph_ensemble_set_group_size(self.ens, group_size),
                    "set_group_size")

    def tune_shape(self, steps_per_trial=2):
        """Lanes and walk-group size (fsph_ensemble_tune_shape): returns
        (lanes, group_size, ms_per_step)."""
        l, g, ms = C.c_int32(0), C.c_int32(0), C.c_double(0)
        self._check(self.lib.fsph_ensemble_tune_shape(self.ens, steps_per_trial, C.byref(l),
                                                      C.byref(g), C.byref(ms)),
                    "tune_shape")
        return l.value, g.value, ms.value

    def tune(self, steps_per_trial=3):
        lanes, ms = C.c_int32(0), C.c_double(0)
        self._check(self.lib.fsph_ensemble_tune(self.ens, steps_per_trial, C.byref(lanes),
                                                C.byref(ms)), "ensemble_tune")
        return lanes.value, ms.value

    def close(self):
        if getattr(self, "ens", None):
            for m in self.members:
                m.ctx = None
            self.lib.fsph_ensemble_destroy(self.ens)
            self.ens = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_external_force(params, external_force_type):
    """Fill params.external_force from an external_force_type string, as
    external_force::select parses it (fsph_params_set_external_force)."""
    st = library().fsph_params_set_external_force(C.byref(params),
                                                  external_force_type.encode())
    if st:
        raise FsphError(st, "set_external_force", external_force_type)
    return params


def capacity_for(params, n, state=None, margin=0.25):
    """Capacity that holds n real particles and their periodic copies.

    A particle within the halo (2.5 h_max) of the faces of k periodic axes
    gets one copy per non-empty subset of them (faces, edges, corner):
    2^k - 1.  Without `state` this is the bound n * 2^k; with it, the copies
    the current positions make, plus `margin` for particles that move into
    the halo later."""
    axes = [a for a in range(3) if getattr(params, "periodic_boundary_" + "xyz"[a])]
    if not axes:
        return n
    if state is None:
        return n << len(axes)
    halo = 2.5 * float(np.max(state["h"]))
    size = [params.box_length, params.box_width, params.box_height]
    k = np.zeros(n, np.int64)
    for a in axes:
        x = state["xyz"[a]]
        hi, lo = 0.5 * size[a], -0.5 * size[a]
        k += ((x + halo > hi) | (x - halo <= lo)).astype(np.int64)
    copies = int(((1 << k) - 1).sum())
    return min(n << len(axes), n + int(copies * (1.0 + margin)) + 1024)


def host_register(arr):
    """Pin a numpy array's memory for full-speed host<->device copies."""
    st = library().fsph_host_register(arr.ctypes.data, arr.nbytes)
    if st:
        raise FsphError(st, "host_register")


def host_unregister(arr):
    library().fsph_host_unregister(arr.ctypes.data)


def measure_peak(kind, device=0):
    """Measured FMA throughput of the device in TFLOP/s: kind 0 FP64, 1 FP32."""
    v = C.c_double()
    st = library().fsph_measure_peak(device, kind, C.byref(v))
    if st:
        raise FsphError(st, "measure_peak")
    return v.value


def mixed_available():
    """The mixed-precision pair kernels are part of this build."""
    return True
