"""ctypes binding of the CPU oracle (oracle/fsph_oracle.h).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, as the checker or the timed CPU
baseline.  The GPU product (flecsph_gb300/) never imports this module.

``Oracle("port")`` loads oracle/liboracle.so (the C restatement);
``Oracle("reference", dim)`` loads oracle/_ref/libfsph_ref{dim}.so (the
reference's own headers compiled here), when that was built.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from flecsph_gb300.abi import FsphError, Params, make_view, new_state

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")


def ref_lib_path(dim):
    return os.path.join(HERE, "_ref", f"libfsph_ref{dim}.so")


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def reference_root():
    """Where the reference's sources are: $FSPH_REFERENCE, else a checkout
    named `reference` beside this repository; None when neither exists."""
    cand = os.environ.get("FSPH_REFERENCE") or os.path.join(
        os.path.dirname(os.path.dirname(HERE)), "reference")
    return cand if os.path.isdir(cand) else None


def build_ref(ref_root=None):
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return True


def have_ref(dim=3):
    return os.path.exists(ref_lib_path(dim))


_FUNCS0 = ["update_iteration", "reset_ghosts", "density_pressure_soundspeed",
           "acceleration", "dudt", "dedt", "eos_init", "set_total_energy",
           "save_velocityhalf", "leapfrog_kick_v", "leapfrog_kick_u",
           "leapfrog_kick_e", "leapfrog_drift", "recompute_pressure_soundspeed",
           "recompute_pressure_soundspeed_thermokinetic", "compute_dt",
           "set_adaptive_timestep", "compute_smoothinglength",
           "compute_average_smoothinglength", "check_nans", "check_negativity",
           "advance_time", "step", "compute_alpha", "initialize_alpha",
           "add_drag_acceleration", "add_short_range_repulsion", "add_drag_dedt",
           "add_drag_dudt"]

_libs = {}


def _load(path):
    if path in _libs:
        return _libs[path]
    lib = C.CDLL(path)
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.POINTER(Params)]
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_destroy.restype = None
    for f in _FUNCS0:
        fn = getattr(lib, "orc_" + f)
        fn.argtypes = [C.c_void_p]
        fn.restype = C.c_int
    lib.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
    lib.orc_upload.argtypes = [C.c_void_p, C.c_void_p]
    lib.orc_download.argtypes = [C.c_void_p, C.c_void_p]
    lib.orc_get_time.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.orc_set_time.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int64]
    lib.orc_get_range.argtypes = [C.c_void_p, C.c_void_p]
    lib.orc_gravity_direct.argtypes = [C.c_void_p, C.c_int64, C.c_int64]
    lib.orc_get_neighbors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    lib.orc_get_order.argtypes = [C.c_void_p, C.c_void_p]
    lib.orc_particle_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]
    _libs[path] = lib
    return lib


def _fresh_copy(path):
    """Load a private copy of a library: new globals and function statics.

    The reference's external-force functions keep their parameters in
    function-local statics set at the first call (eforce.h:51-52, 71-72,
    132-133, 156-157, 180, 191, 256, 286, 311), so one loaded copy serves
    one set of external-force parameters."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp(prefix="fsph_ref_")
    dst = os.path.join(d, os.path.basename(path))
    shutil.copy(path, dst)
    return _load(dst)


class Oracle:
    def __init__(self, kind, params, threads=None):
        self.kind = kind
        self.params = params
        path = PORT_LIB if kind == "port" else ref_lib_path(params.dimension)
        if kind != "port" and params.forces():
            self.lib = _fresh_copy(path)
        else:
            self.lib = _load(path)
        self.ctx = self.lib.orc_create(C.byref(params))
        if not self.ctx:
            raise FsphError(1, "orc_create")
        if threads:
            self.lib.orc_set_threads(self.ctx, threads)

    def close(self):
        if self.ctx:
            self.lib.orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __getattr__(self, name):
        if name in _FUNCS0:
            fn = getattr(self.lib, "orc_" + name)

            def call():
                st = fn(self.ctx)
                if st:
                    raise FsphError(st, f"{self.kind}.{name}")
            return call
        raise AttributeError(name)

    @property
    def n(self):
        """Particles held, periodic copies included."""
        return self.count()[0]

    def count(self):
        t, r = C.c_int64(), C.c_int64()
        self.lib.orc_particle_count(self.ctx, C.byref(t), C.byref(r))
        return t.value, r.value

    def upload(self, state):
        self._keep = {k: np.ascontiguousarray(v) for k, v in state.items()}
        v = make_view(self._keep)
        st = self.lib.orc_upload(self.ctx, C.byref(v))
        if st:
            raise FsphError(st, "upload")

    def download(self):
        out = new_state(self.n)
        v = make_view(out)
        st = self.lib.orc_download(self.ctx, C.byref(v))
        if st:
            raise FsphError(st, "download")
        return out

    def time(self):
        dt, t, it = C.c_double(), C.c_double(), C.c_int64()
        self.lib.orc_get_time(self.ctx, C.byref(dt), C.byref(t), C.byref(it))
        return dt.value, t.value, it.value

    def set_time(self, dt, t, it):
        self.lib.orc_set_time(self.ctx, dt, t, it)

    def range(self):
        r = np.zeros(2 * self.params.dimension)
        self.lib.orc_get_range(self.ctx, r.ctypes.data)
        return r

    def gravity_direct(self, s0=0, s1=None):
        s1 = self.n if s1 is None else s1
        st = self.lib.orc_gravity_direct(self.ctx, s0, s1)
        if st:
            raise FsphError(st, "gravity_direct")

    def neighbors(self):
        off = np.zeros(self.n + 1, np.int64)
        st = self.lib.orc_get_neighbors(self.ctx, off.ctypes.data, None, 0)
        if st:
            raise FsphError(st, "neighbors")
        idx = np.zeros(int(off[-1]), np.int64)
        st = self.lib.orc_get_neighbors(self.ctx, off.ctypes.data, idx.ctypes.data,
                                        len(idx))
        if st:
            raise FsphError(st, "neighbors")
        return off, idx

    def order(self):
        o = np.zeros(self.n, np.int64)
        st = self.lib.orc_get_order(self.ctx, o.ctypes.data)
        if st:
            raise FsphError(st, "order")
        return o
