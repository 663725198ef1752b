"""ctypes mirror of include/fsph.h (the C ABI of libfsph_gb300.so).

Only plain data types live here: the parameter block, the structure-of-arrays
particle view and the status codes.  Field order must match the header
exactly; ``tests/test_abi.py`` checks sizes and offsets against the compiled
library.
"""
import ctypes as C

import numpy as np

FSPH_OK = 0
STATUS_NAMES = {
    0: "FSPH_OK", 1: "FSPH_ERR_ARG", 2: "FSPH_ERR_CUDA", 3: "FSPH_ERR_NAN",
    4: "FSPH_ERR_NEG_DENSITY", 5: "FSPH_ERR_NEG_ENERGY", 6: "FSPH_ERR_NEGATIVITY",
    7: "FSPH_ERR_LIST_OVERFLOW", 8: "FSPH_ERR_STACK_OVERFLOW", 9: "FSPH_ERR_TIMEOUT",
    10: "FSPH_ERR_DUPLICATE_KEY", 11: "FSPH_ERR_DT", 12: "FSPH_ERR_STATE",
    13: "FSPH_ERR_NO_DEVICE", 14: "FSPH_ERR_OOM",
}

KERNEL_CUBIC_SPLINE = 0
KERNEL_QUINTIC_SPLINE = 1
KERNEL_WENDLAND_C2 = 2
KERNEL_WENDLAND_C4 = 3
KERNEL_WENDLAND_C6 = 4
KERNEL_GAUSSIAN = 5
KERNEL_SUPER_GAUSSIAN = 6
KERNEL_SINC = 7
EOS_IDEAL = 0
VISC_CONSTANT = 0
VISC_CULLEN = 1
EOS_POLYTROPIC = 1
EOS_WD = 2
EOS_PPT = 3
EOS_NO_EOS = 4
PRECISION_FP64 = 0
PRECISION_MIXED = 1
# enum fsph_eforce: the terms of external_force::select
EFORCE_NONE = 0
EFORCE_WALLS_X = 1
EFORCE_WALLS_Y = 2
EFORCE_WALLS_Z = 3
EFORCE_SPHERICAL_WALL = 4
EFORCE_SPHERICAL_DENSITY_SUPPORT = 5
EFORCE_GRAVITY = 6
EFORCE_AIRFOIL = 7
EFORCE_ORBIT = 8
EFORCE_POISON = 9
MAX_EFORCE = 8
DENSITY_CONSTANT = 0
DENSITY_PARABOLIC = 1
DENSITY_MESA = 2

TIMER_NAMES = ["range_keys", "sort", "tree", "neighbors", "density", "vsig",
               "accel", "energy", "integrate", "dt", "gravity", "periodic"]
TIMER_COUNT = 16


class FsphError(RuntimeError):
    def __init__(self, status, where="", detail=""):
        self.status = status
        msg = f"{where}: {STATUS_NAMES.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class Params(C.Structure):
    """fsph_params; defaults follow param:: in the reference's params.h."""
    _fields_ = [
        ("dimension", C.c_int32),
        ("sph_kernel", C.c_int32),
        ("eos_type", C.c_int32),
        ("sph_viscosity", C.c_int32),
        ("poly_gamma", C.c_double),
        ("sph_eta", C.c_double),
        ("sph_viscosity_alpha", C.c_double),
        ("sph_viscosity_beta", C.c_double),
        ("sph_viscosity_epsilon", C.c_double),
        ("timestep_cfl_factor", C.c_double),
        ("initial_dt", C.c_double),
        ("initial_time", C.c_double),
        ("final_time", C.c_double),
        ("out_screen_dt", C.c_double),
        ("out_scalar_dt", C.c_double),
        ("out_h5data_dt", C.c_double),
        ("fmm_macangle", C.c_double),
        ("gravitational_constant", C.c_double),
        ("box_length", C.c_double),
        ("box_width", C.c_double),
        ("box_height", C.c_double),
        ("initial_iteration", C.c_int64),
        ("final_iteration", C.c_int64),
        ("adaptive_timestep", C.c_int32),
        ("thermokinetic_formulation", C.c_int32),
        ("evolve_internal_energy", C.c_int32),
        ("pressure_updates_number", C.c_int32),
        ("sph_variable_h", C.c_int32),
        ("sph_update_uniform_h", C.c_int32),
        ("relaxation_steps", C.c_int32),
        ("enable_fmm", C.c_int32),
        ("periodic_boundary_x", C.c_int32),
        ("periodic_boundary_y", C.c_int32),
        ("periodic_boundary_z", C.c_int32),
        ("precision_mode", C.c_int32),
        ("max_neighbors", C.c_int32),
        ("gravity_order", C.c_int32),
        ("group_size", C.c_int32),
        ("sph_viscosity_alpha_max", C.c_double),
        ("sph_viscosity_l", C.c_double),
        ("sph_viscosity_delta", C.c_double),
        ("sph_sinc_index", C.c_double),
        ("poly_gamma2", C.c_double),
        ("ppt_density_thr", C.c_double),
        ("external_force", C.c_int32 * MAX_EFORCE),
        ("density_profile", C.c_int32),
        ("reserved_pad2", C.c_int32),
        ("extforce_wall_powerindex", C.c_double),
        ("extforce_wall_steepness", C.c_double),
        ("sphere_radius", C.c_double),
        ("gravity_acceleration_constant", C.c_double),
        ("orbital_separation", C.c_double),
        ("mass_neutron_star", C.c_double),
        ("mass_white_dwarf", C.c_double),
        ("zero_potential_poison_value", C.c_double),
        ("airfoil_size", C.c_double),
        ("airfoil_thickness", C.c_double),
        ("airfoil_camber", C.c_double),
        ("airfoil_anchor_x", C.c_double),
        ("airfoil_anchor_y", C.c_double),
        ("airfoil_attack_angle", C.c_double),
        ("rho_initial", C.c_double),
        ("pressure_initial", C.c_double),
        ("mesa_rim_width", C.c_double),
        ("relaxation_beta", C.c_double),
        ("relaxation_gamma", C.c_double),
        ("relaxation_repulsion_radius", C.c_double),
        ("relaxation_repulsion_gamma", C.c_double),
        ("reserved", C.c_int32 * 8),
    ]

    @classmethod
    def defaults(cls, **kw):
        p = cls()
        p.dimension = 3
        p.sph_kernel = KERNEL_WENDLAND_C4
        p.eos_type = EOS_IDEAL
        p.sph_viscosity = 0
        p.poly_gamma = 1.4
        p.sph_eta = 1.5
        p.sph_viscosity_alpha = 1.0
        p.sph_viscosity_beta = 2.0
        p.sph_viscosity_epsilon = 0.01
        p.timestep_cfl_factor = 0.25
        p.initial_dt = 0.001
        p.initial_time = 0.0
        p.final_time = 0.0
        p.fmm_macangle = 0.0
        p.gravitational_constant = 1.0
        p.box_length, p.box_width, p.box_height = 3.0, 1.0, 1.0
        p.initial_iteration = 0
        p.final_iteration = 0
        p.adaptive_timestep = 0
        p.thermokinetic_formulation = 1
        p.evolve_internal_energy = 1
        p.pressure_updates_number = 1
        p.sph_variable_h = 0
        p.sph_update_uniform_h = 0
        p.relaxation_steps = 0
        p.enable_fmm = 0
        p.precision_mode = PRECISION_FP64
        p.max_neighbors = 256
        p.gravity_order = 2
        p.sph_viscosity_alpha_max = 1.0
        p.sph_viscosity_l = 0.05
        p.sph_viscosity_delta = 1.0
        p.sph_sinc_index = 4.0
        p.poly_gamma2 = 2.5
        p.ppt_density_thr = 5e14
        p.density_profile = DENSITY_CONSTANT
        p.extforce_wall_powerindex = 5.0
        p.extforce_wall_steepness = 1e12
        p.sphere_radius = 1.0
        p.gravity_acceleration_constant = 9.81
        p.orbital_separation = 2.5e9
        p.mass_neutron_star = 1.26 * 1.988435e33
        p.mass_white_dwarf = 1.10 * 1.988435e33
        p.zero_potential_poison_value = 0.0
        p.airfoil_size = 2.0
        p.airfoil_thickness = 0.05
        p.airfoil_camber = 0.1
        p.airfoil_anchor_x = -1.0
        p.airfoil_anchor_y = 0.0
        p.airfoil_attack_angle = 0.0
        p.rho_initial = 1.0
        p.pressure_initial = 1.0
        p.mesa_rim_width = 0.25
        p.relaxation_beta = 1e-6
        p.relaxation_gamma = 0.0
        p.relaxation_repulsion_radius = 0.25
        p.relaxation_repulsion_gamma = 0.0
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            if k == "external_force":
                p.set_forces(v)
            else:
                setattr(p, k, v)
        return p

    def set_forces(self, codes):
        """Set the ordered external-force list (fsph_eforce codes)."""
        codes = list(codes)
        if len(codes) > MAX_EFORCE:
            raise ValueError("at most %d external-force terms" % MAX_EFORCE)
        self.external_force = (C.c_int32 * MAX_EFORCE)(*(codes + [0] * (MAX_EFORCE - len(codes))))

    def forces(self):
        """The external-force codes in order, without the terminating zeros."""
        out = []
        for c in self.external_force:
            if c == EFORCE_NONE:
                break
            out.append(int(c))
        return out

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            if name in ("reserved", "reserved_pad2"):
                continue
            v = getattr(self, name)
            out[name] = list(v) if name == "external_force" else v
        return out


_DP = C.POINTER(C.c_double)


class SoAView(C.Structure):
    """fsph_soa_view: structure-of-arrays particle state, FP64."""
    _fields_ = [
        ("n", C.c_int64),
        ("x", _DP), ("y", _DP), ("z", _DP),
        ("vx", _DP), ("vy", _DP), ("vz", _DP),
        ("vhx", _DP), ("vhy", _DP), ("vhz", _DP),
        ("ax", _DP), ("ay", _DP), ("az", _DP),
        ("gax", _DP), ("gay", _DP), ("gaz", _DP),
        ("gpot", _DP), ("m", _DP), ("h", _DP), ("rho", _DP), ("P", _DP),
        ("cs", _DP), ("u", _DP), ("e", _DP), ("dudt", _DP), ("dedt", _DP),
        ("K", _DP), ("alpha", _DP), ("vsig", _DP), ("dt", _DP),
        ("divv", _DP), ("ddivvdt", _DP), ("Ye", _DP),
        ("id", C.POINTER(C.c_int64)),
        ("key", C.POINTER(C.c_uint64)),
    ]


class Conserved(C.Structure):
    _fields_ = [("mass", C.c_double), ("energy", C.c_double),
                ("momentum", C.c_double * 3),
                ("angular_momentum", C.c_double * 3)]


# Every double field of the particle state, in header order.
DOUBLE_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "vhx", "vhy", "vhz",
                 "ax", "ay", "az", "gax", "gay", "gaz", "gpot", "m", "h",
                 "rho", "P", "cs", "u", "e", "dudt", "dedt", "K", "alpha",
                 "vsig", "dt", "divv", "ddivvdt", "Ye"]


def new_state(n):
    """A zeroed particle state: dict of contiguous numpy arrays."""
    s = {f: np.zeros(n, np.float64) for f in DOUBLE_FIELDS}
    s["id"] = np.arange(n, dtype=np.int64)
    s["key"] = np.zeros(n, np.uint64)
    return s


def make_view(state, n=None, fields=None):
    """fsph_soa_view over the arrays of `state` (kept alive by the caller).

    `fields` restricts which pointers are set (others stay NULL)."""
    if n is None:
        n = len(state["x"])
    v = SoAView()
    v.n = n
    for f in DOUBLE_FIELDS:
        if fields is not None and f not in fields:
            continue
        a = state.get(f)
        if a is None:
            continue
        assert a.dtype == np.float64 and a.flags.c_contiguous and len(a) == n, f
        setattr(v, f, a.ctypes.data_as(_DP))
    if "id" in state and (fields is None or "id" in fields):
        a = state["id"]
        assert a.dtype == np.int64 and a.flags.c_contiguous
        v.id = a.ctypes.data_as(C.POINTER(C.c_int64))
    if "key" in state and (fields is None or "key" in fields):
        a = state["key"]
        assert a.dtype == np.uint64 and a.flags.c_contiguous
        v.key = a.ctypes.data_as(C.POINTER(C.c_uint64))
    return v


def make_view_tensors(batch, n=None, fields=None):
    """fsph_soa_view over torch tensors (host or device memory; the caller
    keeps them alive): float64 fields, int64 id, int64 key bits."""
    import torch
    if n is None:
        n = int(batch["x"].shape[0])
    v = SoAView()
    v.n = n
    for f in DOUBLE_FIELDS:
        if fields is not None and f not in fields:
            continue
        t = batch.get(f)
        if t is None:
            continue
        assert t.dtype == torch.float64 and t.is_contiguous() and t.shape[0] == n, f
        setattr(v, f, C.cast(C.c_void_p(t.data_ptr()), _DP))
    for f, ct in (("id", C.c_int64), ("key", C.c_uint64)):
        if f in batch and (fields is None or f in fields):
            t = batch[f]
            assert t.dtype == torch.int64 and t.is_contiguous() and t.shape[0] == n, f
            setattr(v, f, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return v
