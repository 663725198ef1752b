"""Seeded synthetic initial conditions for the benchmark problems.

The reference builds its initial data with separate generator executables
that write .h5part files (app/id_generators/*).  Those need HDF5 and are not
part of the per-step path, so the problems are restated here from their
physical description, with every choice recorded in the returned ``meta``.

Smoothing length convention (app/id_generators/sodtube/main.cc:538-539):
h = sph_eta * kernel_width * (m/rho)^(1/D), kernel_width = 2 for the
Wendland kernels (include/physics/kernels.h:753-756).
"""
import math

import numpy as np

from .abi import EOS_IDEAL, EOS_POLYTROPIC, KERNEL_WENDLAND_C6, Params, new_state

KERNEL_WIDTH = 2.0


def _lattice(nx, ny, nz, lo, dx):
    """Cell-centred cubic lattice, x fastest; returns (N,3) positions."""
    ix = (np.arange(nx) + 0.5) * dx + lo[0]
    iy = (np.arange(ny) + 0.5) * dx + lo[1]
    iz = (np.arange(nz) + 0.5) * dx + lo[2]
    Z, Y, X = np.meshgrid(iz, iy, ix, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def _wendland_c6_3d(r, h):
    q = r / h
    w = (1365.0 / (64.0 * math.pi)) / h**3 * (1 - q) ** 8 * (1 + 8 * q + 25 * q**2 + 32 * q**3)
    return np.where(q < 1.0, w, 0.0)


def sod3d(nx=80, ny=20, nz=20, gamma=1.4, eta=1.5, seed=None):
    """3D Sod shock tube on a cubic lattice, dx = 1/nx over x in [-0.5, 0.5].

    Left (x < 0): rho=1, P=1; right: rho=0.125, P=0.1, densities set by the
    particle mass on one uniform lattice; v = 0; ideal gas; Wendland C6;
    h = eta*2*dx (h = 3 dx for eta = 1.5, about 97 neighbours).  The y and z
    extents follow from the cubic spacing: ny*dx and nz*dx, centred on 0.
    """
    dx = 1.0 / nx
    lo = (-0.5, -0.5 * ny * dx, -0.5 * nz * dx)
    pos = _lattice(nx, ny, nz, lo, dx)
    n = len(pos)
    s = new_state(n)
    left = pos[:, 0] < 0.0
    rho = np.where(left, 1.0, 0.125)
    P = np.where(left, 1.0, 0.1)
    s["x"][:], s["y"][:], s["z"][:] = pos[:, 0], pos[:, 1], pos[:, 2]
    s["m"][:] = rho * dx**3
    s["rho"][:] = rho
    s["P"][:] = P
    s["u"][:] = P / ((gamma - 1.0) * rho)
    s["h"][:] = eta * KERNEL_WIDTH * dx
    params = Params.defaults(dimension=3, sph_kernel=KERNEL_WENDLAND_C6,
                             eos_type=EOS_IDEAL, poly_gamma=gamma, sph_eta=eta,
                             adaptive_timestep=1, timestep_cfl_factor=0.25,
                             initial_dt=1.0e-12)
    meta = dict(problem="sod3d", n=n, dx=dx, box=[[lo[0], -lo[0]], [lo[1], -lo[1]], [lo[2], -lo[2]]],
                lattice=[nx, ny, nz])
    return s, params, meta


def sedov3d(n1d=128, gamma=5.0 / 3.0, eta=1.495, jitter=0.01, seed=12345,
            energy=1.0, u0=1.0e-5):
    """3D Sedov blast on a jittered cubic lattice in [-0.5, 0.5]^3.

    rho = 1 (m = dx^3), u = u0, per-axis N(0, jitter*dx) jitter from
    numpy's PCG64(seed); energy E deposited as u_b += E w_b / sum(m w) with
    w_b = W_C6(r_b, 2h), i.e. kernel-weighted over particles within 2h of
    the origin.  eta = 1.495 gives h = 2.99 dx: with the 1% jitter the mean
    neighbour count (self included) is 100 (93 lattice points lie within
    2.83 dx, the next shell of 30 sits at 3 dx).
    """
    dx = 1.0 / n1d
    pos = _lattice(n1d, n1d, n1d, (-0.5, -0.5, -0.5), dx)
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = pos + rng.normal(0.0, jitter * dx, size=pos.shape)
    n = len(pos)
    s = new_state(n)
    s["x"][:], s["y"][:], s["z"][:] = pos[:, 0], pos[:, 1], pos[:, 2]
    m = dx**3
    h = eta * KERNEL_WIDTH * dx
    s["m"][:] = m
    s["rho"][:] = 1.0
    s["h"][:] = h
    r = np.sqrt((pos**2).sum(axis=1))
    w = _wendland_c6_3d(r, 2.0 * h)
    u = np.full(n, u0)
    u += energy * w / (m * w.sum())
    s["u"][:] = u
    s["P"][:] = (gamma - 1.0) * 1.0 * u
    params = Params.defaults(dimension=3, sph_kernel=KERNEL_WENDLAND_C6,
                             eos_type=EOS_IDEAL, poly_gamma=gamma, sph_eta=eta,
                             adaptive_timestep=1, timestep_cfl_factor=0.25,
                             initial_dt=1.0e-6)
    meta = dict(problem="sedov3d", n=n, dx=dx, seed=seed, jitter=jitter, eta=eta,
                energy=energy, u0=u0, box=[[-0.5, 0.5]] * 3)
    return s, params, meta


def polytrope3d(n=1 << 22, seed=2024, eta=1.2, G=1.0, R=1.0, M=1.0, rho_floor=1e-3):
    """n=1 polytrope: rho(r) = rho_c sin(pi r)/(pi r), R = 1, M = 1, G = 1.

    Radii by inverse-CDF sampling of M(r) ~ sin(pi r) - pi r cos(pi r)
    (bisection in FP64), isotropic directions, m = M/n, rho_c = pi M/(4 R^3)
    (so the enclosed mass is M), polytropic EOS with gamma = 2 and
    K = 2 G R^2 / pi (hydrostatic equilibrium), v = 0, h from the local
    density; internal energy evolved by du/dt (thermokinetic off, as the
    reference's self-gravity parfile data/collapse_nx10.par has it).  The density is the analytic profile (the SPH sum recomputes it
    in the first density pass).  The density that sets h is floored at
    rho_floor * rho_c: near the surface the profile goes to zero and h with
    it to the star's size (1e-3 leaves the outermost few particles with
    thousands of neighbours; 1e-2 keeps every list under ~200).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.random(n)
    # invert F(r) = (sin(pi r) - pi r cos(pi r)) / pi on [0, 1] by bisection
    lo = np.zeros(n)
    hi = np.ones(n)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        F = (np.sin(np.pi * mid) - np.pi * mid * np.cos(np.pi * mid)) / np.pi
        mask = F < t
        lo = np.where(mask, mid, lo)
        hi = np.where(mask, hi, mid)
    r = 0.5 * (lo + hi) * R
    cth = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    sth = np.sqrt(1.0 - cth**2)
    s = new_state(n)
    s["x"][:] = r * sth * np.cos(phi)
    s["y"][:] = r * sth * np.sin(phi)
    s["z"][:] = r * cth
    rho_c = math.pi * M / (4.0 * R**3)
    pr = np.pi * r / R
    rho = rho_c * np.where(pr > 1e-12, np.sin(pr) / np.maximum(pr, 1e-300), 1.0)
    rho = np.maximum(rho, rho_floor * rho_c)
    K = 2.0 * G * R**2 / math.pi
    m = M / n
    s["m"][:] = m
    s["rho"][:] = rho
    s["P"][:] = K * rho**2
    s["K"][:] = K
    s["u"][:] = K * rho  # P / ((gamma-1) rho) with gamma = 2
    s["h"][:] = eta * KERNEL_WIDTH * np.cbrt(m / rho)
    params = Params.defaults(dimension=3, sph_kernel=KERNEL_WENDLAND_C6,
                             eos_type=EOS_POLYTROPIC, poly_gamma=2.0, sph_eta=eta,
                             enable_fmm=1, fmm_macangle=0.5, gravitational_constant=G,
                             gravity_order=2, adaptive_timestep=1,
                             initial_dt=1.0e-6, thermokinetic_formulation=0)
    meta = dict(problem="polytrope3d", n=n, seed=seed, K=K, rho_c=rho_c, eta=eta)
    return s, params, meta


def kh3d(n1d=256, gamma=5.0 / 3.0, eta=1.44, amp=0.01, seed=7):
    """Kelvin-Helmholtz in the periodic unit box [-0.5, 0.5]^3 (the box the
    reference's periodic boundaries assume, boundary.h:130-144), cubic
    lattice n1d^3.

    The band |y| < 0.25 has rho = 2, vx = +0.5; elsewhere rho = 1,
    vx = -0.5; density by particle mass on one lattice; P = 2.5;
    vy = amp sin(4 pi x).  `seed` is recorded but unused: the perturbation
    is deterministic.
    """
    dx = 1.0 / n1d
    pos = _lattice(n1d, n1d, n1d, (-0.5, -0.5, -0.5), dx)
    n = len(pos)
    s = new_state(n)
    s["x"][:], s["y"][:], s["z"][:] = pos[:, 0], pos[:, 1], pos[:, 2]
    band = np.abs(pos[:, 1]) < 0.25
    rho = np.where(band, 2.0, 1.0)
    s["m"][:] = rho * dx**3
    s["rho"][:] = rho
    s["P"][:] = 2.5
    s["u"][:] = 2.5 / ((gamma - 1.0) * rho)
    s["vx"][:] = np.where(band, 0.5, -0.5)
    s["vy"][:] = amp * np.sin(4.0 * np.pi * pos[:, 0])
    s["h"][:] = eta * KERNEL_WIDTH * dx
    params = Params.defaults(dimension=3, sph_kernel=KERNEL_WENDLAND_C6,
                             eos_type=EOS_IDEAL, poly_gamma=gamma, sph_eta=eta,
                             periodic_boundary_x=1, periodic_boundary_y=1,
                             periodic_boundary_z=1, box_length=1.0, box_width=1.0,
                             box_height=1.0, adaptive_timestep=1, initial_dt=1e-6)
    meta = dict(problem="kh3d", n=n, dx=dx, seed=seed, band="|y| < 0.25",
                box="[-0.5, 0.5]^3")
    return s, params, meta


def kh2d(n1d=128, gamma=5.0 / 3.0, eta=1.5, amp=0.01):
    """2D analogue of kh3d on [-0.5, 0.5]^2, periodic in x and y."""
    dx = 1.0 / n1d
    ix = (np.arange(n1d) + 0.5) * dx - 0.5
    Y, X = np.meshgrid(ix, ix, indexing="ij")
    x, y = X.ravel(), Y.ravel()
    n = len(x)
    s = new_state(n)
    s["x"][:], s["y"][:] = x, y
    band = np.abs(y) < 0.25
    rho = np.where(band, 2.0, 1.0)
    s["m"][:] = rho * dx**2
    s["rho"][:] = rho
    s["P"][:] = 2.5
    s["u"][:] = 2.5 / ((gamma - 1.0) * rho)
    s["vx"][:] = np.where(band, 0.5, -0.5)
    s["vy"][:] = amp * np.sin(4.0 * np.pi * x)
    s["h"][:] = eta * KERNEL_WIDTH * dx
    params = Params.defaults(dimension=2, sph_kernel=KERNEL_WENDLAND_C6,
                             eos_type=EOS_IDEAL, poly_gamma=gamma, sph_eta=eta,
                             periodic_boundary_x=1, periodic_boundary_y=1,
                             box_length=1.0, box_width=1.0, adaptive_timestep=1,
                             initial_dt=1e-6)
    meta = dict(problem="kh2d", n=n, dx=dx, band="|y| < 0.25", box="[-0.5, 0.5]^2")
    return s, params, meta


def sod2d(nx=200, ny=20, gamma=1.4, eta=1.5):
    """2D Sod tube on a square lattice dx = 1/nx, x in [-0.5,0.5]."""
    dx = 1.0 / nx
    ix = (np.arange(nx) + 0.5) * dx - 0.5
    iy = (np.arange(ny) + 0.5) * dx - 0.5 * ny * dx
    Y, X = np.meshgrid(iy, ix, indexing="ij")
    x, y = X.ravel(), Y.ravel()
    n = len(x)
    s = new_state(n)
    left = x < 0
    rho = np.where(left, 1.0, 0.125)
    P = np.where(left, 1.0, 0.1)
    s["x"][:], s["y"][:] = x, y
    s["m"][:] = rho * dx**2
    s["rho"][:] = rho
    s["P"][:] = P
    s["u"][:] = P / ((gamma - 1.0) * rho)
    s["h"][:] = eta * KERNEL_WIDTH * dx
    params = Params.defaults(dimension=2, sph_kernel=KERNEL_WENDLAND_C6,
                             poly_gamma=gamma, sph_eta=eta, adaptive_timestep=1,
                             initial_dt=1.0e-12)
    return s, params, dict(problem="sod2d", n=n, dx=dx)


def noh2d(n1d=100, gamma=5.0 / 3.0, eta=1.5, P0=1e-6):
    """2D Noh implosion: disc of radius 0.5, rho=1, P=1e-6, v = -r_hat."""
    dx = 1.0 / n1d
    ix = (np.arange(n1d) + 0.5) * dx - 0.5
    Y, X = np.meshgrid(ix, ix, indexing="ij")
    x, y = X.ravel(), Y.ravel()
    r = np.sqrt(x * x + y * y)
    keep = r < 0.5
    x, y, r = x[keep], y[keep], r[keep]
    n = len(x)
    s = new_state(n)
    s["x"][:], s["y"][:] = x, y
    s["m"][:] = dx**2
    s["rho"][:] = 1.0
    s["P"][:] = P0
    s["u"][:] = P0 / (gamma - 1.0)
    rr = np.maximum(r, 1e-12)
    s["vx"][:] = -x / rr
    s["vy"][:] = -y / rr
    s["h"][:] = eta * KERNEL_WIDTH * dx
    params = Params.defaults(dimension=2, sph_kernel=KERNEL_WENDLAND_C6,
                             poly_gamma=gamma, sph_eta=eta, adaptive_timestep=1,
                             initial_dt=1.0e-6)
    return s, params, dict(problem="noh2d", n=n, dx=dx)


def ensemble2d(nproblems=256, nmin=2000, nmax=200000, seed=2020):
    """Many independent 2D problems: particle counts log-uniform in
    [nmin, nmax] (seeded), alternately a Sod tube (10:1 lattice) and a Noh
    disc, all in mixed precision.  Returns a list of (state, params, meta);
    the actual counts follow from the lattices (recorded in meta).  With
    the default seed the 256 problems hold about 12.4M particles."""
    rng = np.random.Generator(np.random.PCG64(seed))
    target = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nproblems))
    out = []
    for k, nt in enumerate(target):
        if k % 2 == 0:
            ny = max(4, int(round(math.sqrt(nt / 10.0))))
            s, p, m = sod2d(10 * ny, ny)
        else:
            n1d = max(8, int(round(math.sqrt(4.0 * nt / math.pi))))
            s, p, m = noh2d(n1d)
        p.precision_mode = 1
        m["target_n"] = float(nt)
        out.append((s, p, m))
    return out


EXTERNAL_FORCE_PROBLEMS = ["gravity_walls_2d", "spherical_wall_3d", "density_support_3d",
                           "mesa_support_2d", "airfoil_2d", "orbit_3d", "relaxation_3d",
                           "relaxation_dudt_2d"]


def external_force_problem(name):
    """Small problems exercising each external force of include/physics/
    eforce.h and the particle relaxation terms; returns (state, params).

    gravity_walls_2d: a Sod tube in uniform gravity (plus a potential shift)
        between walls in y placed inside the lattice, so that the outer rows
        feel them; spherical_wall_3d: a Sedov blast inside a spherical wall of
        radius 0.45 (the corners are outside); density_support_3d /
        mesa_support_2d: a polytrope / disc held by the parabolic / mesa
        support potential; airfoil_2d: a uniform stream past an airfoil tilted
        by 5 degrees; orbit_3d: a Sod tube scaled to 1e8 cm in the
        neutron-star + white-dwarf co-rotating potential; relaxation_3d /
        relaxation_dudt_2d: drag and short-range repulsion while relaxing (e
        and u formulations).
    """
    from .abi import (DENSITY_MESA, DENSITY_PARABOLIC, EFORCE_AIRFOIL, EFORCE_GRAVITY,
                      EFORCE_ORBIT, EFORCE_POISON, EFORCE_SPHERICAL_DENSITY_SUPPORT,
                      EFORCE_SPHERICAL_WALL, EFORCE_WALLS_X, EFORCE_WALLS_Y)
    if name == "gravity_walls_2d":
        s, p, m = sod2d(100, 10)
        p.set_forces([EFORCE_GRAVITY, EFORCE_WALLS_Y, EFORCE_POISON, EFORCE_WALLS_X])
        p.gravity_acceleration_constant = 2.0
        p.zero_potential_poison_value = 0.3
        p.box_length, p.box_width = 0.98, 0.08
    elif name == "spherical_wall_3d":
        s, p, m = sedov3d(16, eta=1.44)
        p.set_forces([EFORCE_SPHERICAL_WALL])
        p.sphere_radius = 0.45
        p.extforce_wall_steepness = 20.0
        p.extforce_wall_powerindex = 3.0
    elif name == "density_support_3d":
        s, p, m = polytrope3d(3000)
        p.enable_fmm = 0
        p.set_forces([EFORCE_SPHERICAL_DENSITY_SUPPORT])
        p.density_profile = DENSITY_PARABOLIC
        p.sphere_radius = 0.9
        p.rho_initial, p.pressure_initial = 2.0, 0.5
        p.extforce_wall_steepness = 10.0
    elif name == "mesa_support_2d":
        s, p, m = noh2d(40)
        for k in ("vx", "vy"):
            s[k][:] = 0.0
        s["u"][:] = 1.0
        s["P"][:] = (p.poly_gamma - 1.0) * s["rho"] * s["u"]
        p.set_forces([EFORCE_SPHERICAL_DENSITY_SUPPORT])
        p.density_profile = DENSITY_MESA
        p.sphere_radius = 0.45
        p.mesa_rim_width = 0.3
        p.extforce_wall_steepness = 100.0
    elif name == "airfoil_2d":
        s, p, m = sod2d(200, 20)
        s["rho"][:] = 1.0
        s["m"][:] = (1.0 / 200) ** 2
        s["P"][:] = 1.0
        s["u"][:] = s["P"] / ((p.poly_gamma - 1.0) * s["rho"])
        s["vx"][:] = 0.5
        p.set_forces([EFORCE_AIRFOIL])
        p.airfoil_size, p.airfoil_thickness, p.airfoil_camber = 0.8, 0.06, 0.02
        p.airfoil_anchor_x, p.airfoil_anchor_y = -0.4, 0.0
        p.airfoil_attack_angle = 5.0
    elif name == "orbit_3d":
        s, p, m = sod3d(20, 10, 10)
        L = 1.0e8
        for k in ("x", "y", "z", "h"):
            s[k] *= L
        s["m"] *= L ** 3
        s["u"] *= 1.0e10
        s["P"] *= 1.0e10
        p.set_forces([EFORCE_ORBIT])
        p.gravitational_constant = 6.674e-8
    elif name == "relaxation_3d":
        s, p, m = sedov3d(16, eta=1.44)
        p.relaxation_steps = 8
        p.relaxation_beta, p.relaxation_gamma = 0.2, 3.0
        p.relaxation_repulsion_radius, p.relaxation_repulsion_gamma = 0.5, 1e-7
        rng = np.random.Generator(np.random.PCG64(5))
        for k in ("vx", "vy", "vz"):
            s[k][:] = rng.normal(0.0, 0.05, len(s["x"]))
    elif name == "relaxation_dudt_2d":
        s, p, m = sod2d(100, 10)
        p.thermokinetic_formulation = 0
        p.relaxation_steps = 8
        p.relaxation_beta, p.relaxation_gamma = 0.1, 1.0
        p.relaxation_repulsion_radius, p.relaxation_repulsion_gamma = 0.6, 1e-6
        s["vx"][:] = 0.1 * np.sin(2 * np.pi * s["x"])
    else:
        raise ValueError(name)
    if p.dimension == 3:
        p.max_neighbors = 1024  # walls and supports compress the outer layers
    return s, p


def shuffled(state, seed=99):
    """The same particles in a seeded random order (ids travel along)."""
    n = len(state["x"])
    perm = np.random.Generator(np.random.PCG64(seed)).permutation(n)
    return {k: np.ascontiguousarray(v[perm]) for k, v in state.items()}
