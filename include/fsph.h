/*
 * fsph.h -- C ABI of the GB300 SPH hot path (libfsph_gb300.so).
 *
 * The entry points replace the call surface FleCSPH's evolution drivers use
 * on the per-step particle path (app/drivers/hydro/main_driver.cc:98-279 and
 * app/drivers/newtonian/main_driver.cc:98-298):
 *
 *   body_system<T,D>   (mpisph/bodies_system.h)
 *     update_iteration()              :152-229  -> fsph_update_iteration
 *     reset_ghosts()                  :273-275  -> fsph_reset_ghosts
 *     apply_in_smoothinglength(f)     :304-307  -> fsph_density_pressure_soundspeed,
 *                                                  fsph_acceleration, fsph_dudt, fsph_dedt
 *     apply_all(f)                    :318-324  -> fsph_eos_init, fsph_set_total_energy,
 *                                                  fsph_save_velocityhalf, fsph_leapfrog_*,
 *                                                  fsph_recompute_pressure_soundspeed[_thermokinetic],
 *                                                  fsph_compute_dt, fsph_check_nans,
 *                                                  fsph_check_negativity
 *     get_all(f)                      :335-338  -> fsph_set_adaptive_timestep,
 *                                                  fsph_compute_smoothinglength,
 *                                                  fsph_compute_average_smoothinglength
 *     gravitation_fmm()               :282-288  -> fsph_gravitation
 *     setMacangle(double)             :70-72    -> fsph_params.fmm_macangle
 *   physics::advance_time()  include/physics/default_physics.h:853-860 -> fsph_advance_time
 *   the whole do{...}while body of mpi_init_task              -> fsph_step
 *
 * All arrays crossing this boundary are host (or device, where stated)
 * pointers owned by the caller; plain C types only.  Every call returns an
 * fsph_status; nothing throws across the boundary.  A context owns one CUDA
 * stream on one device and is not re-entrant: use one context per host
 * thread.  Calls enqueue work asynchronously except where documented as
 * synchronous (download, neighbour export, reductions, status reads).
 *
 * Particle order: after fsph_update_iteration the particles are held sorted
 * by (Morton key, id), as the reference keeps its bodies vector sorted in
 * place (mpisph/bodies_system.h:195-206); fsph_download returns that order,
 * with ids, so the caller can map back.
 */
#ifndef FSPH_H
#define FSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSPH_ABI_VERSION 6

/* Status codes.  They replace the reference's assert()/mpi_assert() aborts
 * (default_physics.h:134-143,215-226,636-651,661-691,918-979;
 * mpisph/utils.h:34-38). */
typedef enum fsph_status {
  FSPH_OK = 0,
  FSPH_ERR_ARG = 1,            /* bad argument / unsupported parameter value */
  FSPH_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  FSPH_ERR_NAN = 3,            /* check_nans found a NaN */
  FSPH_ERR_NEG_DENSITY = 4,    /* compute_density: rho not > 0 */
  FSPH_ERR_NEG_ENERGY = 5,     /* recover_internal_energy / compute_dt: u not > 0 */
  FSPH_ERR_NEGATIVITY = 6,     /* check_negativity: rho, P or u < 0 */
  FSPH_ERR_LIST_OVERFLOW = 7,  /* a neighbour list exceeded max_neighbors */
  FSPH_ERR_STACK_OVERFLOW = 8, /* a tree-walk stack exceeded its capacity */
  FSPH_ERR_TIMEOUT = 9,        /* a bounded device loop gave up */
  FSPH_ERR_DUPLICATE_KEY = 10, /* two particles share a full Morton key */
  FSPH_ERR_DT = 11,            /* compute_dt energy-positivity loop did not converge */
  FSPH_ERR_STATE = 12,         /* call made before the state it needs exists */
  FSPH_ERR_NO_DEVICE = 13,     /* no CUDA device / extension not usable */
  FSPH_ERR_OOM = 14            /* device allocation failed */
} fsph_status;

/* Same numbering as param::sph_kernel_keyword (include/params.h:128-137). */
enum fsph_kernel {
  FSPH_KERNEL_CUBIC_SPLINE = 0,
  FSPH_KERNEL_QUINTIC_SPLINE = 1,
  FSPH_KERNEL_WENDLAND_C2 = 2,
  FSPH_KERNEL_WENDLAND_C4 = 3,
  FSPH_KERNEL_WENDLAND_C6 = 4,
  FSPH_KERNEL_GAUSSIAN = 5,
  FSPH_KERNEL_SUPER_GAUSSIAN = 6,
  FSPH_KERNEL_SINC = 7
};
/* Same numbering as param::eos_type_keyword (include/params.h:139-145). */
/* param::eos_type_keyword (include/params.h:138-144) */
enum fsph_eos {
  FSPH_EOS_IDEAL = 0,
  FSPH_EOS_POLYTROPIC = 1,
  FSPH_EOS_WD = 2,      /* cold white-dwarf matter (CGS units) */
  FSPH_EOS_PPT = 3,     /* piecewise polytrope */
  FSPH_EOS_NO_EOS = 4   /* pressure and sound speed left as they are */
};
/* param::sph_viscosity_keyword (include/params.h:148-152). */
enum fsph_viscosity { FSPH_VISC_CONSTANT = 0, FSPH_VISC_CULLEN = 1 };
/* The terms external_force::select (include/physics/eforce.h:359-434)
 * builds from external_force_type, one code per potential/acceleration in
 * the order the string names them ("walls:xyz" gives three codes). */
enum fsph_eforce {
  FSPH_EFORCE_NONE = 0,                      /* ends the list */
  FSPH_EFORCE_WALLS_X = 1,                   /* eforce.h:46-82, box_length */
  FSPH_EFORCE_WALLS_Y = 2,                   /* box_width */
  FSPH_EFORCE_WALLS_Z = 3,                   /* box_height */
  FSPH_EFORCE_SPHERICAL_WALL = 4,            /* eforce.h:84-121 */
  FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT = 5, /* eforce.h:123-168 */
  FSPH_EFORCE_GRAVITY = 6,                   /* eforce.h:170-192 */
  FSPH_EFORCE_AIRFOIL = 7,                   /* eforce.h:194-271 (2D) */
  FSPH_EFORCE_ORBIT = 8,                     /* eforce.h:273-313 (3D) */
  FSPH_EFORCE_POISON = 9                     /* eforce.h:315-321 (potential only) */
};
#define FSPH_MAX_EFORCE 8
/* param::density_profile (include/physics/density_profiles.h:355-398); the
 * tabulated "from file" profile is not supported. */
enum fsph_density_profile {
  FSPH_DENSITY_CONSTANT = 0,
  FSPH_DENSITY_PARABOLIC = 1,
  FSPH_DENSITY_MESA = 2
};
enum fsph_precision {
  FSPH_PRECISION_FP64 = 0,  /* every pair term in FP64 (plain method) */
  FSPH_PRECISION_MIXED = 1  /* FP32 pair math with compensated sums; FP64 state */
};

/* Physics and run parameters.  Names and defaults follow param:: in
 * include/params.h (line of each DECLARE_PARAM in brackets); the last block
 * is specific to this implementation. */
typedef struct fsph_params {
  int32_t dimension;                 /* gdimension: 2 or 3 */
  int32_t sph_kernel;                /* [227] wendland_c4 */
  int32_t eos_type;                  /* [468] eos_ideal */
  int32_t sph_viscosity;             /* [495] visc_constant */
  double poly_gamma;                 /* [478] 1.4 */
  double sph_eta;                    /* [212] 1.5 */
  double sph_viscosity_alpha;        /* [501] 1.0 */
  double sph_viscosity_beta;         /* [506] 2.0 */
  double sph_viscosity_epsilon;      /* [511] 0.01 */
  double timestep_cfl_factor;        /* [183] 0.25 */
  double initial_dt;                 /* [178] 0.001 */
  double initial_time;               /* [169] 0 */
  double final_time;                 /* [173] 0 */
  double out_screen_dt;              /* [339] 0 */
  double out_scalar_dt;              /* [350] 0 */
  double out_h5data_dt;              /* [366] 0 */
  double fmm_macangle;               /* [542] 0.0 (0: every pair summed directly) */
  double gravitational_constant;     /* [628] 1 */
  double box_length;                 /* [258] 3.0 */
  double box_width;                  /* [262] 1.0 */
  double box_height;                 /* [266] 1.0 */
  int64_t initial_iteration;         /* [160] 0 */
  int64_t final_iteration;           /* [165] 0 */
  int32_t adaptive_timestep;         /* [188] false */
  int32_t thermokinetic_formulation; /* [591] true */
  int32_t evolve_internal_energy;    /* [584] true */
  int32_t pressure_updates_number;   /* [194] 1 */
  int32_t sph_variable_h;            /* [244] false */
  int32_t sph_update_uniform_h;      /* [238] false */
  int32_t relaxation_steps;          /* [563] 0 */
  int32_t enable_fmm;                /* [537] false */
  int32_t periodic_boundary_x;       /* [292] false */
  int32_t periodic_boundary_y;       /* [296] false */
  int32_t periodic_boundary_z;       /* [300] false */
  /* implementation-specific */
  int32_t precision_mode;            /* enum fsph_precision, default FP64 */
  int32_t max_neighbors;             /* neighbour-list capacity per particle, default 256 */
  int32_t gravity_order;             /* multipole order of fsph_gravitation: 1 or 2 (default 2) */
  int32_t group_size;                /* particles per group of the neighbour and
                                        gravity walks (one warp each): 1..32,
                                        0 = 32 */
  /* Cullen & Dehnen adaptive viscosity (visc_cullen), param:: names */
  double sph_viscosity_alpha_max;    /* [516] 1.0 */
  double sph_viscosity_l;            /* [523] 0.05 */
  double sph_viscosity_delta;        /* [529] 1.0 */
  double sph_sinc_index;             /* [232] 4.0, sinc kernel power */
  double poly_gamma2;                /* [483] 2.5, eos_ppt upper segment */
  double ppt_density_thr;            /* [488] 5e14, eos_ppt threshold */
  /* external forces: external_force_type [597] "none" as the list of
   * fsph_eforce codes that external_force::select builds from it
   * (fsph_params_set_external_force parses the string) */
  int32_t external_force[FSPH_MAX_EFORCE];
  int32_t density_profile;           /* [671] "constant" (enum fsph_density_profile) */
  int32_t reserved_pad2;
  double extforce_wall_powerindex;   /* [608] 5.0 */
  double extforce_wall_steepness;    /* [613] 1e12 */
  double sphere_radius;              /* [270] 1.0 */
  double gravity_acceleration_constant; /* [623] 9.81 */
  double orbital_separation;         /* [637] 2.5e9 */
  double mass_neutron_star;          /* [642] 1.26 * 1.988435e33 */
  double mass_white_dwarf;           /* [647] 1.10 * 1.988435e33 */
  double zero_potential_poison_value;/* [603] 0.0 */
  double airfoil_size;               /* [761] 2.0 */
  double airfoil_thickness;          /* [765] 0.05 */
  double airfoil_camber;             /* [769] 0.1 */
  double airfoil_anchor_x;           /* [773] -1.0 */
  double airfoil_anchor_y;           /* [777] 0.0 */
  double airfoil_attack_angle;       /* [781] 0.0 (degrees) */
  double rho_initial;                /* [682] 1.0 */
  double pressure_initial;           /* [687] 1.0 */
  double mesa_rim_width;             /* [618] 0.25 */
  /* particle relaxation, iterations < relaxation_steps */
  double relaxation_beta;            /* [568] 1e-6 */
  double relaxation_gamma;           /* [572] 0.0 */
  double relaxation_repulsion_radius;/* [576] 0.25 */
  double relaxation_repulsion_gamma; /* [580] 0.0 */
  int32_t reserved[8];
} fsph_params;

/* Structure-of-arrays view of the particle state, FP64 throughout.  On
 * upload every pointer marked (in) must be non-NULL; (opt) pointers may be
 * NULL and then start at zero.  On download NULL pointers are skipped.
 * 2D runs ignore the z components.  Field names follow body_u
 * (include/physics/body.h:221-251). */
typedef struct fsph_soa_view {
  int64_t n;
  double *x, *y, *z;       /* (in)  coordinates */
  double *vx, *vy, *vz;    /* (in)  velocity */
  double *vhx, *vhy, *vhz; /* (opt) velocity at the half step */
  double *ax, *ay, *az;    /* (opt) hydro acceleration */
  double *gax, *gay, *gaz; /* (opt) gravitational acceleration */
  double *gpot;            /* (opt) gravitational potential */
  double *m;               /* (in)  mass */
  double *h;               /* (in)  smoothing length (entity radius) */
  double *rho;             /* (opt) density */
  double *P;               /* (opt) pressure */
  double *cs;              /* (opt) sound speed */
  double *u;               /* (opt) specific internal energy */
  double *e;               /* (opt) specific total (thermokinetic) energy */
  double *dudt;            /* (opt) */
  double *dedt;            /* (opt) */
  double *K;               /* (opt) adiabatic invariant */
  double *alpha;           /* (opt) viscosity alpha (unused by visc_constant) */
  double *vsig;            /* (opt) signal speed */
  double *dt;              /* (opt) per-particle timestep estimate */
  double *divv;            /* (opt) velocity divergence (visc_cullen) */
  double *ddivvdt;         /* (opt) its time derivative (visc_cullen) */
  double *Ye;              /* (opt) electron fraction (eos_wd) */
  int64_t *id;             /* (in)  particle id (sort tie-break) */
  uint64_t *key;           /* (out) Morton key, download only */
} fsph_soa_view;

/* Conserved totals over all particles (include/physics/analysis.h:56-214),
 * FP64 reductions on the device. */
typedef struct fsph_conserved {
  double mass;
  double energy;        /* sum m*e (thermokinetic) or m*(u + v^2/2), plus grav. */
  double momentum[3];
  double angular_momentum[3];
} fsph_conserved;

/* Per-kernel device time accumulated since the last reset (CUDA events on
 * the context's stream).  Indices: see FSPH_TIMER_* below. */
enum {
  FSPH_TIMER_RANGE_KEYS = 0,
  FSPH_TIMER_SORT = 1,
  FSPH_TIMER_TREE = 2,
  FSPH_TIMER_NEIGHBORS = 3,
  FSPH_TIMER_DENSITY = 4,
  FSPH_TIMER_VSIG = 5,
  FSPH_TIMER_ACCEL = 6,
  FSPH_TIMER_ENERGY = 7,
  FSPH_TIMER_INTEGRATE = 8,
  FSPH_TIMER_DT = 9,
  FSPH_TIMER_GRAVITY = 10,
  FSPH_TIMER_PERIODIC = 11,
  FSPH_TIMER_COUNT = 16
};

typedef struct fsph_ctx fsph_ctx;

/* -- lifetime ------------------------------------------------------------ */
void fsph_params_default(fsph_params * p);
/* external_force::select (include/physics/eforce.h:359-434): fill
 * p->external_force from an external_force_type string, a comma-separated
 * list of "spherical wall", "airfoil", "spherical density support",
 * "gravity", "orbit", "walls:<xyz>", "poison" (case-insensitive; "none" or
 * "zero" alone for no force).  An unknown term returns FSPH_ERR_ARG, where
 * the reference stops with log_fatal; more than FSPH_MAX_EFORCE terms too. */
fsph_status fsph_params_set_external_force(fsph_params * p,
  const char * external_force_type);
int32_t fsph_abi_version(void);
/* Creates a context on `device` able to hold `capacity` particles. */
fsph_ctx * fsph_create(const fsph_params * p, int32_t device, int64_t capacity,
  fsph_status * status);
void fsph_destroy(fsph_ctx * ctx);
const char * fsph_status_string(int32_t status);
/* Last error detail of this context (CUDA error string etc.). */
const char * fsph_last_error(const fsph_ctx * ctx);

/* -- data movement ------------------------------------------------------- */
/* Host -> device copy of a full particle set (mpisph/bodies_system.h:83-89
 * read_bodies analogue); resets iteration/time to the params' initial ones.
 * With a periodic axis the set holds the real particles only, with ids
 * 0 .. n-1 (the reference's id-sum check, boundary.h:241-246), and the
 * capacity must leave room for the copies update_iteration appends. */
fsph_status fsph_upload(fsph_ctx * ctx, const fsph_soa_view * host);
/* Device -> host copy, current (sorted) order, periodic copies included
 * (host->n = the total of fsph_particle_count).  Synchronous. */
fsph_status fsph_download(fsph_ctx * ctx, fsph_soa_view * host);
/* Host -> device copy of the non-NULL fields of `host` (host->n must equal
 * the uploaded count) into the current particle order, keeping time,
 * iteration and tree state: the per-step input path of a host-side driver. */
fsph_status fsph_upload_fields(fsph_ctx * ctx, const fsph_soa_view * host);
/* The same three copies with the view's arrays in DEVICE memory of the
 * context's device (for instance another library's tensors): device to
 * device on the context's stream, the stream synchronised before
 * fsph_upload_device and fsph_download_device return.  The context's stream
 * does not wait for other streams: work that writes the arrays must be
 * complete before the call (synchronise the producing stream), and with
 * fsph_upload_fields_device the arrays must stay unchanged until the
 * context synchronises.  A multi-rank driver moves its exchanged particles
 * in and out this way without host staging. */
fsph_status fsph_upload_device(fsph_ctx * ctx, const fsph_soa_view * dev);
fsph_status fsph_download_device(fsph_ctx * ctx, fsph_soa_view * dev);
fsph_status fsph_upload_fields_device(fsph_ctx * ctx, const fsph_soa_view * dev);
/* Page-lock (pin) / release a host buffer so the copies above run at full
 * link speed.  Thin wrappers over cudaHostRegister/cudaHostUnregister. */
fsph_status fsph_host_register(void * ptr, int64_t bytes);
fsph_status fsph_host_unregister(void * ptr);
fsph_status fsph_get_time(fsph_ctx * ctx, double * dt, double * totaltime,
  int64_t * iteration);
fsph_status fsph_set_time(fsph_ctx * ctx, double dt, double totaltime,
  int64_t iteration);
/* Range [min0,min1,(min2),max0,max1,(max2)] of the last update_iteration. */
fsph_status fsph_get_range(fsph_ctx * ctx, double * range);

/* One iteration with its host copies: the non-NULL fields of `in` (host,
 * current particle order, as fsph_upload_fields) go in, the step runs, and
 * the non-NULL fields of `out` (host, n = the particle count) come back in
 * the order fsph_download gives.  The result equals fsph_upload_fields +
 * fsph_step + fsph_download; in a regular (not the initial) iteration
 * without periodic copies the copies overlap the step: input fields the
 * kick, drift and key sort do not touch go in on a second stream while those
 * run, and each output field goes out as soon as the step has written it
 * for the last time.  Synchronous: returns after `out` is complete, with the
 * step's device status. */
fsph_status fsph_step_io(fsph_ctx * ctx, const fsph_soa_view * in,
  fsph_soa_view * out);

/* -- body_system --------------------------------------------------------- */
fsph_status fsph_update_iteration(fsph_ctx * ctx);
fsph_status fsph_reset_ghosts(fsph_ctx * ctx);
/* apply_in_smoothinglength(...) */
/* physics::compute_density_pressure_soundspeed (default_physics.h:309-320):
 * density, EOS, signal speed and, with visc_cullen, compute_divv */
fsph_status fsph_density_pressure_soundspeed(fsph_ctx * ctx);
/* viscosity::compute_alpha (viscosity.h:310-363), visc_cullen only */
fsph_status fsph_compute_alpha(fsph_ctx * ctx);
/* apply_all(viscosity::initialize_alpha) (viscosity.h:171-177) */
fsph_status fsph_initialize_alpha(fsph_ctx * ctx);
fsph_status fsph_acceleration(fsph_ctx * ctx);
fsph_status fsph_dudt(fsph_ctx * ctx);
fsph_status fsph_dedt(fsph_ctx * ctx);
/* particle relaxation terms (default_physics.h:571-599,699-753), which the
 * hydro driver adds while iteration < relaxation_steps
 * (hydro/main_driver.cc:129-134,150-165,204-207): */
/* apply_all(physics::add_drag_acceleration) */
fsph_status fsph_add_drag_acceleration(fsph_ctx * ctx);
/* apply_in_smoothinglength(physics::add_short_range_repulsion) */
fsph_status fsph_add_short_range_repulsion(fsph_ctx * ctx);
/* apply_all(physics::add_drag_dedt) / apply_all(physics::add_drag_dudt) */
fsph_status fsph_add_drag_dedt(fsph_ctx * ctx);
fsph_status fsph_add_drag_dudt(fsph_ctx * ctx);
/* apply_all(...) */
fsph_status fsph_eos_init(fsph_ctx * ctx);
fsph_status fsph_set_total_energy(fsph_ctx * ctx);
fsph_status fsph_save_velocityhalf(fsph_ctx * ctx);
fsph_status fsph_leapfrog_kick_v(fsph_ctx * ctx);
fsph_status fsph_leapfrog_kick_u(fsph_ctx * ctx);
fsph_status fsph_leapfrog_kick_e(fsph_ctx * ctx);
fsph_status fsph_leapfrog_drift(fsph_ctx * ctx);
fsph_status fsph_recompute_pressure_soundspeed(fsph_ctx * ctx);
fsph_status fsph_recompute_pressure_soundspeed_thermokinetic(fsph_ctx * ctx);
fsph_status fsph_compute_dt(fsph_ctx * ctx);
fsph_status fsph_check_nans(fsph_ctx * ctx);
fsph_status fsph_check_negativity(fsph_ctx * ctx);
/* get_all(...) */
fsph_status fsph_set_adaptive_timestep(fsph_ctx * ctx);
fsph_status fsph_compute_smoothinglength(fsph_ctx * ctx);
fsph_status fsph_compute_average_smoothinglength(fsph_ctx * ctx);
/* gravitation_fmm(): multipole tree gravity, order params.gravity_order,
 * opening angle params.fmm_macangle; adds into g-acceleration/potential. */
fsph_status fsph_gravitation(fsph_ctx * ctx);
/* Gravity over ranks (a locally essential tree).  The reference shares
 * top-tree branches between MPI ranks and fetches remote subtrees in its
 * FMM walk (tree_topology.h:1142-1542,1550-1744).  Here each rank, after
 * fsph_gravitation on its own particles, exports for every other rank's
 * bounding box [box_lo, box_hi] (dimension doubles each) the cells of its
 * tree that are far enough for that whole box (r_max < theta * distance of
 * the centre of mass to the box) and the particles of the cells that are
 * not, as records of 10 doubles {m, c_x, c_y, c_z, Q_xx, Q_yy, Q_zz, Q_xy,
 * Q_xz, Q_yz} (traceless quadrupole about c, zero for a particle and with
 * gravity_order 1).  *count receives the number of records; at most
 * `capacity` are copied to `cells` (host or device memory; NULL with
 * capacity 0 to query).  Synchronous.  FSPH_ERR_STATE unless
 * fsph_gravitation ran after the last fsph_update_iteration. */
fsph_status fsph_gravity_export(fsph_ctx * ctx, const double * box_lo,
  const double * box_hi, double theta, double * cells, int64_t capacity,
  int64_t * count);
/* Adds the field of `ncell` such records (host or device memory, from the
 * other ranks; device records must be complete, as above) to the
 * g-acceleration and potential of every particle the context holds:
 * monopole plus quadrupole terms, G = gravitational_constant; a record at a
 * particle's own position adds nothing to it. */
fsph_status fsph_gravity_import(fsph_ctx * ctx, const double * cells, int64_t ncell);
/* physics::advance_time() */
fsph_status fsph_advance_time(fsph_ctx * ctx);

/* One whole driver iteration (the initial one when iteration ==
 * initial_iteration, else a leapfrog step), including advance_time. */
fsph_status fsph_step(fsph_ctx * ctx);
/* Synchronises and returns the first error any kernel raised since the
 * last call (device error words), then clears it. */
fsph_status fsph_sync(fsph_ctx * ctx);

/* -- inspection ---------------------------------------------------------- */
/* Neighbour lists of the last update_iteration in CSR form over the sorted
 * particle index: offsets[n+1], indices[total].  Pass indices == NULL to
 * query the total in offsets[n].  Each list is sorted ascending.  Sync. */
fsph_status fsph_get_neighbors(fsph_ctx * ctx, int64_t * offsets,
  int64_t * indices, int64_t capacity);
fsph_status fsph_conserved_sums(fsph_ctx * ctx, fsph_conserved * out);
fsph_status fsph_timers(fsph_ctx * ctx, double * ms, int32_t count,
  int64_t * launches);
fsph_status fsph_timers_reset(fsph_ctx * ctx);
/* Particles held: *total includes the periodic copies (WALL particles of
 * boundary.h) made by the last fsph_update_iteration, *real does not.
 * fsph_download wants total.  Without periodic axes both equal the uploaded
 * count. */
fsph_status fsph_particle_count(fsph_ctx * ctx, int64_t * total, int64_t * real);
/* Number of kernel launches this context has issued (all kinds). */
int64_t fsph_launch_count(const fsph_ctx * ctx);
/* Record CUDA event `slot` (0..63) on the context's stream; elapsed device
 * time between two recorded slots (synchronises on the later one). */
fsph_status fsph_mark(fsph_ctx * ctx, int32_t slot);
fsph_status fsph_mark_elapsed(fsph_ctx * ctx, int32_t from, int32_t to,
  double * ms);
/* Allocation-free variant of the range + Morton-key + radix-sort part of
 * fsph_update_iteration, with no counterpart in the reference.  For callers
 * that must not allocate device memory (an application whose device memory
 * belongs to its own pool allocator, or a time-critical loop where
 * cudaMalloc/cudaFree could synchronise the device).  Inputs x, y, z (NULL
 * in 2D) and h and outputs keys_out[n] (sorted Morton keys) and
 * perm_out[n] (input index of each sorted position) are DEVICE pointers of
 * the caller; work is enqueued on `stream` (a cudaStream_t, NULL = default)
 * of the current device.  Scratch is a fixed 12.25 MiB static device array
 * in the library, so n must be in [2, 1048576] (FSPH_ERR_ARG otherwise),
 * and every call shares it: calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  That address is kept for
 * the life of the process: do not call this entry point again on a device
 * after cudaDeviceReset (or any teardown of its primary context), which can
 * move the array.  Nothing is allocated.  Two differences from
 * fsph_update_iteration: equal keys keep their input order (the tie-break
 * is the input index; the reference's comparator, bodies_system.h:195-206,
 * breaks ties by id, which is the same order when ids ascend with the
 * input), and duplicate full keys are not reported (no
 * FSPH_ERR_DUPLICATE_KEY: the status word would need a synchronisation). */
fsph_status fsph_sort_keys_noalloc(const double * x, const double * y,
  const double * z, const double * h, int64_t n, int32_t dimension,
  uint64_t * keys_out, int32_t * perm_out, void * stream);
/* Measured arithmetic peak of `device`: kind 0 = FP64 FMA, 1 = FP32 FMA,
 * 2 = FP32 FMA through the packed FP32x2 instruction, in TFLOP/s (2 flops
 * per FMA), from a register-resident FMA chain kernel. */
fsph_status fsph_measure_peak(int32_t device, int32_t kind, double * tflops);

/* -- ensembles ----------------------------------------------------------- */
/* Many independent problems on one GPU (the reference runs one problem per
 * MPI job, app/drivers/hydro/main_driver.cc; a parameter study is many jobs).
 * Each member is an ordinary fsph_ctx owned by the ensemble: upload, download
 * and query it with the calls above.  fsph_ensemble_step advances every
 * member by whole driver iterations (fsph_step); after each member's initial
 * iteration and one regular one, the regular iteration of all members runs
 * as CUDA graphs, one launch per lane (stream).  Periodic members and
 * members with timers on step eagerly.  Members' own calls between steps are
 * allowed; a change of a member's state re-captures the graphs. */
typedef struct fsph_ensemble fsph_ensemble;
fsph_ensemble * fsph_ensemble_create(int32_t device, fsph_status * status);
/* Adds a problem with its own parameters and capacity; the returned context
 * is owned by the ensemble (never fsph_destroy it). */
fsph_ctx * fsph_ensemble_add(fsph_ensemble * ens, const fsph_params * params,
  int64_t capacity, fsph_status * status);
int32_t fsph_ensemble_size(const fsph_ensemble * ens);
fsph_ctx * fsph_ensemble_member(fsph_ensemble * ens, int32_t k);
fsph_status fsph_ensemble_step(fsph_ensemble * ens, int32_t nsteps);
/* Waits for every member; the first member with a device-side error gives
 * the status and its index (else -1). */
fsph_status fsph_ensemble_sync(fsph_ensemble * ens, int32_t * failed_member);
/* Members are spread over `lanes` streams by particle count; 0 turns the
 * graphs off (every member steps eagerly on its own stream). */
fsph_status fsph_ensemble_set_lanes(fsph_ensemble * ens, int32_t lanes);
/* Times steps_per_trial steps for 1, 2, 4, 8, 16 lanes (advancing every
 * member meanwhile) and keeps the fastest. */
fsph_status fsph_ensemble_tune(fsph_ensemble * ens, int32_t steps_per_trial,
  int32_t * lanes_chosen, double * ms_per_step);
/* Sets every member's walk-group size (fsph_params.group_size, 0..32). */
fsph_status fsph_ensemble_set_group_size(fsph_ensemble * ens, int32_t group_size);
/* fsph_ensemble_tune for each walk-group size 8, 16 and 32; keeps the
 * fastest (lanes, group size) pair. */
fsph_status fsph_ensemble_tune_shape(fsph_ensemble * ens, int32_t steps_per_trial,
  int32_t * lanes_chosen, int32_t * group_size_chosen, double * ms_per_step);
const char * fsph_ensemble_last_error(const fsph_ensemble * ens);
void fsph_ensemble_destroy(fsph_ensemble * ens);

#ifdef __cplusplus
}
#endif
#endif /* FSPH_H */
