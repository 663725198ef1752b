// fsph_api.cu -- the C ABI (include/fsph.h): context, data movement and the
// body_system / physics call surface, sequenced on one CUDA stream.
#include <cuda_runtime.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fsph_ctx.cuh"
#include "fsph_internal.cuh"
#include "fsph_eforce.cuh"

using namespace fsph;

namespace {

const int GROUP_MAX = 32;

}  // namespace

namespace {

fsph_status cuda_fail(fsph_ctx * c, cudaError_t e, const char * where) {
  if(c) {
    c->last_error = std::string(where) + ": " + cudaGetErrorString(e);
  }
  return e == cudaErrorMemoryAllocation ? FSPH_ERR_OOM : FSPH_ERR_CUDA;
}

#define CK(expr)                                                               \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if(e_ != cudaSuccess)                                                      \
      return cuda_fail(c, e_, #expr);                                          \
  } while(0)

template<class T>
cudaError_t dalloc(fsph_ctx * c, T ** p, size_t count) {
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
  if(e == cudaSuccess)
    c->allocs.push_back(*p);
  return e;
}

void phase_begin(fsph_ctx * c, int phase, int * tok) {
  *tok = -1;
  if(!c->timing)
    return;
  if(c->ev_used + 2 > (int)c->events.size()) {
    // flush: everything recorded so far is accumulated
    cudaStreamSynchronize(c->stream);
    for(auto & r : c->pending) {
      float ms = 0;
      cudaEventElapsedTime(&ms, c->events[r.e0], c->events[r.e1]);
      c->timer_ms[r.phase] += ms;
      c->timer_calls[r.phase] += 1;
    }
    c->pending.clear();
    c->ev_used = 0;
  }
  *tok = c->ev_used;
  cudaEventRecord(c->events[c->ev_used++], c->stream);
  (void)phase;
}

void phase_end(fsph_ctx * c, int phase, int tok) {
  if(!c->timing || tok < 0)
    return;
  int e1 = c->ev_used++;
  cudaEventRecord(c->events[e1], c->stream);
  c->pending.push_back(TimerRec{phase, tok, e1});
}

struct Phase {
  fsph_ctx * c;
  int phase, tok;
  Phase(fsph_ctx * c_, int ph) : c(c_), phase(ph) { phase_begin(c, ph, &tok); }
  ~Phase() { phase_end(c, phase, tok); }
};

void make_phys(const fsph_params * p, PhysParams * pp) {
  pp->dim = p->dimension;
  pp->kernel = p->sph_kernel;
  pp->eos = p->eos_type;
  pp->thermokinetic = p->thermokinetic_formulation;
  pp->evolve_u = p->evolve_internal_energy;
  pp->adaptive = p->adaptive_timestep;
  pp->gamma = p->poly_gamma;
  pp->eta = p->sph_eta;
  // kernels::select (kernels.h:753-786)
  pp->kw = (p->sph_kernel == FSPH_KERNEL_QUINTIC_SPLINE ||
            p->sph_kernel == FSPH_KERNEL_GAUSSIAN ||
            p->sph_kernel == FSPH_KERNEL_SUPER_GAUSSIAN) ? 3.0 : 2.0;
  // set_sinc_kernel_normalization (kernels.h:67-77)
  {
    const double b0[3] = {-1.5404568e-2, 5.2245027e-2, 2.7012593e-2};
    const double b1[3] = {3.6632876e-1, 1.3090245e-1, 2.0410827e-2};
    const double b2[3] = {-4.6519576e-4, 1.9358485e-2, 3.7451957e-3};
    const double b3[3] = {7.3658324e-2, -6.1642906e-3, 4.7013839e-2};
    const double si = p->sph_sinc_index, sq = sqrt(si), s2 = si * si;
    pp->sinc_index = si;
    pp->sinc_sigma[0] = 2. * (b0[0] + b1[0] * sq + b2[0] * si + b3[0] / sq);
    pp->sinc_sigma[1] = 4. * (b0[1] + b1[1] * si + b2[1] / si + b3[1] / s2);
    pp->sinc_sigma[2] = 8. * (b0[2] + b1[2] * sq + b2[2] * si + b3[2] * sq * si);
  }
  pp->alpha = p->sph_viscosity_alpha;
  pp->beta = p->sph_viscosity_beta;
  pp->eps = p->sph_viscosity_epsilon;
  pp->cullen = p->sph_viscosity == FSPH_VISC_CULLEN;
  pp->alpha_max = p->sph_viscosity_alpha_max;
  pp->visc_l = p->sph_viscosity_l;
  pp->visc_delta = p->sph_viscosity_delta;
  pp->cfl = p->timestep_cfl_factor;
  pp->gamma2 = p->poly_gamma2;
  pp->rho_thr = p->ppt_density_thr;
  pp->ppt_k2 = pow(p->ppt_density_thr, p->poly_gamma - p->poly_gamma2);
  pp->out_screen_dt = p->out_screen_dt;
  pp->out_scalar_dt = p->out_scalar_dt;
  pp->out_h5data_dt = p->out_h5data_dt;
  pp->G = p->gravitational_constant;
  // external forces (eforce.h) and the constants their functions cache
  pp->n_eforce = 0;
  pp->has_eacc = 0;
  for(int k = 0; k < FSPH_MAX_EFORCE && p->external_force[k] != FSPH_EFORCE_NONE; ++k) {
    pp->eforce[pp->n_eforce++] = p->external_force[k];
    if(p->external_force[k] != FSPH_EFORCE_POISON)
      pp->has_eacc = 1;
  }
  for(int k = pp->n_eforce; k < 8; ++k)
    pp->eforce[k] = FSPH_EFORCE_NONE;
  pp->ew_n = p->extforce_wall_powerindex;
  pp->ew_a = p->extforce_wall_steepness;
  pp->box_half[0] = .5 * p->box_length;
  pp->box_half[1] = .5 * p->box_width;
  pp->box_half[2] = .5 * p->box_height;
  pp->sphere_r = p->sphere_radius;
  pp->grav_acc = p->gravity_acceleration_constant;
  pp->poison = p->zero_potential_poison_value;
  pp->orb_a = p->orbital_separation;
  pp->orb_mns = p->mass_neutron_star;
  pp->orb_mwd = p->mass_white_dwarf;
  pp->af_size = p->airfoil_size;
  pp->af_thick = p->airfoil_thickness;
  pp->af_camber = p->airfoil_camber;
  pp->af_x = p->airfoil_anchor_x;
  pp->af_y = p->airfoil_anchor_y;
  pp->af_alpha = p->airfoil_attack_angle * FSPH_PI / 180.0;
  pp->dprof = p->density_profile;
  pp->mesa_q = p->mesa_rim_width;
  pp->mesa_rho0 = mesa_rho0_for(p->dimension, p->mesa_rim_width);
  pp->rho_init = p->rho_initial;
  pp->ds_K0 = p->pressure_initial / pow(p->rho_initial, p->poly_gamma);
  pp->ds_rho0 = dprof_rho(p->dimension, p->density_profile, 0., pp->mesa_q,
    pp->mesa_rho0);
  pp->relax_beta = p->relaxation_beta;
  pp->relax_gamma = p->relaxation_gamma;
  pp->rep_radius = p->relaxation_repulsion_radius;
  pp->rep_gamma = p->relaxation_repulsion_gamma;
  pp->relax_steps = p->relaxation_steps;
}

// analysis::set_initial_time_iteration (analysis.h:221-249)
void init_time(const fsph_params * p, DevTime * t) {
  memset(t, 0, sizeof(*t));
  t->iteration = p->initial_iteration;
  t->totaltime = p->initial_time;
  t->dt = p->initial_dt;
  auto snap = [&](double every, double * slot) {
    if(every > 0.0) {
      *slot = every * (double)((int64_t)(t->totaltime / every));
      if(*slot < t->totaltime)
        *slot = t->totaltime;
    }
  };
  snap(p->out_screen_dt, &t->t_screen);
  snap(p->out_scalar_dt, &t->t_scalar);
  snap(p->out_h5data_dt, &t->t_h5);
}

bool params_supported(const fsph_params * p, std::string * why) {
  if(p->dimension != 2 && p->dimension != 3) {
    *why = "dimension must be 2 or 3";
    return false;
  }
  if(p->sph_kernel < FSPH_KERNEL_CUBIC_SPLINE || p->sph_kernel > FSPH_KERNEL_SINC) {
    *why = "unknown sph_kernel";
    return false;
  }
  if(p->sph_kernel == FSPH_KERNEL_SINC && !(p->sph_sinc_index > 1.0)) {
    *why = "sph_sinc_index must exceed 1";
    return false;
  }
  if(p->eos_type < FSPH_EOS_IDEAL || p->eos_type > FSPH_EOS_NO_EOS) {
    *why = "unknown eos_type";
    return false;
  }
  if(p->sph_viscosity != FSPH_VISC_CONSTANT && p->sph_viscosity != FSPH_VISC_CULLEN) {
    *why = "sph_viscosity must be visc_constant or visc_cullen";
    return false;
  }
  if(p->relaxation_steps < 0) {
    *why = "relaxation_steps must be >= 0";
    return false;
  }
  for(int k = 0; k < FSPH_MAX_EFORCE && p->external_force[k] != FSPH_EFORCE_NONE; ++k) {
    const int32_t e = p->external_force[k];
    if(e < FSPH_EFORCE_WALLS_X || e > FSPH_EFORCE_POISON) {
      *why = "unknown external_force code";
      return false;
    }
    if(e == FSPH_EFORCE_WALLS_Z && p->dimension < 3) {
      *why = "walls:z needs three dimensions";
      return false;
    }
    if(e == FSPH_EFORCE_ORBIT && p->dimension != 3) {
      *why = "the orbit force is three-dimensional (eforce.h:279-298)";
      return false;
    }
    if(e == FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT &&
       (p->density_profile < FSPH_DENSITY_CONSTANT || p->density_profile > FSPH_DENSITY_MESA)) {
      *why = "density_profile must be constant, parabolic or mesa";
      return false;
    }
  }
  {
    const int per[3] = {p->periodic_boundary_x, p->periodic_boundary_y,
      p->periodic_boundary_z};
    const double len[3] = {p->box_length, p->box_width, p->box_height};
    for(int d = 0; d < 3; ++d)
      if(per[d] && (d >= p->dimension || !(len[d] > 0))) {
        *why = "a periodic axis needs d < dimension and a positive box size";
        return false;
      }
  }
  if(p->enable_fmm && (p->dimension != 3 || p->gravity_order < 1 ||
                        p->gravity_order > 2 || !(p->fmm_macangle >= 0))) {
    *why = "gravity needs 3D, gravity_order 1 or 2 and fmm_macangle >= 0";
    return false;
  }
  if(p->group_size < 0 || p->group_size > 32) {
    *why = "group_size out of [0, 32]";
    return false;
  }
  if(p->max_neighbors < 8 || p->max_neighbors > 4096) {
    *why = "max_neighbors out of [8, 4096]";
    return false;
  }
  if(p->precision_mode != FSPH_PRECISION_FP64 &&
     p->precision_mode != FSPH_PRECISION_MIXED) {
    *why = "precision_mode";
    return false;
  }
  return true;
}

fsph_status set_device(fsph_ctx * c) {
  CK(cudaSetDevice(c->device));
  return FSPH_OK;
}

}  // namespace

extern "C" {

void fsph_params_default(fsph_params * p) {
  memset(p, 0, sizeof(*p));
  p->dimension = 3;
  p->sph_kernel = FSPH_KERNEL_WENDLAND_C4;
  p->eos_type = FSPH_EOS_IDEAL;
  p->sph_viscosity = FSPH_VISC_CONSTANT;
  p->poly_gamma = 1.4;
  p->sph_eta = 1.5;
  p->sph_viscosity_alpha = 1.0;
  p->sph_viscosity_beta = 2.0;
  p->sph_viscosity_epsilon = 0.01;
  p->timestep_cfl_factor = 0.25;
  p->initial_dt = 0.001;
  p->gravitational_constant = 1.0;
  p->box_length = 3.0;
  p->box_width = 1.0;
  p->box_height = 1.0;
  p->thermokinetic_formulation = 1;
  p->evolve_internal_energy = 1;
  p->pressure_updates_number = 1;
  p->precision_mode = FSPH_PRECISION_FP64;
  p->max_neighbors = 256;
  p->gravity_order = 2;
  p->sph_viscosity_alpha_max = 1.0;
  p->sph_viscosity_l = 0.05;
  p->sph_viscosity_delta = 1.0;
  p->sph_sinc_index = 4.0;
  p->poly_gamma2 = 2.5;
  p->ppt_density_thr = 5e14;
  p->density_profile = FSPH_DENSITY_CONSTANT;
  p->extforce_wall_powerindex = 5.0;
  p->extforce_wall_steepness = 1e12;
  p->sphere_radius = 1.0;
  p->gravity_acceleration_constant = 9.81;
  p->orbital_separation = 2.5e9;
  p->mass_neutron_star = 1.26 * 1.988435e33;
  p->mass_white_dwarf = 1.10 * 1.988435e33;
  p->zero_potential_poison_value = 0.0;
  p->airfoil_size = 2.0;
  p->airfoil_thickness = 0.05;
  p->airfoil_camber = 0.1;
  p->airfoil_anchor_x = -1.0;
  p->airfoil_anchor_y = 0.0;
  p->airfoil_attack_angle = 0.0;
  p->rho_initial = 1.0;
  p->pressure_initial = 1.0;
  p->mesa_rim_width = 0.25;
  p->relaxation_beta = 1.e-6;
  p->relaxation_gamma = 0.0;
  p->relaxation_repulsion_radius = 0.25;
  p->relaxation_repulsion_gamma = 0.0;
}

// external_force::select (eforce.h:359-434): split at commas, match each
// term case-insensitively, "walls:" followed by up to three axis letters.
static bool ieq(const char * a, size_t na, const char * b) {
  if(strlen(b) != na)
    return false;
  for(size_t i = 0; i < na; ++i)
    if(tolower((unsigned char)a[i]) != tolower((unsigned char)b[i]))
      return false;
  return true;
}

fsph_status fsph_params_set_external_force(fsph_params * p, const char * spec) {
  if(!p || !spec)
    return FSPH_ERR_ARG;
  int32_t codes[FSPH_MAX_EFORCE];
  int n = 0;
  const size_t len = strlen(spec);
  auto push = [&](int32_t code) {
    if(n >= FSPH_MAX_EFORCE)
      return false;
    codes[n++] = code;
    return true;
  };
  if(!(ieq(spec, len, "zero") || ieq(spec, len, "none"))) {
    size_t start = 0;
    while(true) {
      size_t end = start;
      while(end < len && spec[end] != ',')
        ++end;
      const char * t = spec + start;
      const size_t tl = end - start;
      bool ok = true;
      if(ieq(t, tl, "spherical wall"))
        ok = push(FSPH_EFORCE_SPHERICAL_WALL);
      else if(ieq(t, tl, "airfoil"))
        ok = push(FSPH_EFORCE_AIRFOIL);
      else if(ieq(t, tl, "spherical density support"))
        ok = push(FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT);
      else if(ieq(t, tl, "gravity"))
        ok = push(FSPH_EFORCE_GRAVITY);
      else if(ieq(t, tl, "orbit"))
        ok = push(FSPH_EFORCE_ORBIT);
      else if(tl >= 6 && ieq(t, 6, "walls:")) {
        const size_t imx = tl - 6 < 3 ? tl - 6 : 3;
        for(size_t i = 0; ok && i < imx; ++i) {
          const char c = (char)tolower((unsigned char)t[6 + i]);
          if(c == 'x')
            ok = push(FSPH_EFORCE_WALLS_X);
          else if(c == 'y')
            ok = push(FSPH_EFORCE_WALLS_Y);
          else if(c == 'z')
            ok = push(FSPH_EFORCE_WALLS_Z);
          else
            ok = false;
        }
      }
      else if(ieq(t, tl, "poison"))
        ok = push(FSPH_EFORCE_POISON);
      else
        ok = false;
      if(!ok)
        return FSPH_ERR_ARG;
      if(end >= len)
        break;
      start = end + 1;
    }
  }
  for(int k = 0; k < FSPH_MAX_EFORCE; ++k)
    p->external_force[k] = k < n ? codes[k] : FSPH_EFORCE_NONE;
  return FSPH_OK;
}

int32_t fsph_abi_version(void) { return FSPH_ABI_VERSION; }

const char * fsph_status_string(int32_t s) {
  switch(s) {
    case FSPH_OK: return "FSPH_OK";
    case FSPH_ERR_ARG: return "FSPH_ERR_ARG";
    case FSPH_ERR_CUDA: return "FSPH_ERR_CUDA";
    case FSPH_ERR_NAN: return "FSPH_ERR_NAN";
    case FSPH_ERR_NEG_DENSITY: return "FSPH_ERR_NEG_DENSITY";
    case FSPH_ERR_NEG_ENERGY: return "FSPH_ERR_NEG_ENERGY";
    case FSPH_ERR_NEGATIVITY: return "FSPH_ERR_NEGATIVITY";
    case FSPH_ERR_LIST_OVERFLOW: return "FSPH_ERR_LIST_OVERFLOW";
    case FSPH_ERR_STACK_OVERFLOW: return "FSPH_ERR_STACK_OVERFLOW";
    case FSPH_ERR_TIMEOUT: return "FSPH_ERR_TIMEOUT";
    case FSPH_ERR_DUPLICATE_KEY: return "FSPH_ERR_DUPLICATE_KEY";
    case FSPH_ERR_DT: return "FSPH_ERR_DT";
    case FSPH_ERR_STATE: return "FSPH_ERR_STATE";
    case FSPH_ERR_NO_DEVICE: return "FSPH_ERR_NO_DEVICE";
    case FSPH_ERR_OOM: return "FSPH_ERR_OOM";
  }
  return "unknown";
}

const char * fsph_last_error(const fsph_ctx * c) {
  return c ? c->last_error.c_str() : "";
}

fsph_ctx * fsph_create(const fsph_params * p, int32_t device, int64_t capacity,
  fsph_status * status) {
  fsph_status dummy;
  if(!status)
    status = &dummy;
  std::string why;
  if(!p || capacity < 2 || capacity > (int64_t)1 << 30 || !params_supported(p, &why)) {
    *status = FSPH_ERR_ARG;
    return nullptr;
  }
  int ndev = 0;
  if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    *status = FSPH_ERR_NO_DEVICE;
    return nullptr;
  }
  fsph_ctx * c = new fsph_ctx();
  c->p = *p;
  make_phys(p, &c->pp);
  c->device = device;
  c->cap = capacity;
  auto fail = [&](fsph_status s) {
    fsph_destroy(c);
    *status = s;
    return (fsph_ctx *)nullptr;
  };
  if(cudaSetDevice(device) != cudaSuccess)
    return fail(FSPH_ERR_CUDA);
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  if(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FSPH_ERR_CUDA);
  const size_t N = (size_t)capacity;
  const size_t Npad = (N + 31) / 32 * 32;
  bool ok = true;
  for(int k = 0; k < NF; ++k) {
    ok &= dalloc(c, &c->P.f[k], N) == cudaSuccess;
    ok &= dalloc(c, &c->Palt.f[k], N) == cudaSuccess;
  }
  ok &= dalloc(c, &c->P.id, N) == cudaSuccess;
  ok &= dalloc(c, &c->Palt.id, N) == cudaSuccess;
  ok &= dalloc(c, &c->P.key, N) == cudaSuccess;
  ok &= dalloc(c, &c->Palt.key, N) == cudaSuccess;
  ok &= dalloc(c, &c->cs_new, N) == cudaSuccess;
  ok &= dalloc(c, &c->skeys, N) == cudaSuccess;
  ok &= dalloc(c, &c->skeys_tmp, N) == cudaSuccess;
  ok &= dalloc(c, &c->svals, N) == cudaSuccess;
  ok &= dalloc(c, &c->svals_tmp, N) == cudaSuccess;
  ok &= dalloc(c, &c->hist, radix_hist_entries((int)N)) == cudaSuccess;
  ok &= dalloc(c, &c->d_range, 8) == cudaSuccess;
  ok &= dalloc(c, &c->T.left, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.right, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.parent, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.leaf_parent, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.first, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.last, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.qbox, 2 * N) == cudaSuccess;
  ok &= dalloc(c, &c->T.box2, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.fbox2, 2 * N) == cudaSuccess;
  ok &= dalloc(c, &c->T.opar, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.gref, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.counter, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.edepth, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.group_first, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.group_last, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.group_start, N) == cudaSuccess;
  ok &= dalloc(c, &c->T.ngroups, 1) == cudaSuccess;
  ok &= dalloc(c, &c->K.qpos, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.vhm, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.vel, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.thermo, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.mass, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.velp, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.rc, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fv1, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fv2, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fdv, N) == cudaSuccess;
  if(c->pp.cullen)
    ok &= dalloc(c, &c->K.visc, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.qscale, 4) == cudaSuccess;
  ok &= dalloc(c, &c->K.fph, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fpl, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fmA, N) == cudaSuccess;
  ok &= dalloc(c, &c->K.fscale, 3) == cudaSuccess;
  // (c->mixed is set further down: decide from the parameters)
  if(p->precision_mode == FSPH_PRECISION_MIXED)
    ok &= dalloc(c, &c->K.ahyd, 3 * N) == cudaSuccess;
  c->periodic = p->periodic_boundary_x || p->periodic_boundary_y ||
                p->periodic_boundary_z;
  if(c->periodic) {
    ok &= dalloc(c, &c->PS.flag, N) == cudaSuccess;
    ok &= dalloc(c, &c->PS.pos, N) == cudaSuccess;
    ok &= dalloc(c, &c->PS.perm, N) == cudaSuccess;
    ok &= dalloc(c, &c->PS.tiles, (size_t)scan_tiles((int)N) + 1) == cudaSuccess;
    ok &= dalloc(c, &c->PS.total, 1) == cudaSuccess;
    ok &= dalloc(c, &c->PS.hbits, 1) == cudaSuccess;
  }
  if(p->enable_fmm) {
    ok &= dalloc(c, &c->grav.gn, N) == cudaSuccess;
    ok &= dalloc(c, &c->grav.gnf, 4 * N) == cudaSuccess;
    ok &= dalloc(c, &c->grav.gpk, 2 * N) == cudaSuccess;
    ok &= dalloc(c, &c->T.gmom, 10 * N) == cudaSuccess;
  }
  c->mixed = p->precision_mode == FSPH_PRECISION_MIXED;
  c->Ls.maxnb = (p->max_neighbors + 3) & ~3;  // whole chunks of four slots
  ok &= dalloc(c, &c->Ls.idx, Npad * (size_t)c->Ls.maxnb) == cudaSuccess;
  ok &= dalloc(c, &c->Ls.cnt, N) == cudaSuccess;
  ok &= dalloc(c, &c->d_time, 1) == cudaSuccess;
  ok &= dalloc(c, &c->d_status, 1) == cudaSuccess;
  ok &= dalloc(c, &c->d_cons, 8 * (1 + CONS_BLOCKS)) == cudaSuccess;
  if(!ok) {
    cudaGetLastError();
    return fail(FSPH_ERR_OOM);
  }
  if(cudaMemset(c->d_status, 0, sizeof(DevStatus)) != cudaSuccess)
    return fail(FSPH_ERR_CUDA);
  // timer and mark events are made on first use: an ensemble holds hundreds
  // of contexts that never time themselves
  *status = FSPH_OK;
  return c;
}

void fsph_destroy(fsph_ctx * c) {
  if(!c)
    return;
  cudaSetDevice(c->device);
  // both streams drain before any buffer they may still touch is freed
  if(c->stream)
    cudaStreamSynchronize(c->stream);
  if(c->io.stream)
    cudaStreamSynchronize(c->io.stream);
  for(void * p : c->allocs)
    cudaFree(p);
  if(c->let_buf)
    cudaFree(c->let_buf);
  for(auto & e : c->events)
    if(e)
      cudaEventDestroy(e);
  for(auto & e : c->marks)
    if(e)
      cudaEventDestroy(e);
  if(c->io.stream) {
    for(auto & e : c->io.ev)
      if(e)
        cudaEventDestroy(e);
    cudaStreamDestroy(c->io.stream);
  }
  if(c->stream)
    cudaStreamDestroy(c->stream);
  delete c;
}

// The view's arrays are host memory (kind cudaMemcpyHostToDevice) or device
// memory of the context's device (cudaMemcpyDeviceToDevice).
static fsph_status upload_impl(fsph_ctx * c, const fsph_soa_view * v,
  cudaMemcpyKind kind) {
  if(!c || !v || v->n < 2 || v->n > c->cap || !v->x || !v->y ||
     (c->p.dimension == 3 && !v->z) || !v->m || !v->h || !v->id)
    return FSPH_ERR_ARG;
  c->ahyd_ok = false;
  c->fv_ok = c->fdv_ok = c->vel_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  const int n = (int)v->n;
  if(c->periodic) {
    // the copies are told apart by id: the real particles must hold 0..n-1
    std::vector<long long> ids((size_t)n);
    if(kind == cudaMemcpyHostToDevice)
      std::memcpy(ids.data(), v->id, sizeof(long long) * n);
    else
      CK(cudaMemcpy(ids.data(), v->id, sizeof(long long) * n, cudaMemcpyDeviceToHost));
    std::vector<char> seen((size_t)n, 0);
    for(int i = 0; i < n; ++i) {
      const long long id = ids[i];
      if(id < 0 || id >= n || seen[(size_t)id]) {
        c->last_error = "periodic boundaries need the ids 0 .. n-1";
        return FSPH_ERR_ARG;
      }
      seen[(size_t)id] = 1;
    }
  }
  c->nreal = n;
  c->n = n;
  c->P.n = c->Palt.n = n;
  const double * src[NF] = {v->x, v->y, v->z, v->vx, v->vy, v->vz, v->vhx,
    v->vhy, v->vhz, v->ax, v->ay, v->az, v->gax, v->gay, v->gaz, v->gpot, v->m,
    v->h, v->rho, v->P, v->cs, v->u, v->e, v->dudt, v->dedt, v->K, v->alpha,
    v->vsig, v->dt, v->divv, v->ddivvdt, v->Ye};
  for(int k = 0; k < NF; ++k) {
    if(src[k])
      CK(cudaMemcpyAsync(c->P.f[k], src[k], sizeof(double) * n, kind, c->stream));
    else
      CK(cudaMemsetAsync(c->P.f[k], 0, sizeof(double) * n, c->stream));
  }
  CK(cudaMemcpyAsync(c->P.id, v->id, sizeof(long long) * n, kind, c->stream));
  CK(cudaMemsetAsync(c->P.key, 0, sizeof(unsigned long long) * n, c->stream));
  DevTime t;
  init_time(&c->p, &t);
  CK(cudaMemcpyAsync(c->d_time, &t, sizeof(t), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(DevStatus), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->iteration = c->p.initial_iteration;
  c->tree_ok = false;
  c->uploaded = true;
  return FSPH_OK;
}

fsph_status fsph_upload(fsph_ctx * c, const fsph_soa_view * v) {
  return upload_impl(c, v, cudaMemcpyHostToDevice);
}

fsph_status fsph_upload_device(fsph_ctx * c, const fsph_soa_view * v) {
  return upload_impl(c, v, cudaMemcpyDeviceToDevice);
}

static fsph_status upload_fields_impl(fsph_ctx * c, const fsph_soa_view * v,
  cudaMemcpyKind kind) {
  if(!c || !v || !c->uploaded || v->n != c->n)
    return FSPH_ERR_ARG;
  c->ahyd_ok = false;
  c->fv_ok = c->fdv_ok = c->vel_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  const int n = c->n;
  const double * src[NF] = {v->x, v->y, v->z, v->vx, v->vy, v->vz, v->vhx,
    v->vhy, v->vhz, v->ax, v->ay, v->az, v->gax, v->gay, v->gaz, v->gpot, v->m,
    v->h, v->rho, v->P, v->cs, v->u, v->e, v->dudt, v->dedt, v->K, v->alpha,
    v->vsig, v->dt, v->divv, v->ddivvdt, v->Ye};
  for(int k = 0; k < NF; ++k)
    if(src[k])
      CK(cudaMemcpyAsync(c->P.f[k], src[k], sizeof(double) * n, kind, c->stream));
  if(v->id)
    CK(cudaMemcpyAsync(c->P.id, v->id, sizeof(long long) * n, kind, c->stream));
  return FSPH_OK;
}

fsph_status fsph_upload_fields(fsph_ctx * c, const fsph_soa_view * v) {
  return upload_fields_impl(c, v, cudaMemcpyHostToDevice);
}

fsph_status fsph_upload_fields_device(fsph_ctx * c, const fsph_soa_view * v) {
  return upload_fields_impl(c, v, cudaMemcpyDeviceToDevice);
}

fsph_status fsph_host_register(void * ptr, int64_t bytes) {
  if(!ptr || bytes <= 0)
    return FSPH_ERR_ARG;
  cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
  return e == cudaSuccess ? FSPH_OK : FSPH_ERR_CUDA;
}

fsph_status fsph_host_unregister(void * ptr) {
  if(!ptr)
    return FSPH_ERR_ARG;
  return cudaHostUnregister(ptr) == cudaSuccess ? FSPH_OK : FSPH_ERR_CUDA;
}

fsph_status fsph_mark(fsph_ctx * c, int32_t slot) {
  if(!c || slot < 0 || slot >= 64)
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  if(!c->marks[slot])
    CK(cudaEventCreate(&c->marks[slot]));
  CK(cudaEventRecord(c->marks[slot], c->stream));
  return FSPH_OK;
}

fsph_status fsph_mark_elapsed(fsph_ctx * c, int32_t a, int32_t b, double * ms) {
  if(!c || !ms || a < 0 || a >= 64 || b < 0 || b >= 64)
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  if(!c->marks[a] || !c->marks[b])
    return FSPH_ERR_STATE;
  CK(cudaEventSynchronize(c->marks[b]));
  float f = 0;
  CK(cudaEventElapsedTime(&f, c->marks[a], c->marks[b]));
  *ms = f;
  return FSPH_OK;
}

fsph_status fsph_sync(fsph_ctx * c) {
  if(!c)
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaGetLastError());
  DevStatus st;
  CK(cudaMemcpy(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost));
  if(st.code) {
    char buf[128];
    snprintf(buf, sizeof(buf), "%s at particle %lld",
      fsph_status_string(st.code), st.index);
    c->last_error = buf;
    CK(cudaMemset(c->d_status, 0, sizeof(DevStatus)));
    return (fsph_status)st.code;
  }
  return FSPH_OK;
}

static fsph_status download_impl(fsph_ctx * c, fsph_soa_view * v,
  cudaMemcpyKind kind) {
  if(!c || !v || v->n != c->n || !c->uploaded)
    return FSPH_ERR_ARG;
  fsph_status s = fsph_sync(c);
  if(s)
    return s;
  const int n = c->n;
  double * dst[NF] = {v->x, v->y, v->z, v->vx, v->vy, v->vz, v->vhx, v->vhy,
    v->vhz, v->ax, v->ay, v->az, v->gax, v->gay, v->gaz, v->gpot, v->m, v->h,
    v->rho, v->P, v->cs, v->u, v->e, v->dudt, v->dedt, v->K, v->alpha, v->vsig,
    v->dt, v->divv, v->ddivvdt, v->Ye};
  for(int k = 0; k < NF; ++k) {
    if(k == F_Z || k == F_VZ || k == F_VHZ || k == F_AZ || k == F_GAZ)
      if(c->p.dimension == 2)
        continue;
    if(dst[k])
      CK(cudaMemcpyAsync(dst[k], c->P.f[k], sizeof(double) * n, kind, c->stream));
  }
  if(v->id)
    CK(cudaMemcpyAsync(v->id, c->P.id, sizeof(long long) * n, kind, c->stream));
  if(v->key)
    CK(cudaMemcpyAsync(v->key, c->P.key, sizeof(unsigned long long) * n, kind,
      c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return FSPH_OK;
}

fsph_status fsph_download(fsph_ctx * c, fsph_soa_view * v) {
  return download_impl(c, v, cudaMemcpyDeviceToHost);
}

fsph_status fsph_download_device(fsph_ctx * c, fsph_soa_view * v) {
  return download_impl(c, v, cudaMemcpyDeviceToDevice);
}

fsph_status fsph_get_time(fsph_ctx * c, double * dt, double * tt,
  int64_t * it) {
  fsph_status s = fsph_sync(c);
  if(s)
    return s;
  DevTime t;
  CK(cudaMemcpy(&t, c->d_time, sizeof(t), cudaMemcpyDeviceToHost));
  if(dt) *dt = t.dt;
  if(tt) *tt = t.totaltime;
  if(it) *it = t.iteration;
  return FSPH_OK;
}

fsph_status fsph_set_time(fsph_ctx * c, double dt, double tt, int64_t it) {
  fsph_status s = fsph_sync(c);
  if(s)
    return s;
  DevTime t;
  CK(cudaMemcpy(&t, c->d_time, sizeof(t), cudaMemcpyDeviceToHost));
  t.dt = dt;
  t.totaltime = tt;
  t.iteration = it;
  CK(cudaMemcpy(c->d_time, &t, sizeof(t), cudaMemcpyHostToDevice));
  c->iteration = it;
  return FSPH_OK;
}

fsph_status fsph_get_range(fsph_ctx * c, double * range) {
  if(!c || !range || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = fsph_sync(c);
  if(s)
    return s;
  unsigned long long bits[6];
  CK(cudaMemcpy(bits, c->d_range, sizeof(bits), cudaMemcpyDeviceToHost));
  const int D = c->p.dimension;
  for(int k = 0; k < 2; ++k)
    for(int d = 0; d < D; ++d) {
      unsigned long long u = bits[3 * k + d];
      long long b = (u & 0x8000000000000000ull)
                      ? (long long)(u & 0x7fffffffffffffffull)
                      : (long long)~u;
      double x;
      memcpy(&x, &b, 8);
      range[k * D + d] = x;
    }
  return FSPH_OK;
}

// ------------------------------------------------------------ body_system
static bool wendland(int k);

fsph_status fsph_update_iteration(fsph_ctx * c) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  c->ahyd_ok = false;
  c->fv_ok = c->fdv_ok = c->vel_ok = false;
  c->grav_nodes_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  if(c->periodic) {
    // boundary::pboundary_clean + pboundary_generate (bodies_system.h:160-169)
    Phase ph(c, FSPH_TIMER_PERIODIC);
    const double len[3] = {c->p.box_length, c->p.box_width, c->p.box_height};
    const int per[3] = {c->p.periodic_boundary_x, c->p.periodic_boundary_y,
      c->p.periodic_boundary_z};
    int ntot = 0;
    const char * why = nullptr;
    CK(launch_periodic(L, c->P, c->Palt, c->pp, len, per, c->nreal, (int)c->cap,
      c->PS, &ntot, &why, c->permute_skip));
    if(why) {
      c->last_error = std::string(why) + ": need " + std::to_string(ntot) +
                      ", capacity " + std::to_string(c->cap);
      c->tree_ok = false;
      c->n = c->P.n;  // the copies of the last iteration are gone
      return FSPH_ERR_ARG;
    }
    c->n = ntot;
  }
  const int n = c->n;
  {
    Phase ph(c, FSPH_TIMER_RANGE_KEYS);
    CK(launch_range_keys(L, c->P, c->pp, (double *)c->d_range, c->skeys, c->svals));
  }
  {
    Phase ph(c, FSPH_TIMER_SORT);
    CK(radix_sort_pairs(L, c->skeys, c->svals, c->skeys_tmp, c->svals_tmp, n,
      c->hist, 0));
    CK(launch_check_duplicates(L, c->skeys, n, c->d_status));
    if(c->io.h2d_pending) {
      // fsph_step_io: input fields copied on the copy stream land first
      CK(cudaStreamWaitEvent(c->stream, c->io.ev[0], 0));
      c->io.h2d_pending = false;
    }
    // the mixed float-float path's {v, c_s} records come out of the permute
    float4 * vel = c->mixed && wendland(c->pp.kernel) ? c->K.vel : nullptr;
    CK(launch_permute(L, c->P, c->Palt, c->svals, c->skeys, c->permute_skip, vel,
      c->pp.dim));
    c->vel_ok = vel != nullptr;
    Particles t = c->P;
    c->P = c->Palt;
    c->Palt = t;
  }
  {
    Phase ph(c, FSPH_TIMER_TREE);
    CK(launch_pack_positions(L, c->P, c->pp, c->d_range, c->K));
    CK(launch_build_tree(L, c->P, c->pp, c->T,
      c->p.group_size > 0 ? c->p.group_size : GROUP_MAX, c->d_range, c->K.qpos,
      c->K.qscale, c->mixed ? 0 : 1));
  }
  {
    // FP64 mode keeps each list in the reference's order so its sums round
    // like the reference's; the mixed path only needs the set
    Phase ph(c, FSPH_TIMER_NEIGHBORS);
    CK(launch_neighbors(L, c->P, c->pp, c->T, c->Ls, c->d_status, c->nsm,
      c->d_range, c->K, c->mixed ? 0 : 1));
  }
  c->tree_ok = true;
  return FSPH_OK;
}

fsph_status fsph_reset_ghosts(fsph_ctx * c) {
  // bodies_system::reset_ghosts rebuilds the tree over unchanged keys to
  // refresh MPI ghosts (mpisph/bodies_system.h:273-275); on one device the
  // tree and the neighbour lists it would produce are the ones held already.
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  return FSPH_OK;
}

static fsph_status elem(fsph_ctx * c, int op, int phase);

// viscosity::initialize_alpha over all particles (viscosity.h:171-177).
fsph_status fsph_initialize_alpha(fsph_ctx * c) {
  return elem(c, OP_INIT_ALPHA, FSPH_TIMER_INTEGRATE);
}

// apply_in_smoothinglength(viscosity::compute_alpha) (viscosity.h:310-363).
fsph_status fsph_compute_alpha(fsph_ctx * c) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  if(!c->pp.cullen) {
    c->last_error = "compute_alpha needs sph_viscosity = visc_cullen";
    return FSPH_ERR_STATE;
  }
  c->ahyd_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_DENSITY);
  if(c->mixed)
    CK(launch_alpha_mixed(L, c->P, c->pp, c->Ls, c->K, c->d_time));
  else
    CK(launch_alpha_cullen(L, c->P, c->pp, c->Ls, c->d_time));
  return FSPH_OK;
}

static fsph_status density_impl(fsph_ctx * c, bool with_vsig) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  c->ahyd_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  if(c->mixed) {
    {
      Phase ph(c, FSPH_TIMER_DENSITY);
      CK(launch_density_mixed(L, c->P, c->pp, c->Ls, c->K, c->cs_new, c->d_status,
        c->d_time, c->vel_ok ? 1 : 0));
    }
    if(with_vsig) {
      Phase ph(c, FSPH_TIMER_VSIG);
      CK(launch_vsig_mixed(L, c->P, c->pp, c->Ls, c->K));
    }
  }
  else {
    {
      Phase ph(c, FSPH_TIMER_DENSITY);
      CK(launch_density_fp64(L, c->P, c->pp, c->Ls, c->cs_new, c->d_status, c->d_time));
    }
    Phase ph(c, FSPH_TIMER_VSIG);
    CK(launch_vsig_fp64(L, c->P, c->pp, c->Ls, c->cs_new));
  }
  // the new sound speed becomes the particle's sound speed
  double * t = c->P.f[F_CS];
  c->P.f[F_CS] = c->cs_new;
  c->cs_new = t;
  // the float-float density pass (Wendland kernels) wrote the fv records;
  // the sound speeds in K.vel are now the previous ones
  c->fv_ok = c->mixed && wendland(c->pp.kernel);
  c->vel_ok = false;
  return FSPH_OK;
}

fsph_status fsph_density_pressure_soundspeed(fsph_ctx * c) {
  return density_impl(c, true);
}

static bool wendland(int k) {
  return k == FSPH_KERNEL_WENDLAND_C2 || k == FSPH_KERNEL_WENDLAND_C4 ||
         k == FSPH_KERNEL_WENDLAND_C6;
}

static fsph_status accel_impl(fsph_ctx * c, int kick, int fused_vsig = 0) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_ACCEL);
  if(c->mixed)
    CK(launch_accel_mixed(L, c->P, c->pp, c->Ls, c->K, kick, c->d_time, fused_vsig,
      c->fv_ok ? 1 : 0));
  else
    CK(launch_accel_fp64(L, c->P, c->pp, c->Ls, kick, c->d_time));
  // the float-float pass (Wendland kernels) leaves the pressure-only
  // acceleration in K.ahyd for the de/dt pass, and with the kick the
  // {v - v_half, m} records of the kicked velocities
  c->ahyd_ok = c->mixed && c->K.ahyd && wendland(c->pp.kernel);
  c->fv_ok = c->fv_ok || (c->mixed && wendland(c->pp.kernel));
  c->fdv_ok = c->mixed && wendland(c->pp.kernel) && kick;
  return FSPH_OK;
}

fsph_status fsph_acceleration(fsph_ctx * c) { return accel_impl(c, 0); }

fsph_status fsph_dudt(fsph_ctx * c) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_ENERGY);
  if(c->mixed)
    CK(launch_dudt_mixed(L, c->P, c->pp, c->Ls, c->K, c->d_time, 0, c->fv_ok ? 1 : 0,
      c->fdv_ok ? 1 : 0));
  else
    CK(launch_dudt_fp64(L, c->P, c->pp, c->Ls, c->d_time));
  return FSPH_OK;
}

fsph_status fsph_dedt(fsph_ctx * c) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_ENERGY);
  if(c->mixed)
    CK(launch_dedt_mixed(L, c->P, c->pp, c->Ls, c->K, 0, c->d_time, c->d_status,
      c->ahyd_ok ? 1 : 0, c->fdv_ok ? 1 : 0));
  else
    CK(launch_dedt_fp64(L, c->P, c->pp, c->Ls));
  return FSPH_OK;
}

// de/dt (du/dt) followed by the element-wise update `op`
// (OP_RECOMPUTE_THERMO or OP_RECOMPUTE_KICK_E; OP_RECOMPUTE or
// OP_RECOMPUTE_KICK_U): one pass on the mixed path, two on the FP64 path
// (whose update stays in the -fmad=false element-wise unit).
static fsph_status energy_then(fsph_ctx * c, bool thermo, int op) {
  if(!c->mixed) {
    const fsph_status s0 = thermo ? fsph_dedt(c) : fsph_dudt(c);
    return s0 ? s0 : elem(c, op, FSPH_TIMER_INTEGRATE);
  }
  if(!c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_ENERGY);
  if(thermo)
    CK(launch_dedt_mixed(L, c->P, c->pp, c->Ls, c->K, op, c->d_time, c->d_status,
      c->ahyd_ok ? 1 : 0, c->fdv_ok ? 1 : 0));
  else
    CK(launch_dudt_mixed(L, c->P, c->pp, c->Ls, c->K, c->d_time, op, c->fv_ok ? 1 : 0,
      c->fdv_ok ? 1 : 0));
  // the pressure update of `op` changes P/rho^2 and c_s
  c->ahyd_ok = false;
  c->fv_ok = c->vel_ok = false;
  return FSPH_OK;
}

fsph_status fsph_add_drag_acceleration(fsph_ctx * c) {
  return elem(c, OP_DRAG_ACC, FSPH_TIMER_ACCEL);
}

fsph_status fsph_add_drag_dedt(fsph_ctx * c) {
  return elem(c, OP_DRAG_DEDT, FSPH_TIMER_ENERGY);
}

fsph_status fsph_add_drag_dudt(fsph_ctx * c) {
  return elem(c, OP_DRAG_DUDT, FSPH_TIMER_ENERGY);
}

fsph_status fsph_add_short_range_repulsion(fsph_ctx * c) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_ACCEL);
  CK(launch_repulsion(L, c->P, c->pp, c->Ls));
  return FSPH_OK;
}

static fsph_status elem(fsph_ctx * c, int op, int phase) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  // every update of positions, P/rho^2, v_half, alpha or h outdates the
  // pressure-only acceleration the de/dt pass would reuse
  // (and the fv records), and any change of v the fdv records
  if(op != OP_KICK_V && op != OP_KICK_E && op != OP_KICK_U &&
     op != OP_SET_TOTAL_ENERGY && op != OP_DRAG_ACC && op != OP_DRAG_DEDT &&
     op != OP_DRAG_DUDT && op != OP_CHECK_NANS && op != OP_CHECK_NEGATIVITY)
    c->ahyd_ok = c->fv_ok = c->fdv_ok = c->vel_ok = false;
  if(op == OP_KICK_V)
    c->fdv_ok = c->vel_ok = false;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, phase);
  CK(launch_elementwise(L, c->P, c->pp, op, c->d_time, c->d_status));
  return FSPH_OK;
}

fsph_status fsph_eos_init(fsph_ctx * c) { return elem(c, OP_EOS_INIT, FSPH_TIMER_INTEGRATE); }
fsph_status fsph_set_total_energy(fsph_ctx * c) {
  return elem(c, OP_SET_TOTAL_ENERGY, FSPH_TIMER_INTEGRATE);
}
fsph_status fsph_save_velocityhalf(fsph_ctx * c) {
  return elem(c, OP_SAVE_VHALF, FSPH_TIMER_INTEGRATE);
}
fsph_status fsph_leapfrog_kick_v(fsph_ctx * c) { return elem(c, OP_KICK_V, FSPH_TIMER_INTEGRATE); }
fsph_status fsph_leapfrog_kick_u(fsph_ctx * c) { return elem(c, OP_KICK_U, FSPH_TIMER_INTEGRATE); }
fsph_status fsph_leapfrog_kick_e(fsph_ctx * c) { return elem(c, OP_KICK_E, FSPH_TIMER_INTEGRATE); }
fsph_status fsph_leapfrog_drift(fsph_ctx * c) { return elem(c, OP_DRIFT, FSPH_TIMER_INTEGRATE); }
fsph_status fsph_recompute_pressure_soundspeed(fsph_ctx * c) {
  return elem(c, OP_RECOMPUTE, FSPH_TIMER_INTEGRATE);
}
fsph_status fsph_recompute_pressure_soundspeed_thermokinetic(fsph_ctx * c) {
  return elem(c, OP_RECOMPUTE_THERMO, FSPH_TIMER_INTEGRATE);
}
fsph_status fsph_check_nans(fsph_ctx * c) { return elem(c, OP_CHECK_NANS, FSPH_TIMER_DT); }
fsph_status fsph_check_negativity(fsph_ctx * c) {
  return elem(c, OP_CHECK_NEGATIVITY, FSPH_TIMER_DT);
}
fsph_status fsph_compute_smoothinglength(fsph_ctx * c) {
  return elem(c, OP_SMOOTHING_LENGTH, FSPH_TIMER_INTEGRATE);
}

fsph_status fsph_compute_average_smoothinglength(fsph_ctx * c) {
  fsph_status s = elem(c, OP_SMOOTHING_LENGTH, FSPH_TIMER_INTEGRATE);
  if(s)
    return s;
  Launch L = c->L();
  CK(launch_hsum(L, c->P, c->d_time));
  return elem(c, OP_SET_H, FSPH_TIMER_INTEGRATE);
}

fsph_status fsph_compute_dt(fsph_ctx * c) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_DT);
  CK(launch_compute_dt(L, c->P, c->pp, c->d_time, c->d_status, 0, c->mixed));
  return FSPH_OK;
}

// compute_dt preceded by check_nans and check_negativity in one pass
static fsph_status checks_and_dt(fsph_ctx * c) {
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_DT);
  CK(launch_compute_dt(L, c->P, c->pp, c->d_time, c->d_status, 1, c->mixed));
  return FSPH_OK;
}

fsph_status fsph_set_adaptive_timestep(fsph_ctx * c) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  CK(launch_set_adaptive_timestep(L, c->pp, c->d_time));
  return FSPH_OK;
}

fsph_status fsph_advance_time(fsph_ctx * c) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  CK(launch_advance_time(L, c->pp, c->d_time));
  c->iteration++;
  return FSPH_OK;
}

fsph_status fsph_gravitation(fsph_ctx * c) {
  if(!c || !c->tree_ok)
    return FSPH_ERR_STATE;
  if(!c->grav.gn) {
    c->last_error = "context created without enable_fmm";
    return FSPH_ERR_STATE;
  }
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_GRAVITY);
  CK(launch_gravity(L, c->P, c->pp, c->T, c->grav, c->d_range, c->p.fmm_macangle,
    c->p.gravity_order, c->mixed ? 1 : 0, c->d_status, c->nsm));
  c->grav_nodes_ok = c->n >= 2;
  return FSPH_OK;
}

static fsph_status let_reserve(fsph_ctx * c, long long records) {
  if(records <= c->let_cap)
    return FSPH_OK;
  if(c->let_buf) {
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(c->let_buf);
    c->let_buf = nullptr;
    c->let_cap = 0;
  }
  CK(cudaMalloc((void **)&c->let_buf, sizeof(double) * 10 * (size_t)records));
  c->let_cap = records;
  return FSPH_OK;
}

fsph_status fsph_gravity_export(fsph_ctx * c, const double * box_lo,
  const double * box_hi, double theta, double * cells, int64_t capacity,
  int64_t * count) {
  if(!c || !box_lo || !box_hi || !count || capacity < 0 || (capacity > 0 && !cells) ||
     !(theta >= 0.0))
    return FSPH_ERR_ARG;
  if(!c->grav_nodes_ok) {
    c->last_error = "gravity_export needs fsph_gravitation after the last tree build";
    return FSPH_ERR_STATE;
  }
  fsph_status s = set_device(c);
  if(s)
    return s;
  // a walk emits at most every node and every particle once
  const long long most = 2ll * c->n;
  s = let_reserve(c, most);
  if(s)
    return s;
  if(!c->let_count)
    CK(dalloc(c, &c->let_count, 1));
  Launch L = c->L();
  CK(launch_let_export(L, c->P, c->p.dimension, c->T, c->grav, box_lo, box_hi, theta,
    c->p.gravity_order, c->let_buf, most, c->let_count, c->d_status));
  unsigned long long got = 0;
  CK(cudaMemcpyAsync(&got, c->let_count, sizeof(got), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  s = fsph_sync(c);
  if(s)
    return s;
  *count = (int64_t)got;
  const long long take = (long long)got < capacity ? (long long)got : capacity;
  if(take > 0)
    CK(cudaMemcpy(cells, c->let_buf, sizeof(double) * 10 * (size_t)take, cudaMemcpyDefault));
  return FSPH_OK;
}

fsph_status fsph_gravity_import(fsph_ctx * c, const double * cells, int64_t ncell) {
  if(!c || ncell < 0 || (ncell > 0 && !cells))
    return FSPH_ERR_ARG;
  if(!c->uploaded)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  if(ncell == 0)
    return FSPH_OK;
  s = let_reserve(c, ncell);
  if(s)
    return s;
  Launch L = c->L();
  Phase ph(c, FSPH_TIMER_GRAVITY);
  CK(cudaMemcpyAsync(c->let_buf, cells, sizeof(double) * 10 * (size_t)ncell,
    cudaMemcpyDefault, c->stream));
  CK(launch_let_apply(L, c->P, c->p.dimension, c->let_buf, ncell,
    c->p.gravitational_constant, c->mixed ? 1 : 0));
  return FSPH_OK;
}

#define TRY(x)                                                                 \
  do {                                                                         \
    fsph_status s_ = (x);                                                      \
    if(s_) return s_;                                                          \
  } while(0)

// One iteration of the driver loop (app/drivers/hydro/main_driver.cc:98-279;
// newtonian/main_driver.cc:103-298 when enable_fmm).  Elementwise steps that
// the reference runs back to back are fused; every fusion only combines
// ---- fsph_step_io ---------------------------------------------------------
enum { IO_UPDATE = 1, IO_DENSITY = 2, IO_ACCEL = 3, IO_ENERGY = 4, IO_END = 5 };

static double ** view_fields(const fsph_soa_view * v, double ** f) {
  double * const src[NF] = {v->x, v->y, v->z, v->vx, v->vy, v->vz, v->vhx,
    v->vhy, v->vhz, v->ax, v->ay, v->az, v->gax, v->gay, v->gaz, v->gpot, v->m,
    v->h, v->rho, v->P, v->cs, v->u, v->e, v->dudt, v->dedt, v->K, v->alpha,
    v->vsig, v->dt, v->divv, v->ddivvdt, v->Ye};
  for(int k = 0; k < NF; ++k)
    f[k] = src[k];
  return f;
}

// The stage of a regular iteration of fsph_step after which field k is not
// written again: the drift and the permute of update_iteration, the density
// pass (and the alpha pass), the acceleration (with gravity, relaxation and
// the velocity kick), the energy passes with the pressure updates and the
// energy kick, and the h and dt updates at the end.
static int io_final_stage(const fsph_ctx * c, int k) {
  const fsph_params & p = c->p;
  const bool thermo = p.thermokinetic_formulation, evolve = p.evolve_internal_energy;
  const bool cullen = c->pp.cullen;
  switch(k) {
    case F_X: case F_Y: case F_Z: case F_VHX: case F_VHY: case F_VHZ:
    case F_M: case F_K: case F_YE:
      return IO_UPDATE;
    case F_H:
      return (p.sph_variable_h || p.sph_update_uniform_h) ? IO_END : IO_UPDATE;
    case F_DUDT:
      return (evolve && !thermo) ? IO_ENERGY : IO_UPDATE;
    case F_DEDT:
      return (evolve && thermo) ? IO_ENERGY : IO_UPDATE;
    case F_E:
      return (evolve && thermo) ? IO_ENERGY : IO_UPDATE;
    case F_U:
      return evolve ? IO_ENERGY : IO_UPDATE;
    case F_P: case F_CS:
      return evolve ? IO_ENERGY : IO_ACCEL;
    case F_ALPHA:
      return cullen ? IO_ACCEL : IO_UPDATE;
    case F_DIVV: case F_DDIVVDT:
      return cullen ? IO_DENSITY : IO_UPDATE;
    case F_RHO:
      return IO_DENSITY;
    case F_AX: case F_AY: case F_AZ: case F_GAX: case F_GAY: case F_GAZ:
    case F_GPOT: case F_VX: case F_VY: case F_VZ: case F_VSIG:
      return IO_ACCEL;
    default:  // dt
      return IO_END;
  }
}

// Send the output fields that are final at `stage` on the copy stream, after
// the work enqueued so far on the context's stream.
static fsph_status io_stage(fsph_ctx * c, int stage) {
  if(!c->io.active)
    return FSPH_OK;
  CK(cudaEventRecord(c->io.ev[stage], c->stream));
  CK(cudaStreamWaitEvent(c->io.stream, c->io.ev[stage], 0));
  double * dst[NF];
  view_fields(&c->io.out, dst);
  const size_t bytes = sizeof(double) * (size_t)c->n;
  for(int k = 0; k < NF; ++k) {
    if(!dst[k] || c->io.sent[k] || io_final_stage(c, k) > stage)
      continue;
    if(c->p.dimension == 2 &&
       (k == F_Z || k == F_VZ || k == F_VHZ || k == F_AZ || k == F_GAZ))
      continue;
    CK(cudaMemcpyAsync(dst[k], c->P.f[k], bytes, cudaMemcpyDeviceToHost, c->io.stream));
    c->io.sent[k] = true;
  }
  if(c->io.out.id && !c->io.sent[NF]) {
    CK(cudaMemcpyAsync(c->io.out.id, c->P.id, sizeof(long long) * c->n,
      cudaMemcpyDeviceToHost, c->io.stream));
    c->io.sent[NF] = true;
  }
  if(c->io.out.key && !c->io.sent[NF + 1]) {
    CK(cudaMemcpyAsync(c->io.out.key, c->P.key, sizeof(unsigned long long) * c->n,
      cudaMemcpyDeviceToHost, c->io.stream));
    c->io.sent[NF + 1] = true;
  }
  return FSPH_OK;
}

fsph_status fsph_step_io(fsph_ctx * c, const fsph_soa_view * in, fsph_soa_view * out) {
  if(!c || !c->uploaded || !out || (in && in->n != c->n))
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  const bool overlap = c->iteration != c->p.initial_iteration && !c->periodic &&
                       out->n == c->n;
  if(!overlap) {
    if(in)
      TRY(fsph_upload_fields(c, in));
    TRY(fsph_step(c));
    return fsph_download(c, out);
  }
  if(!c->io.stream) {
    CK(cudaStreamCreateWithFlags(&c->io.stream, cudaStreamNonBlocking));
    for(int k = 0; k < 8; ++k)
      CK(cudaEventCreateWithFlags(&c->io.ev[k], cudaEventDisableTiming));
  }
  if(in) {
    // fields the kick, drift, range, keys and sort read or write go in
    // first on the context's stream, the rest on the copy stream, which the
    // permute waits for
    double * src[NF];
    view_fields(in, src);
    const size_t bytes = sizeof(double) * (size_t)c->n;
    bool late_any = false;
    CK(cudaEventRecord(c->io.ev[6], c->stream));
    CK(cudaStreamWaitEvent(c->io.stream, c->io.ev[6], 0));
    for(int k = 0; k < NF; ++k) {
      if(!src[k])
        continue;
      const bool early = k <= F_GAZ || k == F_H || k == F_U || k == F_E ||
                         k == F_DUDT || k == F_DEDT;
      CK(cudaMemcpyAsync(c->P.f[k], src[k], bytes, cudaMemcpyHostToDevice,
        early ? c->stream : c->io.stream));
      late_any = late_any || !early;
    }
    if(in->id)
      CK(cudaMemcpyAsync(c->P.id, in->id, sizeof(long long) * c->n,
        cudaMemcpyHostToDevice, c->stream));
    if(late_any) {
      CK(cudaEventRecord(c->io.ev[0], c->io.stream));
      c->io.h2d_pending = true;
    }
  }
  c->io.active = true;
  c->io.out = *out;
  for(int k = 0; k < NF + 2; ++k)
    c->io.sent[k] = false;
  s = fsph_step(c);
  if(!s)
    s = io_stage(c, IO_END);
  c->io.active = false;
  if(c->io.h2d_pending) {  // the step stopped before the permute
    cudaStreamWaitEvent(c->stream, c->io.ev[0], 0);
    c->io.h2d_pending = false;
  }
  // the context's stream continues after the copies
  CK(cudaEventRecord(c->io.ev[7], c->io.stream));
  CK(cudaStreamWaitEvent(c->stream, c->io.ev[7], 0));
  if(s)
    return s;
  return fsph_sync(c);
}

// per-particle updates whose inputs the fused pass does not read from
// neighbours.
fsph_status fsph_step(fsph_ctx * c) {
  if(!c || !c->uploaded)
    return FSPH_ERR_STATE;
  const fsph_params & p = c->p;
  const bool thermo = p.thermokinetic_formulation;
  const bool evolve = p.evolve_internal_energy;
  const bool grav = p.enable_fmm;
  const bool cullen = c->pp.cullen;
  // particle relaxation terms (hydro/main_driver.cc:129-134,150-165,
  // 204-207,219-234); the newtonian driver has none
  const bool relax = !grav && c->iteration < p.relaxation_steps;
  if(c->iteration == p.initial_iteration) {
    TRY(fsph_update_iteration(c));
    TRY(fsph_eos_init(c));
    if(thermo)
      TRY(fsph_set_total_energy(c));
    if(cullen)
      TRY(fsph_initialize_alpha(c));
    // mixed: the signal speed rides in the acceleration loop
    TRY(density_impl(c, !c->mixed));
    TRY(fsph_save_velocityhalf(c));
    if(cullen)
      TRY(fsph_compute_alpha(c));
    TRY(accel_impl(c, 0, c->mixed));
    if(relax) {
      TRY(fsph_add_drag_acceleration(c));
      TRY(fsph_add_short_range_repulsion(c));
    }
    if(grav) {
      // newtonian/main_driver.cc:137-151: gravity, then total energy again
      TRY(fsph_gravitation(c));
      if(thermo)
        TRY(fsph_set_total_energy(c));
    }
    if(p.adaptive_timestep) {
      TRY(fsph_compute_dt(c));
      TRY(fsph_set_adaptive_timestep(c));
    }
    if(evolve) {
      for(int m = 1; m <= p.pressure_updates_number; ++m) {
        if(thermo) {
          if(relax) {
            TRY(fsph_dedt(c));
            TRY(fsph_add_drag_dedt(c));
            TRY(elem(c, OP_RECOMPUTE_THERMO, FSPH_TIMER_INTEGRATE));
          }
          else
            TRY(energy_then(c, true, OP_RECOMPUTE_THERMO));
        }
        else if(relax) {
          TRY(fsph_dudt(c));
          TRY(fsph_add_drag_dudt(c));
          TRY(elem(c, OP_RECOMPUTE, FSPH_TIMER_INTEGRATE));
        }
        else
          TRY(energy_then(c, false, OP_RECOMPUTE));
      }
    }
  }
  else {
    TRY(elem(c, !evolve ? OP_KICK_DRIFT_NONE : (thermo ? OP_KICK_DRIFT_E : OP_KICK_DRIFT_U),
      FSPH_TIMER_INTEGRATE));
    // fields the rest of the iteration writes before reading stay behind
    // in the permute
    unsigned skip = (1u << F_AX) | (1u << F_AY) | (1u << F_GAX) | (1u << F_GAY) |
                    (1u << F_GPOT) | (1u << F_RHO) | (1u << F_VSIG);
    if(p.dimension == 3)
      skip |= (1u << F_AZ) | (1u << F_GAZ);
    if(p.adaptive_timestep)
      skip |= 1u << F_DT;
    if(p.eos_type != FSPH_EOS_NO_EOS)
      skip |= 1u << F_P;
    if(evolve && thermo)
      skip |= (1u << F_DEDT) | (1u << F_U);
    if(evolve && !thermo)
      skip |= 1u << F_DUDT;
    c->permute_skip = skip;
    const fsph_status us = fsph_update_iteration(c);
    c->permute_skip = 0;
    TRY(us);
    TRY(io_stage(c, IO_UPDATE));
    TRY(density_impl(c, !c->mixed));
    if(cullen)
      TRY(fsph_compute_alpha(c));
    TRY(io_stage(c, IO_DENSITY));
    if(grav) {
      // newtonian/main_driver.cc:217-227: gravity between the hydro
      // acceleration and the velocity kick
      TRY(accel_impl(c, 0, c->mixed));
      TRY(fsph_gravitation(c));
      TRY(fsph_leapfrog_kick_v(c));
    }
    else if(relax) {
      TRY(accel_impl(c, 0, c->mixed));
      TRY(fsph_add_drag_acceleration(c));
      TRY(fsph_add_short_range_repulsion(c));
      TRY(fsph_leapfrog_kick_v(c));
    }
    else
      TRY(accel_impl(c, 1, c->mixed));
    TRY(io_stage(c, IO_ACCEL));
    if(evolve) {
      for(int m = 1; m <= p.pressure_updates_number; ++m) {
        const bool lastp = m == p.pressure_updates_number;
        if(thermo) {
          const int op = lastp ? OP_RECOMPUTE_KICK_E : OP_RECOMPUTE_THERMO;
          if(relax) {
            TRY(fsph_dedt(c));
            TRY(fsph_add_drag_dedt(c));
            TRY(elem(c, op, FSPH_TIMER_INTEGRATE));
          }
          else
            TRY(energy_then(c, true, op));
        }
        else {
          const int op = lastp ? OP_RECOMPUTE_KICK_U : OP_RECOMPUTE;
          if(relax) {
            TRY(fsph_dudt(c));
            TRY(fsph_add_drag_dudt(c));
            TRY(elem(c, op, FSPH_TIMER_INTEGRATE));
          }
          else
            TRY(energy_then(c, false, op));
        }
      }
    }
  }
  TRY(io_stage(c, IO_ENERGY));
  if(p.sph_variable_h)
    TRY(fsph_compute_smoothinglength(c));
  else if(p.sph_update_uniform_h)
    TRY(fsph_compute_average_smoothinglength(c));
  if(p.adaptive_timestep) {
    TRY(checks_and_dt(c));
    TRY(fsph_set_adaptive_timestep(c));
  }
  else {
    TRY(fsph_check_nans(c));
    TRY(fsph_check_negativity(c));
  }
  return fsph_advance_time(c);
}

fsph_status fsph_get_neighbors(fsph_ctx * c, int64_t * offsets,
  int64_t * indices, int64_t capacity) {
  if(!c || !offsets || !c->tree_ok)
    return FSPH_ERR_STATE;
  fsph_status s = fsph_sync(c);
  if(s)
    return s;
  const int n = c->n;
  std::vector<int> cnt(n);
  CK(cudaMemcpy(cnt.data(), c->Ls.cnt, sizeof(int) * n, cudaMemcpyDeviceToHost));
  offsets[0] = 0;
  for(int i = 0; i < n; ++i)
    offsets[i + 1] = offsets[i] + cnt[i];
  if(!indices)
    return FSPH_OK;
  if(offsets[n] > capacity)
    return FSPH_ERR_ARG;
  const size_t npad = ((size_t)n + 31) / 32 * 32;
  std::vector<int> raw(npad * (size_t)c->Ls.maxnb);
  CK(cudaMemcpy(raw.data(), c->Ls.idx, sizeof(int) * raw.size(),
    cudaMemcpyDeviceToHost));
  for(int i = 0; i < n; ++i)
    for(int j = 0; j < cnt[i]; ++j)
      indices[offsets[i] + j] = raw[list_slot(i, j, c->Ls.maxnb)];
  return FSPH_OK;
}

fsph_status fsph_conserved_sums(fsph_ctx * c, fsph_conserved * out) {
  if(!c || !out || !c->uploaded)
    return FSPH_ERR_STATE;
  fsph_status s = set_device(c);
  if(s)
    return s;
  Launch L = c->L();
  CK(launch_conserved(L, c->P, c->pp, c->d_cons,
    c->periodic ? c->nreal : (long long)INT64_MAX));
  s = fsph_sync(c);
  if(s)
    return s;
  double v[8];
  CK(cudaMemcpy(v, c->d_cons, sizeof(v), cudaMemcpyDeviceToHost));
  out->mass = v[0];
  out->energy = v[1];
  for(int d = 0; d < 3; ++d) {
    out->momentum[d] = v[2 + d];
    out->angular_momentum[d] = v[5 + d];
  }
  return FSPH_OK;
}

fsph_status fsph_timers(fsph_ctx * c, double * ms, int32_t count,
  int64_t * launches) {
  if(!c)
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  CK(cudaStreamSynchronize(c->stream));
  for(auto & r : c->pending) {
    float e = 0;
    CK(cudaEventElapsedTime(&e, c->events[r.e0], c->events[r.e1]));
    c->timer_ms[r.phase] += e;
    c->timer_calls[r.phase] += 1;
  }
  c->pending.clear();
  c->ev_used = 0;
  for(int k = 0; k < count && k < FSPH_TIMER_COUNT; ++k) {
    if(ms)
      ms[k] = c->timer_ms[k];
    if(launches)
      launches[k] = c->timer_calls[k];
  }
  return FSPH_OK;
}

fsph_status fsph_timers_reset(fsph_ctx * c) {
  if(!c)
    return FSPH_ERR_ARG;
  fsph_status s = set_device(c);
  if(s)
    return s;
  CK(cudaStreamSynchronize(c->stream));
  if(c->events.empty()) {
    c->events.resize(4096);
    for(auto & e : c->events)
      CK(cudaEventCreate(&e));
  }
  c->pending.clear();
  c->ev_used = 0;
  for(int k = 0; k < FSPH_TIMER_COUNT; ++k) {
    c->timer_ms[k] = 0;
    c->timer_calls[k] = 0;
  }
  c->timing = true;
  return FSPH_OK;
}

int64_t fsph_launch_count(const fsph_ctx * c) { return c ? c->launches : 0; }

fsph_status fsph_particle_count(fsph_ctx * c, int64_t * total, int64_t * real) {
  if(!c)
    return FSPH_ERR_ARG;
  if(total)
    *total = c->n;
  if(real)
    *real = c->uploaded ? c->nreal : 0;
  return FSPH_OK;
}

}  // extern "C"
