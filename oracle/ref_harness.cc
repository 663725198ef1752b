/*
 * ref_harness.cc -- the reference's own hot-path code behind the oracle API.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `ref`)
 * directly from the laristra/flecsph headers where they lie, against the
 * single-rank stubs in oracle/stubs/, into oracle/_ref/libfsph_ref{2,3}.so.
 * Nothing of the reference is copied here: this file only calls the
 * reference's tree_topology, physics, eos, integration and viscosity code
 * and replays body_system::update_iteration (mpisph/bodies_system.h:152-229,
 * one-rank branch) and the driver loop (app/drivers/hydro/main_driver.cc:
 * 98-279), because bodies_system.h itself needs HDF5 (mpisph/io.h).
 *
 * The reference keeps its state in globals (param::, physics::), so one
 * context at a time per process.
 */
#include <mpi.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "params.h"
#include "tree.h"
#include "default_physics.h"

extern "C" {
#include "fsph_oracle.h"
}

struct orc_ctx {
  fsph_params p;
  tree_topology_t * tree;
  range_t range;
  bool built;
  std::vector<int64_t> order;
};

/* the external_force_type string whose select() gives the code list */
static std::string external_force_string(const fsph_params * p) {
  static const char * name[] = {"", "walls:x", "walls:y", "walls:z", "spherical wall",
    "spherical density support", "gravity", "airfoil", "orbit", "poison"};
  std::string out;
  for(int k = 0; k < FSPH_MAX_EFORCE && p->external_force[k] != FSPH_EFORCE_NONE; ++k) {
    if(!out.empty())
      out += ",";
    out += name[p->external_force[k]];
  }
  return out.empty() ? std::string("none") : out;
}

static void set_params(const fsph_params * p) {
  using namespace param;
  _poly_gamma = p->poly_gamma;
  _poly_gamma2 = p->poly_gamma2;
  _ppt_density_thr = p->ppt_density_thr;
  _sph_eta = p->sph_eta;
  _sph_kernel = (sph_kernel_keyword)p->sph_kernel;
  _eos_type = (eos_type_keyword)p->eos_type;
  _sph_viscosity = p->sph_viscosity == FSPH_VISC_CULLEN ? visc_cullen : visc_constant;
  _sph_viscosity_alpha_max = p->sph_viscosity_alpha_max;
  _sph_viscosity_l = p->sph_viscosity_l;
  _sph_viscosity_delta = p->sph_viscosity_delta;
  _sph_sinc_index = p->sph_sinc_index;
  _sph_viscosity_alpha = p->sph_viscosity_alpha;
  _sph_viscosity_beta = p->sph_viscosity_beta;
  _sph_viscosity_epsilon = p->sph_viscosity_epsilon;
  _timestep_cfl_factor = p->timestep_cfl_factor;
  _initial_dt = p->initial_dt;
  _initial_time = (int64_t)p->initial_time;
  _final_time = p->final_time;
  _out_screen_dt = p->out_screen_dt;
  _out_scalar_dt = p->out_scalar_dt;
  _out_h5data_dt = p->out_h5data_dt;
  _fmm_macangle = p->fmm_macangle;
  _gravitational_constant = p->gravitational_constant;
  _initial_iteration = p->initial_iteration;
  _final_iteration = p->final_iteration;
  _adaptive_timestep = p->adaptive_timestep;
  _thermokinetic_formulation = p->thermokinetic_formulation;
  _evolve_internal_energy = p->evolve_internal_energy;
  _pressure_updates_number = p->pressure_updates_number;
  _sph_variable_h = p->sph_variable_h;
  _sph_update_uniform_h = p->sph_update_uniform_h;
  _relaxation_steps = p->relaxation_steps;
  _enable_fmm = p->enable_fmm;
  _box_length = p->box_length;
  _box_width = p->box_width;
  _box_height = p->box_height;
  _periodic_boundary_x = p->periodic_boundary_x;
  _periodic_boundary_y = p->periodic_boundary_y;
  _periodic_boundary_z = p->periodic_boundary_z;
  fmm::gc = p->gravitational_constant;
  _extforce_wall_powerindex = p->extforce_wall_powerindex;
  _extforce_wall_steepness = p->extforce_wall_steepness;
  _sphere_radius = p->sphere_radius;
  _gravity_acceleration_constant = p->gravity_acceleration_constant;
  _orbital_separation = p->orbital_separation;
  _mass_neutron_star = p->mass_neutron_star;
  _mass_white_dwarf = p->mass_white_dwarf;
  _zero_potential_poison_value = p->zero_potential_poison_value;
  _airfoil_size = p->airfoil_size;
  _airfoil_thickness = p->airfoil_thickness;
  _airfoil_camber = p->airfoil_camber;
  _airfoil_anchor_x = p->airfoil_anchor_x;
  _airfoil_anchor_y = p->airfoil_anchor_y;
  _airfoil_attack_angle = p->airfoil_attack_angle;
  _rho_initial = p->rho_initial;
  _pressure_initial = p->pressure_initial;
  _mesa_rim_width = p->mesa_rim_width;
  _relaxation_beta = p->relaxation_beta;
  _relaxation_gamma = p->relaxation_gamma;
  _relaxation_repulsion_radius = p->relaxation_repulsion_radius;
  _relaxation_repulsion_gamma = p->relaxation_repulsion_gamma;
  {
    static const char * prof[] = {"constant", "parabolic", "mesa"};
    std::snprintf(_density_profile, STRING_MAXLEN, "%s",
      prof[p->density_profile >= 0 && p->density_profile <= 2 ? p->density_profile : 0]);
  }
  kernels::select();
  viscosity::select();
  eos::select();
  external_force::select(external_force_string(p));
  /* analysis::set_initial_time_iteration (analysis.h:221-249) */
  physics::iteration = initial_iteration;
  physics::totaltime = initial_time;
  physics::dt = initial_dt;
  physics::dt_saved = 0.0;
  physics::t_screen_output = 0;
  physics::t_scalar_output = 0;
  physics::t_h5data_output = 0;
}

template<class F>
static int apply_all(orc_ctx * c, F f) {
  for(auto & b : c->tree->entities())
    f(b);
  return FSPH_OK;
}

extern "C" {

orc_ctx * orc_create(const fsph_params * p) {
  if(!p || p->dimension != (int)gdimension)
    return nullptr;
  orc_ctx * c = new orc_ctx();
  c->p = *p;
  c->tree = new tree_topology_t();
  c->built = false;
  set_params(p);
  return c;
}

void orc_destroy(orc_ctx * c) {
  if(!c)
    return;
  delete c->tree;
  delete c;
}

int orc_set_threads(orc_ctx *, int) { return FSPH_OK; }

int orc_upload(orc_ctx * c, const fsph_soa_view * v) {
  if(!v || v->n < 2)
    return FSPH_ERR_ARG;
  set_params(&c->p);
  auto & ents = c->tree->entities();
  ents.clear();
  ents.resize(v->n);
  const double * xs[3] = {v->x, v->y, v->z};
  const double * vs[3] = {v->vx, v->vy, v->vz};
  const double * vhs[3] = {v->vhx, v->vhy, v->vhz};
  const double * as[3] = {v->ax, v->ay, v->az};
  const double * gas[3] = {v->gax, v->gay, v->gaz};
  auto get = [](const double * a, int64_t i) { return a ? a[i] : 0.0; };
  for(int64_t i = 0; i < v->n; ++i) {
    body & b = ents[i];
    point_t x, vv, vh, a, ga;
    for(size_t d = 0; d < gdimension; ++d) {
      x[d] = xs[d][i];
      vv[d] = get(vs[d], i);
      vh[d] = get(vhs[d], i);
      a[d] = get(as[d], i);
      ga[d] = get(gas[d], i);
    }
    b.set_coordinates(x);
    b.setVelocity(vv);
    b.setVelocityhalf(vh);
    b.setAcceleration(a);
    b.setGAcceleration(ga);
    b.setGPotential(get(v->gpot, i));
    b.set_mass(v->m[i]);
    b.set_radius(v->h[i]);
    b.setDensity(get(v->rho, i));
    b.setPressure(get(v->P, i));
    b.setSoundspeed(get(v->cs, i));
    b.setInternalenergy(get(v->u, i));
    b.setTotalenergy(get(v->e, i));
    b.setDudt(get(v->dudt, i));
    b.setDedt(get(v->dedt, i));
    b.setAdiabatic(get(v->K, i));
    b.setAlpha(get(v->alpha, i));
    b.setSignalspeed(get(v->vsig, i));
    b.setDt(get(v->dt, i));
    b.setDivergenceV(get(v->divv, i));
    b.setDdivvdt(get(v->ddivvdt, i));
    b.setEntropy(0.0);
    b.setTemperature(0.0);
    b.setElectronfraction(get(v->Ye, i));
    b.setDadt(0.0);
    b.set_id(v->id[i]);
    b.setType(NORMAL);
  }
  c->built = false;
  return FSPH_OK;
}

int orc_download(orc_ctx * c, fsph_soa_view * v) {
  auto & ents = c->tree->entities();
  if(!v || v->n != (int64_t)ents.size())
    return FSPH_ERR_ARG;
  double * xs[3] = {v->x, v->y, v->z};
  double * vs[3] = {v->vx, v->vy, v->vz};
  double * vhs[3] = {v->vhx, v->vhy, v->vhz};
  double * as[3] = {v->ax, v->ay, v->az};
  double * gas[3] = {v->gax, v->gay, v->gaz};
  for(int64_t i = 0; i < v->n; ++i) {
    body & b = ents[i];
    for(size_t d = 0; d < gdimension; ++d) {
      if(xs[d]) xs[d][i] = b.coordinates()[d];
      if(vs[d]) vs[d][i] = b.getVelocity()[d];
      if(vhs[d]) vhs[d][i] = b.getVelocityhalf()[d];
      if(as[d]) as[d][i] = b.getAcceleration()[d];
      if(gas[d]) gas[d][i] = b.getGAcceleration()[d];
    }
    if(v->gpot) v->gpot[i] = b.getGPotential();
    if(v->m) v->m[i] = b.mass();
    if(v->h) v->h[i] = b.radius();
    if(v->rho) v->rho[i] = b.getDensity();
    if(v->P) v->P[i] = b.getPressure();
    if(v->cs) v->cs[i] = b.getSoundspeed();
    if(v->u) v->u[i] = b.getInternalenergy();
    if(v->e) v->e[i] = b.getTotalenergy();
    if(v->dudt) v->dudt[i] = b.getDudt();
    if(v->dedt) v->dedt[i] = b.getDedt();
    if(v->K) v->K[i] = b.getAdiabatic();
    if(v->alpha) v->alpha[i] = b.getAlpha();
    if(v->vsig) v->vsig[i] = b.getSignalspeed();
    if(v->dt) v->dt[i] = b.getDt();
    if(v->divv) v->divv[i] = b.getDivergenceV();
    if(v->ddivvdt) v->ddivvdt[i] = b.getDdivvdt();
    if(v->Ye) v->Ye[i] = b.getElectronfraction();
    if(v->id) v->id[i] = (int64_t)b.id();
    if(v->key) v->key[i] = b.key().value();
  }
  return FSPH_OK;
}

int orc_get_time(orc_ctx *, double * dt, double * t, int64_t * it) {
  if(dt) *dt = physics::dt;
  if(t) *t = physics::totaltime;
  if(it) *it = physics::iteration;
  return FSPH_OK;
}

int orc_set_time(orc_ctx *, double dt, double t, int64_t it) {
  physics::dt = dt;
  physics::totaltime = t;
  physics::iteration = it;
  return FSPH_OK;
}

int orc_get_range(orc_ctx * c, double * r) {
  for(size_t d = 0; d < gdimension; ++d) {
    r[d] = c->range[0][d];
    r[gdimension + d] = c->range[1][d];
  }
  return FSPH_OK;
}

/* bodies_system::mpi_compute_range (bodies_system.h:231-268) is a member of
 * a class this harness cannot include; its one-rank arithmetic is replayed. */
static void compute_range(std::vector<body> & bodies, range_t & range) {
  range_t lrange;
  lrange[1] = bodies.back().coordinates();
  lrange[0] = bodies.back().coordinates();
  for(size_t i = 0; i < bodies.size(); ++i)
    for(size_t d = 0; d < gdimension; ++d) {
      if(bodies[i].coordinates()[d] + bodies[i].radius() > lrange[1][d])
        lrange[1][d] = bodies[i].coordinates()[d] + bodies[i].radius();
      if(bodies[i].coordinates()[d] - bodies[i].radius() < lrange[0][d])
        lrange[0][d] = bodies[i].coordinates()[d] - bodies[i].radius();
    }
  range = lrange;
}

int orc_particle_count(orc_ctx * c, int64_t * total, int64_t * real) {
  auto & ents = c->tree->entities();
  int64_t r = 0;
  for(auto & b : ents)
    r += b.getType() == NORMAL;
  if(total)
    *total = (int64_t)ents.size();
  if(real)
    *real = r;
  return FSPH_OK;
}

int orc_update_iteration(orc_ctx * c) {
  tree_topology_t & t = *c->tree;
  t.clean();
  if(param::periodic_boundary_x || param::periodic_boundary_y ||
     param::periodic_boundary_z) {
    // bodies_system.h:160-169 with getSmoothinglength (:112-124) inlined
    boundary::pboundary_clean(t.entities());
    double smoothinglength = 0;
    for(size_t i = 0; i < t.entities().size(); ++i)
      if(smoothinglength < t.entity(i).radius())
        smoothinglength = t.entity(i).radius();
    boundary::pboundary_generate(t.entities(), 2.5 * smoothinglength);
  }
  compute_range(t.entities(), c->range);
  if(c->range[0] == c->range[1])
    return FSPH_ERR_ARG;
  t.set_range(c->range);
  t.compute_keys();
  std::sort(t.entities().begin(), t.entities().end(),
    [](auto & left, auto & right) {
      if(left.key() < right.key())
        return true;
      if(left.key() == right.key())
        return left.id() < right.id();
      return false;
    });
  t.build_tree(physics::compute_cofm);
  c->built = true;
  return FSPH_OK;
}

int orc_reset_ghosts(orc_ctx * c) {
  c->tree->reset_ghosts(physics::compute_cofm);
  return FSPH_OK;
}

int orc_density_pressure_soundspeed(orc_ctx * c) {
  c->tree->traversal_sph(physics::compute_density_pressure_soundspeed);
  return FSPH_OK;
}
int orc_compute_alpha(orc_ctx * c) {
  c->tree->traversal_sph(viscosity::compute_alpha);
  return FSPH_OK;
}
int orc_initialize_alpha(orc_ctx * c) { return apply_all(c, viscosity::initialize_alpha); }
int orc_acceleration(orc_ctx * c) {
  c->tree->traversal_sph(physics::compute_acceleration);
  return FSPH_OK;
}
int orc_dudt(orc_ctx * c) {
  c->tree->traversal_sph(physics::compute_dudt);
  return FSPH_OK;
}
int orc_dedt(orc_ctx * c) {
  c->tree->traversal_sph(physics::compute_dedt);
  return FSPH_OK;
}
int orc_add_drag_acceleration(orc_ctx * c) {
  return apply_all(c, physics::add_drag_acceleration);
}
int orc_add_short_range_repulsion(orc_ctx * c) {
  c->tree->traversal_sph(physics::add_short_range_repulsion);
  return FSPH_OK;
}
int orc_add_drag_dedt(orc_ctx * c) { return apply_all(c, physics::add_drag_dedt); }
int orc_add_drag_dudt(orc_ctx * c) { return apply_all(c, physics::add_drag_dudt); }

int orc_eos_init(orc_ctx * c) { return apply_all(c, eos::init); }
int orc_set_total_energy(orc_ctx * c) {
  return apply_all(c, physics::set_total_energy);
}
int orc_save_velocityhalf(orc_ctx * c) {
  return apply_all(c, integration::save_velocityhalf);
}
int orc_leapfrog_kick_v(orc_ctx * c) {
  return apply_all(c, integration::leapfrog_kick_v);
}
int orc_leapfrog_kick_u(orc_ctx * c) {
  return apply_all(c, integration::leapfrog_kick_u);
}
int orc_leapfrog_kick_e(orc_ctx * c) {
  return apply_all(c, integration::leapfrog_kick_e);
}
int orc_leapfrog_drift(orc_ctx * c) {
  return apply_all(c, integration::leapfrog_drift);
}
int orc_recompute_pressure_soundspeed(orc_ctx * c) {
  return apply_all(c, physics::recompute_pressure_soundspeed);
}
int orc_recompute_pressure_soundspeed_thermokinetic(orc_ctx * c) {
  return apply_all(c, physics::recompute_pressure_soundspeed_thermokinetic);
}
int orc_compute_dt(orc_ctx * c) { return apply_all(c, physics::compute_dt); }
int orc_set_adaptive_timestep(orc_ctx * c) {
  physics::set_adaptive_timestep(c->tree->entities());
  return FSPH_OK;
}
int orc_compute_smoothinglength(orc_ctx * c) {
  physics::compute_smoothinglength(c->tree->entities());
  return FSPH_OK;
}
int orc_compute_average_smoothinglength(orc_ctx * c) {
  physics::compute_average_smoothinglength(
    c->tree->entities(), (int64_t)c->tree->entities().size());
  return FSPH_OK;
}
int orc_check_nans(orc_ctx * c) { return apply_all(c, physics::check_nans); }
int orc_check_negativity(orc_ctx * c) {
  return apply_all(c, physics::check_negativity);
}
int orc_advance_time(orc_ctx *) {
  physics::advance_time();
  return FSPH_OK;
}

int orc_gravity_direct(orc_ctx *, int64_t, int64_t) { return FSPH_ERR_ARG; }

int orc_step(orc_ctx * c) {
  using namespace param;
  /* one pass of the hydro driver loop (hydro/main_driver.cc:98-279) */
  if(physics::iteration == initial_iteration) {
    orc_update_iteration(c);
    orc_eos_init(c);
    if(thermokinetic_formulation)
      orc_set_total_energy(c);
    if(sph_viscosity != visc_constant)
      orc_initialize_alpha(c);
    orc_density_pressure_soundspeed(c);
    orc_save_velocityhalf(c);
    if(sph_viscosity != visc_constant)
      orc_compute_alpha(c);
    orc_reset_ghosts(c);
    orc_acceleration(c);
    if(physics::iteration < relaxation_steps) {
      orc_add_drag_acceleration(c);
      orc_add_short_range_repulsion(c);
    }
    if(adaptive_timestep) {
      orc_compute_dt(c);
      orc_set_adaptive_timestep(c);
    }
    if(evolve_internal_energy) {
      for(int m = 1; m <= pressure_updates_number; ++m) {
        if(thermokinetic_formulation) {
          orc_dedt(c);
          if(physics::iteration < relaxation_steps)
            orc_add_drag_dedt(c);
          orc_recompute_pressure_soundspeed_thermokinetic(c);
        }
        else {
          orc_dudt(c);
          if(physics::iteration < relaxation_steps)
            orc_add_drag_dudt(c);
          orc_recompute_pressure_soundspeed(c);
        }
        if(m < pressure_updates_number)
          orc_reset_ghosts(c);
      }
    }
  }
  else {
    if(evolve_internal_energy) {
      if(thermokinetic_formulation)
        orc_leapfrog_kick_e(c);
      else
        orc_leapfrog_kick_u(c);
    }
    orc_leapfrog_kick_v(c);
    orc_save_velocityhalf(c);
    orc_leapfrog_drift(c);
    orc_update_iteration(c);
    orc_density_pressure_soundspeed(c);
    if(sph_viscosity != visc_constant)
      orc_compute_alpha(c);
    orc_reset_ghosts(c);
    orc_acceleration(c);
    if(physics::iteration < relaxation_steps) {
      orc_add_drag_acceleration(c);
      orc_add_short_range_repulsion(c);
    }
    orc_leapfrog_kick_v(c);
    orc_reset_ghosts(c);
    if(evolve_internal_energy) {
      for(int m = 1; m <= pressure_updates_number; ++m) {
        if(thermokinetic_formulation) {
          orc_dedt(c);
          if(physics::iteration < relaxation_steps)
            orc_add_drag_dedt(c);
          orc_recompute_pressure_soundspeed_thermokinetic(c);
        }
        else {
          orc_dudt(c);
          if(physics::iteration < relaxation_steps)
            orc_add_drag_dudt(c);
          orc_recompute_pressure_soundspeed(c);
        }
        if(m < pressure_updates_number)
          orc_reset_ghosts(c);
      }
      if(thermokinetic_formulation)
        orc_leapfrog_kick_e(c);
      else
        orc_leapfrog_kick_u(c);
    }
  }
  if(sph_variable_h)
    orc_compute_smoothinglength(c);
  else if(sph_update_uniform_h)
    orc_compute_average_smoothinglength(c);
  orc_check_nans(c);
  orc_check_negativity(c);
  if(adaptive_timestep) {
    orc_compute_dt(c);
    orc_set_adaptive_timestep(c);
  }
  physics::advance_time();
  return FSPH_OK;
}

/* Neighbour lists exactly as traversal_sph hands them to the physics
 * callback, recorded by a capturing callback. */
int orc_get_neighbors(orc_ctx * c, int64_t * offsets, int64_t * indices,
  int64_t capacity) {
  auto & ents = c->tree->entities();
  const int64_t n = (int64_t)ents.size();
  body * base = ents.data();
  std::vector<std::vector<int64_t>> lists(n);
  c->order.clear();
  c->tree->traversal_sph([&](body & p, std::vector<body *> & nbs) {
    int64_t a = &p - base;
    c->order.push_back(a);
    auto & l = lists[a];
    l.clear();
    for(body * b : nbs)
      l.push_back(b - base);
  });
  offsets[0] = 0;
  for(int64_t i = 0; i < n; ++i)
    offsets[i + 1] = offsets[i] + (int64_t)lists[i].size();
  if(indices) {
    if(offsets[n] > capacity)
      return FSPH_ERR_ARG;
    for(int64_t i = 0; i < n; ++i)
      std::memcpy(indices + offsets[i], lists[i].data(), 8 * lists[i].size());
  }
  return FSPH_OK;
}

int orc_get_order(orc_ctx * c, int64_t * order) {
  if(c->order.empty()) {
    int64_t n = (int64_t)c->tree->entities().size();
    std::vector<int64_t> off(n + 1);
    orc_get_neighbors(c, off.data(), nullptr, 0);
  }
  std::copy(c->order.begin(), c->order.end(), order);
  return FSPH_OK;
}

} // extern "C"
