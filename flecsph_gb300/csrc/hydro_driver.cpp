// hydro_driver.cpp -- the evolution loop of FleCSPH's hydro driver
// (app/drivers/hydro/main_driver.cc:98-279) written against the C++ mirror
// of body_system (include/fsph_body_system.hpp), each call in the order the
// reference makes it (no fused fsph_step).
//
//   hydro_driver <in.bin> <out.bin> <iterations> [key=value ...]
//
// in/out: raw particle snapshots, little endian:
//   char magic[8] = "FSPHSOA2"; int64 n; int32 dim; int32 nfields(=32);
//   int64 iteration; double dt; double time;
//   32 double arrays of length n in fsph_soa_view order (x..Ye);
//   int64 id[n]
// "FSPHSOA1" files have no time record, and files with 29 to 31 arrays are
// read with the missing ones zero.
// Restart (mpisph/io.h:523-586,818-836): a snapshot written at a non-zero
// iteration restores dt and the total time, and the run starts at that
// iteration with the driver's initial-iteration branch, as the reference's
// read_bodies(..., initial_iteration) and main loop do; an initial_iteration
// given on the command line must name the snapshot's iteration.
// Parameters not given as key=value keep their reference defaults.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fsph_body_system.hpp"

namespace {

constexpr int NFIELDS = 32;
constexpr int NFIELDS_MIN = 29;

struct Snapshot {
  int64_t n = 0;
  int32_t dim = 3;
  bool has_time = false;  // FSPHSOA2: the time record below is valid
  int64_t iteration = 0;
  double dt = 0.0, time = 0.0;
  std::vector<double> f[NFIELDS];
  std::vector<int64_t> id;
  std::vector<uint64_t> key;

  fsph_soa_view view() {
    fsph_soa_view v;
    std::memset(&v, 0, sizeof(v));
    v.n = n;
    double ** slots[NFIELDS] = {&v.x, &v.y, &v.z, &v.vx, &v.vy, &v.vz, &v.vhx,
      &v.vhy, &v.vhz, &v.ax, &v.ay, &v.az, &v.gax, &v.gay, &v.gaz, &v.gpot,
      &v.m, &v.h, &v.rho, &v.P, &v.cs, &v.u, &v.e, &v.dudt, &v.dedt, &v.K,
      &v.alpha, &v.vsig, &v.dt, &v.divv, &v.ddivvdt, &v.Ye};
    for(int k = 0; k < NFIELDS; ++k)
      *slots[k] = f[k].data();
    v.id = id.data();
    v.key = key.data();
    return v;
  }
};

bool read_snapshot(const char * path, Snapshot & s) {
  FILE * fp = std::fopen(path, "rb");
  if(!fp)
    return false;
  char magic[8];
  int32_t nf = 0;
  bool ok = std::fread(magic, 1, 8, fp) == 8;
  const bool v2 = ok && std::memcmp(magic, "FSPHSOA2", 8) == 0;
  ok = ok && (v2 || std::memcmp(magic, "FSPHSOA1", 8) == 0) &&
       std::fread(&s.n, 8, 1, fp) == 1 && std::fread(&s.dim, 4, 1, fp) == 1 &&
       std::fread(&nf, 4, 1, fp) == 1 && nf >= NFIELDS_MIN && nf <= NFIELDS && s.n > 1;
  if(ok && v2)
    ok = std::fread(&s.iteration, 8, 1, fp) == 1 && std::fread(&s.dt, 8, 1, fp) == 1 &&
         std::fread(&s.time, 8, 1, fp) == 1;
  s.has_time = ok && v2;
  for(int k = 0; ok && k < NFIELDS; ++k) {
    s.f[k].assign(s.n, 0.0);
    if(k < nf)
      ok = std::fread(s.f[k].data(), 8, s.n, fp) == (size_t)s.n;
  }
  if(ok) {
    s.id.resize(s.n);
    s.key.resize(s.n);
    ok = std::fread(s.id.data(), 8, s.n, fp) == (size_t)s.n;
  }
  std::fclose(fp);
  return ok;
}

bool write_snapshot(const char * path, Snapshot & s) {
  FILE * fp = std::fopen(path, "wb");
  if(!fp)
    return false;
  int32_t nf = NFIELDS;
  bool ok = std::fwrite("FSPHSOA2", 1, 8, fp) == 8 && std::fwrite(&s.n, 8, 1, fp) == 1 &&
            std::fwrite(&s.dim, 4, 1, fp) == 1 && std::fwrite(&nf, 4, 1, fp) == 1 &&
            std::fwrite(&s.iteration, 8, 1, fp) == 1 && std::fwrite(&s.dt, 8, 1, fp) == 1 &&
            std::fwrite(&s.time, 8, 1, fp) == 1;
  for(int k = 0; ok && k < NFIELDS; ++k)
    ok = std::fwrite(s.f[k].data(), 8, s.n, fp) == (size_t)s.n;
  if(ok)
    ok = std::fwrite(s.id.data(), 8, s.n, fp) == (size_t)s.n;
  std::fclose(fp);
  return ok;
}

// key=value overrides for the parameters a hydro parfile sets
bool set_param(fsph_params & p, const std::string & kv) {
  auto eq = kv.find('=');
  if(eq == std::string::npos)
    return false;
  std::string k = kv.substr(0, eq);
  if(k == "external_force_type")
    return fsph_params_set_external_force(&p, kv.c_str() + eq + 1) == FSPH_OK;
  double v = std::atof(kv.c_str() + eq + 1);
  if(k == "poly_gamma") p.poly_gamma = v;
  else if(k == "sph_viscosity") p.sph_viscosity = (int32_t)v;
  else if(k == "relaxation_steps") p.relaxation_steps = (int32_t)v;
  else if(k == "relaxation_beta") p.relaxation_beta = v;
  else if(k == "relaxation_gamma") p.relaxation_gamma = v;
  else if(k == "relaxation_repulsion_radius") p.relaxation_repulsion_radius = v;
  else if(k == "relaxation_repulsion_gamma") p.relaxation_repulsion_gamma = v;
  else if(k == "gravity_acceleration_constant") p.gravity_acceleration_constant = v;
  else if(k == "sphere_radius") p.sphere_radius = v;
  else if(k == "extforce_wall_powerindex") p.extforce_wall_powerindex = v;
  else if(k == "extforce_wall_steepness") p.extforce_wall_steepness = v;
  else if(k == "box_length") p.box_length = v;
  else if(k == "box_width") p.box_width = v;
  else if(k == "box_height") p.box_height = v;
  else if(k == "sph_eta") p.sph_eta = v;
  else if(k == "sph_kernel") p.sph_kernel = (int32_t)v;
  else if(k == "eos_type") p.eos_type = (int32_t)v;
  else if(k == "initial_dt") p.initial_dt = v;
  else if(k == "timestep_cfl_factor") p.timestep_cfl_factor = v;
  else if(k == "adaptive_timestep") p.adaptive_timestep = (int32_t)v;
  else if(k == "thermokinetic_formulation") p.thermokinetic_formulation = (int32_t)v;
  else if(k == "sph_variable_h") p.sph_variable_h = (int32_t)v;
  else if(k == "sph_update_uniform_h") p.sph_update_uniform_h = (int32_t)v;
  else if(k == "max_neighbors") p.max_neighbors = (int32_t)v;
  else if(k == "precision_mode") p.precision_mode = (int32_t)v;
  else if(k == "evolve_internal_energy") p.evolve_internal_energy = (int32_t)v;
  else if(k == "pressure_updates_number") p.pressure_updates_number = (int32_t)v;
  else if(k == "initial_iteration") p.initial_iteration = (int64_t)std::atoll(kv.c_str() + eq + 1);
  else if(k == "initial_time") p.initial_time = v;
  else if(k == "group_size") p.group_size = (int32_t)v;
  else
    return false;
  return true;
}

// de/dt (thermokinetic) or du/dt, then the pressure predictor, repeated
// pressure_updates_number times with a ghost refresh between passes
// (hydro/main_driver.cc:145-171,214-240)
template<class BS>
void energy_passes(BS & bs, const fsph_params & p, bool relax) {
  using namespace fsph;
  for(int m = 1; m <= p.pressure_updates_number; ++m) {
    if(p.thermokinetic_formulation) {
      bs.apply_in_smoothinglength(physics::compute_dedt);
      if(relax)
        bs.apply_all(physics::add_drag_dedt);
      bs.apply_all(physics::recompute_pressure_soundspeed_thermokinetic);
    }
    else {
      bs.apply_in_smoothinglength(physics::compute_dudt);
      if(relax)
        bs.apply_all(physics::add_drag_dudt);
      bs.apply_all(physics::recompute_pressure_soundspeed);
    }
    if(m < p.pressure_updates_number)
      bs.reset_ghosts();
  }
}

} // namespace

int main(int argc, char ** argv) {
  if(argc < 4) {
    std::fprintf(stderr, "usage: %s in.bin out.bin iterations [key=value ...]\n", argv[0]);
    return 2;
  }
  Snapshot s;
  if(!read_snapshot(argv[1], s)) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  fsph_params p;
  fsph_params_default(&p);
  bool iteration_given = false;
  for(int a = 4; a < argc; ++a) {
    if(!set_param(p, argv[a])) {
      std::fprintf(stderr, "unknown parameter %s\n", argv[a]);
      return 2;
    }
    iteration_given |= std::strncmp(argv[a], "initial_iteration=", 18) == 0;
  }
  // a snapshot of a later iteration restarts the run there
  const bool restart = s.has_time && s.iteration != 0;
  if(restart) {
    if(iteration_given && p.initial_iteration != s.iteration) {
      std::fprintf(stderr, "%s holds iteration %lld, not initial_iteration %lld\n",
        argv[1], (long long)s.iteration, (long long)p.initial_iteration);
      return 2;
    }
    p.initial_iteration = s.iteration;
  }
  const int iterations = std::atoi(argv[3]);
  try {
    if(s.dim != 3) {
      std::fprintf(stderr, "this driver is built for 3D\n");
      return 2;
    }
    using namespace fsph;
    body_system<3> bs(p, s.n);
    fsph_soa_view v = s.view();
    bs.read_bodies(v);
    if(restart)
      check(fsph_set_time(bs.context(), s.dt, s.time, s.iteration), "set_time");
    for(int it = 0; it < iterations; ++it) {
      const bool relax = bs.iteration() < p.relaxation_steps;
      if(bs.iteration() == p.initial_iteration) {
        bs.update_iteration();
        bs.apply_all(eos::init);
        if(p.thermokinetic_formulation)
          bs.apply_all(physics::set_total_energy);
        if(p.sph_viscosity != FSPH_VISC_CONSTANT)
          bs.apply_all(viscosity::initialize_alpha);
        bs.apply_in_smoothinglength(physics::compute_density_pressure_soundspeed);
        bs.apply_all(integration::save_velocityhalf);
        if(p.sph_viscosity != FSPH_VISC_CONSTANT)
          bs.apply_in_smoothinglength(viscosity::compute_alpha);
        bs.reset_ghosts();
        bs.apply_in_smoothinglength(physics::compute_acceleration);
        if(relax) {
          bs.apply_all(physics::add_drag_acceleration);
          bs.apply_in_smoothinglength(physics::add_short_range_repulsion);
        }
        if(p.adaptive_timestep) {
          bs.apply_all(physics::compute_dt);
          bs.get_all(physics::set_adaptive_timestep);
        }
        if(p.evolve_internal_energy)
          energy_passes(bs, p, relax);
      }
      else {
        if(p.evolve_internal_energy) {
          if(p.thermokinetic_formulation)
            bs.apply_all(integration::leapfrog_kick_e);
          else
            bs.apply_all(integration::leapfrog_kick_u);
        }
        bs.apply_all(integration::leapfrog_kick_v);
        bs.apply_all(integration::save_velocityhalf);
        bs.apply_all(integration::leapfrog_drift);
        bs.update_iteration();
        bs.apply_in_smoothinglength(physics::compute_density_pressure_soundspeed);
        if(p.sph_viscosity != FSPH_VISC_CONSTANT)
          bs.apply_in_smoothinglength(viscosity::compute_alpha);
        bs.reset_ghosts();
        bs.apply_in_smoothinglength(physics::compute_acceleration);
        if(relax) {
          bs.apply_all(physics::add_drag_acceleration);
          bs.apply_in_smoothinglength(physics::add_short_range_repulsion);
        }
        bs.apply_all(integration::leapfrog_kick_v);
        bs.reset_ghosts();
        if(p.evolve_internal_energy) {
          energy_passes(bs, p, relax);
          if(p.thermokinetic_formulation)
            bs.apply_all(integration::leapfrog_kick_e);
          else
            bs.apply_all(integration::leapfrog_kick_u);
        }
      }
      if(p.sph_variable_h)
        bs.get_all(physics::compute_smoothinglength);
      else if(p.sph_update_uniform_h)
        bs.get_all(physics::compute_average_smoothinglength);
      bs.apply_all(physics::check_nans);
      bs.apply_all(physics::check_negativity);
      if(p.adaptive_timestep) {
        bs.apply_all(physics::compute_dt);
        bs.get_all(physics::set_adaptive_timestep);
      }
      physics::advance_time(bs.context());
    }
    bs.sync();
    bs.write_bodies(v);
    double dt = 0, t = 0;
    int64_t iter = 0;
    check(fsph_get_time(bs.context(), &dt, &t, &iter), "get_time");
    s.iteration = iter;
    s.dt = dt;
    s.time = t;
    std::printf("iteration %lld time %.17g dt %.17g\n", (long long)iter, t, dt);
  } catch(const fsph::error & e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  if(!write_snapshot(argv[2], s)) {
    std::fprintf(stderr, "cannot write %s\n", argv[2]);
    return 2;
  }
  return 0;
}
