// fsph_body_system.hpp -- C++ host mirror of FleCSPH's body_system<T, D>
// over the C ABI of libfsph_gb300.so (include/fsph.h).
//
// A FleCSPH driver written against mpisph/bodies_system.h keeps its shape:
//
//   fsph::body_system<3> bs(params);                // body_system<double,3>
//   bs.read_bodies(view);                           // read_bodies(...)      :83
//   bs.update_iteration();                          // update_iteration()    :152
//   bs.apply_all(eos::init);                        // apply_all(ef)         :318
//   bs.apply_in_smoothinglength(
//       physics::compute_density_pressure_soundspeed); //                    :304
//   bs.reset_ghosts();                              // reset_ghosts()        :273
//   bs.get_all(physics::set_adaptive_timestep);     // get_all(ef)           :335
//   bs.gravitation_fmm();                           // gravitation_fmm()     :282
//
// The reference passes physics functions as callbacks; here the names in
// fsph::physics / fsph::eos / fsph::integration are tags that select the
// fused GPU pass implementing that function.  Errors come back as
// fsph::error exceptions carrying the fsph_status (the reference asserts).
#pragma once

#include <stdexcept>
#include <string>

#include "fsph.h"

namespace fsph {

struct error : std::runtime_error {
  fsph_status status;
  error(fsph_status s, const std::string & where)
    : std::runtime_error(where + ": " + fsph_status_string(s)), status(s) {}
};

inline void check(fsph_status s, const char * where) {
  if(s != FSPH_OK)
    throw error(s, where);
}

// Tags naming the reference's physics modules.
namespace physics {
struct density_pressure_soundspeed_t {};
struct acceleration_t {};
struct dudt_t {};
struct dedt_t {};
struct set_total_energy_t {};
struct recompute_pressure_soundspeed_t {};
struct recompute_pressure_soundspeed_thermokinetic_t {};
struct compute_dt_t {};
struct check_nans_t {};
struct check_negativity_t {};
struct set_adaptive_timestep_t {};
struct compute_smoothinglength_t {};
struct compute_average_smoothinglength_t {};
struct add_drag_acceleration_t {};
struct add_short_range_repulsion_t {};
struct add_drag_dedt_t {};
struct add_drag_dudt_t {};
constexpr add_drag_acceleration_t add_drag_acceleration{};          // default_physics.h:699-708
constexpr add_short_range_repulsion_t add_short_range_repulsion{};  // :723-753
constexpr add_drag_dedt_t add_drag_dedt{};                          // :571-579
constexpr add_drag_dudt_t add_drag_dudt{};                          // :586-594
constexpr density_pressure_soundspeed_t compute_density_pressure_soundspeed{};
constexpr acceleration_t compute_acceleration{};
constexpr dudt_t compute_dudt{};
constexpr dedt_t compute_dedt{};
constexpr set_total_energy_t set_total_energy{};
constexpr recompute_pressure_soundspeed_t recompute_pressure_soundspeed{};
constexpr recompute_pressure_soundspeed_thermokinetic_t
  recompute_pressure_soundspeed_thermokinetic{};
constexpr compute_dt_t compute_dt{};
constexpr check_nans_t check_nans{};
constexpr check_negativity_t check_negativity{};
constexpr set_adaptive_timestep_t set_adaptive_timestep{};
constexpr compute_smoothinglength_t compute_smoothinglength{};
constexpr compute_average_smoothinglength_t compute_average_smoothinglength{};
inline void advance_time(fsph_ctx * c) { check(fsph_advance_time(c), "advance_time"); }
} // namespace physics

namespace eos {
struct init_t {};
constexpr init_t init{};
} // namespace eos

namespace integration {
struct save_velocityhalf_t {};
struct leapfrog_kick_v_t {};
struct leapfrog_kick_u_t {};
struct leapfrog_kick_e_t {};
struct leapfrog_drift_t {};
constexpr save_velocityhalf_t save_velocityhalf{};
constexpr leapfrog_kick_v_t leapfrog_kick_v{};
constexpr leapfrog_kick_u_t leapfrog_kick_u{};
constexpr leapfrog_kick_e_t leapfrog_kick_e{};
constexpr leapfrog_drift_t leapfrog_drift{};
} // namespace integration

namespace viscosity {
struct compute_alpha_t {};
struct initialize_alpha_t {};
constexpr compute_alpha_t compute_alpha{};        // viscosity.h:310-363
constexpr initialize_alpha_t initialize_alpha{};  // viscosity.h:171-177
} // namespace viscosity

template<int D>
class body_system {
public:
  explicit body_system(fsph_params p, int64_t capacity, int device = 0) {
    p.dimension = D;
    fsph_status s = FSPH_OK;
    ctx_ = fsph_create(&p, device, capacity, &s);
    if(!ctx_)
      throw error(s, "fsph_create");
    params_ = p;
  }
  ~body_system() { fsph_destroy(ctx_); }
  body_system(const body_system &) = delete;
  body_system & operator=(const body_system &) = delete;

  fsph_ctx * context() { return ctx_; }

  // setMacangle (bodies_system.h:70-72): the opening angle is part of the
  // parameter block fixed at construction.
  double macangle() const { return params_.fmm_macangle; }

  void read_bodies(const fsph_soa_view & v) { check(fsph_upload(ctx_, &v), "read_bodies"); }
  void write_bodies(fsph_soa_view & v) { check(fsph_download(ctx_, &v), "write_bodies"); }

  void update_iteration() { check(fsph_update_iteration(ctx_), "update_iteration"); }
  void reset_ghosts() { check(fsph_reset_ghosts(ctx_), "reset_ghosts"); }
  void gravitation_fmm() { check(fsph_gravitation(ctx_), "gravitation_fmm"); }

  void apply_in_smoothinglength(physics::density_pressure_soundspeed_t) {
    check(fsph_density_pressure_soundspeed(ctx_), "compute_density_pressure_soundspeed");
  }
  void apply_in_smoothinglength(physics::acceleration_t) {
    check(fsph_acceleration(ctx_), "compute_acceleration");
  }
  void apply_in_smoothinglength(physics::dudt_t) { check(fsph_dudt(ctx_), "compute_dudt"); }
  void apply_in_smoothinglength(physics::dedt_t) { check(fsph_dedt(ctx_), "compute_dedt"); }

  void apply_in_smoothinglength(viscosity::compute_alpha_t) {
    check(fsph_compute_alpha(ctx_), "viscosity::compute_alpha");
  }
  void apply_all(viscosity::initialize_alpha_t) {
    check(fsph_initialize_alpha(ctx_), "viscosity::initialize_alpha");
  }
  void apply_all(eos::init_t) { check(fsph_eos_init(ctx_), "eos::init"); }
  void apply_all(physics::set_total_energy_t) {
    check(fsph_set_total_energy(ctx_), "set_total_energy");
  }
  void apply_all(integration::save_velocityhalf_t) {
    check(fsph_save_velocityhalf(ctx_), "save_velocityhalf");
  }
  void apply_all(integration::leapfrog_kick_v_t) {
    check(fsph_leapfrog_kick_v(ctx_), "leapfrog_kick_v");
  }
  void apply_all(integration::leapfrog_kick_u_t) {
    check(fsph_leapfrog_kick_u(ctx_), "leapfrog_kick_u");
  }
  void apply_all(integration::leapfrog_kick_e_t) {
    check(fsph_leapfrog_kick_e(ctx_), "leapfrog_kick_e");
  }
  void apply_all(integration::leapfrog_drift_t) {
    check(fsph_leapfrog_drift(ctx_), "leapfrog_drift");
  }
  void apply_all(physics::recompute_pressure_soundspeed_t) {
    check(fsph_recompute_pressure_soundspeed(ctx_), "recompute_pressure_soundspeed");
  }
  void apply_all(physics::recompute_pressure_soundspeed_thermokinetic_t) {
    check(fsph_recompute_pressure_soundspeed_thermokinetic(ctx_),
      "recompute_pressure_soundspeed_thermokinetic");
  }
  void apply_all(physics::compute_dt_t) { check(fsph_compute_dt(ctx_), "compute_dt"); }
  void apply_all(physics::add_drag_acceleration_t) {
    check(fsph_add_drag_acceleration(ctx_), "add_drag_acceleration");
  }
  void apply_in_smoothinglength(physics::add_short_range_repulsion_t) {
    check(fsph_add_short_range_repulsion(ctx_), "add_short_range_repulsion");
  }
  void apply_all(physics::add_drag_dedt_t) { check(fsph_add_drag_dedt(ctx_), "add_drag_dedt"); }
  void apply_all(physics::add_drag_dudt_t) { check(fsph_add_drag_dudt(ctx_), "add_drag_dudt"); }
  void apply_all(physics::check_nans_t) { check(fsph_check_nans(ctx_), "check_nans"); }
  void apply_all(physics::check_negativity_t) {
    check(fsph_check_negativity(ctx_), "check_negativity");
  }
  void get_all(physics::set_adaptive_timestep_t) {
    check(fsph_set_adaptive_timestep(ctx_), "set_adaptive_timestep");
  }
  void get_all(physics::compute_smoothinglength_t) {
    check(fsph_compute_smoothinglength(ctx_), "compute_smoothinglength");
  }
  void get_all(physics::compute_average_smoothinglength_t) {
    check(fsph_compute_average_smoothinglength(ctx_), "compute_average_smoothinglength");
  }

  // One pass of mpi_init_task's loop, fused on the device.
  void step() { check(fsph_step(ctx_), "step"); }
  void sync() { check(fsph_sync(ctx_), "sync"); }

  int64_t iteration() {
    int64_t it = 0;
    check(fsph_get_time(ctx_, nullptr, nullptr, &it), "get_time");
    return it;
  }

private:
  fsph_ctx * ctx_ = nullptr;
  fsph_params params_{};
};

} // namespace fsph
