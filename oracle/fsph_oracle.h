/*
 * fsph_oracle.h -- CPU oracle of the FleCSPH per-step particle path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm may load this library, and only as
 * the checker or the timed CPU baseline -- never as part of the GPU product
 * path.
 *
 * Two libraries implement this API:
 *   oracle/liboracle.so      -- fsph_oracle.c, a plain-C restatement of the
 *                               reference algorithm (each function cites the
 *                               reference file:line it follows);
 *   oracle/_ref/libfsph_ref.so -- ref_harness.cc, the reference's own headers
 *                               compiled against single-rank stubs (built only
 *                               where the reference sources are present).
 * Both take the same fsph_params / fsph_soa_view types as the GPU boundary
 * (include/fsph.h) so one harness drives all three.
 */
#ifndef FSPH_ORACLE_H
#define FSPH_ORACLE_H
#include <stdint.h>
#include "../include/fsph.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

orc_ctx * orc_create(const fsph_params * p);
void orc_destroy(orc_ctx * c);
int orc_set_threads(orc_ctx * c, int nthreads);
int orc_upload(orc_ctx * c, const fsph_soa_view * v);
int orc_download(orc_ctx * c, fsph_soa_view * v);
int orc_get_time(orc_ctx * c, double * dt, double * totaltime, int64_t * it);
int orc_set_time(orc_ctx * c, double dt, double totaltime, int64_t it);
int orc_get_range(orc_ctx * c, double * range);

/* Particles held: total includes the periodic copies (WALL) of the last
 * update_iteration; real = the uploaded count. */
int orc_particle_count(orc_ctx * c, int64_t * total, int64_t * real);

int orc_update_iteration(orc_ctx * c);
int orc_reset_ghosts(orc_ctx * c);
int orc_density_pressure_soundspeed(orc_ctx * c);
int orc_compute_alpha(orc_ctx * c);
int orc_initialize_alpha(orc_ctx * c);
int orc_acceleration(orc_ctx * c);
int orc_dudt(orc_ctx * c);
int orc_dedt(orc_ctx * c);
int orc_add_drag_acceleration(orc_ctx * c);
int orc_add_short_range_repulsion(orc_ctx * c);
int orc_add_drag_dedt(orc_ctx * c);
int orc_add_drag_dudt(orc_ctx * c);
int orc_eos_init(orc_ctx * c);
int orc_set_total_energy(orc_ctx * c);
int orc_save_velocityhalf(orc_ctx * c);
int orc_leapfrog_kick_v(orc_ctx * c);
int orc_leapfrog_kick_u(orc_ctx * c);
int orc_leapfrog_kick_e(orc_ctx * c);
int orc_leapfrog_drift(orc_ctx * c);
int orc_recompute_pressure_soundspeed(orc_ctx * c);
int orc_recompute_pressure_soundspeed_thermokinetic(orc_ctx * c);
int orc_compute_dt(orc_ctx * c);
int orc_set_adaptive_timestep(orc_ctx * c);
int orc_compute_smoothinglength(orc_ctx * c);
int orc_compute_average_smoothinglength(orc_ctx * c);
int orc_check_nans(orc_ctx * c);
int orc_check_negativity(orc_ctx * c);
int orc_advance_time(orc_ctx * c);
int orc_step(orc_ctx * c);
/* Direct-summation gravity (unsoftened, include/physics/fmm.h:37-46) for the
 * sinks [s0, s1) of the current order over all sources; overwrites
 * g-acceleration and potential of those sinks. */
int orc_gravity_direct(orc_ctx * c, int64_t s0, int64_t s1);

/* Neighbour lists of the current tree in the reference's order (CSR over the
 * sorted index).  indices == NULL: only offsets (total in offsets[n]). */
int orc_get_neighbors(orc_ctx * c, int64_t * offsets, int64_t * indices,
  int64_t capacity);
/* Particle processing order of apply_in_smoothinglength (sorted indices). */
int orc_get_order(orc_ctx * c, int64_t * order);

#ifdef __cplusplus
}
#endif
#endif
