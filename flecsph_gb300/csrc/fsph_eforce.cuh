// fsph_eforce.cuh -- external forces and potentials (include/physics/
// eforce.h), the radial density profiles the density support uses
// (include/physics/density_profiles.h:64-230), and the relaxation drag
// (eforce.h:441-451).  FP64, with the reference's operand order; the
// profiles are also called on the host to set the support's constants.
#pragma once
#include "fsph_internal.cuh"

namespace fsph {

#define FSPH_HD __host__ __device__ __forceinline__
#define FSPH_PI 3.14159265358979323846

FSPH_HD double sq_(double x) { return x * x; }
FSPH_HD double cu_(double x) { return x * x * x; }

// mesa_mass_helper (density_profiles.h:163-177)
FSPH_HD double mesa_mass_helper(int D, double r, double q) {
  const double dr = q, r0 = 1. - q;
  double mm = 0.0;
  if(D == 2)
    mm = sq_(r) * (1. - (.5 * sq_(r) + sq_(r0)) / sq_(dr)) +
         (.5 * cu_(r0) + 4. * cu_(r)) * r0 / (3. * sq_(dr));
  if(D == 3)
    mm = cu_(r0) / 3. + (cu_(r) - cu_(r0)) / 3. * (1. - sq_(r0) / sq_(dr)) +
         r0 * (sq_(r) - sq_(r0)) * (sq_(r) + sq_(r0)) / (2. * sq_(dr)) -
         (sq_(r) * cu_(r) - sq_(r0) * cu_(r0)) / (5 * sq_(dr));
  return mm;
}

// mesa_rho0 as density_profiles::select sets it (:366-374)
FSPH_HD double mesa_rho0_for(int D, double q) {
  return D == 2 ? 1. / (FSPH_PI * mesa_mass_helper(2, 1., q))
                : 1. / (4. * FSPH_PI * mesa_mass_helper(3, 1., q));
}

// spherical_density_profile (density_profiles.h:69-80, 107-120, 179-188)
FSPH_HD double dprof_rho(int D, int prof, double r, double q, double rho0) {
  if(prof == FSPH_DENSITY_PARABOLIC)
    return D == 2 ? 2. / FSPH_PI * (1. - sq_(r)) : 15. / (8. * FSPH_PI) * (1. - sq_(r));
  if(prof == FSPH_DENSITY_MESA) {
    double rho = 0.0;
    const double r0 = 1. - q;
    if(r < 1. - q)
      rho = rho0;
    else if(r < .9999)
      rho = rho0 * (1. - sq_(r - r0) / sq_(q));
    return rho;
  }
  return D == 2 ? 1.0 / FSPH_PI : 0.75 / FSPH_PI;
}

// spherical_drho_dr (density_profiles.h:98-101, 137-150, 215-222)
FSPH_HD double dprof_drho(int D, int prof, double r, double q, double rho0) {
  if(prof == FSPH_DENSITY_PARABOLIC)
    return D == 2 ? -4. / FSPH_PI * r : -15. / (4. * FSPH_PI) * r;
  if(prof == FSPH_DENSITY_MESA) {
    double drhodr = 0.0;
    const double r0 = 1. - q;
    if(r > 1. - q && r < .9999)
      drhodr = -2. * rho0 * (r - r0) / sq_(q);
    return drhodr;
  }
  return 0.;
}

template<int D>
__device__ __forceinline__ double radius_of(const double * rp) {
  double r = rp[0] * rp[0];
  for(int i = 1; i < D; ++i)
    r += rp[i] * rp[i];
  return sqrt(r);
}

// airfoil geometry shared by the force and the potential (eforce.h:213-271)
struct AirfoilGeom {
  double x, y, ca, sa, camber_line, phi;
  bool inside;
};
__device__ __forceinline__ AirfoilGeom airfoil_geom(const PhysParams & pp,
  const double * rp) {
  AirfoilGeom g;
  const double x1 = rp[0] - pp.af_x, y1 = rp[1] - pp.af_y;
  g.ca = cos(pp.af_alpha);
  g.sa = sin(pp.af_alpha);
  g.x = x1 * g.ca + y1 * g.sa;
  g.y = -x1 * g.sa + y1 * g.ca;
  g.inside = fabs(g.y) < 5.0 * pp.af_thick && g.x > -pp.af_size * 0.02 &&
             g.x < pp.af_size * 1.02;
  const double upper = pp.af_thick * g.x * sqrt(pp.af_size * pp.af_size - g.x * g.x);
  g.camber_line = pp.af_camber * sin(FSPH_PI * g.x / 2.);
  g.phi = sq_(upper) - sq_(g.y - g.camber_line) + 0.002;
  return g;
}

// one potential term
template<int D>
__device__ double eforce_potential_term(const PhysParams & pp, int code,
  const double * rp) {
  switch(code) {
    case FSPH_EFORCE_WALLS_X:
    case FSPH_EFORCE_WALLS_Y:
    case FSPH_EFORCE_WALLS_Z: {  // potential_square_well<I> (:46-58)
      const int I = code - FSPH_EFORCE_WALLS_X;
      const double b = pp.box_half[I];
      return (((rp[I] < -b) ? pow(-rp[I] - b, pp.ew_n) : 0.0) +
              ((rp[I] > b) ? pow(rp[I] - b, pp.ew_n) : 0.0)) *
             pp.ew_a;
    }
    case FSPH_EFORCE_SPHERICAL_WALL: {  // potential_spherical_wall (:108-121)
      double phi = 0.0;
      const double r = radius_of<D>(rp);
      if(r > pp.sphere_r)
        phi = pp.ew_a * pow(r - pp.sphere_r, pp.ew_n);
      return phi;
    }
    case FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT: {  // (:153-168)
      const double r = radius_of<D>(rp);
      const double x = r / pp.sphere_r;
      const double rho = pp.rho_init / pp.ds_rho0 *
                         dprof_rho(D, pp.dprof, x, pp.mesa_q, pp.mesa_rho0);
      const double g = pp.gamma;
      const double phi = (rho > 0) ? (-pp.ds_K0 * g * pow(rho, g - 1.) / (g - 1.)) : 0;
      double wall = 0.0;
      if(r > pp.sphere_r)
        wall = pp.ew_a * pow(r - pp.sphere_r, pp.ew_n);
      return phi + wall;
    }
    case FSPH_EFORCE_GRAVITY: {  // potential_gravity (:186-192)
      double height = rp[0];
      if(D > 1)
        height = rp[1];
      return height * pp.grav_acc;
    }
    case FSPH_EFORCE_AIRFOIL: {  // potential_airfoil (:245-271)
      double phi = 0.0;
      const AirfoilGeom g = airfoil_geom(pp, rp);
      if(g.inside && g.phi > 0.0)
        phi = pp.ew_a * pow(g.phi, pp.ew_n);
      return phi;
    }
    case FSPH_EFORCE_ORBIT: {  // potential_orbit (:300-313)
      const double m_t = pp.orb_mns + pp.orb_mwd;
      double term1 = sqrt(sq_(rp[0] - pp.orb_a) + sq_(rp[1]) + sq_(rp[2]));
      term1 = -pp.G * pp.orb_mns / term1;
      double term2 = -0.5 * pp.G * m_t / cu_(pp.orb_a);
      term2 = term2 * (sq_(rp[0] - pp.orb_a * pp.orb_mns / m_t) + sq_(rp[1]));
      return term1 + term2;
    }
    case FSPH_EFORCE_POISON:  // potential_poison (:319-321)
      return pp.poison;
    default:
      return 0.0;
  }
}

// one acceleration term, added into a[] (which holds the sum so far)
template<int D>
__device__ void eforce_accel_term(const PhysParams & pp, int code,
  const double * rp, double * a) {
  switch(code) {
    case FSPH_EFORCE_WALLS_X:
    case FSPH_EFORCE_WALLS_Y:
    case FSPH_EFORCE_WALLS_Z: {  // acceleration_square_well<I> (:64-79)
      const int I = code - FSPH_EFORCE_WALLS_X;
      const double b = pp.box_half[I];
      double t[3] = {0.0, 0.0, 0.0};
      t[I] = (((rp[I] < -b) ? pow(-rp[I] - b, pp.ew_n - 1) : 0.0) -
              ((rp[I] > b) ? pow(rp[I] - b, pp.ew_n - 1) : 0.0)) *
             pp.ew_n * pp.ew_a;
      for(int i = 0; i < D; ++i)
        a[i] += t[i];
      return;
    }
    case FSPH_EFORCE_SPHERICAL_WALL:
    case FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT: {
      double t[3] = {0.0, 0.0, 0.0};
      const double r = radius_of<D>(rp);
      if(code == FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT) {  // (:128-151)
        const double x = r / pp.sphere_r;
        if(x > 1e-12) {
          const double rho = pp.rho_init / pp.ds_rho0 *
                             dprof_rho(D, pp.dprof, x, pp.mesa_q, pp.mesa_rho0);
          const double drhodr = pp.rho_init / (pp.ds_rho0 * pp.sphere_r) *
                                dprof_drho(D, pp.dprof, x, pp.mesa_q, pp.mesa_rho0);
          const double a_r =
            (rho > 0) ? (pp.ds_K0 * pp.gamma * pow(rho, pp.gamma - 2) * drhodr) : 0;
          for(int i = 0; i < D; ++i)
            t[i] = a_r * rp[i] / r;
        }
      }
      // acceleration_spherical_wall (:88-106); the density support adds it
      double w[3] = {0.0, 0.0, 0.0};
      if(r > pp.sphere_r) {
        const double ar = pp.ew_n * pp.ew_a * pow(r - pp.sphere_r, pp.ew_n - 1);
        for(int i = 0; i < D; ++i)
          w[i] = -rp[i] / r * ar;
      }
      for(int i = 0; i < D; ++i)
        a[i] += code == FSPH_EFORCE_SPHERICAL_WALL ? w[i] : t[i] + w[i];
      return;
    }
    case FSPH_EFORCE_GRAVITY: {  // acceleration_gravity (:176-184)
      double t[3] = {0.0, 0.0, 0.0};
      if(D > 1)
        t[1] = -pp.grav_acc;
      else
        t[0] = -pp.grav_acc;
      for(int i = 0; i < D; ++i)
        a[i] += t[i];
      return;
    }
    case FSPH_EFORCE_AIRFOIL: {  // acceleration_airfoil (:213-243)
      double t[3] = {0.0, 0.0, 0.0};
      const AirfoilGeom g = airfoil_geom(pp, rp);
      if(g.inside && g.phi > 0.0) {
        const double c = pp.af_camber, th = pp.af_thick, sz = pp.af_size, x = g.x;
        const double a0 = pp.ew_n * pp.ew_a * pow(g.phi, pp.ew_n - 1) *
                          (2. * (g.y - g.camber_line) *
                             (-c * FSPH_PI / 2. * cos(FSPH_PI / 2. * x)) -
                           th * th * 2 * x * (sz * sz - 2 * x * x));
        const double a1 = pp.ew_n * pp.ew_a * pow(g.phi, pp.ew_n - 1) * 2. *
                          (g.y - g.camber_line);
        t[0] = a0 * g.ca - a1 * g.sa;
        t[1] = a0 * g.sa + a1 * g.ca;
      }
      for(int i = 0; i < D; ++i)
        a[i] += t[i];
      return;
    }
    case FSPH_EFORCE_ORBIT: {  // acceleration_orbit (:279-298), 3D
      const double m_t = pp.orb_mns + pp.orb_mwd;
      double t[3] = {0.0, 0.0, 0.0};
      double temp = sq_(rp[0] - pp.orb_a) + sq_(rp[1]) + sq_(rp[2]);
      temp = cu_(temp);
      temp = sqrt(temp);
      const double term1 = -pp.G * pp.orb_mns / temp;
      t[0] += term1 * (rp[0] - pp.orb_a);
      t[1] += term1 * rp[1];
      t[2] += term1 * rp[2];
      const double term2 = pp.G * m_t / cu_(pp.orb_a);
      t[0] += term2 * (rp[0] - pp.orb_a * pp.orb_mns / m_t);
      t[1] += term2 * rp[1];
      for(int i = 0; i < D; ++i)
        a[i] += t[i];
      return;
    }
    default:  // poison: a potential only
      return;
  }
}

// external_force::potential (eforce.h:336-346)
template<int D>
__device__ __forceinline__ double ext_potential(const PhysParams & pp,
  const double * rp) {
  double phi = 0.0;
  for(int k = 0; k < pp.n_eforce; ++k)
    phi += eforce_potential_term<D>(pp, pp.eforce[k], rp);
  return phi;
}

// The potential at particle i's position; no loads without external forces.
template<int D>
__device__ __forceinline__ double ext_potential_of(const PhysParams & pp,
  double * const * f, int i) {
  if(pp.n_eforce == 0)
    return 0.0;
  const double pos[3] = {f[F_X][i], f[F_Y][i], D == 3 ? f[F_Z][i] : 0.0};
  return ext_potential<D>(pp, pos);
}

// external_force::acceleration (eforce.h:325-334): the sum of the terms,
// starting from zero
template<int D>
__device__ __forceinline__ void ext_acceleration(const PhysParams & pp,
  const double * rp, double * a) {
  for(int i = 0; i < D; ++i)
    a[i] = 0.0;
  for(int k = 0; k < pp.n_eforce; ++k)
    eforce_accel_term<D>(pp, pp.eforce[k], rp, a);
}

// external_force::acceleration_drag (eforce.h:441-451)
template<int D>
__device__ __forceinline__ void drag_acceleration(const PhysParams & pp,
  const double * vel, double * acc) {
  double v2 = vel[0] * vel[0];
  for(int i = 1; i < D; ++i)
    v2 += vel[i] * vel[i];
  for(int i = 0; i < D; ++i)
    acc[i] = 0.0 - (pp.relax_beta + pp.relax_gamma * v2) * vel[i];
}

}  // namespace fsph
