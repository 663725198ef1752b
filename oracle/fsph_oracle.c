/*
 * fsph_oracle.c -- plain-C restatement of FleCSPH's per-step particle path.
 *
 * TEST INFRASTRUCTURE: the CPU oracle the GPU library is checked against and
 * the timed CPU baseline.  It is never linked into, loaded by or called from
 * the GPU product path (flecsph_gb300/).
 *
 * What it restates (paths inside the laristra/flecsph tree):
 *   range              mpisph/bodies_system.h:231-268
 *   Morton keys        include/tree_topology/filling_curve.h:503-525
 *   sort (key, id)     mpisph/bodies_system.h:195-206, mpisph/psort.h:247-253
 *   octree + COM data  include/tree_topology/tree_topology.h:878-997,1894-1970
 *                      include/physics/default_physics.h:59-119
 *   groups + walk      include/tree_topology/tree_topology.h:212-442
 *   geometry tests     include/tree_topology/tree_geometry.h:152-366
 *   physics            include/physics/default_physics.h, kernels.h,
 *                      viscosity.h, eos/eos.h, integration.h
 *   driver step        app/drivers/hydro/main_driver.cc:98-279
 *
 * Every floating-point expression keeps the reference's operand order; build
 * with -ffp-contract=off so no multiply-add is fused (the reference's x86
 * build has no FMA).  The result: neighbour lists in the reference's own
 * order and bit-identical FP64 fields on the same input (up to ulp-level
 * differences of libm pow/sqrt/cbrt between platforms).
 *
 * Two implementation choices keep results identical while allowing threads:
 *  - the reference walks groups in descending Morton order and, inside the
 *    density pass, computes the signal speed of a particle right after its
 *    own sound speed, so a neighbour b already visited (sorted index
 *    b > a) contributes its new sound speed and any other neighbour its old
 *    one (default_physics.h:236-265,309-320, tree_topology.h:220-235,
 *    401-408).  This file evaluates that rule explicitly instead of relying
 *    on visiting order;
 *  - the reference's compressed chains of single-child nodes are kept
 *    implicitly: a node records the top and bottom level of its chain and
 *    the COM/radius/lap of the chain's top node are derived with the same
 *    arithmetic compute_cofm applies to a one-child node.
 */
#include "fsph_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define GROUP_MAX 128 /* tree_topology.h:2121 sub_entities_ */
static const double TINY = 1e10 * DBL_MIN; /* kernels.h:64, viscosity.h:36 */

/* ---------------------------------------------------------------- tree -- */
typedef struct {
  int64_t s, e;      /* particle range [s, e) in sorted order */
  int ltop, lbot;    /* level of the chain's top node and of the branching node */
  double com[3], mass, radius, lap;          /* branching (bottom) node */
  double tcom[3], tmass, tradius, tlap;      /* chain top node */
  double bmin[3], bmax[3];
  int64_t sub;
  int nchild;
  int64_t child[8]; /* >= 0: node index; < 0: ~particle index */
} onode;

typedef struct {
  int64_t * q;
  int64_t * nq;
  int64_t qcap;
  int64_t ** nb; /* per member neighbour lists */
  int64_t * nbn;
  int64_t * nbcap;
} scratch;

struct orc_ctx {
  fsph_params p;
  int D;
  int64_t n, cap;
  int64_t nreal; /* real particles hold ids [0, nreal); WALL copies above */
  double *x[3], *v[3], *vh[3], *a[3], *ga[3];
  double *gpot, *m, *h, *rho, *P, *cs, *u, *e, *dudt, *dedt, *K, *alpha, *vsig,
    *dtp, *divv, *ddivvdt, *Ye;
  int64_t * id;
  uint64_t * key;
  double * csnew;
  /* time (physics:: globals, default_physics.h:32-39) */
  double dt, dt_saved, totaltime, totaltime_next;
  double t_screen, t_scalar, t_h5;
  int64_t iteration;
  double range[2][3];
  double kernel_width;
  /* tree */
  onode * nodes;
  int64_t nnodes, node_cap;
  int * edepth;
  int64_t * groups;
  int64_t ngroups;
  int tree_ok;
  int nthreads;
  int err;
};

static int max_depth_of(int D) { return 63 / D; }

static int digit_of(const orc_ctx * c, uint64_t key, int level) {
  int md = max_depth_of(c->D);
  return (int)((key >> ((md - level) * c->D)) & ((1u << c->D) - 1));
}

static int lcp_levels(const orc_ctx * c, uint64_t a, uint64_t b) {
  int md = max_depth_of(c->D);
  int l = 0;
  while(l < md && digit_of(c, a, l + 1) == digit_of(c, b, l + 1))
    ++l;
  return l;
}

/* ------------------------------------------------------ small helpers -- */
static inline double dmax_(double a, double b) { return (a < b) ? b : a; } /* std::max */
static inline double dmin_(double a, double b) { return (b < a) ? b : a; } /* std::min */

static double dist_pts(int D, const double * a, const double * b) {
  /* flecsi::distance (space_vector.h:47-58) */
  double sum = 0;
  for(int d = 0; d < D; ++d)
    sum += (a[d] - b[d]) * (a[d] - b[d]);
  return sqrt(sum);
}

static void getx(const orc_ctx * c, int64_t i, double * o) {
  for(int d = 0; d < c->D; ++d)
    o[d] = c->x[d][i];
}

/* ------------------------------------------------------------ kernels -- */
static const double cubic_sigma[3] = {4. / 3., 40. / (7. * M_PI), 8. / M_PI};
static const double wc2_sigma[3] = {1.25, 7. / M_PI, 21. / (2. * M_PI)};
static const double wc4_sigma[3] = {1.5, 9. / M_PI, 495. / (32. * M_PI)};
static const double wc6_sigma[3] = {55. / 32., 78. / (7. * M_PI),
  1365. / (64. * M_PI)};
static const double quintic_sigma[3] = {1. / 40., 63. / (478. * M_PI),
  81. / (359. * M_PI)};
/* kernels.h:47-55 writes these as long-double literals; the doubles they
 * round to */
static const double gaussian_sigma[3] = {0x1.b14ea2d5440dap+0,
  0x1.6ebcfdd1ce67cp+1, 0x1.36768dfdddb6bp+2};
static const double super_gaussian_sigma[3] = {0x1.b13778577c0efp+0,
  0x1.6e54d13f8aff2p+1, 0x1.354cb7a91e8ccp+2};

/* kernel<K,D>(r, h): kernels.h:106-121 (cubic), :282-312 (C2), :375-410
 * (C4), :477-512 (C6). */
/* set_sinc_kernel_normalization (kernels.h:67-77) */
static double sinc_sigma(const orc_ctx * c) {
  static const double b0[3] = {-1.5404568e-2, 5.2245027e-2, 2.7012593e-2};
  static const double b1[3] = {3.6632876e-1, 1.3090245e-1, 2.0410827e-2};
  static const double b2[3] = {-4.6519576e-4, 1.9358485e-2, 3.7451957e-3};
  static const double b3[3] = {7.3658324e-2, -6.1642906e-3, 4.7013839e-2};
  const double si = c->p.sph_sinc_index, sq = sqrt(si), s2 = si * si;
  if(c->D == 1)
    return 2. * (b0[0] + b1[0] * sq + b2[0] * si + b3[0] / sq);
  if(c->D == 2)
    return 4. * (b0[1] + b1[1] * si + b2[1] / si + b3[1] / s2);
  return 8. * (b0[2] + b1[2] * sq + b2[2] * si + b3[2] * sq * si);
}

static double kfun(const orc_ctx * c, double r, double h) {
  const int D = c->D;
  switch(c->p.sph_kernel) {
    case FSPH_KERNEL_SINC: { /* kernels.h:633-661 */
      double rh = fabs(r / h), rh2;
      const double eps = 1e-24;
      const double eps_root = sqrt(eps);
      const double eps_root4 = sqrt(eps_root);
      double result = 0.;
      if(rh < 1.) {
        double hd = h;
        for(int i = 1; i < D; i++)
          hd *= h;
        double sinc = 1.0;
        rh *= M_PI;
        if(rh > eps_root4)
          sinc = sin(rh) / rh;
        else if(rh > eps) {
          rh2 = rh * rh;
          sinc += rh2 * (.05 * rh2 - 1.) / 6.;
        }
        result = sinc_sigma(c) / hd * pow(sinc, c->p.sph_sinc_index);
      }
      return result;
    }
    case FSPH_KERNEL_QUINTIC_SPLINE: { /* kernels.h:217-235 */
      double rh = 3. * r / h;
      double result = 0.;
      if(rh < 3.) {
        result = pow(3 - rh, 5);
        if(rh < 2.)
          result += -6 * pow(2 - rh, 5);
        if(rh < 1.)
          result += 15 * pow(1 - rh, 5);
        double sigma = quintic_sigma[D - 1] / pow(h, D);
        result *= sigma;
      }
      return result;
    }
    case FSPH_KERNEL_GAUSSIAN: { /* kernels.h:167-179 */
      double rh = 3. * r / h;
      double result = 0.;
      if(rh <= 3.) {
        double sigma = gaussian_sigma[D - 1] / pow(h, D);
        result = sigma * exp(-rh * rh);
      }
      return result;
    }
    case FSPH_KERNEL_SUPER_GAUSSIAN: { /* kernels.h:581-590 */
      double rh = 3. * r / h, rh2 = rh * rh;
      double sigma = super_gaussian_sigma[D - 1] / pow(h, D);
      double result = sigma * exp(-rh2) * (D / 2.0 + 1 - rh2);
      return result * (fabs(rh) < 3.);
    }
    case FSPH_KERNEL_CUBIC_SPLINE: {
      double rh = 2. * r / h;
      double result = 0.;
      if(rh < 2.0) {
        if(rh < 1.0)
          result = 1.0 - 1.5 * rh * rh + .75 * rh * rh * rh;
        else
          result = 0.25 * (2 - rh) * (2 - rh) * (2 - rh);
        result *= cubic_sigma[D - 1] / pow(h, D);
      }
      return result;
    }
    case FSPH_KERNEL_WENDLAND_C2: {
      double rh = r / h;
      double hd = (D == 3) ? h * h * h : h * h;
      double rh2 = (1 - rh) * (1 - rh);
      double sigma = wc2_sigma[D - 1] / hd;
      double result = sigma * rh2 * rh2 * (4 * rh + 1);
      return result * (rh < 1.0);
    }
    case FSPH_KERNEL_WENDLAND_C4: {
      double rh = r / h;
      double hd = (D == 3) ? h * h * h : h * h;
      double rh1 = 1 - rh;
      double rh2 = rh1 * rh1;
      double rh6 = rh2 * rh2 * rh2;
      double sigma = wc4_sigma[D - 1] / hd;
      double result = sigma * rh6 * (1 + rh * (6 + rh * 35 / 3));
      return result * (rh < 1.0);
    }
    case FSPH_KERNEL_WENDLAND_C6:
    default: {
      double rh = r / h;
      double hd = (D == 3) ? h * h * h : h * h;
      double rh2 = (1 - rh) * (1 - rh);
      double rh4 = rh2 * rh2;
      double sigma = wc6_sigma[D - 1] / hd;
      double result = sigma * rh4 * rh4 * (1 + rh * (8 + rh * (25 + rh * 32)));
      return result * (rh < 1.0);
    }
  }
}

/* kernel_gradient<K,D>(vecP, h): kernels.h:132-153 (cubic), :322-361 (C2),
 * :435-463 (C4), :536-566 (C6). */
static void kgrad(const orc_ctx * c, const double * p, double h, double * out) {
  const int D = c->D;
  double r = 0;
  for(int d = 0; d < D; ++d)
    r += p[d] * p[d];
  r = sqrt(r); /* flecsi::magnitude */
  switch(c->p.sph_kernel) {
    case FSPH_KERNEL_SINC: { /* kernels.h:671-698 */
      double rh = fabs(r / h), rh2;
      const double eps = 1e-24;
      const double eps_root = sqrt(eps);
      const double eps_root4 = sqrt(eps_root);
      const double n = c->p.sph_sinc_index;
      for(int d = 0; d < D; ++d)
        out[d] = 0.0;
      if(rh < 1.) {
        double hd = h * h;
        for(int i = 1; i < D; i++)
          hd *= h;
        double sigma = sinc_sigma(c) / hd;
        rh *= M_PI;
        double dWdr = 0.0;
        if(rh > eps_root4) {
          double sinc = sin(rh) / rh, cosx = cos(rh) / rh;
          dWdr = -n * pow(sinc, n - 1) * M_PI * (sinc / rh - cosx);
        }
        else if(rh > eps) {
          rh2 = rh * rh;
          dWdr = -n * rh / 3. * M_PI * (1 - .5 * rh2 * (.2 - (n - 1) / 18));
        }
        for(int d = 0; d < D; ++d)
          out[d] = p[d] * sigma * dWdr / (r + TINY);
      }
      return;
    }
    case FSPH_KERNEL_QUINTIC_SPLINE:   /* kernels.h:246-270 */
    case FSPH_KERNEL_GAUSSIAN: {       /* kernels.h:189-205 */
      double rh = 3. * r / h;
      for(int d = 0; d < D; ++d)
        out[d] = 0.0;
      if(rh < 3.) {
        double sigma, dWdr;
        if(c->p.sph_kernel == FSPH_KERNEL_QUINTIC_SPLINE) {
          sigma = 3. * quintic_sigma[D - 1] / pow(h, D + 1);
          dWdr = -5. * pow(3 - rh, 4);
          if(rh < 2.)
            dWdr += 30. * pow(2 - rh, 4);
          if(rh < 1.)
            dWdr += -75. * pow(1 - rh, 4);
        }
        else {
          sigma = 3. * gaussian_sigma[D - 1] / pow(h, D + 1);
          dWdr = -2. * rh * exp(-rh * rh);
        }
        for(int d = 0; d < D; ++d)
          out[d] = p[d] * sigma * dWdr / (r + TINY);
      }
      return;
    }
    case FSPH_KERNEL_SUPER_GAUSSIAN: { /* kernels.h:600-613 */
      double rh = 3. * r / h;
      double sigma = 3. * super_gaussian_sigma[D - 1] / pow(h, D + 1);
      double dWdr = exp(-rh * rh) * (2. * pow(rh, 3.) - (D + 4.) * rh);
      double f = (rh < 3.0) * (sigma * dWdr / (r + TINY));
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * f;
      return;
    }
    case FSPH_KERNEL_CUBIC_SPLINE: {
      double rh = 2. * r / h;
      for(int d = 0; d < D; ++d)
        out[d] = 0.0;
      if(rh < 2.0) {
        double dWdr;
        double sigma = 2. * cubic_sigma[D - 1] / pow(h, D + 1);
        if(rh < 1.0)
          dWdr = -3.0 * rh + 9. / 4. * rh * rh;
        else
          dWdr = -.75 * (2 - rh) * (2 - rh);
        for(int d = 0; d < D; ++d)
          out[d] = p[d] * sigma * dWdr / (r + TINY);
      }
      return;
    }
    case FSPH_KERNEL_WENDLAND_C2: {
      double rh = r / h;
      double hd1 = (D == 3) ? h * h * h * h : h * h * h;
      double rh2 = (1 - rh) * (1 - rh);
      double sigma = 2. * wc2_sigma[D - 1] / hd1;
      double dWdr = -10. * rh * rh2 * (1 - rh);
      double f = (rh < 1.0) * (sigma * dWdr / (r + TINY));
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * f;
      return;
    }
    case FSPH_KERNEL_WENDLAND_C4: {
      double rh = r / h;
      double hd1 = (D == 3) ? h * h * h * h : h * h * h;
      double rh2 = (1 - rh) * (1 - rh);
      double rh3 = rh2 * (1 - rh);
      double sigma = 14. * wc4_sigma[D - 1] / hd1;
      double dWdr = -4. / 3. * rh * rh3 * rh2 * (1 + 5. * rh);
      double f = (rh < 1.0) * (sigma * dWdr / (r + TINY));
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * f;
      return;
    }
    case FSPH_KERNEL_WENDLAND_C6:
    default: {
      double rh = r / h;
      double hd1 = (D == 3) ? h * h * h * h : h * h * h;
      double rh2 = (1 - rh) * (1 - rh);
      double rh3 = rh2 * (1 - rh);
      double rh4 = rh2 * rh2;
      double sigma = wc6_sigma[D - 1] / hd1;
      double dWdr = -22. * rh * rh4 * rh3 * (1 + rh * (7 + rh * 16));
      double f = (rh < 1.0) * (sigma * dWdr / (r + TINY));
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * f;
      return;
    }
  }
}

/* viscosity::mu (viscosity.h:81-93) */
static double visc_mu(const orc_ctx * c, double h_ab, const double * vel_ab,
  const double * pos_ab) {
  double dotp = 0, dist2 = 0;
  for(int d = 0; d < c->D; ++d)
    dotp += vel_ab[d] * pos_ab[d];
  for(int d = 0; d < c->D; ++d)
    dist2 += pos_ab[d] * pos_ab[d];
  double result = h_ab * dotp /
                  (dist2 + c->p.sph_viscosity_epsilon * h_ab * h_ab + TINY);
  return result * (dotp < 0.0);
}

/* sph_artificial_viscosity: viscosity_function<visc_constant>
 * (viscosity.h:128-137) ignores alpha_ab; <visc_cullen> (:150-158) uses
 * alpha_ab = (alpha_a + alpha_b) / 2 (default_physics.h:388). */
static double visc_pi(const orc_ctx * c, int64_t a, int64_t b, double rho_ab,
  double c_ab, double mu_ab) {
  if(c->p.sph_viscosity == FSPH_VISC_CULLEN) {
    const double alpha_ab = .5 * (c->alpha[a] + c->alpha[b]);
    return -alpha_ab * (c_ab - 2.0 * mu_ab) * mu_ab / rho_ab;
  }
  return (-c->p.sph_viscosity_alpha * c_ab + c->p.sph_viscosity_beta * mu_ab) *
         mu_ab / rho_ab;
}

/* ---------------------------------------------------------------- EOS -- */
/* eos_t<wd> constants and functions (eos/eos.h:225-315) */
#define WD_A 6.00233181e22
#define WD_B 9.73932099e5
#define C_LIGHT_CGS 2.99792458e10
static double wd_x(double rho, double Ye) { return cbrt(rho * Ye / WD_B); }
static double wd_pressure(double rho, double Ye) {
  double x = wd_x(rho, Ye), x2 = x * x;
  return WD_A * (x * (2. * x2 - 3.) * sqrt(x2 + 1.) + 3. * asinh(x));
}
static double wd_soundspeed(double rho, double Ye) {
  double x = wd_x(rho, Ye), x2 = x * x;
  double numer = (1. + x2) * (6. * x2 - 3.) + 3. + x2 * (2. * x2 - 3.);
  double denom = (1. + x2) * (6. * x2 + 1.) - 1. + x2 * (2. * x2 + 1.);
  return sqrt(numer / (3. * denom)) * C_LIGHT_CGS;
}
static double wd_internal_energy(double rho, double Ye) {
  const double x = wd_x(rho, Ye), x2 = x * x, x3 = x * x * x;
  return WD_A / rho * (8. * x3 * (sqrt(x2 + 1.) - 1.) -
                       (x * (2. * x2 - 3.) * sqrt(x2 + 1.) + 3. * asinh(x)));
}

/* eos_t<>::compute_pressure + compute_soundspeed (eos/eos.h:57-431):
 * ideal, polytropic, wd, ppt; no_eos leaves both as they are. */
static void eos_pressure(orc_ctx * c, int64_t i, double uval, double * P,
  double * cs) {
  const double g = c->p.poly_gamma;
  const double rho = c->rho[i];
  switch(c->p.eos_type) {
    case FSPH_EOS_POLYTROPIC:
      *P = c->K[i] * pow(rho, g);
      *cs = sqrt(c->K[i] * g * pow(rho, g - 1.));
      return;
    case FSPH_EOS_WD:
      *P = wd_pressure(rho, c->Ye[i]);
      *cs = wd_soundspeed(rho, c->Ye[i]);
      return;
    case FSPH_EOS_PPT: {
      const double g2 = c->p.poly_gamma2, thr = c->p.ppt_density_thr;
      const double K1 = c->K[i];
      if(rho < thr)
        *P = K1 * pow(rho, g);
      else
        *P = K1 * pow(thr, g - g2) * pow(rho, g2);
      if(rho < thr)
        *cs = sqrt(K1 * g * pow(rho, g - 1.));
      else {
        double K2 = K1 * pow(thr, g - g2);
        *cs = sqrt(K2 * g2 * pow(rho, g2 - 1.));
      }
      return;
    }
    case FSPH_EOS_NO_EOS:
      *P = c->P[i];
      *cs = c->cs[i];
      return;
    default:
      *P = (g - 1.) * rho * uval;
      *cs = sqrt(g * (g - 1.) * uval);
  }
}

/* ------------------------------------------------------------ context -- */
/* ---- external forces (include/physics/eforce.h), density profiles
 * (include/physics/density_profiles.h:64-230) and the relaxation drag ---- */
#define ORC_PI 3.14159265358979323846
static double sq_(double x) { return x * x; }
static double cu_(double x) { return x * x * x; }

/* mesa_mass_helper (density_profiles.h:163-177) */
static double mesa_mass_helper(int D, double r, double q) {
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
/* density_profiles::select (:355-398) sets mesa_rho0 this way */
static double mesa_rho0(const orc_ctx * c) {
  const double q = c->p.mesa_rim_width;
  return c->D == 2 ? 1. / (ORC_PI * mesa_mass_helper(2, 1., q))
                   : 1. / (4. * ORC_PI * mesa_mass_helper(3, 1., q));
}
/* spherical_density_profile (:69-80, 107-120, 179-188) */
static double prof_rho(const orc_ctx * c, double r) {
  const int D = c->D;
  if(c->p.density_profile == FSPH_DENSITY_PARABOLIC)
    return D == 2 ? 2. / ORC_PI * (1. - sq_(r)) : 15. / (8. * ORC_PI) * (1. - sq_(r));
  if(c->p.density_profile == FSPH_DENSITY_MESA) {
    const double q = c->p.mesa_rim_width, rho0 = mesa_rho0(c), r0 = 1. - q;
    double rho = 0.0;
    if(r < 1. - q)
      rho = rho0;
    else if(r < .9999)
      rho = rho0 * (1. - sq_(r - r0) / sq_(q));
    return rho;
  }
  return D == 2 ? 1.0 / ORC_PI : 0.75 / ORC_PI;
}
/* spherical_drho_dr (:98-101, 137-150, 215-222) */
static double prof_drho(const orc_ctx * c, double r) {
  const int D = c->D;
  if(c->p.density_profile == FSPH_DENSITY_PARABOLIC)
    return D == 2 ? -4. / ORC_PI * r : -15. / (4. * ORC_PI) * r;
  if(c->p.density_profile == FSPH_DENSITY_MESA) {
    const double q = c->p.mesa_rim_width, rho0 = mesa_rho0(c), r0 = 1. - q;
    double drhodr = 0.0;
    if(r > 1. - q && r < .9999)
      drhodr = -2. * rho0 * (r - r0) / sq_(q);
    return drhodr;
  }
  return 0.;
}

static double radius3(int D, const double * rp) {
  double r = rp[0] * rp[0];
  for(int i = 1; i < D; ++i)
    r += rp[i] * rp[i];
  return sqrt(r);
}

/* wall potentials and accelerations (eforce.h:46-121) */
static double wall_pot(const orc_ctx * c, int I, const double * rp) {
  const double box[3] = {.5 * c->p.box_length, .5 * c->p.box_width, .5 * c->p.box_height};
  const double pw_n = c->p.extforce_wall_powerindex, pw_a = c->p.extforce_wall_steepness;
  return (((rp[I] < -box[I]) ? pow(-rp[I] - box[I], pw_n) : 0.0) +
          ((rp[I] > box[I]) ? pow(rp[I] - box[I], pw_n) : 0.0)) * pw_a;
}
static double wall_acc(const orc_ctx * c, int I, const double * rp) {
  const double box[3] = {.5 * c->p.box_length, .5 * c->p.box_width, .5 * c->p.box_height};
  const double pw_n = c->p.extforce_wall_powerindex, pw_a = c->p.extforce_wall_steepness;
  return (((rp[I] < -box[I]) ? pow(-rp[I] - box[I], pw_n - 1) : 0.0) -
          ((rp[I] > box[I]) ? pow(rp[I] - box[I], pw_n - 1) : 0.0)) * pw_n * pw_a;
}
static void sphwall_acc(const orc_ctx * c, const double * rp, double * a) {
  const double pw_n = c->p.extforce_wall_powerindex, pw_a = c->p.extforce_wall_steepness;
  const double R = c->p.sphere_radius;
  for(int i = 0; i < 3; ++i)
    a[i] = 0.0;
  double r = radius3(c->D, rp);
  if(r > R) {
    const double ar = pw_n * pw_a * pow(r - R, pw_n - 1);
    for(int i = 0; i < c->D; ++i)
      a[i] = -rp[i] / r * ar;
  }
}
static double sphwall_pot(const orc_ctx * c, const double * rp) {
  double phi = 0.0;
  double r = radius3(c->D, rp);
  if(r > c->p.sphere_radius)
    phi = c->p.extforce_wall_steepness * pow(r - c->p.sphere_radius, c->p.extforce_wall_powerindex);
  return phi;
}

/* airfoil (eforce.h:213-271) */
static int airfoil(const orc_ctx * c, const double * rp, double * xo, double * yo,
  double * cam, double * phi) {
  const fsph_params * p = &c->p;
  const double x1 = rp[0] - p->airfoil_anchor_x, y1 = rp[1] - p->airfoil_anchor_y,
               alpha = p->airfoil_attack_angle * ORC_PI / 180.0;
  const double x = x1 * cos(alpha) + y1 * sin(alpha), y = -x1 * sin(alpha) + y1 * cos(alpha);
  const int inside = fabs(y) < 5.0 * p->airfoil_thickness && x > -p->airfoil_size * 0.02 &&
                     x < p->airfoil_size * 1.02;
  double upper = p->airfoil_thickness * x * sqrt(p->airfoil_size * p->airfoil_size - x * x);
  double camber_line = p->airfoil_camber * sin(ORC_PI * x / 2.);
  *phi = sq_(upper) - sq_(y - camber_line) + 0.002;
  *xo = x;
  *yo = y;
  *cam = camber_line;
  return inside;
}

/* one term of external_force::potential (eforce.h:336-346) */
static double eforce_pot(const orc_ctx * c, int code, const double * rp) {
  const fsph_params * p = &c->p;
  const int D = c->D;
  switch(code) {
    case FSPH_EFORCE_WALLS_X: return wall_pot(c, 0, rp);
    case FSPH_EFORCE_WALLS_Y: return wall_pot(c, 1, rp);
    case FSPH_EFORCE_WALLS_Z: return wall_pot(c, 2, rp);
    case FSPH_EFORCE_SPHERICAL_WALL: return sphwall_pot(c, rp);
    case FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT: {
      const double K0 = p->pressure_initial / pow(p->rho_initial, p->poly_gamma);
      const double rho0 = prof_rho(c, 0.);
      double r = radius3(D, rp);
      const double x = r / p->sphere_radius;
      double rho = p->rho_initial / rho0 * prof_rho(c, x);
      double phi = (rho > 0) ? (-K0 * p->poly_gamma * pow(rho, p->poly_gamma - 1.) /
                                (p->poly_gamma - 1.)) : 0;
      return phi + sphwall_pot(c, rp);
    }
    case FSPH_EFORCE_GRAVITY: {
      double height = rp[0];
      if(D > 1)
        height = rp[1];
      return height * p->gravity_acceleration_constant;
    }
    case FSPH_EFORCE_AIRFOIL: {
      double x, y, cam, aux, phi = 0.0;
      int inside = airfoil(c, rp, &x, &y, &cam, &aux);
      if(inside && aux > 0.0)
        phi = p->extforce_wall_steepness * pow(aux, p->extforce_wall_powerindex);
      return phi;
    }
    case FSPH_EFORCE_ORBIT: {
      const double grav = p->gravitational_constant, a_sp = p->orbital_separation,
                   m_ns = p->mass_neutron_star, m_wd = p->mass_white_dwarf;
      const double m_t = m_ns + m_wd;
      double term1 = sqrt(sq_(rp[0] - a_sp) + sq_(rp[1]) + sq_(rp[2]));
      term1 = -grav * m_ns / term1;
      double term2 = -0.5 * grav * m_t / cu_(a_sp);
      term2 = term2 * (sq_(rp[0] - a_sp * m_ns / m_t) + sq_(rp[1]));
      return term1 + term2;
    }
    case FSPH_EFORCE_POISON: return p->zero_potential_poison_value;
  }
  return 0.0;
}

static double ext_potential(const orc_ctx * c, const double * rp) {
  double phi = 0.0;
  for(int k = 0; k < FSPH_MAX_EFORCE && c->p.external_force[k] != FSPH_EFORCE_NONE; ++k)
    phi += eforce_pot(c, c->p.external_force[k], rp);
  return phi;
}

/* external_force::acceleration (eforce.h:325-334) */
static void ext_acceleration(const orc_ctx * c, const double * rp, double * a) {
  const fsph_params * p = &c->p;
  const int D = c->D;
  for(int i = 0; i < 3; ++i)
    a[i] = 0.0;
  for(int k = 0; k < FSPH_MAX_EFORCE && p->external_force[k] != FSPH_EFORCE_NONE; ++k) {
    double t[3] = {0.0, 0.0, 0.0};
    switch(p->external_force[k]) {
      case FSPH_EFORCE_WALLS_X: t[0] = wall_acc(c, 0, rp); break;
      case FSPH_EFORCE_WALLS_Y: t[1] = wall_acc(c, 1, rp); break;
      case FSPH_EFORCE_WALLS_Z: t[2] = wall_acc(c, 2, rp); break;
      case FSPH_EFORCE_SPHERICAL_WALL: sphwall_acc(c, rp, t); break;
      case FSPH_EFORCE_SPHERICAL_DENSITY_SUPPORT: {
        const double K0 = p->pressure_initial / pow(p->rho_initial, p->poly_gamma);
        const double rho0 = prof_rho(c, 0.);
        double r = radius3(D, rp);
        const double x = r / p->sphere_radius;
        if(x > 1e-12) {
          double rho = p->rho_initial / rho0 * prof_rho(c, x);
          double drhodr = p->rho_initial / (rho0 * p->sphere_radius) * prof_drho(c, x);
          double a_r = (rho > 0) ? (K0 * p->poly_gamma * pow(rho, p->poly_gamma - 2) * drhodr) : 0;
          for(int i = 0; i < D; ++i)
            t[i] = a_r * rp[i] / r;
        }
        double w[3];
        sphwall_acc(c, rp, w);
        for(int i = 0; i < D; ++i)
          t[i] = t[i] + w[i];
        break;
      }
      case FSPH_EFORCE_GRAVITY:
        if(D > 1)
          t[1] = -p->gravity_acceleration_constant;
        else
          t[0] = -p->gravity_acceleration_constant;
        break;
      case FSPH_EFORCE_AIRFOIL: {
        double x, y, cam, phi;
        int inside = airfoil(c, rp, &x, &y, &cam, &phi);
        if(inside && phi > 0.0) {
          const double alpha = p->airfoil_attack_angle * ORC_PI / 180.0;
          const double pw_n = p->extforce_wall_powerindex, pw_a = p->extforce_wall_steepness;
          const double ac = p->airfoil_camber, th = p->airfoil_thickness, sz = p->airfoil_size;
          double a0 = pw_n * pw_a * pow(phi, pw_n - 1) *
                      (2. * (y - cam) * (-ac * ORC_PI / 2. * cos(ORC_PI / 2. * x)) -
                       th * th * 2 * x * (sz * sz - 2 * x * x));
          double a1 = pw_n * pw_a * pow(phi, pw_n - 1) * 2. * (y - cam);
          t[0] = a0 * cos(alpha) - a1 * sin(alpha);
          t[1] = a0 * sin(alpha) + a1 * cos(alpha);
        }
        break;
      }
      case FSPH_EFORCE_ORBIT: {
        const double grav = p->gravitational_constant, a_sp = p->orbital_separation,
                     m_ns = p->mass_neutron_star, m_wd = p->mass_white_dwarf;
        const double m_t = m_ns + m_wd;
        double temp = sq_(rp[0] - a_sp) + sq_(rp[1]) + sq_(rp[2]);
        temp = cu_(temp);
        temp = sqrt(temp);
        double term1 = -grav * m_ns / temp;
        t[0] += term1 * (rp[0] - a_sp);
        t[1] += term1 * rp[1];
        t[2] += term1 * rp[2];
        double term2 = grav * m_t / cu_(a_sp);
        t[0] += term2 * (rp[0] - a_sp * m_ns / m_t);
        t[1] += term2 * rp[1];
        break;
      }
      default: /* poison: no acceleration term */
        continue;
    }
    for(int i = 0; i < D; ++i)
      a[i] += t[i];
  }
}

/* external_force::acceleration_drag (eforce.h:441-451) */
static void drag_acc(const orc_ctx * c, const double * vel, double * acc) {
  double v2 = vel[0] * vel[0];
  for(int i = 1; i < c->D; ++i)
    v2 += vel[i] * vel[i];
  for(int i = 0; i < c->D; ++i)
    acc[i] = 0.0 - (c->p.relaxation_beta + c->p.relaxation_gamma * v2) * vel[i];
}

static void * xalloc(size_t n) {
  void * p = calloc(n ? n : 1, 1);
  return p;
}

orc_ctx * orc_create(const fsph_params * p) {
  if(!p || (p->dimension != 2 && p->dimension != 3))
    return NULL;
  orc_ctx * c = (orc_ctx *)xalloc(sizeof(orc_ctx));
  c->p = *p;
  c->D = p->dimension;
  c->nthreads = 1;
  /* kernels::select (kernels.h:753-767) */
  c->kernel_width = (p->sph_kernel == FSPH_KERNEL_QUINTIC_SPLINE ||
                     p->sph_kernel == FSPH_KERNEL_GAUSSIAN ||
                     p->sph_kernel == FSPH_KERNEL_SUPER_GAUSSIAN) ? 3.0 : 2.0;
  return c;
}

static void free_tree(orc_ctx * c) {
  free(c->nodes);
  free(c->edepth);
  free(c->groups);
  c->nodes = NULL;
  c->edepth = NULL;
  c->groups = NULL;
  c->nnodes = c->node_cap = c->ngroups = 0;
  c->tree_ok = 0;
}

static void free_state(orc_ctx * c) {
  for(int d = 0; d < 3; ++d) {
    free(c->x[d]); free(c->v[d]); free(c->vh[d]); free(c->a[d]); free(c->ga[d]);
  }
  free(c->gpot); free(c->m); free(c->h); free(c->rho); free(c->P); free(c->cs);
  free(c->u); free(c->e); free(c->dudt); free(c->dedt); free(c->K);
  free(c->alpha); free(c->vsig); free(c->dtp); free(c->id); free(c->key);
  free(c->divv); free(c->ddivvdt); free(c->Ye);
  free(c->csnew);
}

void orc_destroy(orc_ctx * c) {
  if(!c)
    return;
  free_state(c);
  free_tree(c);
  free(c);
}

int orc_set_threads(orc_ctx * c, int nthreads) {
  c->nthreads = nthreads > 0 ? nthreads : 1;
  return FSPH_OK;
}

/* analysis::set_initial_time_iteration (analysis.h:221-249) */
static void init_time(orc_ctx * c) {
  const fsph_params * p = &c->p;
  c->iteration = p->initial_iteration;
  c->totaltime = p->initial_time;
  c->dt = p->initial_dt;
  c->dt_saved = 0.0;
  c->totaltime_next = 0.0;
  c->t_screen = c->t_scalar = c->t_h5 = 0.0;
  if(p->out_screen_dt > 0.0) {
    c->t_screen = p->out_screen_dt * ((int64_t)(c->totaltime / p->out_screen_dt));
    if(c->t_screen < c->totaltime) c->t_screen = c->totaltime;
  }
  if(p->out_scalar_dt > 0.0) {
    c->t_scalar = p->out_scalar_dt * ((int64_t)(c->totaltime / p->out_scalar_dt));
    if(c->t_scalar < c->totaltime) c->t_scalar = c->totaltime;
  }
  if(p->out_h5data_dt > 0.0) {
    c->t_h5 = p->out_h5data_dt * ((int64_t)(c->totaltime / p->out_h5data_dt));
    if(c->t_h5 < c->totaltime) c->t_h5 = c->totaltime;
  }
}

static int is_periodic(const orc_ctx * c) {
  return c->p.periodic_boundary_x || c->p.periodic_boundary_y ||
         c->p.periodic_boundary_z;
}

#define CPY_IN(dst, src)                                                       \
  do {                                                                         \
    if(src) memcpy(dst, src, sizeof(double) * n);                              \
    else memset(dst, 0, sizeof(double) * n);                                   \
  } while(0)

int orc_upload(orc_ctx * c, const fsph_soa_view * v) {
  if(!v || v->n < 2 || !v->x || !v->y || (c->D == 3 && !v->z) || !v->m ||
     !v->h || !v->id)
    return FSPH_ERR_ARG;
  const int64_t n = v->n;
  free_state(c);
  free_tree(c);
  c->n = c->cap = n;
  for(int d = 0; d < 3; ++d) {
    c->x[d] = xalloc(8 * n); c->v[d] = xalloc(8 * n); c->vh[d] = xalloc(8 * n);
    c->a[d] = xalloc(8 * n); c->ga[d] = xalloc(8 * n);
  }
  c->gpot = xalloc(8 * n); c->m = xalloc(8 * n); c->h = xalloc(8 * n);
  c->rho = xalloc(8 * n); c->P = xalloc(8 * n); c->cs = xalloc(8 * n);
  c->u = xalloc(8 * n); c->e = xalloc(8 * n); c->dudt = xalloc(8 * n);
  c->dedt = xalloc(8 * n); c->K = xalloc(8 * n); c->alpha = xalloc(8 * n);
  c->vsig = xalloc(8 * n); c->dtp = xalloc(8 * n); c->id = xalloc(8 * n);
  c->divv = xalloc(8 * n); c->ddivvdt = xalloc(8 * n); c->Ye = xalloc(8 * n);
  c->key = xalloc(8 * n); c->csnew = xalloc(8 * n);
  double * const xs[3] = {v->x, v->y, v->z};
  double * const vs[3] = {v->vx, v->vy, v->vz};
  double * const vhs[3] = {v->vhx, v->vhy, v->vhz};
  double * const as[3] = {v->ax, v->ay, v->az};
  double * const gas[3] = {v->gax, v->gay, v->gaz};
  for(int d = 0; d < c->D; ++d) {
    CPY_IN(c->x[d], xs[d]); CPY_IN(c->v[d], vs[d]); CPY_IN(c->vh[d], vhs[d]);
    CPY_IN(c->a[d], as[d]); CPY_IN(c->ga[d], gas[d]);
  }
  CPY_IN(c->gpot, v->gpot); CPY_IN(c->m, v->m); CPY_IN(c->h, v->h);
  CPY_IN(c->rho, v->rho); CPY_IN(c->P, v->P); CPY_IN(c->cs, v->cs);
  CPY_IN(c->u, v->u); CPY_IN(c->e, v->e); CPY_IN(c->dudt, v->dudt);
  CPY_IN(c->dedt, v->dedt); CPY_IN(c->K, v->K); CPY_IN(c->alpha, v->alpha);
  CPY_IN(c->vsig, v->vsig); CPY_IN(c->dtp, v->dt);
  CPY_IN(c->divv, v->divv); CPY_IN(c->ddivvdt, v->ddivvdt); CPY_IN(c->Ye, v->Ye);
  memcpy(c->id, v->id, 8 * n);
  c->nreal = n;
  if(is_periodic(c)) {
    /* the reference's id-sum check (boundary.h:241-246) wants 0..n-1 */
    char * seen = (char *)xalloc(n);
    for(int64_t i = 0; i < n; ++i) {
      if(c->id[i] < 0 || c->id[i] >= n || seen[c->id[i]]) {
        free(seen);
        return FSPH_ERR_ARG;
      }
      seen[c->id[i]] = 1;
    }
    free(seen);
  }
  init_time(c);
  return FSPH_OK;
}

int orc_particle_count(orc_ctx * c, int64_t * total, int64_t * real) {
  if(total) *total = c->n;
  if(real) *real = c->nreal;
  return FSPH_OK;
}

#define CPY_OUT(dst, src)                                                      \
  do {                                                                         \
    if(dst) memcpy(dst, src, sizeof(double) * n);                             \
  } while(0)

int orc_download(orc_ctx * c, fsph_soa_view * v) {
  if(!v || v->n != c->n)
    return FSPH_ERR_ARG;
  const int64_t n = c->n;
  double * const xs[3] = {v->x, v->y, v->z};
  double * const vs[3] = {v->vx, v->vy, v->vz};
  double * const vhs[3] = {v->vhx, v->vhy, v->vhz};
  double * const as[3] = {v->ax, v->ay, v->az};
  double * const gas[3] = {v->gax, v->gay, v->gaz};
  for(int d = 0; d < c->D; ++d) {
    CPY_OUT(xs[d], c->x[d]); CPY_OUT(vs[d], c->v[d]); CPY_OUT(vhs[d], c->vh[d]);
    CPY_OUT(as[d], c->a[d]); CPY_OUT(gas[d], c->ga[d]);
  }
  CPY_OUT(v->gpot, c->gpot); CPY_OUT(v->m, c->m); CPY_OUT(v->h, c->h);
  CPY_OUT(v->rho, c->rho); CPY_OUT(v->P, c->P); CPY_OUT(v->cs, c->cs);
  CPY_OUT(v->u, c->u); CPY_OUT(v->e, c->e); CPY_OUT(v->dudt, c->dudt);
  CPY_OUT(v->dedt, c->dedt); CPY_OUT(v->K, c->K); CPY_OUT(v->alpha, c->alpha);
  CPY_OUT(v->vsig, c->vsig); CPY_OUT(v->dt, c->dtp);
  CPY_OUT(v->divv, c->divv); CPY_OUT(v->ddivvdt, c->ddivvdt); CPY_OUT(v->Ye, c->Ye);
  if(v->id) memcpy(v->id, c->id, 8 * n);
  if(v->key) memcpy(v->key, c->key, 8 * n);
  return FSPH_OK;
}

int orc_get_time(orc_ctx * c, double * dt, double * t, int64_t * it) {
  if(dt) *dt = c->dt;
  if(t) *t = c->totaltime;
  if(it) *it = c->iteration;
  return FSPH_OK;
}

int orc_set_time(orc_ctx * c, double dt, double t, int64_t it) {
  c->dt = dt;
  c->totaltime = t;
  c->iteration = it;
  return FSPH_OK;
}

int orc_get_range(orc_ctx * c, double * r) {
  for(int d = 0; d < c->D; ++d) {
    r[d] = c->range[0][d];
    r[c->D + d] = c->range[1][d];
  }
  return FSPH_OK;
}

/* ------------------------------------------------- update_iteration -- */
typedef struct {
  uint64_t key;
  int64_t id;
  int64_t idx;
} sortrec;

static int cmp_sortrec(const void * a, const void * b) {
  const sortrec * l = (const sortrec *)a;
  const sortrec * r = (const sortrec *)b;
  /* comparator of bodies_system.h:197-205 */
  if(l->key < r->key) return -1;
  if(l->key > r->key) return 1;
  if(l->id < r->id) return -1;
  if(l->id > r->id) return 1;
  return 0;
}

static void permute_d(double ** f, const sortrec * rec, int64_t n, double * tmp) {
  for(int64_t i = 0; i < n; ++i)
    tmp[i] = (*f)[rec[i].idx];
  memcpy(*f, tmp, 8 * n);
}

/* compute_cofm for a chain (one child node, no entities), as
 * default_physics.h:59-119 evaluates it. */
static void chain_up(int D, double * com, double * mass, double * radius,
  double * lap) {
  double nc[3];
  double cm = *mass;
  for(int d = 0; d < D; ++d)
    nc[d] = 0.0 + cm * com[d];
  double nm = 0.0 + cm;
  for(int d = 0; d < D; ++d)
    nc[d] /= nm;
  double dist = dist_pts(D, nc, com);
  double nr = dmax_(0.0, dist + *radius);
  double nl = dmax_(0.0, dist + *radius + *lap);
  for(int d = 0; d < D; ++d)
    com[d] = nc[d];
  *mass = nm;
  *radius = nr;
  *lap = nl;
}

static int64_t build_node(orc_ctx * c, int64_t s, int64_t e, int ltop) {
  const int D = c->D;
  const int md = max_depth_of(D);
  int lbot = lcp_levels(c, c->key[s], c->key[e - 1]);
  if(lbot >= md) {
    c->err = FSPH_ERR_DUPLICATE_KEY;
    return -1;
  }
  if(c->nnodes == c->node_cap) {
    c->node_cap = c->node_cap ? 2 * c->node_cap : 1024;
    c->nodes = (onode *)realloc(c->nodes, sizeof(onode) * c->node_cap);
  }
  int64_t me = c->nnodes++;
  onode nd;
  memset(&nd, 0, sizeof(nd));
  nd.s = s;
  nd.e = e;
  nd.ltop = ltop;
  nd.lbot = lbot;
  /* children: split [s,e) by the digit at level lbot+1 */
  int64_t i = s;
  while(i < e) {
    int dg = digit_of(c, c->key[i], lbot + 1);
    int64_t j = i + 1;
    while(j < e && digit_of(c, c->key[j], lbot + 1) == dg)
      ++j;
    if(j - i == 1) {
      nd.child[nd.nchild++] = ~i;
      c->edepth[i] = lbot + 1;
    }
    else {
      int64_t ci = build_node(c, i, j, lbot + 1);
      if(ci < 0)
        return -1;
      nd.child[nd.nchild++] = ci;
    }
    i = j;
  }
  /* compute_cofm (default_physics.h:59-119): entities first, then nodes,
   * each in child order */
  double coord[3] = {0, 0, 0};
  double mass = 0, radius = 0, lap = 0;
  int64_t sub = 0;
  for(int d = 0; d < D; ++d) {
    nd.bmax[d] = -DBL_MAX;
    nd.bmin[d] = DBL_MAX;
  }
  for(int k = 0; k < nd.nchild; ++k) {
    if(nd.child[k] >= 0)
      continue;
    int64_t p = ~nd.child[k];
    for(int d = 0; d < D; ++d)
      coord[d] += c->m[p] * c->x[d][p];
    mass += c->m[p];
    ++sub;
    for(int d = 0; d < D; ++d) {
      nd.bmin[d] = dmin_(nd.bmin[d], c->x[d][p] - c->h[p] / 2.);
      nd.bmax[d] = dmax_(nd.bmax[d], c->x[d][p] + c->h[p] / 2.);
    }
  }
  for(int k = 0; k < nd.nchild; ++k) {
    if(nd.child[k] < 0)
      continue;
    const onode * ch = &c->nodes[nd.child[k]];
    for(int d = 0; d < D; ++d)
      coord[d] += ch->tmass * ch->tcom[d];
    mass += ch->tmass;
    sub += ch->sub;
    for(int d = 0; d < D; ++d) {
      nd.bmin[d] = dmin_(nd.bmin[d], ch->bmin[d]);
      nd.bmax[d] = dmax_(nd.bmax[d], ch->bmax[d]);
    }
  }
  for(int d = 0; d < D; ++d)
    coord[d] /= mass;
  for(int k = 0; k < nd.nchild; ++k) {
    if(nd.child[k] >= 0)
      continue;
    int64_t p = ~nd.child[k];
    double xp[3];
    getx(c, p, xp);
    double dist = dist_pts(D, coord, xp);
    radius = dmax_(radius, dist);
    lap = dmax_(lap, dist + c->h[p]);
  }
  for(int k = 0; k < nd.nchild; ++k) {
    if(nd.child[k] < 0)
      continue;
    const onode * ch = &c->nodes[nd.child[k]];
    double dist = dist_pts(D, coord, ch->tcom);
    radius = dmax_(radius, dist + ch->tradius);
    lap = dmax_(lap, dist + ch->tradius + ch->tlap);
  }
  for(int d = 0; d < D; ++d)
    nd.com[d] = nd.tcom[d] = coord[d];
  nd.mass = nd.tmass = mass;
  nd.radius = nd.tradius = radius;
  nd.lap = nd.tlap = lap;
  nd.sub = sub;
  for(int l = lbot; l > ltop; --l)
    chain_up(D, nd.tcom, &nd.tmass, &nd.tradius, &nd.tlap);
  c->nodes[me] = nd;
  return me;
}

/* groups in the order traversal_sph visits them (tree_topology.h:220-235):
 * depth-first, highest child first. */
static void collect_groups(orc_ctx * c, int64_t node) {
  const onode * nd = &c->nodes[node];
  if(nd->sub <= GROUP_MAX) {
    c->groups[c->ngroups++] = node;
    return;
  }
  for(int k = nd->nchild - 1; k >= 0; --k) {
    int64_t ch = c->nodes[node].child[k];
    if(ch < 0)
      c->groups[c->ngroups++] = ch;
    else
      collect_groups(c, ch);
  }
}

/* Every per-particle array, for moves of whole particles. */
#define ORC_NFIELDS 30
static void field_list(orc_ctx * c, double *** out) {
  int k = 0;
  for(int d = 0; d < 3; ++d) {
    out[k++] = &c->x[d]; out[k++] = &c->v[d]; out[k++] = &c->vh[d];
    out[k++] = &c->a[d]; out[k++] = &c->ga[d];
  }
  out[k++] = &c->gpot; out[k++] = &c->m; out[k++] = &c->h; out[k++] = &c->rho;
  out[k++] = &c->P; out[k++] = &c->cs; out[k++] = &c->u; out[k++] = &c->e;
  out[k++] = &c->dudt; out[k++] = &c->dedt; out[k++] = &c->K;
  out[k++] = &c->alpha;
  out[k++] = &c->divv; out[k++] = &c->ddivvdt; out[k++] = &c->Ye;
}

static void ensure_cap(orc_ctx * c, int64_t need) {
  if(need <= c->cap)
    return;
  int64_t cap = need + need / 4;
  double ** fs[ORC_NFIELDS];
  field_list(c, fs);
  for(int k = 0; k < ORC_NFIELDS; ++k)
    *fs[k] = (double *)realloc(*fs[k], 8 * cap);
  double ** more[] = {&c->vsig, &c->dtp, &c->csnew};
  for(int k = 0; k < 3; ++k)
    *more[k] = (double *)realloc(*more[k], 8 * cap);
  c->id = (int64_t *)realloc(c->id, 8 * cap);
  c->key = (uint64_t *)realloc(c->key, 8 * cap);
  c->cap = cap;
}

static void copy_particle(orc_ctx * c, int64_t dst, int64_t src) {
  double ** fs[ORC_NFIELDS];
  field_list(c, fs);
  for(int k = 0; k < ORC_NFIELDS; ++k)
    (*fs[k])[dst] = (*fs[k])[src];
  c->vsig[dst] = c->vsig[src];
  c->dtp[dst] = c->dtp[src];
  c->csnew[dst] = c->csnew[src];
  c->id[dst] = c->id[src];
  c->key[dst] = c->key[src];
}

/* Copy of particle i with the given position appended as a WALL particle. */
static void append_copy(orc_ctx * c, int64_t i, const double * pos) {
  const int64_t j = c->n++;
  copy_particle(c, j, i);
  for(int d = 0; d < c->D; ++d)
    c->x[d][j] = pos[d];
  c->id[j] = j; /* c->nreal + running index of the copies (boundary.h:236-240) */
}

/* boundary::add_corner_XX / add_corner_XXX (boundary.h:72-118): the copy
 * across the corner of the axes in dims[0..k). */
static void add_corner(orc_ctx * c, const int * on_edge, const int * dims,
  int k, const double (*box)[3], double halo, int64_t i) {
  for(int t = 0; t < k; ++t)
    if(!on_edge[dims[t]])
      return;
  double pos[3] = {c->x[0][i], c->x[1][i], c->D == 3 ? c->x[2][i] : 0.0};
  for(int t = 0; t < k; ++t) {
    const int d = dims[t];
    const double x = c->x[d][i];
    if(x + halo > box[1][d])
      pos[d] = box[0][d] - fabs(x + box[0][d]);
    else
      pos[d] = box[1][d] + fabs(x + box[1][d]);
  }
  append_copy(c, i, pos);
}

/* boundary::pboundary_clean + pboundary_generate (boundary.h:45-248), as
 * body_system::update_iteration calls them (bodies_system.h:160-169). */
static int periodic_boundaries(orc_ctx * c) {
  const int D = c->D;
  /* clean: keep the real particles in their order (stable_partition) */
  int64_t w = 0;
  for(int64_t i = 0; i < c->n; ++i)
    if(c->id[i] < c->nreal) {
      if(w != i)
        copy_particle(c, w, i);
      ++w;
    }
  if(w == 0)
    return FSPH_ERR_STATE;
  c->n = w;
  /* getSmoothinglength (bodies_system.h:112-124): the largest h */
  double hmax = 0;
  for(int64_t i = 0; i < c->n; ++i)
    if(hmax < c->h[i])
      hmax = c->h[i];
  const double halo = 2.5 * hmax;
  const int periodic[3] = {c->p.periodic_boundary_x, c->p.periodic_boundary_y,
    c->p.periodic_boundary_z};
  const double half = 0.5;
  double box[2][3];
  box[0][0] = -half * c->p.box_length;
  box[1][0] = half * c->p.box_length;
  box[0][1] = -half * c->p.box_width;
  box[1][1] = half * c->p.box_width;
  box[0][2] = -half * c->p.box_height;
  box[1][2] = half * c->p.box_height;
  /* step 1: teleport to the other side */
  for(int64_t i = 0; i < c->n; ++i)
    for(int d = 0; d < D; ++d) {
      if(!periodic[d])
        continue;
      if(c->x[d][i] > box[1][d])
        c->x[d][i] -= box[1][d] - box[0][d];
      else if(c->x[d][i] <= box[0][d])
        c->x[d][i] += box[1][d] - box[0][d];
    }
  /* copies near the faces, then edges and corners */
  const int64_t nreal_now = c->n;
  for(int64_t i = 0; i < nreal_now; ++i) {
    int on_edge[3] = {0, 0, 0};
    for(int d = 0; d < D; ++d) {
      if(!periodic[d])
        continue;
      const double x = c->x[d][i];
      if(x + halo > box[1][d] || x - halo <= box[0][d]) {
        on_edge[d] = 1;
        double pos[3] = {c->x[0][i], c->x[1][i], D == 3 ? c->x[2][i] : 0.0};
        if(x + halo > box[1][d])
          pos[d] -= (box[1][d] - box[0][d]);
        else
          pos[d] += (box[1][d] - box[0][d]);
        ensure_cap(c, c->n + 1);
        append_copy(c, i, pos);
      }
    }
    ensure_cap(c, c->n + 4);
    const int d01[2] = {0, 1}, d02[2] = {0, 2}, d21[2] = {2, 1};
    const int d012[3] = {0, 1, 2};
    if(D == 2)
      add_corner(c, on_edge, d01, 2, (const double (*)[3])box, halo, i);
    if(D == 3) {
      add_corner(c, on_edge, d01, 2, (const double (*)[3])box, halo, i);
      add_corner(c, on_edge, d02, 2, (const double (*)[3])box, halo, i);
      add_corner(c, on_edge, d21, 2, (const double (*)[3])box, halo, i);
      add_corner(c, on_edge, d012, 3, (const double (*)[3])box, halo, i);
    }
  }
  return FSPH_OK;
}

int orc_update_iteration(orc_ctx * c) {
  const int D = c->D;
  free_tree(c);
  if(is_periodic(c)) {
    int st = periodic_boundaries(c);
    if(st)
      return st;
  }
  const int64_t n = c->n;
  if(n < 2)
    return FSPH_ERR_STATE;
  /* mpi_compute_range (bodies_system.h:231-268) */
  double lo[3], hi[3];
  for(int d = 0; d < D; ++d)
    lo[d] = hi[d] = c->x[d][n - 1];
  for(int64_t i = 0; i < n; ++i)
    for(int d = 0; d < D; ++d) {
      if(c->x[d][i] + c->h[i] > hi[d]) hi[d] = c->x[d][i] + c->h[i];
      if(c->x[d][i] - c->h[i] < lo[d]) lo[d] = c->x[d][i] - c->h[i];
    }
  int same = 1;
  for(int d = 0; d < D; ++d) {
    c->range[0][d] = lo[d];
    c->range[1][d] = hi[d];
    if(lo[d] != hi[d]) same = 0;
  }
  if(same)
    return FSPH_ERR_ARG;
  /* keys: morton_curve_u(range, p) (filling_curve.h:503-525) */
  const int md = max_depth_of(D);
  const uint64_t one = 1;
  const uint64_t max_val = (one << (63 / D)) - 1;
  for(int64_t i = 0; i < n; ++i) {
    uint64_t coords[3];
    for(int d = 0; d < D; ++d) {
      double mn = c->range[0][d];
      double scale = c->range[1][d] - mn;
      uint64_t q = (uint64_t)((c->x[d][i] - mn) / scale *
                              (double)(one << (63 / D)));
      coords[d] = q < max_val ? q : max_val;
    }
    uint64_t value = one << (md * D);
    for(int l = 0; l < md; ++l)
      for(int d = 0; d < D; ++d)
        value |= ((coords[d] >> l) & one) << (l * D + d);
    c->key[i] = value;
  }
  /* sort by (key, id) and permute every field */
  sortrec * rec = (sortrec *)malloc(sizeof(sortrec) * n);
  for(int64_t i = 0; i < n; ++i) {
    rec[i].key = c->key[i];
    rec[i].id = c->id[i];
    rec[i].idx = i;
  }
  qsort(rec, n, sizeof(sortrec), cmp_sortrec);
  double * tmp = (double *)malloc(8 * n);
  for(int d = 0; d < 3; ++d) {
    permute_d(&c->x[d], rec, n, tmp); permute_d(&c->v[d], rec, n, tmp);
    permute_d(&c->vh[d], rec, n, tmp); permute_d(&c->a[d], rec, n, tmp);
    permute_d(&c->ga[d], rec, n, tmp);
  }
  double ** fs[] = {&c->gpot, &c->m, &c->h, &c->rho, &c->P, &c->cs, &c->u,
    &c->e, &c->dudt, &c->dedt, &c->K, &c->alpha, &c->vsig, &c->dtp, &c->divv,
    &c->ddivvdt, &c->Ye};
  for(size_t k = 0; k < sizeof(fs) / sizeof(fs[0]); ++k)
    permute_d(fs[k], rec, n, tmp);
  for(int64_t i = 0; i < n; ++i) {
    c->id[i] = rec[i].id;
    c->key[i] = rec[i].key;
  }
  free(tmp);
  free(rec);
  /* tree (tree_topology.h:878-997) */
  c->edepth = (int *)xalloc(sizeof(int) * n);
  c->err = FSPH_OK;
  int64_t root = build_node(c, 0, n, 0);
  if(root != 0 || c->err)
    return c->err ? c->err : FSPH_ERR_STATE;
  c->groups = (int64_t *)xalloc(sizeof(int64_t) * n);
  c->ngroups = 0;
  collect_groups(c, 0);
  c->tree_ok = 1;
  return FSPH_OK;
}

int orc_reset_ghosts(orc_ctx * c) {
  /* bodies_system.h:273-275: clean + build_tree over unchanged keys.  The
   * reference re-runs the build; repeat it so the CPU baseline pays the same
   * cost (results are identical). */
  if(!c->tree_ok)
    return FSPH_ERR_STATE;
  free(c->nodes);
  c->nodes = NULL;
  c->nnodes = c->node_cap = 0;
  c->err = FSPH_OK;
  build_node(c, 0, c->n, 0);
  c->ngroups = 0;
  collect_groups(c, 0);
  return c->err;
}

/* -------------------------------------------------------- the walk -- */
static int within_distance2(int D, const double * p1, const double * p2,
  double r) {
  double s = 0;
  for(int d = 0; d < D; ++d)
    s += (p1[d] - p2[d]) * (p1[d] - p2[d]);
  return s <= r * r;
}

static int intersects_box_box(int D, const double * min1, const double * max1,
  const double * min2, const double * max2) {
  int sep = 0;
  for(int d = 0; d < D; ++d)
    sep |= (max1[d] < min2[d]);
  for(int d = 0; d < D; ++d)
    sep |= (max2[d] < min1[d]);
  return !sep;
}

static int intersects_sphere_box(int D, const double * mn, const double * mx,
  const double * ctr, double r) {
  if(D == 3) { /* tree_geometry.h:329-341 */
    double x[3];
    for(int d = 0; d < 3; ++d)
      x[d] = ctr[d] < mx[d] ? ctr[d] : mx[d];
    for(int d = 0; d < 3; ++d)
      x[d] = x[d] < mn[d] ? mn[d] : x[d];
    double dist = (x[0] - ctr[0]) * (x[0] - ctr[0]) +
                  (x[1] - ctr[1]) * (x[1] - ctr[1]) +
                  (x[2] - ctr[2]) * (x[2] - ctr[2]);
    return dist <= r * r;
  }
  /* 2D: tree_geometry.h:219-227, tol = 10 eps */
  double x[2];
  for(int d = 0; d < 2; ++d)
    x[d] = dmax_(mn[d], dmin_(ctr[d], mx[d]));
  double dist = dist_pts(2, x, ctr);
  return dist - r <= DBL_EPSILON * 10.;
}

static void scratch_init(scratch * s) { memset(s, 0, sizeof(*s)); }

static void scratch_free(scratch * s) {
  free(s->q);
  free(s->nq);
  for(int k = 0; k < GROUP_MAX; ++k)
    if(s->nb) free(s->nb[k]);
  free(s->nb);
  free(s->nbn);
  free(s->nbcap);
}

static void push_nb(scratch * s, int k, int64_t v) {
  if(s->nbn[k] == s->nbcap[k]) {
    s->nbcap[k] = s->nbcap[k] ? 2 * s->nbcap[k] : 256;
    s->nb[k] = (int64_t *)realloc(s->nb[k], sizeof(int64_t) * s->nbcap[k]);
  }
  s->nb[k][s->nbn[k]++] = v;
}

static void push_q(scratch * s, int64_t ** q, int64_t * qn, int64_t v) {
  if(*qn == s->qcap) {
    int64_t nc = s->qcap ? 2 * s->qcap : 4096;
    s->q = (int64_t *)realloc(s->q, sizeof(int64_t) * nc);
    s->nq = (int64_t *)realloc(s->nq, sizeof(int64_t) * nc);
    s->qcap = nc;
    *q = s->nq; /* caller always pushes into nq */
  }
  (*q)[(*qn)++] = v;
}

static const int * g_edepth_sort; /* for the (depth, index) sort */
static int cmp_depth_idx(const void * a, const void * b) {
  int64_t l = *(const int64_t *)a, r = *(const int64_t *)b;
  int dl = g_edepth_sort[l], dr = g_edepth_sort[r];
  if(dl != dr) return dl < dr ? -1 : 1;
  return l < r ? -1 : (l > r ? 1 : 0);
}

static void sort_by_depth(const orc_ctx * c, int64_t * v, int64_t n) {
  /* insertion sort on (edepth, index): lists are short and mostly ordered */
  for(int64_t i = 1; i < n; ++i) {
    int64_t x = v[i];
    int dx = c->edepth[x];
    int64_t j = i - 1;
    while(j >= 0 &&
          (c->edepth[v[j]] > dx || (c->edepth[v[j]] == dx && v[j] > x))) {
      v[j + 1] = v[j];
      --j;
    }
    v[j + 1] = x;
  }
  (void)cmp_depth_idx;
}

/* Neighbour search of one group (tree_topology.h:292-400).  Fills
 * s->nb[k] for members k in cur_entities order (descending index); returns
 * the member count and writes the members to `mem`. */
static int walk_group(const orc_ctx * c, int64_t g, scratch * s, int64_t * mem) {
  const int D = c->D;
  int nm = 0;
  const onode * G = NULL;
  if(g >= 0) {
    G = &c->nodes[g];
    for(int64_t i = G->e - 1; i >= G->s; --i)
      mem[nm++] = i;
  }
  else
    mem[nm++] = ~g;
  if(!s->nb) {
    s->nb = (int64_t **)xalloc(sizeof(int64_t *) * GROUP_MAX);
    s->nbn = (int64_t *)xalloc(sizeof(int64_t) * GROUP_MAX);
    s->nbcap = (int64_t *)xalloc(sizeof(int64_t) * GROUP_MAX);
  }
  for(int k = 0; k < nm; ++k)
    s->nbn[k] = 0;
  double xm[GROUP_MAX][3];
  for(int k = 0; k < nm; ++k)
    getx(c, mem[k], xm[k]);
  int64_t * q;
  int64_t qn = 0, nqn;
  if(s->qcap == 0) {
    s->qcap = 4096;
    s->q = (int64_t *)malloc(sizeof(int64_t) * s->qcap);
    s->nq = (int64_t *)malloc(sizeof(int64_t) * s->qcap);
  }
  s->q[qn++] = 0; /* root */
  while(qn > 0) {
    nqn = 0;
    q = s->nq;
    for(int64_t j = 0; j < qn; ++j) {
      int64_t cell = s->q[j];
      if(cell >= 0) {
        const onode * nd = &c->nodes[cell];
        if(G && !intersects_box_box(D, nd->bmin, nd->bmax, G->bmin, G->bmax))
          continue;
        for(int k = 0; k < nm; ++k) {
          if(intersects_sphere_box(D, nd->bmin, nd->bmax, xm[k], c->h[mem[k]])) {
            for(int l = 0; l < nd->nchild; ++l)
              push_q(s, &q, &nqn, nd->child[l]);
            break;
          }
        }
      }
      else {
        int64_t e = ~cell;
        double xe[3];
        getx(c, e, xe);
        if(G) {
          double extent = dmax_(c->h[e], G->tlap) + G->tradius;
          if(!within_distance2(D, xe, G->tcom, extent))
            continue;
        }
        for(int k = 0; k < nm; ++k) {
          double extent = dmax_(c->h[mem[k]], c->h[e]);
          if(within_distance2(D, xm[k], xe, extent))
            push_nb(s, k, e);
        }
      }
    }
    /* swap queues */
    int64_t * t = s->q;
    s->q = s->nq;
    s->nq = t;
    qn = nqn;
  }
  for(int k = 0; k < nm; ++k)
    sort_by_depth(c, s->nb[k], s->nbn[k]);
  return nm;
}

/* ----------------------------------------------------- pair physics -- */
/* compute_density + recover_internal_energy + EOS (default_physics.h:193-228,
 * 126-145, 309-316); writes rho, u, P and the NEW sound speed into csnew. */
static int density_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double h_a = c->h[a];
  double pa[3];
  getx(c, a, pa);
  double rho_a = 0.0;
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double r = 0;
    for(int d = 0; d < D; ++d) {
      double dd = pa[d] - c->x[d][b];
      r += dd * dd;
    }
    r = sqrt(r);
    double Wab = kfun(c, r, .5 * (h_a + c->h[b]));
    rho_a += c->m[b] * Wab;
  }
  if(!(rho_a > 0))
    return FSPH_ERR_NEG_DENSITY;
  c->rho[a] = rho_a;
  if(c->p.evolve_internal_energy && c->p.thermokinetic_formulation) {
    double vv = 0;
    for(int d = 0; d < D; ++d)
      vv += c->v[d][a] * c->v[d][a];
    double ekin = .5 * vv;
    double eint = c->e[a] - ekin - ext_potential(c, pa);
    if(!(eint > 0))
      return FSPH_ERR_NEG_ENERGY;
    c->u[a] = eint;
  }
  double P, cs;
  eos_pressure(c, a, c->u[a], &P, &cs);
  c->P[a] = P;
  c->csnew[a] = cs;
  if(c->p.sph_viscosity == FSPH_VISC_CULLEN) {
    /* compute_divv (default_physics.h:273-299) */
    double div_v = 0.0;
    for(int64_t j = 0; j < nn; ++j) {
      int64_t b = nb[j];
      double pos_ab[3], DiWab[3];
      for(int d = 0; d < D; ++d)
        pos_ab[d] = pa[d] - c->x[d][b];
      kgrad(c, pos_ab, .5 * (h_a + c->h[b]), DiWab);
      double dot = 0.0;
      for(int d = 0; d < D; ++d)
        dot += c->v[d][a] * DiWab[d];
      div_v += c->m[b] * dot;
    }
    div_v /= c->rho[a];
    const double div_v_p = c->divv[a];
    c->ddivvdt[a] = (div_v - div_v_p) / c->dt;
    c->divv[a] = div_v;
  }
  return FSPH_OK;
}

/* viscosity::compute_alpha with A_trigger and compute_xi (viscosity.h:
 * 185-363). */
static void alpha_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double c_a = c->cs[a], h_a = c->h[a], alpha_a = c->alpha[a];
  const double rho_a = c->rho[a];
  double pa[3];
  getx(c, a, pa);
  /* signal speed (:324-333) */
  double vsig = 0.0;
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pb[3];
    getx(c, b, pb);
    double dist = dist_pts(D, pa, pb);
    double dotv = 0.0;
    for(int d = 0; d < D; ++d)
      dotv += (c->v[d][a] - c->v[d][b]) * ((pa[d] - pb[d]) / dist);
    double cab = dmax_(c_a, c->cs[b]);
    vsig = dmax_(vsig, cab - dmin_(dotv, 0.0));
  }
  /* compute_xi (:200-285) */
  const double divV_a = c->divv[a];
  double R_a = 0.0;
  double gradV[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pb[3], pos_ab[3], vab[3], DiWa[3];
    getx(c, b, pb);
    for(int d = 0; d < D; ++d) {
      pos_ab[d] = pa[d] - pb[d];
      vab[d] = c->v[d][a] - c->v[d][b];
    }
    const double h_ab = .5 * (h_a + c->h[b]);
    kgrad(c, pos_ab, h_ab, DiWa);
    const double Wab = kfun(c, dist_pts(D, pa, pb), h_ab);
    const double dvb = c->divv[b];
    const double sgn = dvb > 0.0 ? 1.0 : (dvb < 0.0 ? -1.0 : dvb);
    R_a += sgn * c->m[b] * Wab;
    for(int i = 0; i < D; ++i)
      for(int k = 0; k < D; ++k)
        gradV[D * i + k] += c->m[b] * (-vab[i]) * DiWa[k];
  }
  R_a /= rho_a;
  for(int k = 0; k < D * D; ++k)
    gradV[k] /= rho_a;
  double traceSS = 0.0;
  for(int i = 0; i < D; ++i) {
    double row[3];
    for(int k = 0; k < D; ++k)
      row[k] = 0.5 * (gradV[D * i + k] + gradV[D * k + i]);
    row[i] -= divV_a / D;
    for(int k = 0; k < D; ++k)
      traceSS += row[k] * row[k];
  }
  const double om = 1.0 - R_a;
  const double t = 2.0 * (om * om * om * om) * divV_a;
  const double res = t * t;
  const double xi = (res < 1e-16) ? 0.0 : res / (res + traceSS);
  /* A_trigger (:293-306) */
  const double Atrig = xi * dmax_(-c->ddivvdt[a], 0.0);
  const double vh = vsig / h_a;
  const double alpha_loc = c->p.sph_viscosity_alpha_max * Atrig /
                           (c->p.sph_viscosity_delta * (vh * vh) + Atrig);
  if(alpha_a <= alpha_loc)
    c->alpha[a] = alpha_loc;
  else {
    const double decayt = h_a / (2.0 * c->p.sph_viscosity_l * vsig);
    const double dalphadt = (alpha_a - alpha_loc) / decayt;
    c->alpha[a] = alpha_a * exp(-dalphadt * c->dt);
  }
}

/* compute_signalspeed (default_physics.h:236-265) with the visiting-order
 * rule for the neighbours' sound speed. */
static void vsig_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double c_a = c->csnew[a];
  double pa[3];
  getx(c, a, pa);
  double vsig = 0.0;
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pb[3];
    getx(c, b, pb);
    double dist = dist_pts(D, pa, pb);
    double dotv = 0;
    for(int d = 0; d < D; ++d) {
      double n_d = (pa[d] - pb[d]) / dist;
      double v_d = c->v[d][a] - c->v[d][b];
      dotv += v_d * n_d;
    }
    double c_b = (b > a || b == a) ? c->csnew[b] : c->cs[b];
    double cab = dmax_(c_a, c_b);
    vsig = dmax_(vsig, cab - dmin_(dotv, 0.0));
  }
  c->vsig[a] = vsig;
}

/* compute_acceleration (default_physics.h:348-408) */
static void accel_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double h_a = c->h[a], rho_a = c->rho[a], P_a = c->P[a], c_a = c->cs[a];
  double pa[3], v12a[3];
  getx(c, a, pa);
  for(int d = 0; d < D; ++d)
    v12a[d] = c->vh[d][a];
  const double Prho2_a = P_a / (rho_a * rho_a);
  double acc[3] = {0, 0, 0};
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pos_ab[3], v12_ab[3], DiWa[3];
    int same = 1;
    for(int d = 0; d < D; ++d) {
      if(c->x[d][b] != pa[d]) same = 0;
      pos_ab[d] = pa[d] - c->x[d][b];
      v12_ab[d] = v12a[d] - c->vh[d][b];
    }
    double m_b = c->m[b] * (!same);
    double h_ab = .5 * (h_a + c->h[b]);
    double mu_ab = visc_mu(c, h_ab, v12_ab, pos_ab);
    double rho_ab = .5 * (rho_a + c->rho[b]);
    double c_ab = .5 * (c_a + c->cs[b]);
    double Pi = visc_pi(c, a, b, rho_ab, c_ab, mu_ab);
    kgrad(c, pos_ab, h_ab, DiWa);
    double Prho2_b = c->P[b] / (c->rho[b] * c->rho[b]);
    double s = -m_b * (Prho2_a + Prho2_b + Pi);
    for(int d = 0; d < D; ++d)
      acc[d] += DiWa[d] * s;
  }
  double ext[3] = {0.0, 0.0, 0.0};
  ext_acceleration(c, pa, ext); /* acc_a += external_force::acceleration (:404) */
  for(int d = 0; d < D; ++d) {
    c->a[d][a] = acc[d] + ext[d];
    c->ga[d][a] = 0;
  }
  c->gpot[a] = 0;
}

/* compute_dudt (default_physics.h:421-487) */
static void dudt_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  if(c->iteration < c->p.relaxation_steps) {
    c->dudt[a] = 0.0;
    return;
  }
  const double h_a = c->h[a], rho_a = c->rho[a], P_a = c->P[a], c_a = c->cs[a];
  double pa[3], va[3], v12a[3];
  getx(c, a, pa);
  for(int d = 0; d < D; ++d) {
    va[d] = c->v[d][a];
    v12a[d] = c->vh[d][a];
  }
  double dp = 0.0, dv = 0.0;
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pos_ab[3], v12_ab[3], vel_ab[3], DiWab[3];
    int same = 1;
    for(int d = 0; d < D; ++d) {
      if(c->x[d][b] != pa[d]) same = 0;
      pos_ab[d] = pa[d] - c->x[d][b];
      v12_ab[d] = v12a[d] - c->vh[d][b];
      vel_ab[d] = va[d] - c->v[d][b];
    }
    double m_b = c->m[b] * (!same);
    double h_ab = .5 * (h_a + c->h[b]);
    double mu_ab = visc_mu(c, h_ab, v12_ab, pos_ab);
    double rho_ab = .5 * (rho_a + c->rho[b]);
    double c_ab = .5 * (c_a + c->cs[b]);
    double Pi = visc_pi(c, a, b, rho_ab, c_ab, mu_ab);
    kgrad(c, pos_ab, h_ab, DiWab);
    double vdw = 0;
    for(int d = 0; d < D; ++d)
      vdw += vel_ab[d] * DiWab[d];
    dp += m_b * vdw;
    dv += m_b * vdw * Pi;
  }
  c->dudt[a] = P_a / (rho_a * rho_a) * dp + .5 * dv;
}

/* compute_dedt (default_physics.h:502-566) */
static void dedt_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double h_a = c->h[a], rho_a = c->rho[a], P_a = c->P[a], c_a = c->cs[a];
  double pa[3], va[3], v12a[3];
  getx(c, a, pa);
  double gv = 0;
  for(int d = 0; d < D; ++d) {
    va[d] = c->v[d][a];
    v12a[d] = c->vh[d][a];
    gv += c->ga[d][a] * va[d];
  }
  const double Prho2_a = P_a / (rho_a * rho_a);
  double dedt = 0;
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    double pos_ab[3], v12_ab[3], DiWab[3];
    int same = 1;
    for(int d = 0; d < D; ++d) {
      if(c->x[d][b] != pa[d]) same = 0;
      pos_ab[d] = pa[d] - c->x[d][b];
      v12_ab[d] = v12a[d] - c->vh[d][b];
    }
    double m_b = c->m[b] * (!same);
    double h_ab = .5 * (h_a + c->h[b]);
    double mu_ab = visc_mu(c, h_ab, v12_ab, pos_ab);
    double rho_ab = .5 * (rho_a + c->rho[b]);
    double c_ab = .5 * (c_a + c->cs[b]);
    double Pi = visc_pi(c, a, b, rho_ab, c_ab, mu_ab);
    kgrad(c, pos_ab, h_ab, DiWab);
    double vad = 0, vbd = 0;
    for(int d = 0; d < D; ++d)
      vad += va[d] * DiWab[d];
    for(int d = 0; d < D; ++d)
      vbd += c->v[d][b] * DiWab[d];
    double Prho2_b = c->P[b] / (c->rho[b] * c->rho[b]);
    dedt -= m_b * (Prho2_a * vbd + vad * Prho2_b + .5 * Pi * (vbd + vad));
  }
  dedt += gv;
  c->dedt[a] = dedt;
}

/* add_short_range_repulsion (default_physics.h:723-753) */
static void repulsion_one(orc_ctx * c, int64_t a, const int64_t * nb, int64_t nn) {
  const int D = c->D;
  const double h_a = c->h[a];
  const int64_t id_a = c->id[a];
  double pa[3], acc_r[3] = {0.0, 0.0, 0.0};
  getx(c, a, pa);
  for(int64_t j = 0; j < nn; ++j) {
    int64_t b = nb[j];
    if(c->id[b] == id_a)
      continue;
    double dx[3], r = 0.0;
    for(int d = 0; d < D; ++d) {
      dx[d] = pa[d] - c->x[d][b];
      r += dx[d] * dx[d];
    }
    double h_ab = .5 * (h_a + c->h[b]);
    double r_ab = sqrt(r);
    if(r_ab > h_ab * c->p.relaxation_repulsion_radius)
      continue;
    double m_b = c->m[b];
    for(int d = 0; d < D; ++d)
      acc_r[d] += m_b * dx[d] / (r_ab * r_ab * r_ab);
  }
  for(int d = 0; d < D; ++d)
    c->a[d][a] = c->a[d][a] + acc_r[d] * c->p.relaxation_repulsion_gamma;
}

enum { PASS_DENSITY, PASS_VSIG, PASS_ACCEL, PASS_DUDT, PASS_DEDT, PASS_ALPHA,
       PASS_REPULSION };

/* apply_in_smoothinglength: walk every group and apply the pass to its
 * members (tree_topology.h:253-409). */
static int run_pass(orc_ctx * c, int pass) {
  if(!c->tree_ok)
    return FSPH_ERR_STATE;
  int status = FSPH_OK;
  const int64_t ng = c->ngroups;
#ifdef _OPENMP
#pragma omp parallel num_threads(c->nthreads)
#endif
  {
    scratch s;
    scratch_init(&s);
    int64_t mem[GROUP_MAX];
    int local = FSPH_OK;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for(int64_t g = 0; g < ng; ++g) {
      int nm = walk_group(c, c->groups[g], &s, mem);
      for(int k = 0; k < nm; ++k) {
        int64_t a = mem[k];
        switch(pass) {
          case PASS_DENSITY: {
            int st = density_one(c, a, s.nb[k], s.nbn[k]);
            if(st && !local) local = st;
            break;
          }
          case PASS_VSIG: vsig_one(c, a, s.nb[k], s.nbn[k]); break;
          case PASS_ACCEL: accel_one(c, a, s.nb[k], s.nbn[k]); break;
          case PASS_DUDT: dudt_one(c, a, s.nb[k], s.nbn[k]); break;
          case PASS_DEDT: dedt_one(c, a, s.nb[k], s.nbn[k]); break;
          case PASS_ALPHA: alpha_one(c, a, s.nb[k], s.nbn[k]); break;
          case PASS_REPULSION: repulsion_one(c, a, s.nb[k], s.nbn[k]); break;
        }
      }
    }
    scratch_free(&s);
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      if(local && !status) status = local;
    }
  }
  return status;
}

int orc_density_pressure_soundspeed(orc_ctx * c) {
  /* compute_density_pressure_soundspeed (default_physics.h:309-320).  The
   * signal speed needs every new sound speed of the pass first; the visiting
   * order rule inside vsig_one reproduces the reference's in-place update. */
  int st = run_pass(c, PASS_DENSITY);
  if(st)
    return st;
  run_pass(c, PASS_VSIG);
  memcpy(c->cs, c->csnew, 8 * c->n);
  return FSPH_OK;
}

int orc_acceleration(orc_ctx * c) { return run_pass(c, PASS_ACCEL); }
int orc_compute_alpha(orc_ctx * c) {
  if(c->p.sph_viscosity != FSPH_VISC_CULLEN)
    return FSPH_ERR_STATE;
  return run_pass(c, PASS_ALPHA);
}
int orc_initialize_alpha(orc_ctx * c) {
  /* viscosity::initialize_alpha (viscosity.h:171-177) */
  const double v = c->p.sph_viscosity == FSPH_VISC_CULLEN ? 0.0 : c->p.sph_viscosity_alpha;
  for(int64_t i = 0; i < c->n; ++i)
    c->alpha[i] = v;
  return FSPH_OK;
}
int orc_dudt(orc_ctx * c) { return run_pass(c, PASS_DUDT); }
int orc_add_short_range_repulsion(orc_ctx * c) { return run_pass(c, PASS_REPULSION); }

/* add_drag_acceleration, add_drag_dedt, add_drag_dudt
 * (default_physics.h:571-594, 699-708) */
static int drag(orc_ctx * c, int which) {
  for(int64_t i = 0; i < c->n; ++i) {
    double vel[3] = {0.0, 0.0, 0.0}, acc[3];
    for(int d = 0; d < c->D; ++d)
      vel[d] = c->v[d][i];
    drag_acc(c, vel, acc);
    if(which == 0) {
      for(int d = 0; d < c->D; ++d)
        c->a[d][i] = c->a[d][i] + acc[d];
    }
    else {
      double v_dot_a = 0.0;
      for(int d = 0; d < c->D; ++d)
        v_dot_a += vel[d] * acc[d];
      double * f = which == 1 ? c->dedt : c->dudt;
      f[i] = f[i] + v_dot_a;
    }
  }
  return FSPH_OK;
}
int orc_add_drag_acceleration(orc_ctx * c) { return drag(c, 0); }
int orc_add_drag_dedt(orc_ctx * c) { return drag(c, 1); }
int orc_add_drag_dudt(orc_ctx * c) { return drag(c, 2); }
int orc_dedt(orc_ctx * c) { return run_pass(c, PASS_DEDT); }

/* ------------------------------------------------------- apply_all -- */
int orc_eos_init(orc_ctx * c) {
  /* eos_t<>::init (eos.h:67-92, 157-159, 240-243, 345-364) */
  const double g = c->p.poly_gamma, g2 = c->p.poly_gamma2;
  const double thr = c->p.ppt_density_thr;
  for(int64_t i = 0; i < c->n; ++i) {
    if(c->p.eos_type == FSPH_EOS_WD)
      c->u[i] = wd_internal_energy(c->rho[i], c->Ye[i]);
    else if(c->p.eos_type == FSPH_EOS_PPT) {
      if(c->rho[i] < thr)
        c->K[i] = c->P[i] / pow(c->rho[i], g);
      else {
        double K2 = c->P[i] / pow(c->rho[i], g2);
        c->K[i] = K2 * pow(thr, g2 - g);
      }
    }
    else if(c->p.eos_type != FSPH_EOS_NO_EOS)
      c->K[i] = c->P[i] / pow(c->rho[i], g);
  }
  return FSPH_OK;
}

int orc_set_total_energy(orc_ctx * c) {
  /* default_physics.h:327-335 */
  for(int64_t i = 0; i < c->n; ++i) {
    double vv = 0;
    for(int d = 0; d < c->D; ++d)
      vv += c->v[d][i] * c->v[d][i];
    double ekin = .5 * vv, pos[3];
    getx(c, i, pos);
    c->e[i] = ekin + c->u[i] + ext_potential(c, pos);
  }
  return FSPH_OK;
}

int orc_save_velocityhalf(orc_ctx * c) {
  /* integration.h:52-55 */
  for(int d = 0; d < c->D; ++d)
    memcpy(c->vh[d], c->v[d], 8 * c->n);
  return FSPH_OK;
}

int orc_leapfrog_kick_v(orc_ctx * c) {
  /* integration.h:65-70 */
  const double s = 0.5 * c->dt;
  for(int64_t i = 0; i < c->n; ++i)
    for(int d = 0; d < c->D; ++d)
      c->v[d][i] = c->v[d][i] + (c->a[d][i] + c->ga[d][i]) * s;
  return FSPH_OK;
}

int orc_leapfrog_kick_u(orc_ctx * c) {
  /* integration.h:80-84 */
  for(int64_t i = 0; i < c->n; ++i)
    c->u[i] = c->u[i] + 0.5 * c->dt * c->dudt[i];
  return FSPH_OK;
}

int orc_leapfrog_kick_e(orc_ctx * c) {
  /* integration.h:94-98 */
  for(int64_t i = 0; i < c->n; ++i)
    c->e[i] = c->e[i] + 0.5 * c->dt * c->dedt[i];
  return FSPH_OK;
}

int orc_leapfrog_drift(orc_ctx * c) {
  /* integration.h:106-110 */
  for(int64_t i = 0; i < c->n; ++i)
    for(int d = 0; d < c->D; ++d)
      c->x[d][i] = c->x[d][i] + c->v[d][i] * c->dt;
  return FSPH_OK;
}

int orc_recompute_pressure_soundspeed(orc_ctx * c) {
  /* default_physics.h:153-161 */
  for(int64_t i = 0; i < c->n; ++i) {
    double uint = c->u[i];
    double P, cs;
    eos_pressure(c, i, uint + 0.5 * c->dt * c->dudt[i], &P, &cs);
    c->P[i] = P;
    c->cs[i] = cs;
  }
  return FSPH_OK;
}

int orc_recompute_pressure_soundspeed_thermokinetic(orc_ctx * c) {
  /* default_physics.h:169-182 */
  for(int64_t i = 0; i < c->n; ++i) {
    double vv = 0;
    for(int d = 0; d < c->D; ++d)
      vv += c->v[d][i] * c->v[d][i];
    double ekin = .5 * vv;
    double pos[3];
    getx(c, i, pos);
    double eint = c->e[i] - ekin - ext_potential(c, pos);
    if(!(eint > 0))
      return FSPH_ERR_NEG_ENERGY;
    c->u[i] = eint;
    double vda = 0;
    for(int d = 0; d < c->D; ++d)
      vda += c->v[d][i] * c->a[d][i];
    double P, cs;
    eos_pressure(c, i, eint + 0.5 * c->dt * (c->dedt[i] - vda), &P, &cs);
    c->P[i] = P;
    c->cs[i] = cs;
  }
  return FSPH_OK;
}

int orc_compute_dt(orc_ctx * c) {
  /* default_physics.h:602-695 */
  const double tiny = 1e-24, mc = 0.6;
  const fsph_params * p = &c->p;
  for(int64_t i = 0; i < c->n; ++i) {
    const double dx = c->h[i] / (p->sph_eta * c->kernel_width);
    double vn = 0;
    for(int d = 0; d < c->D; ++d)
      vn += c->v[d][i] * c->v[d][i];
    vn = sqrt(vn);
    const double dt_v = dx / (vn + tiny);
    double acc = 0;
    for(int d = 0; d < c->D; ++d) {
      double ad = c->a[d][i] + c->ga[d][i];
      acc += ad * ad;
    }
    acc = sqrt(acc);
    const double dt_a = sqrt(dx / (acc + tiny));
    const double dt_c =
      dx / (tiny + c->vsig[i] * (1 + mc * p->sph_viscosity_alpha));
    double dtmin = p->timestep_cfl_factor * dmin_(dmin_(dt_v, dt_a), dt_c);
    if(p->evolve_internal_energy && p->thermokinetic_formulation) {
      const double eint = c->u[i];
      if(!(eint > 0))
        return FSPH_ERR_NEG_ENERGY;
      double pos[3];
      getx(c, i, pos);
      const double epot = ext_potential(c, pos);
      int it;
      for(it = 0; it < 20; ++it) {
        double gdv = 0;
        for(int d = 0; d < c->D; ++d)
          gdv += c->v[d][i] * c->ga[d][i];
        double p1[3] = {0.0, 0.0, 0.0};
        for(int d = 0; d < c->D; ++d)
          p1[d] = pos[d] + dtmin * c->v[d][i];
        double delta_epot = ext_potential(c, p1) - epot;
        double delta_egrv = -dtmin * gdv;
        if(delta_epot + delta_egrv < eint * 0.5)
          break;
        dtmin *= 0.25;
      }
      if(it >= 20)
        return FSPH_ERR_DT;
    }
    c->dtp[i] = dtmin;
  }
  return FSPH_OK;
}

int orc_set_adaptive_timestep(orc_ctx * c) {
  /* default_physics.h:761-823 */
  const fsph_params * p = &c->p;
  double dtmin = 1e24;
  for(int64_t i = 0; i < c->n; ++i)
    dtmin = dmin_(dtmin, c->dtp[i]);
  if(dtmin < c->dt)
    c->dt = dmin_(dtmin, c->dt / 2.0);
  if(dtmin > 2.0 * c->dt)
    c->dt = c->dt * 2.0;
  c->totaltime_next = c->totaltime + c->dt;
  if(p->out_screen_dt > 0) {
    if(c->totaltime == c->t_screen) {
      if(c->dt_saved > 0) c->dt = c->dt_saved;
      c->t_screen += p->out_screen_dt;
    }
    if(c->totaltime + c->dt > c->t_screen - 0.1 * p->out_screen_dt) {
      c->dt_saved = c->dt;
      c->totaltime_next = c->t_screen;
    }
  }
  if(p->out_scalar_dt > 0) {
    if(c->totaltime == c->t_scalar) {
      if(c->dt_saved > 0) c->dt = c->dt_saved;
      c->t_scalar += p->out_scalar_dt;
    }
    if(c->totaltime + c->dt > c->t_scalar - 0.1 * p->out_scalar_dt) {
      c->dt_saved = c->dt;
      c->totaltime_next = dmin_(c->totaltime_next, c->t_scalar);
    }
  }
  if(p->out_h5data_dt > 0) {
    if(c->totaltime == c->t_h5) {
      if(c->dt_saved > 0) c->dt = c->dt_saved;
      c->t_h5 += p->out_h5data_dt;
    }
    if(c->totaltime + c->dt > c->t_h5 - 0.1 * p->out_h5data_dt) {
      c->dt_saved = c->dt;
      c->totaltime_next = dmin_(c->totaltime_next, c->t_h5);
    }
  }
  c->dt = c->totaltime_next - c->totaltime;
  return FSPH_OK;
}

int orc_compute_smoothinglength(orc_ctx * c) {
  /* default_physics.h:825-848 */
  for(int64_t i = 0; i < c->n; ++i) {
    double q = c->m[i] / c->rho[i];
    double r = (c->D == 3) ? cbrt(q) : sqrt(q);
    c->h[i] = r * c->p.sph_eta * c->kernel_width;
  }
  return FSPH_OK;
}

int orc_compute_average_smoothinglength(orc_ctx * c) {
  /* default_physics.h:879-898 */
  orc_compute_smoothinglength(c);
  double total = 0.;
  for(int64_t i = 0; i < c->n; ++i)
    total += c->h[i];
  double new_h = 1. / (double)c->n * total;
  for(int64_t i = 0; i < c->n; ++i)
    c->h[i] = new_h;
  return FSPH_OK;
}

int orc_check_nans(orc_ctx * c) {
  /* default_physics.h:918-945 */
  for(int64_t i = 0; i < c->n; ++i) {
    for(int d = 0; d < c->D; ++d)
      if(c->x[d][i] != c->x[d][i] || c->v[d][i] != c->v[d][i] ||
         c->vh[d][i] != c->vh[d][i] || c->a[d][i] != c->a[d][i] ||
         c->ga[d][i] != c->ga[d][i])
        return FSPH_ERR_NAN;
    double f[] = {c->m[i], c->gpot[i], c->rho[i], c->P[i], c->e[i], c->dedt[i],
      c->dudt[i], c->K[i], c->vsig[i]};
    for(size_t k = 0; k < sizeof(f) / sizeof(f[0]); ++k)
      if(f[k] != f[k])
        return FSPH_ERR_NAN;
    if(c->p.evolve_internal_energy && c->u[i] != c->u[i])
      return FSPH_ERR_NAN;
  }
  return FSPH_OK;
}

int orc_check_negativity(orc_ctx * c) {
  /* default_physics.h:953-979 */
  for(int64_t i = 0; i < c->n; ++i)
    if(c->rho[i] < 0 || c->P[i] < 0 ||
       (c->p.evolve_internal_energy && c->u[i] < 0))
      return FSPH_ERR_NEGATIVITY;
  return FSPH_OK;
}

int orc_advance_time(orc_ctx * c) {
  /* default_physics.h:853-860 */
  c->iteration++;
  if(c->p.adaptive_timestep)
    c->totaltime = c->totaltime_next;
  else
    c->totaltime = c->totaltime + c->dt;
  return FSPH_OK;
}

int orc_gravity_direct(orc_ctx * c, int64_t s0, int64_t s1) {
  /* fmm::gravitation_p2p (fmm.h:37-46) summed over every source, skipping
   * the sink's own id (fmm.h:136-137). */
  const int D = c->D;
  const double G = c->p.gravitational_constant;
  if(s0 < 0 || s1 > c->n || s0 > s1)
    return FSPH_ERR_ARG;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(c->nthreads)
#endif
  for(int64_t i = s0; i < s1; ++i) {
    double pi[3], acc[3] = {0, 0, 0}, pot = 0;
    getx(c, i, pi);
    for(int64_t j = 0; j < c->n; ++j) {
      if(c->id[j] == c->id[i])
        continue;
      double pj[3];
      getx(c, j, pj);
      double dist = dist_pts(D, pi, pj);
      pot += -G * c->m[j] / dist;
      double f = -G * c->m[j] / (dist * dist * dist);
      for(int d = 0; d < D; ++d)
        acc[d] += f * (pi[d] - pj[d]);
    }
    for(int d = 0; d < D; ++d)
      c->ga[d][i] = acc[d];
    c->gpot[i] = pot;
  }
  return FSPH_OK;
}

#define TRY(x)                                                                 \
  do {                                                                         \
    int st_ = (x);                                                             \
    if(st_) return st_;                                                        \
  } while(0)

/* One iteration of mpi_init_task's loop (hydro/main_driver.cc:98-279;
 * newtonian/main_driver.cc:98-298 when enable_fmm, with direct-summation
 * gravity standing in for the FMM). */
int orc_step(orc_ctx * c) {
  const fsph_params * p = &c->p;
  if(p->sph_viscosity != FSPH_VISC_CONSTANT && p->sph_viscosity != FSPH_VISC_CULLEN)
    return FSPH_ERR_ARG;
  const int cullen = p->sph_viscosity == FSPH_VISC_CULLEN;
  /* relaxation terms: hydro driver only (hydro/main_driver.cc:129-134,
   * 150-165, 204-207, 219-234) */
  const int relax = !p->enable_fmm && c->iteration < p->relaxation_steps;
  if(c->iteration == p->initial_iteration) {
    TRY(orc_update_iteration(c));
    TRY(orc_eos_init(c));
    if(p->thermokinetic_formulation)
      TRY(orc_set_total_energy(c));
    if(cullen)
      TRY(orc_initialize_alpha(c));
    TRY(orc_density_pressure_soundspeed(c));
    TRY(orc_save_velocityhalf(c));
    if(cullen)
      TRY(orc_compute_alpha(c));
    TRY(orc_reset_ghosts(c));
    TRY(orc_acceleration(c));
    if(relax) {
      TRY(orc_add_drag_acceleration(c));
      TRY(orc_add_short_range_repulsion(c));
    }
    if(p->enable_fmm)
      TRY(orc_gravity_direct(c, 0, c->n));
    if(p->thermokinetic_formulation && p->enable_fmm)
      TRY(orc_set_total_energy(c));
    if(p->adaptive_timestep) {
      TRY(orc_compute_dt(c));
      TRY(orc_set_adaptive_timestep(c));
    }
    if(p->evolve_internal_energy) {
      for(int m = 1; m <= p->pressure_updates_number; ++m) {
        if(p->thermokinetic_formulation) {
          TRY(orc_dedt(c));
          if(relax)
            TRY(orc_add_drag_dedt(c));
          TRY(orc_recompute_pressure_soundspeed_thermokinetic(c));
        }
        else {
          TRY(orc_dudt(c));
          if(relax)
            TRY(orc_add_drag_dudt(c));
          TRY(orc_recompute_pressure_soundspeed(c));
        }
        if(m < p->pressure_updates_number)
          TRY(orc_reset_ghosts(c));
      }
    }
  }
  else {
    if(p->evolve_internal_energy) {
      if(p->thermokinetic_formulation)
        TRY(orc_leapfrog_kick_e(c));
      else
        TRY(orc_leapfrog_kick_u(c));
    }
    TRY(orc_leapfrog_kick_v(c));
    TRY(orc_save_velocityhalf(c));
    TRY(orc_leapfrog_drift(c));
    TRY(orc_update_iteration(c));
    TRY(orc_density_pressure_soundspeed(c));
    if(cullen)
      TRY(orc_compute_alpha(c));
    TRY(orc_reset_ghosts(c));
    TRY(orc_acceleration(c));
    if(relax) {
      TRY(orc_add_drag_acceleration(c));
      TRY(orc_add_short_range_repulsion(c));
    }
    if(p->enable_fmm)
      TRY(orc_gravity_direct(c, 0, c->n));
    TRY(orc_leapfrog_kick_v(c));
    TRY(orc_reset_ghosts(c));
    if(p->evolve_internal_energy) {
      for(int m = 1; m <= p->pressure_updates_number; ++m) {
        if(p->thermokinetic_formulation) {
          TRY(orc_dedt(c));
          if(relax)
            TRY(orc_add_drag_dedt(c));
          TRY(orc_recompute_pressure_soundspeed_thermokinetic(c));
        }
        else {
          TRY(orc_dudt(c));
          if(relax)
            TRY(orc_add_drag_dudt(c));
          TRY(orc_recompute_pressure_soundspeed(c));
        }
        if(m < p->pressure_updates_number)
          TRY(orc_reset_ghosts(c));
      }
      if(p->thermokinetic_formulation)
        TRY(orc_leapfrog_kick_e(c));
      else
        TRY(orc_leapfrog_kick_u(c));
    }
  }
  if(p->sph_variable_h)
    TRY(orc_compute_smoothinglength(c));
  else if(p->sph_update_uniform_h)
    TRY(orc_compute_average_smoothinglength(c));
  TRY(orc_check_nans(c));
  TRY(orc_check_negativity(c));
  if(p->adaptive_timestep) {
    TRY(orc_compute_dt(c));
    TRY(orc_set_adaptive_timestep(c));
  }
  return orc_advance_time(c);
}

int orc_get_neighbors(orc_ctx * c, int64_t * offsets, int64_t * indices,
  int64_t capacity) {
  if(!c->tree_ok)
    return FSPH_ERR_STATE;
  scratch s;
  scratch_init(&s);
  int64_t mem[GROUP_MAX];
  /* counts first */
  int64_t * cnt = (int64_t *)xalloc(sizeof(int64_t) * c->n);
  for(int64_t g = 0; g < c->ngroups; ++g) {
    int nm = walk_group(c, c->groups[g], &s, mem);
    for(int k = 0; k < nm; ++k)
      cnt[mem[k]] = s.nbn[k];
  }
  offsets[0] = 0;
  for(int64_t i = 0; i < c->n; ++i)
    offsets[i + 1] = offsets[i] + cnt[i];
  free(cnt);
  if(indices) {
    if(offsets[c->n] > capacity) {
      scratch_free(&s);
      return FSPH_ERR_ARG;
    }
    for(int64_t g = 0; g < c->ngroups; ++g) {
      int nm = walk_group(c, c->groups[g], &s, mem);
      for(int k = 0; k < nm; ++k)
        memcpy(indices + offsets[mem[k]], s.nb[k], 8 * s.nbn[k]);
    }
  }
  scratch_free(&s);
  return FSPH_OK;
}

int orc_get_order(orc_ctx * c, int64_t * order) {
  if(!c->tree_ok)
    return FSPH_ERR_STATE;
  int64_t k = 0;
  for(int64_t g = 0; g < c->ngroups; ++g) {
    int64_t gg = c->groups[g];
    if(gg < 0)
      order[k++] = ~gg;
    else
      for(int64_t i = c->nodes[gg].e - 1; i >= c->nodes[gg].s; --i)
        order[k++] = i;
  }
  return FSPH_OK;
}
