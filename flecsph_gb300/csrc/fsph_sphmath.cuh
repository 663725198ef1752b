// fsph_sphmath.cuh -- FP64 device restatement of the reference's SPH
// kernels, viscosity and EOS.  Every expression keeps the reference's
// operand order; the including translation units are compiled with
// -fmad=false, so each operation rounds exactly as the reference's does.
#pragma once

#include "fsph_internal.cuh"
#include "fsph_eforce.cuh"

namespace fsph {

// kernels::TINY (include/physics/kernels.h:64) and viscosity::TINY
// (include/physics/viscosity.h:36): 1e10 * DBL_MIN.
#define FSPH_TINY (1e10 * 2.2250738585072014e-308)
#define FSPH_PI 3.14159265358979323846

// Normalisations sigma[D-1] (kernels.h:40-46)
__device__ __forceinline__ double cubic_sigma(int D) {
  return D == 1 ? 4. / 3. : (D == 2 ? 40. / (7. * FSPH_PI) : 8. / FSPH_PI);
}
__device__ __forceinline__ double wc2_sigma(int D) {
  return D == 1 ? 1.25 : (D == 2 ? 7. / FSPH_PI : 21. / (2. * FSPH_PI));
}
__device__ __forceinline__ double wc4_sigma(int D) {
  return D == 1 ? 1.5 : (D == 2 ? 9. / FSPH_PI : 495. / (32. * FSPH_PI));
}
__device__ __forceinline__ double wc6_sigma(int D) {
  return D == 1 ? 55. / 32.
                : (D == 2 ? 78. / (7. * FSPH_PI) : 1365. / (64. * FSPH_PI));
}
__device__ __forceinline__ double quintic_sigma(int D) {
  return D == 1 ? 1. / 40.
                : (D == 2 ? 63. / (478. * FSPH_PI) : 81. / (359. * FSPH_PI));
}
// kernels.h:47-55 gives these as long-double literals; the doubles they
// round to, exactly
__device__ __forceinline__ double gaussian_sigma(int D) {
  return D == 1 ? 0x1.b14ea2d5440dap+0
                : (D == 2 ? 0x1.6ebcfdd1ce67cp+1 : 0x1.36768dfdddb6bp+2);
}
__device__ __forceinline__ double super_gaussian_sigma(int D) {
  return D == 1 ? 0x1.b13778577c0efp+0
                : (D == 2 ? 0x1.6e54d13f8aff2p+1 : 0x1.354cb7a91e8ccp+2);
}

// kernel<K,D>(r, h) -- kernels.h:106-121, 167-179, 217-235, 282-312,
// 375-410, 477-512, 581-590
template<int D, int K>
__device__ __forceinline__ double kfun(double r, double h, const PhysParams & pp) {
  if(K == FSPH_KERNEL_SINC) {  // kernels.h:633-661
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
      rh *= FSPH_PI;
      if(rh > eps_root4)
        sinc = sin(rh) / rh;
      else if(rh > eps) {
        rh2 = rh * rh;
        sinc += rh2 * (.05 * rh2 - 1.) / 6.;
      }
      result = pp.sinc_sigma[D - 1] / hd * pow(sinc, pp.sinc_index);
    }
    return result;
  }
  if(K == FSPH_KERNEL_QUINTIC_SPLINE) {
    double rh = 3. * r / h;
    double result = 0.;
    if(rh < 3.) {
      result = pow(3 - rh, 5);
      if(rh < 2.)
        result += -6 * pow(2 - rh, 5);
      if(rh < 1.)
        result += 15 * pow(1 - rh, 5);
      double sigma = quintic_sigma(D) / pow(h, (double)D);
      result *= sigma;
    }
    return result;
  }
  if(K == FSPH_KERNEL_GAUSSIAN) {
    double rh = 3. * r / h;
    double result = 0.;
    if(rh <= 3.) {
      double sigma = gaussian_sigma(D) / pow(h, (double)D);
      result = sigma * exp(-rh * rh);
    }
    return result;
  }
  if(K == FSPH_KERNEL_SUPER_GAUSSIAN) {
    double rh = 3. * r / h, rh2 = rh * rh;
    double sigma = super_gaussian_sigma(D) / pow(h, (double)D);
    double result = sigma * exp(-rh2) * (D / 2.0 + 1 - rh2);
    return result * (fabs(rh) < 3.);
  }
  if(K == FSPH_KERNEL_CUBIC_SPLINE) {
    double rh = 2. * r / h;
    double result = 0.;
    if(rh < 2.0) {
      if(rh < 1.0)
        result = 1.0 - 1.5 * rh * rh + .75 * rh * rh * rh;
      else
        result = 0.25 * (2 - rh) * (2 - rh) * (2 - rh);
      result *= cubic_sigma(D) / pow(h, (double)D);
    }
    return result;
  }
  else if(K == FSPH_KERNEL_WENDLAND_C2) {
    double rh = r / h;
    double hd = D == 3 ? h * h * h : h * h;
    double rh2 = (1 - rh) * (1 - rh);
    double sigma = wc2_sigma(D) / hd;
    double result = sigma * rh2 * rh2 * (4 * rh + 1);
    return result * (rh < 1.0);
  }
  else if(K == FSPH_KERNEL_WENDLAND_C4) {
    double rh = r / h;
    double hd = D == 3 ? h * h * h : h * h;
    double rh1 = 1 - rh;
    double rh2 = rh1 * rh1;
    double rh6 = rh2 * rh2 * rh2;
    double sigma = wc4_sigma(D) / hd;
    double result = sigma * rh6 * (1 + rh * (6 + rh * 35 / 3));
    return result * (rh < 1.0);
  }
  else {
    double rh = r / h;
    double hd = D == 3 ? h * h * h : h * h;
    double rh2 = (1 - rh) * (1 - rh);
    double rh4 = rh2 * rh2;
    double sigma = wc6_sigma(D) / hd;
    double result = sigma * rh4 * rh4 * (1 + rh * (8 + rh * (25 + rh * 32)));
    return result * (rh < 1.0);
  }
}

// kernel_gradient<K,D>(vecP, h) -- kernels.h:132-153, 189-205, 246-270,
// 322-361, 435-463, 536-566, 600-613
template<int D, int K>
__device__ __forceinline__ void kgrad(const double * p, double h, double * out,
  const PhysParams & pp) {
  double r = 0;
  for(int d = 0; d < D; ++d)
    r += p[d] * p[d];
  r = sqrt(r);
  if(K == FSPH_KERNEL_SINC) {  // kernels.h:671-698
    double rh = fabs(r / h), rh2;
    const double eps = 1e-24;
    const double eps_root = sqrt(eps);
    const double eps_root4 = sqrt(eps_root);
    const double n = pp.sinc_index;
    for(int d = 0; d < D; ++d)
      out[d] = 0.0;
    if(rh < 1.) {
      double hd = h * h;
      for(int i = 1; i < D; i++)
        hd *= h;
      double sigma = pp.sinc_sigma[D - 1] / hd;
      rh *= FSPH_PI;
      double dWdr = 0.0;
      if(rh > eps_root4) {
        double sinc = sin(rh) / rh, cosx = cos(rh) / rh;
        dWdr = -n * pow(sinc, n - 1) * FSPH_PI * (sinc / rh - cosx);
      }
      else if(rh > eps) {
        rh2 = rh * rh;
        dWdr = -n * rh / 3. * FSPH_PI * (1 - .5 * rh2 * (.2 - (n - 1) / 18));
      }
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * sigma * dWdr / (r + FSPH_TINY);
    }
    return;
  }
  if(K == FSPH_KERNEL_QUINTIC_SPLINE || K == FSPH_KERNEL_GAUSSIAN) {
    double rh = 3. * r / h;
    for(int d = 0; d < D; ++d)
      out[d] = 0.0;
    if(rh < 3.) {
      double sigma, dWdr;
      if(K == FSPH_KERNEL_QUINTIC_SPLINE) {
        sigma = 3. * quintic_sigma(D) / pow(h, (double)(D + 1));
        dWdr = -5. * pow(3 - rh, 4);
        if(rh < 2.)
          dWdr += 30. * pow(2 - rh, 4);
        if(rh < 1.)
          dWdr += -75. * pow(1 - rh, 4);
      }
      else {
        sigma = 3. * gaussian_sigma(D) / pow(h, (double)(D + 1));
        dWdr = -2. * rh * exp(-rh * rh);
      }
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * sigma * dWdr / (r + FSPH_TINY);
    }
    return;
  }
  if(K == FSPH_KERNEL_SUPER_GAUSSIAN) {
    double rh = 3. * r / h;
    double sigma = 3. * super_gaussian_sigma(D) / pow(h, (double)(D + 1));
    double dWdr = exp(-rh * rh) * (2. * pow(rh, 3.) - (D + 4.) * rh);
    double f = (rh < 3.0) * (sigma * dWdr / (r + FSPH_TINY));
    for(int d = 0; d < D; ++d)
      out[d] = p[d] * f;
    return;
  }
  if(K == FSPH_KERNEL_CUBIC_SPLINE) {
    double rh = 2. * r / h;
    for(int d = 0; d < D; ++d)
      out[d] = 0.0;
    if(rh < 2.0) {
      double dWdr;
      double sigma = 2. * cubic_sigma(D) / pow(h, (double)(D + 1));
      if(rh < 1.0)
        dWdr = -3.0 * rh + 9. / 4. * rh * rh;
      else
        dWdr = -.75 * (2 - rh) * (2 - rh);
      for(int d = 0; d < D; ++d)
        out[d] = p[d] * sigma * dWdr / (r + FSPH_TINY);
    }
    return;
  }
  double f;
  if(K == FSPH_KERNEL_WENDLAND_C2) {
    double rh = r / h;
    double hd1 = D == 3 ? h * h * h * h : h * h * h;
    double rh2 = (1 - rh) * (1 - rh);
    double sigma = 2. * wc2_sigma(D) / hd1;
    double dWdr = -10. * rh * rh2 * (1 - rh);
    f = (rh < 1.0) * (sigma * dWdr / (r + FSPH_TINY));
  }
  else if(K == FSPH_KERNEL_WENDLAND_C4) {
    double rh = r / h;
    double hd1 = D == 3 ? h * h * h * h : h * h * h;
    double rh2 = (1 - rh) * (1 - rh);
    double rh3 = rh2 * (1 - rh);
    double sigma = 14. * wc4_sigma(D) / hd1;
    double dWdr = -4. / 3. * rh * rh3 * rh2 * (1 + 5. * rh);
    f = (rh < 1.0) * (sigma * dWdr / (r + FSPH_TINY));
  }
  else {
    double rh = r / h;
    double hd1 = D == 3 ? h * h * h * h : h * h * h;
    double rh2 = (1 - rh) * (1 - rh);
    double rh3 = rh2 * (1 - rh);
    double rh4 = rh2 * rh2;
    double sigma = wc6_sigma(D) / hd1;
    double dWdr = -22. * rh * rh4 * rh3 * (1 + rh * (7 + rh * 16));
    f = (rh < 1.0) * (sigma * dWdr / (r + FSPH_TINY));
  }
  for(int d = 0; d < D; ++d)
    out[d] = p[d] * f;
}

// viscosity::mu (viscosity.h:81-93)
template<int D>
__device__ __forceinline__ double visc_mu(double eps, double h_ab,
  const double * vel_ab, const double * pos_ab) {
  double dotp = 0, dist2 = 0;
  for(int d = 0; d < D; ++d)
    dotp += vel_ab[d] * pos_ab[d];
  for(int d = 0; d < D; ++d)
    dist2 += pos_ab[d] * pos_ab[d];
  double result = h_ab * dotp / (dist2 + eps * h_ab * h_ab + FSPH_TINY);
  return result * (dotp < 0.0);
}

// viscosity_function<visc_constant> (viscosity.h:128-137)
__device__ __forceinline__ double visc_pi(double alpha, double beta,
  double rho_ab, double c_ab, double mu_ab) {
  return (-alpha * c_ab + beta * mu_ab) * mu_ab / rho_ab;
}

// sph_artificial_viscosity for the configured viscosity: visc_constant
// ignores alpha_ab (viscosity.h:128-137); visc_cullen is
// viscosity_function<visc_cullen> (viscosity.h:150-158) with
// alpha_ab = (alpha_a + alpha_b) / 2 (default_physics.h:388).
__device__ __forceinline__ double visc_pi_pp(const PhysParams & pp,
  const double * ALPHA, int a, int b, double rho_ab, double c_ab, double mu_ab) {
  if(pp.cullen) {
    const double alpha_ab = .5 * (ALPHA[a] + ALPHA[b]);
    return -alpha_ab * (c_ab - 2.0 * mu_ab) * mu_ab / rho_ab;
  }
  return visc_pi(pp.alpha, pp.beta, rho_ab, c_ab, mu_ab);
}

// eos_t<wd> (eos/eos.h:225-315): pressure function constants and the
// pressure, sound speed and internal energy of cold degenerate matter
#define FSPH_WD_A 6.00233181e22       // [dynes/cm^2]
#define FSPH_WD_B 9.73932099e5        // [moles/cm^3]
#define FSPH_C_LIGHT_CGS 2.99792458e10

__device__ __forceinline__ double wd_internal_energy(double rho, double Ye) {
  const double x = cbrt(rho * Ye / FSPH_WD_B), x2 = x * x, x3 = x * x * x;
  return FSPH_WD_A / rho * (8. * x3 * (sqrt(x2 + 1.) - 1.) -
                            (x * (2. * x2 - 3.) * sqrt(x2 + 1.) + 3. * asinh(x)));
}

// eos_t<>::compute_pressure + compute_soundspeed for every eos_type
// (eos/eos.h:102-119 polytropic, 166-183 ideal, 262-289 wd, 362-392 ppt,
// 425-431 no_eos).  P_old and cs_old are returned by eos_no_eos.
__device__ __forceinline__ void eos_p_cs(const PhysParams & pp, double rho,
  double u, double K, double Ye, double P_old, double cs_old, double & P,
  double & cs) {
  // The sound speed of a polytrope, sqrt(K gamma rho^(gamma - 1)), is taken
  // as sqrt(gamma P / rho): one FP64 pow per particle instead of two (pow
  // is long on this part's FP64 pipe), equal to rounding.
  const double g = pp.gamma;
  if(pp.eos == FSPH_EOS_POLYTROPIC) {
    P = K * pow(rho, g);
    cs = sqrt(g * P / rho);
  }
  else if(pp.eos == FSPH_EOS_WD) {
    // both from one x = (rho Ye / B)^(1/3)
    const double x = cbrt(rho * Ye / FSPH_WD_B), x2 = x * x;
    P = FSPH_WD_A * (x * (2. * x2 - 3.) * sqrt(x2 + 1.) + 3. * asinh(x));
    const double numer = (1. + x2) * (6. * x2 - 3.) + 3. + x2 * (2. * x2 - 3.);
    const double denom = (1. + x2) * (6. * x2 + 1.) - 1. + x2 * (2. * x2 + 1.);
    cs = sqrt(numer / (3. * denom)) * FSPH_C_LIGHT_CGS;
  }
  else if(pp.eos == FSPH_EOS_PPT) {
    // K2 = K1 rho_thr^(gamma - gamma2): the power is a constant of the run
    if(rho < pp.rho_thr) {
      P = K * pow(rho, g);
      cs = sqrt(g * P / rho);
    }
    else {
      P = K * pp.ppt_k2 * pow(rho, pp.gamma2);
      cs = sqrt(pp.gamma2 * P / rho);
    }
  }
  else if(pp.eos == FSPH_EOS_NO_EOS) {
    P = P_old;
    cs = cs_old;
  }
  else {
    P = (g - 1.) * rho * u;
    cs = sqrt(g * (g - 1.) * u);
  }
}

__device__ __forceinline__ void raise_status(DevStatus * st, int code,
  long long index) {
  if(atomicCAS(&st->code, 0, code) == 0)
    st->index = index;
}

}  // namespace fsph
