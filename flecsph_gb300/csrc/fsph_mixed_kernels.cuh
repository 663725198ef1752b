// fsph_mixed_kernels.cuh -- the mixed-precision neighbour-pair kernels
// (density, acceleration, du/dt, de/dt) as templates over the dimension,
// the smoothing kernel and the viscosity (Monaghan's constant alpha, or
// Cullen & Dehnen's per-particle alpha).  fsph_mixed.cu instantiates the
// constant-alpha kernels and fsph_mixed_cullen.cu the adaptive ones, so
// the two sets compile in parallel.
//
// Pair arithmetic runs in FP32 on packed per-particle records; the density,
// force and energy sums are Kahan-compensated; every per-particle quantity
// the integrator carries stays FP64 (EOS, kicks, stored fields).  Positions
// enter as 31-bit fixed point over the step's range, so the separation of a
// pair is an exact integer difference scaled once: ~1e-9 of the range
// instead of the 6e-8 an FP32 coordinate would give.
//
// Formulas are those of the reference (default_physics.h:193-566,
// kernels.h, viscosity.h:81-158); algebraic rewrites only (grad W / r
// folded into one factor, which stays finite at r = 0).  The self pair and
// coincident pairs contribute exactly zero to forces and energies (x_ab = 0
// and mu = 0), as the reference's m_b = 0 makes them (:378,456,534), and
// are masked out of the signal speed, where the reference drops a NaN
// (:254-262): FP32 has no equivalent of the reference's TINY guards.
#pragma once
#include <cuda_runtime.h>

#include "fsph_internal.cuh"
#include "fsph_sphmath.cuh"  // the FP64 EOS the density pass applies
#include "fsph_ff.cuh"

namespace fsph {

#define MIX_THREADS 256
#define FPI 3.14159265358979323846f

__device__ __forceinline__ void kahan(float & sum, float & comp, float term) {
  float y = term - comp;
  float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// ------------------------------------------------------- FP32 kernels --
__device__ __forceinline__ float sig_cubic(int D) {
  return D == 2 ? 40.f / (7.f * FPI) : 8.f / FPI;
}
__device__ __forceinline__ float sig_c2(int D) {
  return D == 2 ? 7.f / FPI : 21.f / (2.f * FPI);
}
__device__ __forceinline__ float sig_c4(int D) {
  return D == 2 ? 9.f / FPI : 495.f / (32.f * FPI);
}
__device__ __forceinline__ float sig_c6(int D) {
  return D == 2 ? 78.f / (7.f * FPI) : 1365.f / (64.f * FPI);
}
__device__ __forceinline__ float sig_quintic(int D) {
  return D == 2 ? 63.f / (478.f * FPI) : 81.f / (359.f * FPI);
}
__device__ __forceinline__ float sig_gauss(int D) {
  return D == 2 ? 2.86514256f : 4.85098600f;
}
__device__ __forceinline__ float sig_sgauss(int D) {
  return D == 2 ? 2.86196342f : 4.83280746f;
}

// W(r, h) for the kernel families of kernels.h (FP32).
template<int D, int K>
__device__ __forceinline__ float wfun(float r, float h, float inv_h,
  const PhysParams & pp) {
  const float ihD = D == 3 ? inv_h * inv_h * inv_h : inv_h * inv_h;
  if(K == FSPH_KERNEL_SINC) {
    const float q = r * inv_h;
    if(q >= 1.f)
      return 0.f;
    const float x = FPI * q;
    const float sinc = x > 1e-4f ? sinf(x) / x : 1.f - x * x * (1.f / 6.f);
    return (float)pp.sinc_sigma[D - 1] * ihD * powf(sinc, (float)pp.sinc_index);
  }
  if(K == FSPH_KERNEL_QUINTIC_SPLINE || K == FSPH_KERNEL_GAUSSIAN ||
     K == FSPH_KERNEL_SUPER_GAUSSIAN) {
    const float q = 3.f * r * inv_h;
    if(K == FSPH_KERNEL_GAUSSIAN)
      return q <= 3.f ? sig_gauss(D) * ihD * expf(-q * q) : 0.f;
    if(q >= 3.f)
      return 0.f;
    if(K == FSPH_KERNEL_SUPER_GAUSSIAN)
      return sig_sgauss(D) * ihD * expf(-q * q) * ((float)D * 0.5f + 1.f - q * q);
    const float t3 = 3.f - q, t3s = t3 * t3;
    float w = t3s * t3s * t3;
    if(q < 2.f) {
      const float t2 = 2.f - q, t2s = t2 * t2;
      w -= 6.f * t2s * t2s * t2;
    }
    if(q < 1.f) {
      const float t1 = 1.f - q, t1s = t1 * t1;
      w += 15.f * t1s * t1s * t1;
    }
    return w * sig_quintic(D) * ihD;
  }
  if(K == FSPH_KERNEL_CUBIC_SPLINE) {
    float q = 2.f * r * inv_h;
    if(q >= 2.f)
      return 0.f;
    float w = q < 1.f ? 1.f - 1.5f * q * q + 0.75f * q * q * q
                      : 0.25f * (2.f - q) * (2.f - q) * (2.f - q);
    return w * sig_cubic(D) * ihD;
  }
  const float q = r * inv_h;
  if(q >= 1.f)
    return 0.f;
  const float t = 1.f - q;
  const float t2 = t * t;
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return sig_c2(D) * ihD * t2 * t2 * (4.f * q + 1.f);
  if(K == FSPH_KERNEL_WENDLAND_C4)
    return sig_c4(D) * ihD * t2 * t2 * t2 * (1.f + q * (6.f + q * (35.f / 3.f)));
  const float t4 = t2 * t2;
  return sig_c6(D) * ihD * t4 * t4 * (1.f + q * (8.f + q * (25.f + q * 32.f)));
}

// grad_a W = x_ab * F(r, h); returns F = (dW/dr) / r.
template<int D, int K>
__device__ __forceinline__ float gfac(float r, float h, float inv_h,
  const PhysParams & pp) {
  const float ihD1 = D == 3 ? inv_h * inv_h * inv_h * inv_h : inv_h * inv_h * inv_h;
  if(K == FSPH_KERNEL_SINC) {
    // (dW/dr) / r = sigma / h^(D+2) (-n pi^2 sinc^(n-1)) (sin x - x cos x) / x^3
    const float q = r * inv_h;
    if(q >= 1.f)
      return 0.f;
    const float x = FPI * q, x2 = x * x;
    const float n = (float)pp.sinc_index;
    float sinc, g3;
    if(x > 0.05f) {
      float sx, cx;
      sincosf(x, &sx, &cx);
      sinc = sx / x;
      g3 = (sx - x * cx) / (x2 * x);
    }
    else {
      sinc = 1.f - x2 * (1.f / 6.f);
      g3 = 1.f / 3.f - x2 * (1.f / 30.f - x2 * (1.f / 840.f));
    }
    return (float)pp.sinc_sigma[D - 1] * ihD1 * inv_h * (-n * FPI * FPI) *
           powf(sinc, n - 1.f) * g3;
  }
  if(K == FSPH_KERNEL_QUINTIC_SPLINE || K == FSPH_KERNEL_GAUSSIAN ||
     K == FSPH_KERNEL_SUPER_GAUSSIAN) {
    // q = 3 r / h: (dW/dr) / r = 3 sigma / h^(D+1) * g(q) * (3 / h) / q,
    // with g(q) / q written out so that r = 0 gives a finite factor
    const float q = 3.f * r * inv_h;
    if(q >= 3.f)
      return 0.f;
    const float e = (K == FSPH_KERNEL_QUINTIC_SPLINE) ? 0.f : expf(-q * q);
    float gq;
    if(K == FSPH_KERNEL_GAUSSIAN)
      gq = -2.f * e * sig_gauss(D);
    else if(K == FSPH_KERNEL_SUPER_GAUSSIAN)
      gq = e * (2.f * q * q - ((float)D + 4.f)) * sig_sgauss(D);
    else {
      if(q < 1.f)  // -5(3-q)^4 + 30(2-q)^4 - 75(1-q)^4 = q (-120 + 120 q^2 - 50 q^3)
        gq = -120.f + q * q * (120.f - 50.f * q);
      else {
        const float t3 = 3.f - q, t3s = t3 * t3;
        float g = -5.f * t3s * t3s;
        if(q < 2.f) {
          const float t2 = 2.f - q, t2s = t2 * t2;
          g += 30.f * t2s * t2s;
        }
        gq = g / q;
      }
      gq *= sig_quintic(D);
    }
    return 9.f * ihD1 * inv_h * gq;
  }
  if(K == FSPH_KERNEL_CUBIC_SPLINE) {
    float q = 2.f * r * inv_h;
    if(q >= 2.f)
      return 0.f;
    // sigma' = 2 sigma / h^(D+1); dW/dr = sigma' * g(q); g / r
    float s = 2.f * sig_cubic(D) * ihD1;
    if(q < 1.f)
      return s * (-3.f + 2.25f * q) * 2.f * inv_h;
    float g = -0.75f * (2.f - q) * (2.f - q);
    return s * g / r;
  }
  const float q = r * inv_h;
  if(q >= 1.f)
    return 0.f;
  const float t = 1.f - q;
  const float t2 = t * t;
  // dW/dr / r with rh / r = 1 / h folded in
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return -20.f * sig_c2(D) * ihD1 * inv_h * t2 * t;
  if(K == FSPH_KERNEL_WENDLAND_C4)
    return 14.f * sig_c4(D) * ihD1 * inv_h * (-4.f / 3.f) * t2 * t2 * t * (1.f + 5.f * q);
  const float t4 = t2 * t2;
  return -22.f * sig_c6(D) * ihD1 * inv_h * t4 * t2 * t * (1.f + q * (7.f + q * 16.f));
}

// viscosity_function (viscosity.h:128-158): Monaghan's constant alpha and
// beta, or Cullen & Dehnen's Pi with alpha_ab = (alpha_a + alpha_b) / 2
// (default_physics.h:388).  The FP32 pair terms divide with __fdividef
// (two ulps, no special-case path): they carry FP32 rounding in any case.
template<bool CULL>
__device__ __forceinline__ float visc_pi_f(float alpha, float beta, float alpha_a,
  const Packed & Kp, int b, float rho_ab, float c_ab, float mu) {
  if(CULL) {
    const float al = 0.5f * (alpha_a + Kp.visc[b].x);
    return __fdividef(-al * (c_ab - 2.f * mu) * mu, rho_ab);
  }
  return __fdividef((-alpha * c_ab + beta * mu) * mu, rho_ab);
}

struct PairGeom {
  float dx, dy, dz, r2;
};

// (vh_a - vh_b) . d from the high words (fv1) and low words (fv2) of
// v_half: the high-word and low-word differences are one rounding each, so
// the difference keeps ~2^-24 of itself
__device__ __forceinline__ float vdiff_dot(const float4 & ah, const float4 & al,
  const float4 & bh, const float4 & bl, float dx, float dy, float dz) {
  return ((ah.x - bh.x) + (al.x - bl.x)) * dx + ((ah.y - bh.y) + (al.y - bl.y)) * dy +
         ((ah.z - bh.z) + (al.z - bl.z)) * dz;
}

// (v_a - v_b) . d with v = v_half + (v - v_half) (fv1, fv2, fdv)
__device__ __forceinline__ float vel_diff_dot(const float4 & h1a, const float4 & h2a,
  const float4 & dva, const float4 & h1b, const float4 & h2b, const float4 & dvb,
  float dx, float dy, float dz) {
  return vdiff_dot(h1a, h2a, h1b, h2b, dx, dy, dz) +
         ((dva.x - dvb.x) * dx + (dva.y - dvb.y) * dy + (dva.z - dvb.z) * dz);
}

template<int D>
__device__ __forceinline__ PairGeom geom(const int4 & qa, const int4 & qb,
  float s0, float s1, float s2) {
  PairGeom g;
  g.dx = (float)(qa.x - qb.x) * s0;
  g.dy = (float)(qa.y - qb.y) * s1;
  g.dz = D == 3 ? (float)(qa.z - qb.z) * s2 : 0.f;
  g.r2 = g.dx * g.dx + g.dy * g.dy + g.dz * g.dz;
  return g;
}

// ------------------------------------------------------------- density --
// With CULL the same loop also sums m_b grad_a W_ab for compute_divv
// (default_physics.h:273-299), whose divergence is v_a . that sum / rho_a.
// That sum runs in FP64 from the FP64 positions: on a symmetric
// neighbourhood it cancels to FP64 rounding, and Cullen & Dehnen's limiter
// compares (2 (1 - R)^4 div v)^2 against an absolute 1e-16
// (viscosity.h:265-266), so FP32 rounding noise in a uniform flow would
// switch the viscosity on where the reference keeps it off.
template<int D, int K, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS) k_density_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, double * cs_new, DevStatus * st,
  const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const int cnt = Ls.cnt[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  float sum = 0.f, comp = 0.f;
  double gsum[3] = {0.0, 0.0, 0.0};
  double pa[3] = {0.0, 0.0, 0.0}, h_a = 0.0;
  if(CULL) {
    for(int d = 0; d < D; ++d)
      pa[d] = P.f[F_X + d][a];
    h_a = P.f[F_H][a];
  }
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const float mb = Kp.mass[b];
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = __fdividef(1.f, hab);
      const float r = sqrtf(g.r2);
      const float w = mb * wfun<D, K>(r, hab, ih, pp);
      kahan(sum, comp, j0 + u < cnt ? w : 0.f);
      if(CULL) {
        // padding slots and the self pair have x_ab = 0 and add nothing
        double pos_ab[3] = {0.0, 0.0, 0.0}, DiW[3];
        for(int d = 0; d < D; ++d)
          pos_ab[d] = pa[d] - P.f[F_X + d][b];
        kgrad<D, K>(pos_ab, .5 * (h_a + P.f[F_H][b]), DiW, pp);
        const double mbd = P.f[F_M][b];
        for(int d = 0; d < D; ++d)
          gsum[d] += mbd * DiW[d];
      }
    }
  }
  const double rho = (double)sum - (double)comp;
  if(!(rho > 0)) {
    if(atomicCAS(&st->code, 0, (int)FSPH_ERR_NEG_DENSITY) == 0)
      st->index = a;
  }
  P.f[F_RHO][a] = rho;
  double u = P.f[F_U][a];
  if(pp.evolve_u && pp.thermokinetic) {
    double vv = 0;
    for(int d = 0; d < D; ++d)
      vv += P.f[F_VX + d][a] * P.f[F_VX + d][a];
    double eint = P.f[F_E][a] - .5 * vv - ext_potential_of<D>(pp, P.f, a);
    if(!(eint > 0)) {
      if(atomicCAS(&st->code, 0, (int)FSPH_ERR_NEG_ENERGY) == 0)
        st->index = a;
    }
    u = eint;
    P.f[F_U][a] = u;
  }
  double Pa, cs;
  eos_p_cs(pp, rho, u, P.f[F_K][a], P.f[F_YE][a], P.f[F_P][a], P.f[F_CS][a], Pa, cs);
  P.f[F_P][a] = Pa;
  cs_new[a] = cs;
  Kp.thermo[a] = make_float4((float)rho, (float)(Pa / (rho * rho)), (float)cs,
    (float)P.f[F_CS][a]);
  if(CULL) {
    double div_v = 0.0;
    for(int d = 0; d < D; ++d)
      div_v += P.f[F_VX + d][a] * gsum[d];
    div_v /= rho;
    P.f[F_DDIVVDT][a] = (div_v - P.f[F_DIVV][a]) / tm->dt;
    P.f[F_DIVV][a] = div_v;
  }
}

// -------------------------------------------------------- acceleration --
// With VSIG the signal speed of the density pass (same neighbours, same
// rule as k_vsig_mixed) is evaluated in this loop instead of a pass of its
// own; it reads the pre-kick velocities packed for the density pass, so the
// kick below cannot race with it.
// Three blocks of 256 per SM (<= 85 registers): the pass waits on neighbour
// gathers, and 24 warps hide more of them than 16.
template<int D, int K, bool VSIG, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS, 3) k_accel_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, int kick, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const float alpha_a = CULL ? Kp.visc[a].x : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 vha = Kp.vhm[a];
  const float4 ta = Kp.thermo[a];
  const int cnt = Ls.cnt[a];
  float ax = 0.f, ay = 0.f, az = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float4 va = make_float4(0.f, 0.f, 0.f, 0.f);
  if(VSIG)
    va = Kp.vel[a];
  float vsig = 0.f;
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  // The self pair and coincident pairs add exactly zero (x_ab = 0, mu = 0),
  // as the reference's m_b = 0 makes them; the loop needs no branch.
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = __fdividef(1.f, hab);
      const float r = sqrtf(g.r2);
      const float f = gfac<D, K>(r, hab, ih, pp);
      const float4 vhb = Kp.vhm[b];
      const float4 tb = Kp.thermo[b];
      const float dotp = (vha.x - vhb.x) * g.dx + (vha.y - vhb.y) * g.dy +
                         (vha.z - vhb.z) * g.dz;
      const float mu = dotp < 0.f ? __fdividef(hab * dotp, g.r2 + eps * hab * hab) : 0.f;
      const float rho_ab = 0.5f * (ta.x + tb.x);
      const float c_ab = 0.5f * (ta.z + tb.z);
      const float Pi = visc_pi_f<CULL>(alpha, beta, alpha_a, Kp, b, rho_ab, c_ab, mu);
      const float sc = -vhb.w * (ta.y + tb.y + Pi) * f;
      if(VSIG) {
        const float4 vb = Kp.vel[b];
        const float dotv = ((va.x - vb.x) * g.dx + (va.y - vb.y) * g.dy +
                             (va.z - vb.z) * g.dz) * rsqrtf(g.r2);
        const float cb = b > a ? tb.z : tb.w;
        const float cand = fmaxf(ta.z, cb) - fminf(dotv, 0.f);
        vsig = fmaxf(vsig, (b != a && g.r2 > 0.f) ? cand : 0.f);
      }
      kahan(ax, cx, g.dx * sc);
      kahan(ay, cy, g.dy * sc);
      if(D == 3)
        kahan(az, cz, g.dz * sc);
    }
  }
  double acc[3] = {(double)ax - (double)cx, (double)ay - (double)cy,
    D == 3 ? (double)az - (double)cz : 0.0};
  if(pp.has_eacc) {  // acc_a += external_force::acceleration (:404)
    const double pos[3] = {P.f[F_X][a], P.f[F_Y][a], D == 3 ? P.f[F_Z][a] : 0.0};
    double ext[3];
    ext_acceleration<D>(pp, pos, ext);
    for(int d = 0; d < D; ++d)
      acc[d] += ext[d];
  }
  const double half_dt = kick ? 0.5 * tm->dt : 0.0;
  double v[3] = {0, 0, 0};
  for(int d = 0; d < D; ++d) {
    P.f[F_AX + d][a] = acc[d];
    P.f[F_GAX + d][a] = 0.0;
    v[d] = P.f[F_VX + d][a];
    if(kick) {
      v[d] = v[d] + acc[d] * half_dt;
      P.f[F_VX + d][a] = v[d];
    }
  }
  P.f[F_GPOT][a] = 0.0;
  if(VSIG)
    P.f[F_VSIG][a] = (double)vsig;
}

// --------------------------------------------------------------- du/dt --
// The same records as the de/dt pass ({v, .} and {rho, c_s}: 56 B per pair);
// then_op (OP_RECOMPUTE or OP_RECOMPUTE_KICK_U, else 0) applies the
// element-wise update that follows du/dt in the driver to the particle.
// Resident blocks of 256 per SM of the du/dt and de/dt (through a^P)
// passes: 3 gives them 80 registers, enough for four pairs' records in
// flight with the velocities' low words and no spills.
#ifndef FSPH_ENERGY_BLOCKS
#define FSPH_ENERGY_BLOCKS 3
#endif

template<int D, int K, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS, FSPH_ENERGY_BLOCKS) k_dudt_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, const DevTime * tm, int then_op) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  // no internal energy change while relaxing (default_physics.h:423-427)
  if(tm->iteration < pp.relax_steps) {
    P.f[F_DUDT][a] = 0.0;
    return;
  }
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const float alpha_a = CULL ? Kp.visc[a].x : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 h1a = Kp.fv1[a], h2a = Kp.fv2[a], dva = Kp.fdv[a];
  const int cnt = Ls.cnt[a];
  float dp = 0.f, cp = 0.f, dv = 0.f, cv = 0.f;
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = __fdividef(1.f, hab);
      const float f = gfac<D, K>(sqrtf(g.r2), hab, ih, pp);
      const float4 h1b = Kp.fv1[b], h2b = Kp.fv2[b], dvb = Kp.fdv[b];
      const float dotp = vdiff_dot(h1a, h2a, h1b, h2b, g.dx, g.dy, g.dz);
      const float mu = dotp < 0.f ? __fdividef(hab * dotp, g.r2 + eps * hab * hab) : 0.f;
      const float Pi = visc_pi_f<CULL>(alpha, beta, alpha_a, Kp, b, 0.5f * (h1a.w + h1b.w),
        0.5f * (h2a.w + h2b.w), mu);
      const float vdw = f * vel_diff_dot(h1a, h2a, dva, h1b, h2b, dvb, g.dx, g.dy, g.dz);
      kahan(dp, cp, dvb.w * vdw);
      kahan(dv, cv, dvb.w * vdw * Pi);
    }
  }
  const double sp = (double)dp - (double)cp, sv = (double)dv - (double)cv;
  const double rho_a = P.f[F_RHO][a];
  const double dudt = P.f[F_P][a] / (rho_a * rho_a) * sp + .5 * sv;
  P.f[F_DUDT][a] = dudt;
  if(then_op) {
    // recompute_pressure_soundspeed (default_physics.h:153-161) and, with
    // the kick, leapfrog_kick_u (integration.h:80-84)
    const double dt = tm->dt, uint = P.f[F_U][a];
    double Pn, cs;
    eos_p_cs(pp, rho_a, uint + 0.5 * dt * dudt, P.f[F_K][a], P.f[F_YE][a],
      P.f[F_P][a], P.f[F_CS][a], Pn, cs);
    P.f[F_P][a] = Pn;
    P.f[F_CS][a] = cs;
    if(then_op == OP_RECOMPUTE_KICK_U)
      P.f[F_U][a] = uint + 0.5 * dt * dudt;
  }
}

// --------------------------------------------------------------- de/dt --
// then_op (OP_RECOMPUTE_THERMO or OP_RECOMPUTE_KICK_E, else 0) applies the
// element-wise update that follows de/dt in the driver to the particle
// right away: it reads only the particle's own fields, and the pass reads
// the neighbours' P and c_s from the packed records, not the fields.
template<int D, int K, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS, 4) k_dedt_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, int then_op, const DevTime * tm,
  DevStatus * st) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const float alpha_a = CULL ? Kp.visc[a].x : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 vha = Kp.vhm[a];
  const float4 va = Kp.velp[a];  // .w = P_a / rho_a^2
  const float2 ra = Kp.rc[a];
  const int cnt = Ls.cnt[a];
  float sum = 0.f, comp = 0.f;
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = __fdividef(1.f, hab);
      const float f = gfac<D, K>(sqrtf(g.r2), hab, ih, pp);
      const float4 vhb = Kp.vhm[b];
      const float4 vb = Kp.velp[b];
      const float2 rb = Kp.rc[b];
      const float dotp = (vha.x - vhb.x) * g.dx + (vha.y - vhb.y) * g.dy +
                         (vha.z - vhb.z) * g.dz;
      const float mu = dotp < 0.f ? __fdividef(hab * dotp, g.r2 + eps * hab * hab) : 0.f;
      const float Pi = visc_pi_f<CULL>(alpha, beta, alpha_a, Kp, b, 0.5f * (ra.x + rb.x),
        0.5f * (ra.y + rb.y), mu);
      const float vad = f * (va.x * g.dx + va.y * g.dy + va.z * g.dz);
      const float vbd = f * (vb.x * g.dx + vb.y * g.dy + vb.z * g.dz);
      kahan(sum, comp, vhb.w * (va.w * vbd + vad * vb.w + 0.5f * Pi * (vbd + vad)));
    }
  }
  double gv = 0;
  for(int d = 0; d < D; ++d)
    gv += P.f[F_GAX + d][a] * P.f[F_VX + d][a];
  const double dedt = -((double)sum - (double)comp) + gv;
  P.f[F_DEDT][a] = dedt;
  if(then_op) {
    // recompute_pressure_soundspeed_thermokinetic (default_physics.h:169-182)
    // and, with the kick, leapfrog_kick_e (integration.h:94-98)
    const double dt = tm->dt;
    double vv = 0, vda = 0;
    for(int d = 0; d < D; ++d) {
      const double v = P.f[F_VX + d][a];
      vv += v * v;
      vda += v * P.f[F_AX + d][a];
    }
    const double e = P.f[F_E][a];
    const double eint = e - .5 * vv - ext_potential_of<D>(pp, P.f, a);
    if(!(eint > 0))
      raise_status(st, FSPH_ERR_NEG_ENERGY, a);
    P.f[F_U][a] = eint;
    double Pn, cs;
    eos_p_cs(pp, P.f[F_RHO][a], eint + 0.5 * dt * (dedt - vda), P.f[F_K][a],
      P.f[F_YE][a], P.f[F_P][a], P.f[F_CS][a], Pn, cs);
    P.f[F_P][a] = Pn;
    P.f[F_CS][a] = cs;
    if(then_op == OP_RECOMPUTE_KICK_E)
      P.f[F_E][a] = e + 0.5 * dt * dedt;
  }
}

// ------------------------------------------- float-float Wendland passes --
// The density sum and the acceleration's pressure-gradient sum for the
// Wendland kernels, in float-float arithmetic (fsph_ff.cuh): pair geometry
// from the float-float positions, the kernel polynomial, m_b and
// P/rho^2 + Pi, and the running sums.  Viscosity (mu, Pi) and the signal
// speed stay FP32: they are small beside the pressure terms or enter
// through a maximum.  In t = 1 - q the Wendland polynomials are
//   W h^D / sigma:             C2 t^4 (5 - 4t)
//                              C4 t^6 (56 - 88t + 35t^2) / 3
//                              C6 t^8 (66 - 154t + 121t^2 - 32t^3)
//   (dW/dr)/r h^(D+2) / sigma: C2 -20 t^3
//                              C4 -56/3 t^5 (6 - 5t)
//                              C6 -22 t^7 (24 - 39t + 16t^2)
// (kernels.h's q-forms expanded about q = 1).  Each Horner step adds a
// constant larger in magnitude than the running value for t in [0, 1], so
// the fast two-sum applies.  The constant factors and the unit scale E of
// the positions multiply the finished sums once, in FP64.
template<int K>
__host__ __device__ constexpr bool ff_kernel() {
  return K == FSPH_KERNEL_WENDLAND_C2 || K == FSPH_KERNEL_WENDLAND_C4 ||
         K == FSPH_KERNEL_WENDLAND_C6;
}

template<int K>
__device__ __forceinline__ ffloat ff_wpoly(ffloat t) {
  const ffloat t2 = ff_sqr(t);
  const ffloat t4 = ff_sqr(t2);
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return ff_mul(t4, ff_cadd(5.f, ff_scale2(t, -4.f)));
  if(K == FSPH_KERNEL_WENDLAND_C4) {
    const ffloat p = ff_cadd(56.f, ff_mul(ff_cadd(-88.f, ff_mul_f(t, 35.f)), t));
    return ff_mul(ff_mul(t4, t2), p);
  }
  const ffloat a1 = ff_cadd(121.f, ff_scale2(t, -32.f));
  const ffloat a2 = ff_cadd(-154.f, ff_mul(a1, t));
  const ffloat p = ff_cadd(66.f, ff_mul(a2, t));
  return ff_mul(ff_sqr(t4), p);
}

// ff_wpoly on two values at once (packed FP32x2)
template<int K>
__device__ __forceinline__ ffloat2 ff2_wpoly(ffloat2 t) {
  const ffloat2 t2 = ff2_sqr(t);
  const ffloat2 t4 = ff2_sqr(t2);
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return ff2_mul(t4, ff2_cadd(5.f, ff2_scale2(t, -4.f)));
  if(K == FSPH_KERNEL_WENDLAND_C4) {
    const ffloat2 c35 = ff2_make(f2s(35.f), f2s(0.f));
    const ffloat2 p = ff2_cadd(56.f, ff2_mul(ff2_cadd(-88.f, ff2_mul(t, c35)), t));
    return ff2_mul(ff2_mul(t4, t2), p);
  }
  const ffloat2 a1 = ff2_cadd(121.f, ff2_scale2(t, -32.f));
  const ffloat2 a2 = ff2_cadd(-154.f, ff2_mul(a1, t));
  const ffloat2 p = ff2_cadd(66.f, ff2_mul(a2, t));
  return ff2_mul(ff2_sqr(t4), p);
}

template<int K>
__device__ __forceinline__ ffloat ff_gpoly(ffloat t) {
  const ffloat t2 = ff_sqr(t);
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return ff_mul(t2, t);
  const ffloat t4 = ff_sqr(t2);
  if(K == FSPH_KERNEL_WENDLAND_C4)
    return ff_mul(ff_mul(t4, t), ff_cadd(6.f, ff_mul_f(t, -5.f)));
  const ffloat b1 = ff_cadd(-39.f, ff_scale2(t, 16.f));
  const ffloat p = ff_cadd(24.f, ff_mul(b1, t));
  return ff_mul(ff_mul(ff_mul(t4, t2), t), p);
}


// W = wconst / h^D * wpoly(t);  (dW/dr)/r = gconst / h^(D+2) * gpoly(t)
template<int D, int K>
__device__ __forceinline__ double ff_wconst() {
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return wc2_sigma(D);
  if(K == FSPH_KERNEL_WENDLAND_C4)
    return wc4_sigma(D) / 3.;
  return wc6_sigma(D);
}
template<int D, int K>
__device__ __forceinline__ double ff_gconst() {
  if(K == FSPH_KERNEL_WENDLAND_C2)
    return -20. * wc2_sigma(D);
  if(K == FSPH_KERNEL_WENDLAND_C4)
    return -56. / 3. * wc4_sigma(D);
  return -22. * wc6_sigma(D);
}

// Pair geometry from the float-float positions: the separation (high words
// exact, low words the difference of the residuals, so not normalised), its
// FP32 rounding for the viscosity and signal speed, r^2 and r.
template<int D>
struct FFGeom {
  ffloat dx[3];
  float dxr[3];
  float r2f;
  ffloat r;
};

template<int D>
__device__ __forceinline__ FFGeom<D> ff_geom(const float4 & pa, const float4 & la,
  const float4 & pb, const float4 & lb) {
  FFGeom<D> g;
  g.dx[0] = ff_make(__fsub_rn(pa.x, pb.x), __fsub_rn(la.x, lb.x));
  g.dx[1] = ff_make(__fsub_rn(pa.y, pb.y), __fsub_rn(la.y, lb.y));
  g.dx[2] = D == 3 ? ff_make(__fsub_rn(pa.z, pb.z), __fsub_rn(la.z, lb.z))
                   : ff_make(0.f, 0.f);
  ffloat r2 = ff_add(ff_sqr_wide(g.dx[0]), ff_sqr_wide(g.dx[1]));
  if(D == 3)
    r2 = ff_add(r2, ff_sqr_wide(g.dx[2]));
  r2 = ff_norm(r2);
  g.r2f = r2.h;
  for(int d = 0; d < 3; ++d)
    g.dxr[d] = __fadd_rn(g.dx[d].h, g.dx[d].l);
  g.r = ff_sqrt(r2);
  return g;
}

// 1/h_ab and 1/h_ab^P for P = D or D + 2: the particle's own values when the
// neighbour's h is the same (every pair of a uniform-h run), else from
// h_a + h_b.
template<int P>
__device__ __forceinline__ ffloat ff_ipow(ffloat ih) {
  const ffloat i2 = ff_sqr(ih);
  if(P == 2)
    return i2;
  if(P == 3)
    return ff_mul(i2, ih);
  const ffloat i4 = ff_sqr(i2);
  if(P == 4)
    return i4;
  return ff_mul(i4, ih);  // P == 5
}

// The density sum of one particle: sum_b m_b wpoly(t_ab) / h_ab^D, or, with
// UNI (every h equal), sum_b m_b wpoly(t_ab), the particle's 1/h^D applied
// once afterwards.
template<int D, int K, bool UNI>
__device__ __forceinline__ ffloat density_ff_sum(const Packed & Kp, const int * lp,
  int cnt, const float4 & pa, const float4 & la, const ffloat & iha,
  const ffloat & ihDa) {
  ffloat sum = ff_make(0.f, 0.f);
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const float4 pb = Kp.fph[b], lb = Kp.fpl[b];
      const float2 mb = ((const float2 *)Kp.fmA)[2 * b];
      const FFGeom<D> g = ff_geom<D>(pa, la, pb, lb);
      ffloat ih = iha, ihD = ihDa;
      if(!UNI && (pb.w != pa.w || lb.w != la.w)) {
        ih = ff_rcp_scaled(ff_add(ff_make(pa.w, la.w), ff_make(pb.w, lb.w)), 2.f);
        ihD = ff_ipow<D>(ih);
      }
      const ffloat q = ff_mul(g.r, ih);
      const ffloat t = ff_cadd(1.f, ff_make(-q.h, -q.l));
      ffloat w = ff_mul(ff_wpoly<K>(t), ff_make(mb.x, mb.y));
      if(!UNI)
        w = ff_mul(w, ihD);
      if(!(q.h < 1.f) || j0 + u >= cnt)
        w = ff_make(0.f, 0.f);
      ff_acc(sum, w);
    }
  }
  if(UNI)
    sum = ff_mul(sum, ihDa);
  return sum;
}

// 1: the density pass takes two neighbours per step in packed FP32x2
#ifndef FSPH_DENSITY_PAIRED
#define FSPH_DENSITY_PAIRED 1
#endif

// density_ff_sum with two neighbours per step in packed FP32x2 (the list's
// four-slot chunks hold two pairs of neighbours).  The two lanes keep their
// own running sums, added at the end.
template<int D, int K, bool UNI>
__device__ __forceinline__ ffloat density_ff_sum2(const Packed & Kp, const int * lp,
  int cnt, const float4 & pa, const float4 & la, const ffloat & iha,
  const ffloat & ihDa) {
  ffloat2 sum = ff2_make(f2s(0.f), f2s(0.f));
  const ffloat2 ih1 = ff2_bcast(iha);
  const float2 xa = f2s(pa.x), ya = f2s(pa.y), za = f2s(pa.z);
  const float2 xal = f2s(la.x), yal = f2s(la.y), zal = f2s(la.z);
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; u += 2) {
      const int b0 = u == 0 ? q4.x : q4.z, b1 = u == 0 ? q4.y : q4.w;
      const float4 p0 = Kp.fph[b0], p1 = Kp.fph[b1];
      const float4 l0 = Kp.fpl[b0], l1 = Kp.fpl[b1];
      const float2 m0 = ((const float2 *)Kp.fmA)[2 * b0];
      const float2 m1 = ((const float2 *)Kp.fmA)[2 * b1];
      // separations: exact high-word differences, low-word differences
      const ffloat2 dx = ff2_make(sub2(xa, f2(p0.x, p1.x)), sub2(xal, f2(l0.x, l1.x)));
      const ffloat2 dy = ff2_make(sub2(ya, f2(p0.y, p1.y)), sub2(yal, f2(l0.y, l1.y)));
      ffloat2 r2 = ff2_add(ff2_sqr_wide(dx), ff2_sqr_wide(dy));
      if(D == 3) {
        const ffloat2 dz = ff2_make(sub2(za, f2(p0.z, p1.z)), sub2(zal, f2(l0.z, l1.z)));
        r2 = ff2_add(r2, ff2_sqr_wide(dz));
      }
      const ffloat2 r = ff2_sqrt(ff2_norm(r2));
      ffloat2 ih = ih1;
      if(!UNI)
        ih = ff2_rcp_scaled(ff2_add(ff2_make(f2s(pa.w), f2s(la.w)),
                                    ff2_make(f2(p0.w, p1.w), f2(l0.w, l1.w))), 2.f);
      const ffloat2 q = ff2_mul(r, ih);
      const ffloat2 t = ff2_cadd(1.f, ff2_make(neg2(q.h), neg2(q.l)));
      ffloat2 w = ff2_mul(ff2_wpoly<K>(t), ff2_make(f2(m0.x, m1.x), f2(m0.y, m1.y)));
      if(!UNI) {
        // 1 / h_ab^D per lane
        const ffloat2 i2 = ff2_sqr(ih);
        w = ff2_mul(w, D == 3 ? ff2_mul(i2, ih) : i2);
      }
      const bool k0 = q.h.x < 1.f && j0 + u < cnt, k1 = q.h.y < 1.f && j0 + u + 1 < cnt;
      w.h = f2(k0 ? w.h.x : 0.f, k1 ? w.h.y : 0.f);
      w.l = f2(k0 ? w.l.x : 0.f, k1 ? w.l.y : 0.f);
      ff2_acc(sum, w);
    }
  }
  ffloat s1 = ff_add(ff2_lane(sum, 0), ff2_lane(sum, 1));
  if(UNI)
    s1 = ff_mul(s1, ihDa);
  return s1;
}

template<int D, int K, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS, 3) k_density_ff(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, double * cs_new, DevStatus * st,
  const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float4 pa = Kp.fph[a], la = Kp.fpl[a];
  const ffloat iha = ff_rcp_scaled(ff_make(pa.w, la.w), 1.f);
  const ffloat ihDa = ff_ipow<D>(iha);
  const int cnt = Ls.cnt[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
#if FSPH_DENSITY_PAIRED
  const ffloat sum = Kp.fscale[2] != 0.0
                       ? density_ff_sum2<D, K, true>(Kp, lp, cnt, pa, la, iha, ihDa)
                       : density_ff_sum2<D, K, false>(Kp, lp, cnt, pa, la, iha, ihDa);
#else
  const ffloat sum = Kp.fscale[2] != 0.0
                       ? density_ff_sum<D, K, true>(Kp, lp, cnt, pa, la, iha, ihDa)
                       : density_ff_sum<D, K, false>(Kp, lp, cnt, pa, la, iha, ihDa);
#endif
  double gsum[3] = {0.0, 0.0, 0.0};
  if(CULL) {
    // m_b grad_a W_ab for compute_divv, in FP64 (see k_density_mixed)
    double pa64[3] = {0.0, 0.0, 0.0};
    for(int d = 0; d < D; ++d)
      pa64[d] = P.f[F_X + d][a];
    const double h_a = P.f[F_H][a];
    for(int j = 0; j < cnt; ++j) {
      const int b = lp[slot_off(j)];
      double pos_ab[3] = {0.0, 0.0, 0.0}, DiW[3];
      for(int d = 0; d < D; ++d)
        pos_ab[d] = pa64[d] - P.f[F_X + d][b];
      kgrad<D, K>(pos_ab, .5 * (h_a + P.f[F_H][b]), DiW, pp);
      const double mbd = P.f[F_M][b];
      for(int d = 0; d < D; ++d)
        gsum[d] += mbd * DiW[d];
    }
  }
  const double iE = Kp.fscale[1];
  const double iED = D == 3 ? iE * iE * iE : iE * iE;
  const double rho = ff_wconst<D, K>() * iED * ff_to_double(sum);
  if(!(rho > 0)) {
    if(atomicCAS(&st->code, 0, (int)FSPH_ERR_NEG_DENSITY) == 0)
      st->index = a;
  }
  P.f[F_RHO][a] = rho;
  double u = P.f[F_U][a];
  if(pp.evolve_u && pp.thermokinetic) {
    double vv = 0;
    for(int d = 0; d < D; ++d)
      vv += P.f[F_VX + d][a] * P.f[F_VX + d][a];
    double eint = P.f[F_E][a] - .5 * vv - ext_potential_of<D>(pp, P.f, a);
    if(!(eint > 0)) {
      if(atomicCAS(&st->code, 0, (int)FSPH_ERR_NEG_ENERGY) == 0)
        st->index = a;
    }
    u = eint;
    P.f[F_U][a] = u;
  }
  double Pa, cs;
  eos_p_cs(pp, rho, u, P.f[F_K][a], P.f[F_YE][a], P.f[F_P][a], P.f[F_CS][a], Pa, cs);
  P.f[F_P][a] = Pa;
  cs_new[a] = cs;
  const double A = Pa / (rho * rho);
  Kp.thermo[a] = make_float4((float)rho, (float)A, (float)cs, (float)P.f[F_CS][a]);
  const float Ah = (float)A;
  ((float2 *)Kp.fmA)[2 * a + 1] = make_float2(Ah, (float)(A - (double)Ah));
  {
    // the acceleration and energy passes' v_half records (high and low
    // words) with this pass's rho and new c_s
    float vh[3] = {0.f, 0.f, 0.f}, vl[3] = {0.f, 0.f, 0.f};
    for(int d = 0; d < D; ++d) {
      const double v = P.f[F_VHX + d][a];
      vh[d] = (float)v;
      vl[d] = (float)(v - (double)vh[d]);
    }
    Kp.fv1[a] = make_float4(vh[0], vh[1], vh[2], (float)rho);
    Kp.fv2[a] = make_float4(vl[0], vl[1], vl[2], (float)cs);
  }
  if(CULL) {
    double div_v = 0.0;
    for(int d = 0; d < D; ++d)
      div_v += P.f[F_VX + d][a] * gsum[d];
    div_v /= rho;
    P.f[F_DDIVVDT][a] = (div_v - P.f[F_DIVV][a]) / tm->dt;
    P.f[F_DIVV][a] = div_v;
  }
}

// Acceleration
//   a_a = -sum_b m_b (P_a/rho_a^2 + P_b/rho_b^2 + Pi_ab) grad_a W_ab
// as two sums: the pressure terms, which cancel, in float-float, and the
// viscous terms (Pi is FP32) in FP32 with Kahan compensation; with VSIG,
// also the signal speed of the density pass (FP32, as k_vsig_mixed).  With
// UNI (every h equal) 1/h^(D+2) multiplies the finished sums instead of
// every pair.  The pressure sum alone is the pressure-only acceleration the
// de/dt pass takes.
// pairs of a four-slot list chunk the acceleration pass unrolls: all four
// (128 registers, no spills) measured 2 % faster than two at Sedov 128^3
// (2.01 against 2.05 ms per pass), one 10 % slower
#ifndef FSPH_ACCEL_FF_UNROLL
#define FSPH_ACCEL_FF_UNROLL 4
#endif
constexpr int accel_ff_unroll = FSPH_ACCEL_FF_UNROLL;

struct AccelFFState {
  ffloat sx, sy, sz;     // the pressure sum
  float vx, vy, vz;      // the viscous sum
  float vsig;
};

template<int D, int K, bool VSIG, bool CULL, bool UNI>
__device__ __forceinline__ void accel_ff_sum(const Packed & Kp, const int * lp,
  int cnt, int a, const float4 & pa, const float4 & la, const ffloat & iha,
  const ffloat & ihPa, const ffloat & Aa, const float4 & h1a, const float4 & h2a,
  const float4 & va, float eps, float alpha, float beta, float alpha_a,
  AccelFFState & out) {
  ffloat sx = ff_make(0.f, 0.f), sy = sx, sz = sx;
  float vx = 0.f, vy = 0.f, vz = 0.f, cvx = 0.f, cvy = 0.f, cvz = 0.f;
  float vsig = 0.f;
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll(accel_ff_unroll)
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const float4 pb = Kp.fph[b], lb = Kp.fpl[b];
      const FFGeom<D> g = ff_geom<D>(pa, la, pb, lb);
      ffloat ih = iha, ihP = ihPa;
      if(!UNI && (pb.w != pa.w || lb.w != la.w)) {
        ih = ff_rcp_scaled(ff_add(ff_make(pa.w, la.w), ff_make(pb.w, lb.w)), 2.f);
        ihP = ff_ipow<D + 2>(ih);
      }
      const ffloat q = ff_mul(g.r, ih);
      const ffloat t = ff_cadd(1.f, ff_make(-q.h, -q.l));
      const float4 h1b = Kp.fv1[b], h2b = Kp.fv2[b];  // v_half, rho, c_s
      const float4 mAb = Kp.fmA[b];
      // viscosity in FP32 (the position unit cancels in mu)
      const float hab = 0.5f * (pa.w + pb.w);
      const float dotp = vdiff_dot(h1a, h2a, h1b, h2b, g.dxr[0], g.dxr[1], g.dxr[2]);
      const float mu = dotp < 0.f ? __fdividef(hab * dotp, g.r2f + eps * hab * hab) : 0.f;
      const float rho_ab = 0.5f * (h1a.w + h1b.w);
      const float c_ab = 0.5f * (h2a.w + h2b.w);
      const float Pi = visc_pi_f<CULL>(alpha, beta, alpha_a, Kp, b, rho_ab, c_ab, mu);
      const ffloat gp = ff_gpoly<K>(t);
      ffloat S = ff_mul(ff_mul(ff_add(Aa, ff_make(mAb.z, mAb.w)), ff_make(mAb.x, mAb.y)),
        gp);
      float V = mAb.x * Pi * gp.h;
      if(!UNI) {
        S = ff_mul(S, ihP);
        V *= ihP.h;
      }
      if(!(q.h < 1.f)) {
        S = ff_make(0.f, 0.f);
        V = 0.f;
      }
      if(VSIG) {
        const float4 vb = Kp.vel[b];  // .w: c_s before the density pass
        const float dotv = ((va.x - vb.x) * g.dxr[0] + (va.y - vb.y) * g.dxr[1] +
                             (va.z - vb.z) * g.dxr[2]) * rsqrtf(g.r2f);
        const float cb = b > a ? h2b.w : vb.w;
        const float cand = fmaxf(h2a.w, cb) - fminf(dotv, 0.f);
        vsig = fmaxf(vsig, (b != a && g.r2f > 0.f) ? cand : 0.f);
      }
      // padding slots and the self pair have dx = 0 and add nothing
      ff_acc(sx, ff_mul(S, g.dx[0]));
      ff_acc(sy, ff_mul(S, g.dx[1]));
      kahan(vx, cvx, V * g.dxr[0]);
      kahan(vy, cvy, V * g.dxr[1]);
      if(D == 3) {
        ff_acc(sz, ff_mul(S, g.dx[2]));
        kahan(vz, cvz, V * g.dxr[2]);
      }
    }
  }
  if(UNI) {
    sx = ff_mul(sx, ihPa);
    sy = ff_mul(sy, ihPa);
    sz = ff_mul(sz, ihPa);
  }
  const float ihs = UNI ? ihPa.h : 1.f;
  out.sx = sx;
  out.sy = sy;
  out.sz = sz;
  out.vx = (vx - cvx) * ihs;
  out.vy = (vy - cvy) * ihs;
  out.vz = (vz - cvz) * ihs;
  out.vsig = vsig;
}

// Resident blocks of 256 per SM the acceleration pass is compiled for.  2
// gives it up to 128 registers; 3 caps it at 80 for 24 warps to hide the
// neighbour gathers, which measured slower on Sedov 128^3 (2.23 against
// 1.94 ms per pass: the spills and the lost unrolling cost more than the
// extra warps gain).
#ifndef FSPH_ACCEL_FF_BLOCKS
#define FSPH_ACCEL_FF_BLOCKS 2
#endif
#ifndef FSPH_ACCEL_FF_THREADS
#define FSPH_ACCEL_FF_THREADS MIX_THREADS
#endif

template<int D, int K, bool VSIG, bool CULL>
__global__ void __launch_bounds__(FSPH_ACCEL_FF_THREADS, FSPH_ACCEL_FF_BLOCKS) k_accel_ff(
  Particles P, PhysParams pp, Lists Ls, Packed Kp, int kick, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const float alpha_a = CULL ? Kp.visc[a].x : 0.f;
  const float4 pa = Kp.fph[a], la = Kp.fpl[a];
  const float2 Aa2 = ((const float2 *)Kp.fmA)[2 * a + 1];
  const ffloat Aa = ff_make(Aa2.x, Aa2.y);
  const ffloat iha = ff_rcp_scaled(ff_make(pa.w, la.w), 1.f);
  const ffloat ihPa = ff_ipow<D + 2>(iha);
  const float4 h1a = Kp.fv1[a], h2a = Kp.fv2[a];
  const int cnt = Ls.cnt[a];
  float4 va = make_float4(0.f, 0.f, 0.f, 0.f);
  if(VSIG)
    va = Kp.vel[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  AccelFFState r;
  if(Kp.fscale[2] != 0.0)
    accel_ff_sum<D, K, VSIG, CULL, true>(Kp, lp, cnt, a, pa, la, iha, ihPa, Aa, h1a,
      h2a, va, eps, alpha, beta, alpha_a, r);
  else
    accel_ff_sum<D, K, VSIG, CULL, false>(Kp, lp, cnt, a, pa, la, iha, ihPa, Aa, h1a,
      h2a, va, eps, alpha, beta, alpha_a, r);
  const double iE = Kp.fscale[1];
  const double iE2 = iE * iE;
  // a = -gconst / E^(D+1) * sum
  const double scale = -ff_gconst<D, K>() * (D == 3 ? iE2 * iE2 : iE2 * iE);
  const double ap[3] = {scale * ff_to_double(r.sx), scale * ff_to_double(r.sy),
    D == 3 ? scale * ff_to_double(r.sz) : 0.0};
  double acc[3] = {ap[0] + scale * (double)r.vx, ap[1] + scale * (double)r.vy,
    D == 3 ? ap[2] + scale * (double)r.vz : 0.0};
  if(Kp.ahyd) {
    // the pressure-only hydro acceleration for the de/dt pass
    for(int d = 0; d < D; ++d)
      Kp.ahyd[(size_t)d * P.n + a] = ap[d];
  }
  if(pp.has_eacc) {  // acc_a += external_force::acceleration (:404)
    const double pos[3] = {P.f[F_X][a], P.f[F_Y][a], D == 3 ? P.f[F_Z][a] : 0.0};
    double ext[3];
    ext_acceleration<D>(pp, pos, ext);
    for(int d = 0; d < D; ++d)
      acc[d] += ext[d];
  }
  const double half_dt = kick ? 0.5 * tm->dt : 0.0;
  float dv[3] = {0.f, 0.f, 0.f};
  for(int d = 0; d < D; ++d) {
    P.f[F_AX + d][a] = acc[d];
    P.f[F_GAX + d][a] = 0.0;
    if(kick) {
      const double v = P.f[F_VX + d][a] + acc[d] * half_dt;
      P.f[F_VX + d][a] = v;
      dv[d] = (float)(v - P.f[F_VHX + d][a]);
    }
  }
  // the energy passes' {v - v_half, m} record of the kicked velocity
  if(kick)
    Kp.fdv[a] = make_float4(dv[0], dv[1], dv[2], (float)P.f[F_M][a]);
  P.f[F_GPOT][a] = 0.0;
  if(VSIG)
    P.f[F_VSIG][a] = (double)r.vsig;
}

// de/dt through the pressure-only acceleration of the float-float pass.
// With a^P_a = -sum_b m_b (A_a + A_b) grad W_ab (A = P/rho^2), the
// reference's
//   de/dt_a = -sum_b m_b (A_a v_b + A_b v_a + Pi_ab (v_a + v_b) / 2) . grad W_ab
//             + g_a . v_a                      (default_physics.h:502-566)
// is, exactly (A_a v_b + A_b v_a = (A_a + A_b) v_a + A_a (v_b - v_a)),
//   de/dt_a = v_a . a^P_a
//             - sum_b m_b (A_a (v_b - v_a) + Pi_ab (v_a + v_b) / 2) . grad W_ab
//             + g_a . v_a.
// The pressure terms, which cancel on lattices and in equilibrium, are then
// those of a^P (float-float, less an FP32 viscous part); the remaining sum,
// over velocity differences and the viscosity, stays FP32.  Valid while
// positions, P/rho^2, v_half and alpha are those of the acceleration pass
// (the caller tracks that).
template<int D, int K, bool CULL>
__global__ void __launch_bounds__(MIX_THREADS, FSPH_ENERGY_BLOCKS) k_dedt_ahyd(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, int then_op, const DevTime * tm,
  DevStatus * st) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const float alpha_a = CULL ? Kp.visc[a].x : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 h1a = Kp.fv1[a], h2a = Kp.fv2[a], dva = Kp.fdv[a];
  const float Aa = Kp.fmA[a].z;  // P_a / rho_a^2 (high word)
  const int cnt = Ls.cnt[a];
  float sum = 0.f, comp = 0.f;
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = __fdividef(1.f, hab);
      const float f = gfac<D, K>(sqrtf(g.r2), hab, ih, pp);
      const float4 h1b = Kp.fv1[b], h2b = Kp.fv2[b], dvb = Kp.fdv[b];
      const float dotp = vdiff_dot(h1a, h2a, h1b, h2b, g.dx, g.dy, g.dz);
      const float mu = dotp < 0.f ? __fdividef(hab * dotp, g.r2 + eps * hab * hab) : 0.f;
      const float Pi = visc_pi_f<CULL>(alpha, beta, alpha_a, Kp, b, 0.5f * (h1a.w + h1b.w),
        0.5f * (h2a.w + h2b.w), mu);
      // v_b - v_a and v_a + v_b, v = v_half + (v - v_half)
      const float vbad = f * vel_diff_dot(h1b, h2b, dvb, h1a, h2a, dva, g.dx, g.dy, g.dz);
      const float vsd = f * (((h1a.x + h1b.x) + (dva.x + dvb.x)) * g.dx +
                             ((h1a.y + h1b.y) + (dva.y + dvb.y)) * g.dy +
                             ((h1a.z + h1b.z) + (dva.z + dvb.z)) * g.dz);
      kahan(sum, comp, dvb.w * (Aa * vbad + 0.5f * Pi * vsd));
    }
  }
  double gv = 0, vah = 0;
  for(int d = 0; d < D; ++d) {
    gv += P.f[F_GAX + d][a] * P.f[F_VX + d][a];
    vah += P.f[F_VX + d][a] * Kp.ahyd[(size_t)d * P.n + a];
  }
  const double dedt = vah - ((double)sum - (double)comp) + gv;
  P.f[F_DEDT][a] = dedt;
  if(then_op) {
    // recompute_pressure_soundspeed_thermokinetic (default_physics.h:169-182)
    // and, with the kick, leapfrog_kick_e (integration.h:94-98)
    const double dt = tm->dt;
    double vv = 0, vda = 0;
    for(int d = 0; d < D; ++d) {
      const double v = P.f[F_VX + d][a];
      vv += v * v;
      vda += v * P.f[F_AX + d][a];
    }
    const double e = P.f[F_E][a];
    const double eint = e - .5 * vv - ext_potential_of<D>(pp, P.f, a);
    if(!(eint > 0))
      raise_status(st, FSPH_ERR_NEG_ENERGY, a);
    P.f[F_U][a] = eint;
    double Pn, cs;
    eos_p_cs(pp, P.f[F_RHO][a], eint + 0.5 * dt * (dedt - vda), P.f[F_K][a],
      P.f[F_YE][a], P.f[F_P][a], P.f[F_CS][a], Pn, cs);
    P.f[F_P][a] = Pn;
    P.f[F_CS][a] = cs;
    if(then_op == OP_RECOMPUTE_KICK_E)
      P.f[F_E][a] = e + 0.5 * dt * dedt;
  }
}

// ------------------------------------------------------------ dispatch --
#define MIX_DISPATCH(KERNEL_T, TA, ...)                                            \
  do {                                                                         \
    const int nb_ = (P.n + MIX_THREADS - 1) / MIX_THREADS;                     \
    if(pp.dim == 3) {                                                          \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<3, FSPH_KERNEL_CUBIC_SPLINE, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<3, FSPH_KERNEL_QUINTIC_SPLINE, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<3, FSPH_KERNEL_GAUSSIAN, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<3, FSPH_KERNEL_SUPER_GAUSSIAN, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<3, FSPH_KERNEL_SINC, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C2, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C4, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C6, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    else {                                                                     \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<2, FSPH_KERNEL_CUBIC_SPLINE, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<2, FSPH_KERNEL_QUINTIC_SPLINE, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<2, FSPH_KERNEL_GAUSSIAN, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<2, FSPH_KERNEL_SUPER_GAUSSIAN, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<2, FSPH_KERNEL_SINC, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C2, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C4, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C6, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    *L.counter += 1;                                                           \
  } while(0)


// Launch the pair kernels of one viscosity choice for the step's dimension
// and smoothing kernel.
// The float-float passes serve the Wendland kernels; the other kernels
// (cubic and quintic splines, Gaussians, sinc) keep the FP32 passes.
#define FF_DISPATCH(KERNEL_T, TA, ...)                                         \
  do {                                                                         \
    const int nb_ = (P.n + MIX_THREADS - 1) / MIX_THREADS;                     \
    if(pp.dim == 3) {                                                          \
      if(pp.kernel == FSPH_KERNEL_WENDLAND_C2)                                 \
        KERNEL_T<3, FSPH_KERNEL_WENDLAND_C2, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
      else if(pp.kernel == FSPH_KERNEL_WENDLAND_C4)                            \
        KERNEL_T<3, FSPH_KERNEL_WENDLAND_C4, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
      else                                                                     \
        KERNEL_T<3, FSPH_KERNEL_WENDLAND_C6, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
    }                                                                          \
    else {                                                                     \
      if(pp.kernel == FSPH_KERNEL_WENDLAND_C2)                                 \
        KERNEL_T<2, FSPH_KERNEL_WENDLAND_C2, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
      else if(pp.kernel == FSPH_KERNEL_WENDLAND_C4)                            \
        KERNEL_T<2, FSPH_KERNEL_WENDLAND_C4, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
      else                                                                     \
        KERNEL_T<2, FSPH_KERNEL_WENDLAND_C6, TA><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); \
    }                                                                          \
    *L.counter += 1;                                                           \
  } while(0)

inline bool wendland_kernel(int k) {
  return k == FSPH_KERNEL_WENDLAND_C2 || k == FSPH_KERNEL_WENDLAND_C4 ||
         k == FSPH_KERNEL_WENDLAND_C6;
}

template<bool CULL>
inline void run_density_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st, const DevTime * tm) {
  if(wendland_kernel(pp.kernel))
    FF_DISPATCH(k_density_ff, CULL, P, pp, Ls, K, cs_new, st, tm);
  else
    MIX_DISPATCH(k_density_mixed, CULL, P, pp, Ls, K, cs_new, st, tm);
}

template<bool CULL>
inline void run_dudt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t,
  int then_op) {
  MIX_DISPATCH(k_dudt_mixed, CULL, P, pp, Ls, K, t, then_op);
}

template<bool CULL>
inline void run_dedt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int then_op,
  const DevTime * t, DevStatus * st, int use_ahyd) {
  if(use_ahyd && wendland_kernel(pp.kernel))
    FF_DISPATCH(k_dedt_ahyd, CULL, P, pp, Ls, K, then_op, t, st);
  else
    MIX_DISPATCH(k_dedt_mixed, CULL, P, pp, Ls, K, then_op, t, st);
}

template<bool CULL>
inline void run_accel_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int kick,
  const DevTime * t, int fused_vsig) {
  int threads = MIX_THREADS;
  void (*fn)(Particles, PhysParams, Lists, Packed, int, const DevTime *) = nullptr;
#define PICK(D, KK)                                                            \
  fn = fused_vsig ? k_accel_mixed<D, KK, true, CULL> : k_accel_mixed<D, KK, false, CULL>
  if(pp.dim == 3) {
    switch(pp.kernel) {
      case FSPH_KERNEL_CUBIC_SPLINE: PICK(3, FSPH_KERNEL_CUBIC_SPLINE); break;
      case FSPH_KERNEL_QUINTIC_SPLINE: PICK(3, FSPH_KERNEL_QUINTIC_SPLINE); break;
      case FSPH_KERNEL_GAUSSIAN: PICK(3, FSPH_KERNEL_GAUSSIAN); break;
      case FSPH_KERNEL_SUPER_GAUSSIAN: PICK(3, FSPH_KERNEL_SUPER_GAUSSIAN); break;
      case FSPH_KERNEL_SINC: PICK(3, FSPH_KERNEL_SINC); break;
      case FSPH_KERNEL_WENDLAND_C2: PICK(3, FSPH_KERNEL_WENDLAND_C2); break;
      case FSPH_KERNEL_WENDLAND_C4: PICK(3, FSPH_KERNEL_WENDLAND_C4); break;
      default: PICK(3, FSPH_KERNEL_WENDLAND_C6); break;
    }
  }
  else {
    switch(pp.kernel) {
      case FSPH_KERNEL_CUBIC_SPLINE: PICK(2, FSPH_KERNEL_CUBIC_SPLINE); break;
      case FSPH_KERNEL_QUINTIC_SPLINE: PICK(2, FSPH_KERNEL_QUINTIC_SPLINE); break;
      case FSPH_KERNEL_GAUSSIAN: PICK(2, FSPH_KERNEL_GAUSSIAN); break;
      case FSPH_KERNEL_SUPER_GAUSSIAN: PICK(2, FSPH_KERNEL_SUPER_GAUSSIAN); break;
      case FSPH_KERNEL_SINC: PICK(2, FSPH_KERNEL_SINC); break;
      case FSPH_KERNEL_WENDLAND_C2: PICK(2, FSPH_KERNEL_WENDLAND_C2); break;
      case FSPH_KERNEL_WENDLAND_C4: PICK(2, FSPH_KERNEL_WENDLAND_C4); break;
      default: PICK(2, FSPH_KERNEL_WENDLAND_C6); break;
    }
  }
#undef PICK
#define PICK(D, KK)                                                            \
  fn = fused_vsig ? k_accel_ff<D, KK, true, CULL> : k_accel_ff<D, KK, false, CULL>
  if(wendland_kernel(pp.kernel)) {
    if(pp.dim == 3) {
      if(pp.kernel == FSPH_KERNEL_WENDLAND_C2) PICK(3, FSPH_KERNEL_WENDLAND_C2);
      else if(pp.kernel == FSPH_KERNEL_WENDLAND_C4) PICK(3, FSPH_KERNEL_WENDLAND_C4);
      else PICK(3, FSPH_KERNEL_WENDLAND_C6);
    }
    else {
      if(pp.kernel == FSPH_KERNEL_WENDLAND_C2) PICK(2, FSPH_KERNEL_WENDLAND_C2);
      else if(pp.kernel == FSPH_KERNEL_WENDLAND_C4) PICK(2, FSPH_KERNEL_WENDLAND_C4);
      else PICK(2, FSPH_KERNEL_WENDLAND_C6);
    }
    threads = FSPH_ACCEL_FF_THREADS;
  }
#undef PICK
  fn<<<(P.n + threads - 1) / threads, threads, 0, L.stream>>>(P, pp, Ls, K, kick, t);
  *L.counter += 1;
}

// The Cullen & Dehnen instances, compiled in fsph_mixed_cullen.cu.
void run_density_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st, const DevTime * tm);
void run_accel_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int kick,
  const DevTime * t, int fused_vsig);
void run_dudt_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t,
  int then_op);
void run_dedt_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int then_op,
  const DevTime * t, DevStatus * st, int use_ahyd);
void run_alpha_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t);

}  // namespace fsph
