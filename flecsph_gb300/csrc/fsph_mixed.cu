// fsph_mixed.cu -- the mixed-precision neighbour-pair kernels.
//
// Pair arithmetic runs in FP32 on packed per-particle records; the density,
// force and energy sums are Kahan-compensated; every per-particle quantity
// the integrator carries stays FP64 (EOS, kicks, stored fields).  Positions
// enter as 31-bit fixed point over the step's range, so the separation of a
// pair is an exact integer difference scaled once: ~1e-9 of the range
// instead of the 6e-8 an FP32 coordinate would give.
//
// Formulas are those of the reference (default_physics.h:193-566,
// kernels.h, viscosity.h:81-137); algebraic rewrites only (grad W / r
// folded into one factor, which stays finite at r = 0).  The self pair and
// coincident pairs contribute exactly zero to forces and energies (x_ab = 0
// and mu = 0), as the reference's m_b = 0 makes them (:378,456,534), and
// are masked out of the signal speed, where the reference drops a NaN
// (:254-262): FP32 has no equivalent of the reference's TINY guards.
#include <cuda_runtime.h>

#include "fsph_internal.cuh"
#include "fsph_sphmath.cuh"  // the FP64 EOS the density pass applies

namespace fsph {

#define MIX_THREADS 256
#define FPI 3.14159265358979323846f

__device__ __forceinline__ double ord_dec_m(unsigned long long u) {
  return (u & 0x8000000000000000ull)
           ? __longlong_as_double((long long)(u & 0x7fffffffffffffffull))
           : __longlong_as_double((long long)~u);
}

__device__ __forceinline__ void kahan(float & sum, float & comp, float term) {
  float y = term - comp;
  float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// ------------------------------------------------------------- packing --
__global__ void k_pack_pos(Particles P, int dim,
  const unsigned long long * rbits, Packed K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < 3 && i < dim) {
    double ext = ord_dec_m(rbits[3 + i]) - ord_dec_m(rbits[i]);
    K.qscale[i] = (float)(ext / 2147483648.0);
  }
  if(i >= P.n)
    return;
  int q[3] = {0, 0, 0};
  for(int d = 0; d < dim; ++d) {
    // any monotone mapping shared by all particles will do: multiply by the
    // reciprocal instead of dividing (FP64 division is costly on this part)
    double lo = ord_dec_m(rbits[d]), hi = ord_dec_m(rbits[3 + d]);
    double t = (P.f[F_X + d][i] - lo) * (2147483648.0 / (hi - lo));
    t = fmin(fmax(t, 0.0), 2147483647.0);
    q[d] = __double2int_rn(t);
  }
  K.qpos[i] = make_int4(q[0], q[1], q[2], __float_as_int((float)P.f[F_H][i]));
}

enum { PACK_VHM = 1, PACK_VEL = 2, PACK_THERMO = 4 };

// Refresh the packed records a pass reads from the FP64 state, so every
// pass sees the current v_half, v, rho, P and c_s whatever the caller did
// in between (separate kicks, repeated pressure updates).
__global__ void k_pack_state(Particles P, int dim, Packed K, int what) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  if(what & PACK_VHM)
    K.vhm[i] = make_float4((float)P.f[F_VHX][i], (float)P.f[F_VHY][i],
      dim == 3 ? (float)P.f[F_VHZ][i] : 0.f, (float)P.f[F_M][i]);
  if(what & PACK_VEL)
    K.vel[i] = make_float4((float)P.f[F_VX][i], (float)P.f[F_VY][i],
      dim == 3 ? (float)P.f[F_VZ][i] : 0.f, 0.f);
  if(what & PACK_THERMO) {
    const double rho = P.f[F_RHO][i], cs = P.f[F_CS][i];
    K.thermo[i] = make_float4((float)rho, (float)(P.f[F_P][i] / (rho * rho)),
      (float)cs, (float)cs);
  }
}

cudaError_t launch_pack_positions(const Launch & L, const Particles & P,
  const PhysParams & pp, const unsigned long long * rbits, const Packed & K) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  k_pack_pos<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, rbits, K);
  *L.counter += 1;
  return cudaGetLastError();
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

struct PairGeom {
  float dx, dy, dz, r2;
};

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
template<int D, int K>
__global__ void __launch_bounds__(MIX_THREADS) k_density_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, double * cs_new, DevStatus * st) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const int cnt = Ls.cnt[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  float sum = 0.f, comp = 0.f;
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const int4 qb = Kp.qpos[b];
      const float mb = Kp.vhm[b].w;
      const PairGeom g = geom<D>(qa, qb, s0, s1, s2);
      const float hab = 0.5f * (ha + __int_as_float(qb.w));
      const float ih = 1.0f / hab;
      const float w = mb * wfun<D, K>(sqrtf(g.r2), hab, ih, pp);
      kahan(sum, comp, j0 + u < cnt ? w : 0.f);
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
    double eint = P.f[F_E][a] - .5 * vv;
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
}

// -------------------------------------------------------- signal speed --
// Same visiting-order rule as the FP64 pass: neighbours with a higher
// sorted index contribute their new sound speed (thermo.z), the others the
// previous one (thermo.w).
template<int D>
__global__ void __launch_bounds__(MIX_THREADS) k_vsig_mixed(Particles P,
  Lists Ls, Packed Kp) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const int4 qa = Kp.qpos[a];
  const float4 va = Kp.vel[a];
  const float ca = Kp.thermo[a].z;
  const int cnt = Ls.cnt[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  float vsig = 0.f;
  for(int j0 = 0; j0 < cnt; j0 += 4) {
    // four slots per 16-byte load; padding slots hold a itself
    const int4 q4 = *(const int4 *)(lp + (j0 << 5));
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      const int b = u == 0 ? q4.x : u == 1 ? q4.y : u == 2 ? q4.z : q4.w;
      const PairGeom g = geom<D>(qa, Kp.qpos[b], s0, s1, s2);
      const float4 vb = Kp.vel[b];
      const float4 tb = Kp.thermo[b];
      const float dotv = ((va.x - vb.x) * g.dx + (va.y - vb.y) * g.dy +
                           (va.z - vb.z) * g.dz) * rsqrtf(g.r2);
      const float cb = b > a ? tb.z : tb.w;
      // the self pair and coincident pairs are NaN in the reference and drop out
      const float cand = fmaxf(ca, cb) - fminf(dotv, 0.f);
      vsig = fmaxf(vsig, (b != a && g.r2 > 0.f) ? cand : 0.f);
    }
  }
  P.f[F_VSIG][a] = (double)vsig;
}

// -------------------------------------------------------- acceleration --
// With VSIG the signal speed of the density pass (same neighbours, same
// rule as k_vsig_mixed) is evaluated in this loop instead of a pass of its
// own; it reads the pre-kick velocities packed for the density pass, so the
// kick below cannot race with it.
template<int D, int K, bool VSIG>
__global__ void __launch_bounds__(MIX_THREADS) k_accel_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, int kick, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
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
      const float ih = 1.0f / hab;
      const float r = sqrtf(g.r2);
      const float f = gfac<D, K>(r, hab, ih, pp);
      const float4 vhb = Kp.vhm[b];
      const float4 tb = Kp.thermo[b];
      const float dotp = (vha.x - vhb.x) * g.dx + (vha.y - vhb.y) * g.dy +
                         (vha.z - vhb.z) * g.dz;
      const float mu = dotp < 0.f ? hab * dotp / (g.r2 + eps * hab * hab) : 0.f;
      const float rho_ab = 0.5f * (ta.x + tb.x);
      const float c_ab = 0.5f * (ta.z + tb.z);
      const float Pi = (-alpha * c_ab + beta * mu) * mu / rho_ab;
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
  const double acc[3] = {(double)ax - (double)cx, (double)ay - (double)cy,
    D == 3 ? (double)az - (double)cz : 0.0};
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
template<int D, int K>
__global__ void __launch_bounds__(MIX_THREADS) k_dudt_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 vha = Kp.vhm[a];
  const float4 va = Kp.vel[a];
  const float4 ta = Kp.thermo[a];
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
      const float ih = 1.0f / hab;
      const float f = gfac<D, K>(sqrtf(g.r2), hab, ih, pp);
      const float4 vhb = Kp.vhm[b];
      const float4 vb = Kp.vel[b];
      const float4 tb = Kp.thermo[b];
      const float dotp = (vha.x - vhb.x) * g.dx + (vha.y - vhb.y) * g.dy +
                         (vha.z - vhb.z) * g.dz;
      const float mu = dotp < 0.f ? hab * dotp / (g.r2 + eps * hab * hab) : 0.f;
      const float rho_ab = 0.5f * (ta.x + tb.x);
      const float c_ab = 0.5f * (ta.z + tb.z);
      const float Pi = (-alpha * c_ab + beta * mu) * mu / rho_ab;
      const float vdw = f * ((va.x - vb.x) * g.dx + (va.y - vb.y) * g.dy +
                             (va.z - vb.z) * g.dz);
      kahan(dp, cp, vhb.w * vdw);
      kahan(dv, cv, vhb.w * vdw * Pi);
    }
  }
  const double sp = (double)dp - (double)cp, sv = (double)dv - (double)cv;
  const double rho_a = P.f[F_RHO][a];
  P.f[F_DUDT][a] = P.f[F_P][a] / (rho_a * rho_a) * sp + .5 * sv;
}

// --------------------------------------------------------------- de/dt --
template<int D, int K>
__global__ void __launch_bounds__(MIX_THREADS) k_dedt_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const float eps = (float)pp.eps, alpha = (float)pp.alpha, beta = (float)pp.beta;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 vha = Kp.vhm[a];
  const float4 va = Kp.vel[a];
  const float4 ta = Kp.thermo[a];
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
      const float ih = 1.0f / hab;
      const float f = gfac<D, K>(sqrtf(g.r2), hab, ih, pp);
      const float4 vhb = Kp.vhm[b];
      const float4 vb = Kp.vel[b];
      const float4 tb = Kp.thermo[b];
      const float dotp = (vha.x - vhb.x) * g.dx + (vha.y - vhb.y) * g.dy +
                         (vha.z - vhb.z) * g.dz;
      const float mu = dotp < 0.f ? hab * dotp / (g.r2 + eps * hab * hab) : 0.f;
      const float rho_ab = 0.5f * (ta.x + tb.x);
      const float c_ab = 0.5f * (ta.z + tb.z);
      const float Pi = (-alpha * c_ab + beta * mu) * mu / rho_ab;
      const float vad = f * (va.x * g.dx + va.y * g.dy + va.z * g.dz);
      const float vbd = f * (vb.x * g.dx + vb.y * g.dy + vb.z * g.dz);
      kahan(sum, comp, vhb.w * (ta.y * vbd + vad * tb.y + 0.5f * Pi * (vbd + vad)));
    }
  }
  double gv = 0;
  for(int d = 0; d < D; ++d)
    gv += P.f[F_GAX + d][a] * P.f[F_VX + d][a];
  P.f[F_DEDT][a] = -((double)sum - (double)comp) + gv;
}

// ------------------------------------------------------------ dispatch --
#define MIX_DISPATCH(KERNEL_T, ...)                                            \
  do {                                                                         \
    const int nb_ = (P.n + MIX_THREADS - 1) / MIX_THREADS;                     \
    if(pp.dim == 3) {                                                          \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<3, FSPH_KERNEL_CUBIC_SPLINE><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<3, FSPH_KERNEL_QUINTIC_SPLINE><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<3, FSPH_KERNEL_GAUSSIAN><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<3, FSPH_KERNEL_SUPER_GAUSSIAN><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<3, FSPH_KERNEL_SINC><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C2><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C4><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C6><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    else {                                                                     \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<2, FSPH_KERNEL_CUBIC_SPLINE><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<2, FSPH_KERNEL_QUINTIC_SPLINE><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<2, FSPH_KERNEL_GAUSSIAN><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<2, FSPH_KERNEL_SUPER_GAUSSIAN><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<2, FSPH_KERNEL_SINC><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C2><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C4><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C6><<<nb_, MIX_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    *L.counter += 1;                                                           \
  } while(0)

cudaError_t launch_density_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // masses for the density sum, velocities of this step for the signal speed
  k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K,
    PACK_VHM | PACK_VEL);
  *L.counter += 1;
  MIX_DISPATCH(k_density_mixed, P, pp, Ls, K, cs_new, st);
  return cudaGetLastError();
}

cudaError_t launch_vsig_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  if(pp.dim == 3)
    k_vsig_mixed<3><<<nb, MIX_THREADS, 0, L.stream>>>(P, Ls, K);
  else
    k_vsig_mixed<2><<<nb, MIX_THREADS, 0, L.stream>>>(P, Ls, K);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_accel_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int kick,
  const DevTime * t, int fused_vsig) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // v_half of this step (set by the caller's save_velocityhalf); the thermo
  // records are refreshed unless they come straight from the density pass
  // (fused signal speed needs their previous-sound-speed slot)
  k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K,
    fused_vsig ? PACK_VHM : (PACK_VHM | PACK_THERMO));
  *L.counter += 1;
  void (*fn)(Particles, PhysParams, Lists, Packed, int, const DevTime *) = nullptr;
#define PICK(D, KK)                                                            \
  fn = fused_vsig ? k_accel_mixed<D, KK, true> : k_accel_mixed<D, KK, false>
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
  fn<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp, Ls, K, kick, t);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_dudt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K,
    PACK_VHM | PACK_VEL | PACK_THERMO);
  *L.counter += 1;
  MIX_DISPATCH(k_dudt_mixed, P, pp, Ls, K);
  return cudaGetLastError();
}

cudaError_t launch_dedt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K,
    PACK_VHM | PACK_VEL | PACK_THERMO);
  *L.counter += 1;
  MIX_DISPATCH(k_dedt_mixed, P, pp, Ls, K);
  return cudaGetLastError();
}

}  // namespace fsph
