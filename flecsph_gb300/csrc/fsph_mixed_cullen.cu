// fsph_mixed_cullen.cu -- Cullen & Dehnen's adaptive viscosity on the
// mixed-precision path: the pair kernels of fsph_mixed_kernels.cuh with a
// per-particle alpha, and the alpha pass itself.
#include <cuda_runtime.h>

#include "fsph_internal.cuh"
#include "fsph_mixed_kernels.cuh"

namespace fsph {

void run_density_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st, const DevTime * tm) {
  run_density_mixed<true>(L, P, pp, Ls, K, cs_new, st, tm);
}

void run_accel_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int kick,
  const DevTime * t, int fused_vsig) {
  run_accel_mixed<true>(L, P, pp, Ls, K, kick, t, fused_vsig);
}

void run_dudt_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t,
  int then_op) {
  run_dudt_mixed<true>(L, P, pp, Ls, K, t, then_op);
}

void run_dedt_mixed_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int then_op,
  const DevTime * t, DevStatus * st, int use_ahyd) {
  run_dedt_mixed<true>(L, P, pp, Ls, K, then_op, t, st, use_ahyd);
}

// viscosity::compute_alpha with A_trigger and compute_xi (viscosity.h:
// 185-363).  The neighbour sums (the signal speed over all new sound
// speeds, R_a = sum sign(div v_b) m_b W_ab, the velocity gradient
// sum m_b (v_b - v_a) (x) grad_a W_ab) run in FP32 on the packed records,
// R_a Kahan-compensated; the limiter and the alpha update run in FP64 in
// the reference's operand order.  Padding slots repeat the particle itself:
// they are masked out of R_a and the signal speed and add zero to the
// gradient (v_ab = 0).
template<int D, int K>
__global__ void __launch_bounds__(MIX_THREADS) k_alpha_mixed(Particles P,
  PhysParams pp, Lists Ls, Packed Kp, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const float s0 = Kp.qscale[0], s1 = Kp.qscale[1], s2 = D == 3 ? Kp.qscale[2] : 0.f;
  const int4 qa = Kp.qpos[a];
  const float ha = __int_as_float(qa.w);
  const float4 va = Kp.vel[a];
  const float ca = Kp.visc[a].x;
  const int cnt = Ls.cnt[a];
  const int * lp = Ls.idx + list_slot(a, 0, Ls.maxnb);
  float vsig = 0.f, R = 0.f, cR = 0.f;
  float gv[D * D];
#pragma unroll
  for(int k = 0; k < D * D; ++k)
    gv[k] = 0.f;
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
      const float4 vb = Kp.vel[b];
      const float2 sb = Kp.visc[b];
      const float mb = Kp.vhm[b].w;
      const float vab[3] = {va.x - vb.x, va.y - vb.y, va.z - vb.z};
      const float dx[3] = {g.dx, g.dy, g.dz};
      // vsig = max(vsig, max(c_a, c_b) - min(v_ab . n_ab, 0)); the self
      // pair and coincident pairs are NaN in the reference and drop out
      const float dotv = (vab[0] * g.dx + vab[1] * g.dy + vab[2] * g.dz) * rsqrtf(g.r2);
      const float cand = fmaxf(ca, sb.x) - fminf(dotv, 0.f);
      vsig = fmaxf(vsig, (b != a && g.r2 > 0.f) ? cand : 0.f);
      const float w = wfun<D, K>(r, hab, ih, pp);
      kahan(R, cR, j0 + u < cnt ? sb.y * mb * w : 0.f);
      const float fm = mb * gfac<D, K>(r, hab, ih, pp);
#pragma unroll
      for(int i = 0; i < D; ++i)
#pragma unroll
        for(int k = 0; k < D; ++k)
          gv[D * i + k] += -vab[i] * (dx[k] * fm);
    }
  }
  const double rho_a = P.f[F_RHO][a];
  const double h_a = P.f[F_H][a];
  const double alpha_a = P.f[F_ALPHA][a];
  const double R_a = ((double)R - (double)cR) / rho_a;
  double gradV[D * D];
  for(int k = 0; k < D * D; ++k)
    gradV[k] = (double)gv[k] / rho_a;
  const double divV_a = P.f[F_DIVV][a];
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
  const double q4 = om * om * om * om;
  const double t = 2.0 * q4 * divV_a;
  const double res = t * t;
  const double xi = (res < 1e-16) ? 0.0 : res / (res + traceSS);
  const double ddv = P.f[F_DDIVVDT][a];
  const double trig = -ddv < 0.0 ? 0.0 : -ddv;
  const double Atrig = xi * trig;
  const double vs = (double)vsig;
  const double vh = vs / h_a;
  const double alpha_loc = pp.alpha_max * Atrig / (pp.visc_delta * (vh * vh) + Atrig);
  double alpha;
  if(alpha_a <= alpha_loc)
    alpha = alpha_loc;
  else {
    const double decayt = h_a / (2.0 * pp.visc_l * vs);
    const double dalphadt = (alpha_a - alpha_loc) / decayt;
    alpha = alpha_a * exp(-dalphadt * tm->dt);
  }
  P.f[F_ALPHA][a] = alpha;
}

#define ALPHA_LAUNCH(DD, KK) \
  k_alpha_mixed<DD, KK><<<nb, MIX_THREADS, 0, L.stream>>>(P, pp, Ls, K, t)

void run_alpha_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  if(pp.dim == 3) {
    switch(pp.kernel) {
      case FSPH_KERNEL_CUBIC_SPLINE: ALPHA_LAUNCH(3, FSPH_KERNEL_CUBIC_SPLINE); break;
      case FSPH_KERNEL_QUINTIC_SPLINE: ALPHA_LAUNCH(3, FSPH_KERNEL_QUINTIC_SPLINE); break;
      case FSPH_KERNEL_GAUSSIAN: ALPHA_LAUNCH(3, FSPH_KERNEL_GAUSSIAN); break;
      case FSPH_KERNEL_SUPER_GAUSSIAN: ALPHA_LAUNCH(3, FSPH_KERNEL_SUPER_GAUSSIAN); break;
      case FSPH_KERNEL_SINC: ALPHA_LAUNCH(3, FSPH_KERNEL_SINC); break;
      case FSPH_KERNEL_WENDLAND_C2: ALPHA_LAUNCH(3, FSPH_KERNEL_WENDLAND_C2); break;
      case FSPH_KERNEL_WENDLAND_C4: ALPHA_LAUNCH(3, FSPH_KERNEL_WENDLAND_C4); break;
      default: ALPHA_LAUNCH(3, FSPH_KERNEL_WENDLAND_C6); break;
    }
  }
  else {
    switch(pp.kernel) {
      case FSPH_KERNEL_CUBIC_SPLINE: ALPHA_LAUNCH(2, FSPH_KERNEL_CUBIC_SPLINE); break;
      case FSPH_KERNEL_QUINTIC_SPLINE: ALPHA_LAUNCH(2, FSPH_KERNEL_QUINTIC_SPLINE); break;
      case FSPH_KERNEL_GAUSSIAN: ALPHA_LAUNCH(2, FSPH_KERNEL_GAUSSIAN); break;
      case FSPH_KERNEL_SUPER_GAUSSIAN: ALPHA_LAUNCH(2, FSPH_KERNEL_SUPER_GAUSSIAN); break;
      case FSPH_KERNEL_SINC: ALPHA_LAUNCH(2, FSPH_KERNEL_SINC); break;
      case FSPH_KERNEL_WENDLAND_C2: ALPHA_LAUNCH(2, FSPH_KERNEL_WENDLAND_C2); break;
      case FSPH_KERNEL_WENDLAND_C4: ALPHA_LAUNCH(2, FSPH_KERNEL_WENDLAND_C4); break;
      default: ALPHA_LAUNCH(2, FSPH_KERNEL_WENDLAND_C6); break;
    }
  }
  *L.counter += 1;
}
#undef ALPHA_LAUNCH

}  // namespace fsph
