// fsph_fp64.cu -- the plain-FP64 neighbour-pair kernels (density/EOS,
// signal speed, acceleration, du/dt, de/dt).
//
// One thread per particle walks its neighbour list (interleaved layout, so
// a warp reads 32 consecutive slots per step).  Compiled with -fmad=false and
// evaluated in the reference's operand order: with lists in the reference's
// order the results are bit-identical to the reference on the CPU except
// where libm and CUDA's pow/cbrt differ in the last bit.
#include <cuda_runtime.h>

#include "fsph_sphmath.cuh"

namespace fsph {

#define PAIR_THREADS 256

// compute_density + recover_internal_energy + eos (default_physics.h:193-228,
// 126-145, 309-316).  The new sound speed goes to cs_new: the signal speed
// pass still needs the old one (see k_vsig).
template<int D, int K>
__global__ void __launch_bounds__(PAIR_THREADS) k_density(Particles P,
  PhysParams pp, Lists Ls, double * cs_new, DevStatus * st, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double pa0 = X[a], pa1 = Y[a], pa2 = D == 3 ? Z[a] : 0.0;
  const double h_a = H[a];
  const int cnt = Ls.cnt[a];
  double rho_a = 0.0;
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    double r = 0;
    double d0 = pa0 - X[b];
    r += d0 * d0;
    double d1 = pa1 - Y[b];
    r += d1 * d1;
    if(D == 3) {
      double d2 = pa2 - Z[b];
      r += d2 * d2;
    }
    r = sqrt(r);
    double Wab = kfun<D, K>(r, .5 * (h_a + H[b]), pp);
    rho_a += M[b] * Wab;
  }
  if(!(rho_a > 0))
    raise_status(st, FSPH_ERR_NEG_DENSITY, a);
  P.f[F_RHO][a] = rho_a;
  double u = P.f[F_U][a];
  if(pp.evolve_u && pp.thermokinetic) {
    double vv = 0;
    for(int d = 0; d < D; ++d)
      vv += P.f[F_VX + d][a] * P.f[F_VX + d][a];
    double ekin = .5 * vv;
    const double pos_a[3] = {pa0, pa1, pa2};
    double eint = P.f[F_E][a] - ekin - ext_potential<D>(pp, pos_a);
    if(!(eint > 0))
      raise_status(st, FSPH_ERR_NEG_ENERGY, a);
    u = eint;
    P.f[F_U][a] = u;
  }
  double Pa, cs;
  eos_p_cs(pp, rho_a, u, P.f[F_K][a], P.f[F_YE][a], P.f[F_P][a], P.f[F_CS][a], Pa,
    cs);
  P.f[F_P][a] = Pa;
  cs_new[a] = cs;
  if(pp.cullen) {
    // compute_divv (default_physics.h:273-299), same traversal
    double va[3] = {P.f[F_VX][a], P.f[F_VY][a], D == 3 ? P.f[F_VZ][a] : 0.0};
    double pa[3] = {pa0, pa1, pa2};
    double div_v = 0.0;
    for(int j = 0; j < cnt; ++j) {
      const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
      double pos_ab[3] = {pa[0] - X[b], pa[1] - Y[b], D == 3 ? pa[2] - Z[b] : 0.0};
      const double h_ab = .5 * (h_a + H[b]);
      double DiWab[3];
      kgrad<D, K>(pos_ab, h_ab, DiWab, pp);
      double dot = 0.0;
      for(int d = 0; d < D; ++d)
        dot += va[d] * DiWab[d];
      div_v += M[b] * dot;
    }
    div_v /= rho_a;
    const double div_v_p = P.f[F_DIVV][a];
    P.f[F_DDIVVDT][a] = (div_v - div_v_p) / tm->dt;
    P.f[F_DIVV][a] = div_v;
  }
}

// viscosity::compute_alpha with A_trigger and compute_xi (viscosity.h:
// 185-363): Cullen & Dehnen's adaptive alpha from the velocity divergence,
// its rate and the traceless shear, in the reference's operand order.
template<int D, int K>
__global__ void __launch_bounds__(PAIR_THREADS) k_alpha_cullen(Particles P,
  PhysParams pp, Lists Ls, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double * CS = P.f[F_CS];
  const double * DV = P.f[F_DIVV];
  const double * V[3] = {P.f[F_VX], P.f[F_VY], P.f[F_VZ]};
  const double c_a = CS[a], h_a = H[a], alpha_a = P.f[F_ALPHA][a];
  const double rho_a = P.f[F_RHO][a];
  const double pa[3] = {X[a], Y[a], D == 3 ? Z[a] : 0.0};
  double va[3] = {0, 0, 0};
  for(int d = 0; d < D; ++d)
    va[d] = V[d][a];
  const int cnt = Ls.cnt[a];
  // signal speed of this pass: all sound speeds are the new ones here
  double vsig = 0.0;
  // compute_xi accumulations
  double R_a = 0.0;
  double gradV[D * D];
  for(int k = 0; k < D * D; ++k)
    gradV[k] = 0.0;
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    const double pb[3] = {X[b], Y[b], D == 3 ? Z[b] : 0.0};
    double pos_ab[3] = {0, 0, 0}, vab[3] = {0, 0, 0};
    double dist = 0.0;
    for(int d = 0; d < D; ++d) {
      pos_ab[d] = pa[d] - pb[d];
      vab[d] = va[d] - V[d][b];
      dist += pos_ab[d] * pos_ab[d];
    }
    dist = sqrt(dist);
    // vsig = max(vsig, max(c_a, c_b) - min(v_ab . n_ab, 0)); the self pair
    // (0/0) is a NaN that std::max drops
    double vn = 0.0;
    for(int d = 0; d < D; ++d)
      vn += vab[d] * (pos_ab[d] / dist);
    const double cmax = c_a < CS[b] ? CS[b] : c_a;
    const double mn = 0.0 < vn ? 0.0 : vn;   // std::min(vn, 0.0)
    const double cand = cmax - mn;
    vsig = vsig < cand ? cand : vsig;        // std::max(vsig, cand)
    const double h_ab = .5 * (h_a + H[b]);
    double DiWa[3];
    kgrad<D, K>(pos_ab, h_ab, DiWa, pp);
    const double Wab = kfun<D, K>(dist, h_ab, pp);
    const double dvb = DV[b];
    const double sgn = dvb > 0.0 ? 1.0 : (dvb < 0.0 ? -1.0 : dvb);
    R_a += sgn * M[b] * Wab;
    for(int i = 0; i < D; ++i)
      for(int k = 0; k < D; ++k)
        gradV[D * i + k] += M[b] * (-vab[i]) * DiWa[k];
  }
  R_a /= rho_a;
  for(int k = 0; k < D * D; ++k)
    gradV[k] /= rho_a;
  const double divV_a = DV[a];
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
  const double trig = -ddv < 0.0 ? 0.0 : -ddv;   // std::max(-dDivVdt, 0.0)
  const double Atrig = xi * trig;
  const double vh = vsig / h_a;
  const double alpha_loc = pp.alpha_max * Atrig / (pp.visc_delta * (vh * vh) + Atrig);
  double alpha;
  if(alpha_a <= alpha_loc)
    alpha = alpha_loc;
  else {
    const double decayt = h_a / (2.0 * pp.visc_l * vsig);
    const double dalphadt = (alpha_a - alpha_loc) / decayt;
    alpha = alpha_a * exp(-dalphadt * tm->dt);
  }
  P.f[F_ALPHA][a] = alpha;
}

// compute_signalspeed (default_physics.h:236-265).  The reference visits
// particles in descending key order and sets each particle's sound speed
// just before its signal speed (tree_topology.h:220-235,401-408;
// default_physics.h:309-317), so a neighbour with a higher sorted index
// (visited earlier) contributes its new sound speed, any other its old one.
template<int D>
__global__ void __launch_bounds__(PAIR_THREADS) k_vsig(Particles P, Lists Ls,
  const double * cs_new) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * VX = P.f[F_VX];
  const double * VY = P.f[F_VY];
  const double * VZ = P.f[F_VZ];
  const double * CS = P.f[F_CS];
  const double pa0 = X[a], pa1 = Y[a], pa2 = D == 3 ? Z[a] : 0.0;
  const double va0 = VX[a], va1 = VY[a], va2 = D == 3 ? VZ[a] : 0.0;
  const double c_a = cs_new[a];
  const int cnt = Ls.cnt[a];
  double vsig = 0.0;
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    double q0 = pa0 - X[b], q1 = pa1 - Y[b], q2 = D == 3 ? pa2 - Z[b] : 0.0;
    double dist = 0;
    dist += q0 * q0;
    dist += q1 * q1;
    if(D == 3)
      dist += q2 * q2;
    dist = sqrt(dist);
    double dotv = 0;
    dotv += (va0 - VX[b]) * (q0 / dist);
    dotv += (va1 - VY[b]) * (q1 / dist);
    if(D == 3)
      dotv += (va2 - VZ[b]) * (q2 / dist);
    const double c_b = b >= a ? cs_new[b] : CS[b];
    const double cab = c_a < c_b ? c_b : c_a;
    const double mn = 0.0 < dotv ? 0.0 : dotv;
    const double cand = cab - mn;
    vsig = vsig < cand ? cand : vsig;
  }
  P.f[F_VSIG][a] = vsig;
}

// compute_acceleration (default_physics.h:348-408); optionally followed by
// leapfrog_kick_v (integration.h:65-70) for the same particle: the pass
// reads only v_half of neighbours, never v.
template<int D, int K>
__global__ void __launch_bounds__(PAIR_THREADS) k_accel(Particles P,
  PhysParams pp, Lists Ls, int kick, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double * RHO = P.f[F_RHO];
  const double * PR = P.f[F_P];
  const double * CS = P.f[F_CS];
  const double * VH[3] = {P.f[F_VHX], P.f[F_VHY], P.f[F_VHZ]};
  const double h_a = H[a], rho_a = RHO[a], P_a = PR[a], c_a = CS[a];
  double pa[3] = {X[a], Y[a], D == 3 ? Z[a] : 0.0};
  double v12a[3];
  for(int d = 0; d < D; ++d)
    v12a[d] = VH[d][a];
  const double Prho2_a = P_a / (rho_a * rho_a);
  double acc[3] = {0, 0, 0};
  const int cnt = Ls.cnt[a];
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    double xb[3] = {X[b], Y[b], D == 3 ? Z[b] : 0.0};
    double pos_ab[3], v12_ab[3], DiWa[3];
    bool same = true;
    for(int d = 0; d < D; ++d) {
      same = same && (xb[d] == pa[d]);
      pos_ab[d] = pa[d] - xb[d];
      v12_ab[d] = v12a[d] - VH[d][b];
    }
    const double rho_b = RHO[b];
    const double m_b = M[b] * (!same);
    const double h_ab = .5 * (h_a + H[b]);
    const double mu_ab = visc_mu<D>(pp.eps, h_ab, v12_ab, pos_ab);
    const double rho_ab = .5 * (rho_a + rho_b);
    const double c_ab = .5 * (c_a + CS[b]);
    const double Pi = visc_pi_pp(pp, P.f[F_ALPHA], a, b, rho_ab, c_ab, mu_ab);
    kgrad<D, K>(pos_ab, h_ab, DiWa, pp);
    const double Prho2_b = PR[b] / (rho_b * rho_b);
    const double s = -m_b * (Prho2_a + Prho2_b + Pi);
    for(int d = 0; d < D; ++d)
      acc[d] += DiWa[d] * s;
  }
  // acc_a += external_force::acceleration(particle) (:404)
  double ext[3] = {0.0, 0.0, 0.0};
  if(pp.has_eacc)
    ext_acceleration<D>(pp, pa, ext);
  const double half_dt = kick ? 0.5 * tm->dt : 0.0;
  for(int d = 0; d < D; ++d) {
    const double ad = acc[d] + ext[d];
    P.f[F_AX + d][a] = ad;
    P.f[F_GAX + d][a] = 0.0;
    if(kick)
      P.f[F_VX + d][a] = P.f[F_VX + d][a] + (ad + 0.0) * half_dt;
  }
  P.f[F_GPOT][a] = 0.0;
}

// compute_dudt (default_physics.h:421-487)
template<int D, int K>
__global__ void __launch_bounds__(PAIR_THREADS) k_dudt(Particles P,
  PhysParams pp, Lists Ls, const DevTime * tm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  // no internal energy change while relaxing (:423-427)
  if(tm->iteration < pp.relax_steps) {
    P.f[F_DUDT][a] = 0.0;
    return;
  }
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double * RHO = P.f[F_RHO];
  const double * PR = P.f[F_P];
  const double * CS = P.f[F_CS];
  const double * V[3] = {P.f[F_VX], P.f[F_VY], P.f[F_VZ]};
  const double * VH[3] = {P.f[F_VHX], P.f[F_VHY], P.f[F_VHZ]};
  const double h_a = H[a], rho_a = RHO[a], P_a = PR[a], c_a = CS[a];
  double pa[3] = {X[a], Y[a], D == 3 ? Z[a] : 0.0};
  double va[3], v12a[3];
  for(int d = 0; d < D; ++d) {
    va[d] = V[d][a];
    v12a[d] = VH[d][a];
  }
  double dp = 0.0, dv = 0.0;
  const int cnt = Ls.cnt[a];
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    double xb[3] = {X[b], Y[b], D == 3 ? Z[b] : 0.0};
    double pos_ab[3], v12_ab[3], vel_ab[3], DiWab[3];
    bool same = true;
    for(int d = 0; d < D; ++d) {
      same = same && (xb[d] == pa[d]);
      pos_ab[d] = pa[d] - xb[d];
      v12_ab[d] = v12a[d] - VH[d][b];
      vel_ab[d] = va[d] - V[d][b];
    }
    const double m_b = M[b] * (!same);
    const double h_ab = .5 * (h_a + H[b]);
    const double mu_ab = visc_mu<D>(pp.eps, h_ab, v12_ab, pos_ab);
    const double rho_ab = .5 * (rho_a + RHO[b]);
    const double c_ab = .5 * (c_a + CS[b]);
    const double Pi = visc_pi_pp(pp, P.f[F_ALPHA], a, b, rho_ab, c_ab, mu_ab);
    kgrad<D, K>(pos_ab, h_ab, DiWab, pp);
    double vdw = 0;
    for(int d = 0; d < D; ++d)
      vdw += vel_ab[d] * DiWab[d];
    dp += m_b * vdw;
    dv += m_b * vdw * Pi;
  }
  P.f[F_DUDT][a] = P_a / (rho_a * rho_a) * dp + .5 * dv;
}

// compute_dedt (default_physics.h:502-566)
template<int D, int K>
__global__ void __launch_bounds__(PAIR_THREADS) k_dedt(Particles P,
  PhysParams pp, Lists Ls) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double * RHO = P.f[F_RHO];
  const double * PR = P.f[F_P];
  const double * CS = P.f[F_CS];
  const double * V[3] = {P.f[F_VX], P.f[F_VY], P.f[F_VZ]};
  const double * VH[3] = {P.f[F_VHX], P.f[F_VHY], P.f[F_VHZ]};
  const double h_a = H[a], rho_a = RHO[a], P_a = PR[a], c_a = CS[a];
  double pa[3] = {X[a], Y[a], D == 3 ? Z[a] : 0.0};
  double va[3], v12a[3];
  double gv = 0;
  for(int d = 0; d < D; ++d) {
    va[d] = V[d][a];
    v12a[d] = VH[d][a];
    gv += P.f[F_GAX + d][a] * va[d];
  }
  const double Prho2_a = P_a / (rho_a * rho_a);
  double dedt = 0;
  const int cnt = Ls.cnt[a];
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    double xb[3] = {X[b], Y[b], D == 3 ? Z[b] : 0.0};
    double pos_ab[3], v12_ab[3], DiWab[3], vb[3];
    bool same = true;
    for(int d = 0; d < D; ++d) {
      same = same && (xb[d] == pa[d]);
      pos_ab[d] = pa[d] - xb[d];
      v12_ab[d] = v12a[d] - VH[d][b];
      vb[d] = V[d][b];
    }
    const double rho_b = RHO[b];
    const double m_b = M[b] * (!same);
    const double h_ab = .5 * (h_a + H[b]);
    const double mu_ab = visc_mu<D>(pp.eps, h_ab, v12_ab, pos_ab);
    const double rho_ab = .5 * (rho_a + rho_b);
    const double c_ab = .5 * (c_a + CS[b]);
    const double Pi = visc_pi_pp(pp, P.f[F_ALPHA], a, b, rho_ab, c_ab, mu_ab);
    kgrad<D, K>(pos_ab, h_ab, DiWab, pp);
    double vad = 0, vbd = 0;
    for(int d = 0; d < D; ++d)
      vad += va[d] * DiWab[d];
    for(int d = 0; d < D; ++d)
      vbd += vb[d] * DiWab[d];
    const double Prho2_b = PR[b] / (rho_b * rho_b);
    dedt -= m_b * (Prho2_a * vbd + vad * Prho2_b + .5 * Pi * (vbd + vad));
  }
  dedt += gv;
  P.f[F_DEDT][a] = dedt;
}

// ------------------------------------------------------------ dispatch --
#define DISPATCH_DK(KERNEL_T, ...)                                             \
  do {                                                                         \
    const int nb_ = (P.n + PAIR_THREADS - 1) / PAIR_THREADS;                   \
    if(pp.dim == 3) {                                                          \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<3, FSPH_KERNEL_CUBIC_SPLINE><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<3, FSPH_KERNEL_QUINTIC_SPLINE><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<3, FSPH_KERNEL_GAUSSIAN><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<3, FSPH_KERNEL_SUPER_GAUSSIAN><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<3, FSPH_KERNEL_SINC><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C2><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C4><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<3, FSPH_KERNEL_WENDLAND_C6><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    else {                                                                     \
      switch(pp.kernel) {                                                      \
        case FSPH_KERNEL_CUBIC_SPLINE:                                         \
          KERNEL_T<2, FSPH_KERNEL_CUBIC_SPLINE><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_QUINTIC_SPLINE:                                       \
          KERNEL_T<2, FSPH_KERNEL_QUINTIC_SPLINE><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_GAUSSIAN:                                             \
          KERNEL_T<2, FSPH_KERNEL_GAUSSIAN><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SUPER_GAUSSIAN:                                       \
          KERNEL_T<2, FSPH_KERNEL_SUPER_GAUSSIAN><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_SINC:                                                 \
          KERNEL_T<2, FSPH_KERNEL_SINC><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C2:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C2><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        case FSPH_KERNEL_WENDLAND_C4:                                          \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C4><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
        default:                                                               \
          KERNEL_T<2, FSPH_KERNEL_WENDLAND_C6><<<nb_, PAIR_THREADS, 0, L.stream>>>(__VA_ARGS__); break; \
      }                                                                        \
    }                                                                          \
    *L.counter += 1;                                                           \
  } while(0)

cudaError_t launch_density_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, double * cs_new, DevStatus * st,
  const DevTime * t) {
  DISPATCH_DK(k_density, P, pp, Ls, cs_new, st, t);
  return cudaGetLastError();
}

cudaError_t launch_alpha_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const DevTime * t) {
  DISPATCH_DK(k_alpha_cullen, P, pp, Ls, t);
  return cudaGetLastError();
}

// add_short_range_repulsion (default_physics.h:723-753): neighbours other
// than the particle itself (by id) within relaxation_repulsion_radius of
// h_ab push it away with m_b x_ab / r_ab^3, scaled by
// relaxation_repulsion_gamma.  FP64 on both precision paths (it runs in
// relaxation iterations only).
template<int D>
__global__ void __launch_bounds__(PAIR_THREADS) k_repulsion(Particles P,
  PhysParams pp, Lists Ls) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a >= P.n)
    return;
  const double * H = P.f[F_H];
  const double * M = P.f[F_M];
  const double h_a = H[a];
  const long long id_a = P.id[a];
  double pa[3] = {0.0, 0.0, 0.0}, acc_r[3] = {0.0, 0.0, 0.0};
  for(int d = 0; d < D; ++d)
    pa[d] = P.f[F_X + d][a];
  const int cnt = Ls.cnt[a];
  for(int j = 0; j < cnt; ++j) {
    const int b = Ls.idx[list_slot(a, j, Ls.maxnb)];
    if(P.id[b] == id_a)
      continue;
    double dx[3] = {0.0, 0.0, 0.0};
    double r2 = 0.0;
    for(int d = 0; d < D; ++d) {
      dx[d] = pa[d] - P.f[F_X + d][b];
      r2 += dx[d] * dx[d];
    }
    const double h_ab = .5 * (h_a + H[b]);
    const double r_ab = sqrt(r2);
    if(r_ab > h_ab * pp.rep_radius)
      continue;
    const double m_b = M[b];
    const double r3 = r_ab * r_ab * r_ab;
    for(int d = 0; d < D; ++d)
      acc_r[d] += m_b * dx[d] / r3;
  }
  for(int d = 0; d < D; ++d)
    P.f[F_AX + d][a] = P.f[F_AX + d][a] + acc_r[d] * pp.rep_gamma;
}

cudaError_t launch_repulsion(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls) {
  const int nb = (P.n + PAIR_THREADS - 1) / PAIR_THREADS;
  if(pp.dim == 3)
    k_repulsion<3><<<nb, PAIR_THREADS, 0, L.stream>>>(P, pp, Ls);
  else
    k_repulsion<2><<<nb, PAIR_THREADS, 0, L.stream>>>(P, pp, Ls);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_vsig_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const double * cs_new) {
  const int nb = (P.n + PAIR_THREADS - 1) / PAIR_THREADS;
  if(pp.dim == 3)
    k_vsig<3><<<nb, PAIR_THREADS, 0, L.stream>>>(P, Ls, cs_new);
  else
    k_vsig<2><<<nb, PAIR_THREADS, 0, L.stream>>>(P, Ls, cs_new);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_accel_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, int kick, const DevTime * t) {
  DISPATCH_DK(k_accel, P, pp, Ls, kick, t);
  return cudaGetLastError();
}

cudaError_t launch_dudt_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const DevTime * t) {
  DISPATCH_DK(k_dudt, P, pp, Ls, t);
  return cudaGetLastError();
}

cudaError_t launch_dedt_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls) {
  DISPATCH_DK(k_dedt, P, pp, Ls);
  return cudaGetLastError();
}

}  // namespace fsph
