// fsph_mixed.cu -- the mixed-precision path: packing of the FP32 records,
// the signal-speed pass, and the launchers of the pair kernels of
// fsph_mixed_kernels.cuh (constant-alpha instances here, Cullen & Dehnen
// instances in fsph_mixed_cullen.cu).
#include <cuda_runtime.h>

#include "fsph_internal.cuh"
#include "fsph_mixed_kernels.cuh"

namespace fsph {

__device__ __forceinline__ double ord_dec_m(unsigned long long u) {
  return (u & 0x8000000000000000ull)
           ? __longlong_as_double((long long)(u & 0x7fffffffffffffffull))
           : __longlong_as_double((long long)~u);
}

// ------------------------------------------------------------- packing --
__global__ void k_pack_pos(Particles P, int dim,
  const unsigned long long * rbits, Packed K) {
  // Every position as one 48-bit fixed-point word per axis,
  //   F = round((x - lo) / E * 2^48),  E = the largest range extent
  //   enlarged by 2^-19 (so F < 2^48 - 2^28),
  // from which both packed forms follow by integer operations:
  //   float-float X = 1 + F / 2^48 in [1, 2): the high word takes F's top
  //     23 bits (exactly), the low word the other 25 (rounded to 24 bits);
  //   the walk's 31-bit fixed point q = F / 2^17 rounded to nearest, one
  //     step = E / 2^31 on every axis.
  // Three FP64 operations per axis (subtract, scale, convert): this kernel
  // runs on GB300's FP64 pipe, where divisions and splits cost most.
  __shared__ double s_lo[3], s_sc, s_iE;
  if(threadIdx.x < dim)
    s_lo[threadIdx.x] = ord_dec_m(rbits[threadIdx.x]);
  if(threadIdx.x == 0) {
    double E = 0.0;
    for(int d = 0; d < dim; ++d)
      E = fmax(E, ord_dec_m(rbits[3 + d]) - ord_dec_m(rbits[d]));
    E *= 1.0 + 0x1p-19;
    s_iE = 1.0 / E;
    s_sc = s_iE * 0x1p48;
    if(blockIdx.x == 0) {
      K.fscale[0] = E;
      K.fscale[1] = s_iE;
      // h_min == h_max: the pair passes take h_ab = h_a throughout
      K.fscale[2] = rbits[6] == rbits[7] ? 1.0 : 0.0;
      for(int d = 0; d < 3; ++d)
        K.qscale[d] = d < dim ? (float)(E * 0x1p-31) : 0.f;
    }
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  const long long fmax48 = (1LL << 48) - (1LL << 28);
  int q[3] = {0, 0, 0};
  float xh[4] = {1.f, 1.f, 1.f, 0.f}, xl[4] = {0.f, 0.f, 0.f, 0.f};
  for(int d = 0; d < dim; ++d) {
    long long F = __double2ll_rn((P.f[F_X + d][i] - s_lo[d]) * s_sc);
    F = F < 0 ? 0 : F > fmax48 ? fmax48 : F;
    q[d] = (int)((F + (1LL << 16)) >> 17);
    xh[d] = __int_as_float(0x3f800000 | (int)(F >> 25));
    xl[d] = (float)(int)(F & ((1LL << 25) - 1)) * 0x1p-48f;
  }
  const double h = P.f[F_H][i];
  const double hX = h * s_iE;
  xh[3] = (float)hX;
  xl[3] = (float)(hX - (double)xh[3]);
  K.qpos[i] = make_int4(q[0], q[1], q[2], __float_as_int((float)h));
  K.fph[i] = make_float4(xh[0], xh[1], xh[2], xh[3]);
  K.fpl[i] = make_float4(xl[0], xl[1], xl[2], xl[3]);
  const double m = P.f[F_M][i];
  const float mh = (float)m;
  ((float2 *)K.fmA)[2 * i] = make_float2(mh, (float)(m - (double)mh));
}

// PACK_VHM: {v_half, m} and m alone (the FP32 passes, the alpha pass);
// PACK_VEL: {v, c_s before the density pass} (the signal speed);
// PACK_AV_IN: {c_s, sign(div v)} for the Cullen & Dehnen alpha pass;
// PACK_AV: {alpha, 0} for the pair passes that weight the viscosity by it;
// PACK_DEDT: the FP32 de/dt pass's {v, P/rho^2} and {rho, c_s} records;
// PACK_FV: v_half's high and low words with rho and c_s (the float-float
// acceleration pass, the energy passes); PACK_FDV: {v - v_half, m} (the
// energy passes); PACK_VEL_V: v alone into the PACK_VEL record, its c_s
// slot left as the density pass found it (the alpha pass, between the
// density pass and the acceleration pass that reads that slot).  Each pass
// packs only what its kernels read.
enum { PACK_VHM = 1, PACK_VEL = 2, PACK_THERMO = 4, PACK_AV_IN = 8, PACK_AV = 16,
       PACK_DEDT = 32, PACK_FV = 64, PACK_FDV = 128, PACK_VEL_V = 256 };

// Refresh the packed records a pass reads from the FP64 state, so every
// pass sees the current v_half, v, rho, P and c_s whatever the caller did
// in between (separate kicks, repeated pressure updates).
__global__ void k_pack_state(Particles P, int dim, Packed K, int what) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  // FP32 high word and low word of an FP64 velocity component
  auto hl = [&](int f, float & h, float & l) {
    const double v = P.f[f][i];
    h = (float)v;
    l = (float)(v - (double)h);
  };
  if(what & (PACK_VHM | PACK_FV)) {
    float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
    for(int d = 0; d < dim; ++d)
      hl(F_VHX + d, h[d], l[d]);
    if(what & PACK_VHM) {
      const float m = (float)P.f[F_M][i];
      K.vhm[i] = make_float4(h[0], h[1], h[2], m);
      K.mass[i] = m;
    }
    if(what & PACK_FV) {
      // rho and c_s as the state holds them: after the density pass, the
      // new c_s
      K.fv1[i] = make_float4(h[0], h[1], h[2], (float)P.f[F_RHO][i]);
      K.fv2[i] = make_float4(l[0], l[1], l[2], (float)P.f[F_CS][i]);
    }
  }
  if(what & PACK_VEL)
    K.vel[i] = make_float4((float)P.f[F_VX][i], (float)P.f[F_VY][i],
      dim == 3 ? (float)P.f[F_VZ][i] : 0.f, (float)P.f[F_CS][i]);
  if(what & PACK_VEL_V) {
    float * v = (float *)&K.vel[i];
    v[0] = (float)P.f[F_VX][i];
    v[1] = (float)P.f[F_VY][i];
    v[2] = dim == 3 ? (float)P.f[F_VZ][i] : 0.f;
  }
  if(what & PACK_THERMO) {
    const double rho = P.f[F_RHO][i], cs = P.f[F_CS][i];
    const double A = P.f[F_P][i] / (rho * rho);
    K.thermo[i] = make_float4((float)rho, (float)A, (float)cs, (float)cs);
    const float Ah = (float)A;
    ((float2 *)K.fmA)[2 * i + 1] = make_float2(Ah, (float)(A - (double)Ah));
  }
  if(what & PACK_AV_IN) {
    // signnum_c of the reference (viscosity.h:63-67), taken in FP64
    const double dv = P.f[F_DIVV][i];
    const float sgn = dv > 0.0 ? 1.f : (dv < 0.0 ? -1.f : (float)dv);
    K.visc[i] = make_float2((float)P.f[F_CS][i], sgn);
  }
  if(what & PACK_AV)
    K.visc[i] = make_float2((float)P.f[F_ALPHA][i], 0.f);
  if(what & PACK_DEDT) {
    const double rho = P.f[F_RHO][i];
    K.velp[i] = make_float4((float)P.f[F_VX][i], (float)P.f[F_VY][i],
      dim == 3 ? (float)P.f[F_VZ][i] : 0.f, (float)(P.f[F_P][i] / (rho * rho)));
    K.rc[i] = make_float2((float)rho, (float)P.f[F_CS][i]);
  }
  if(what & PACK_FDV) {
    float dv[3] = {0.f, 0.f, 0.f};
    for(int d = 0; d < dim; ++d)
      dv[d] = (float)(P.f[F_VX + d][i] - P.f[F_VHX + d][i]);
    K.fdv[i] = make_float4(dv[0], dv[1], dv[2], (float)P.f[F_M][i]);
  }
}

cudaError_t launch_pack_positions(const Launch & L, const Particles & P,
  const PhysParams & pp, const unsigned long long * rbits, const Packed & K) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  k_pack_pos<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, rbits, K);
  *L.counter += 1;
  return cudaGetLastError();
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

cudaError_t launch_density_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st, const DevTime * tm, int vel_current) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // velocities of this step for the signal speed (unless the permute of
  // update_iteration wrote them); masses for the FP32 density pass (the
  // float-float one reads them from the position packing)
  const int what = wendland_kernel(pp.kernel) ? (vel_current ? 0 : PACK_VEL)
                                              : PACK_VHM | PACK_VEL;
  if(what) {
    k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K, what);
    *L.counter += 1;
  }
  if(pp.cullen)
    run_density_mixed_cullen(L, P, pp, Ls, K, cs_new, st, tm);
  else
    run_density_mixed<false>(L, P, pp, Ls, K, cs_new, st, tm);
  return cudaGetLastError();
}

cudaError_t launch_alpha_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // current velocities and masses; sound speeds and div v signs of the
  // neighbours
  k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K,
    PACK_VHM | PACK_VEL_V | PACK_AV_IN);
  *L.counter += 1;
  run_alpha_mixed(L, P, pp, Ls, K, t);
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
  const DevTime * t, int fused_vsig, int fv_current) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // v_half of this step (set by the caller's save_velocityhalf); the thermo
  // records are refreshed unless they come straight from the density pass
  // (fused signal speed needs their previous-sound-speed slot)
  const int av = pp.cullen ? PACK_AV : 0;
  const int vh = wendland_kernel(pp.kernel) ? (fv_current ? 0 : PACK_FV) : PACK_VHM;
  const int what = (fused_vsig ? vh : (vh | PACK_THERMO)) | av;
  if(what) {
    k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K, what);
    *L.counter += 1;
  }
  if(pp.cullen)
    run_accel_mixed_cullen(L, P, pp, Ls, K, kick, t, fused_vsig);
  else
    run_accel_mixed<false>(L, P, pp, Ls, K, kick, t, fused_vsig);
  return cudaGetLastError();
}

cudaError_t launch_dudt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t,
  int then_op, int fv_current, int fdv_current) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  const int what = (fv_current ? 0 : PACK_FV) | (fdv_current ? 0 : PACK_FDV) |
                   (pp.cullen ? PACK_AV : 0);
  if(what) {
    k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K, what);
    *L.counter += 1;
  }
  if(pp.cullen)
    run_dudt_mixed_cullen(L, P, pp, Ls, K, t, then_op);
  else
    run_dudt_mixed<false>(L, P, pp, Ls, K, t, then_op);
  return cudaGetLastError();
}

cudaError_t launch_dedt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int then_op,
  const DevTime * t, DevStatus * st, int use_ahyd, int fdv_current) {
  const int nb = (P.n + MIX_THREADS - 1) / MIX_THREADS;
  // through a^P, v_half, rho and c_s are those the acceleration pass packed
  // (the caller's flag says so): only v - v_half is new, and not even that
  // when the acceleration pass's kick wrote it
  const int what = (use_ahyd && wendland_kernel(pp.kernel)
                      ? (fdv_current ? 0 : PACK_FDV) : PACK_VHM | PACK_DEDT) |
                   (pp.cullen ? PACK_AV : 0);
  if(what) {
    k_pack_state<<<nb, MIX_THREADS, 0, L.stream>>>(P, pp.dim, K, what);
    *L.counter += 1;
  }
  if(pp.cullen)
    run_dedt_mixed_cullen(L, P, pp, Ls, K, then_op, t, st, use_ahyd);
  else
    run_dedt_mixed<false>(L, P, pp, Ls, K, then_op, t, st, use_ahyd);
  return cudaGetLastError();
}

}  // namespace fsph
