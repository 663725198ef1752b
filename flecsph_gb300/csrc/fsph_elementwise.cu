// fsph_elementwise.cu -- per-particle (apply_all / get_all) kernels, the
// timestep reduction and the scalar time bookkeeping, all FP64 and
// compiled with -fmad=false so they round like the reference.
#include <cuda_runtime.h>

#include "fsph_sphmath.cuh"

namespace fsph {

#define ELEM_THREADS 256

__device__ __forceinline__ unsigned long long ord_enc_e(double x) {
  long long b = __double_as_longlong(x);
  return b < 0 ? ~(unsigned long long)b
               : ((unsigned long long)b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dec_e(unsigned long long u) {
  return (u & 0x8000000000000000ull)
           ? __longlong_as_double((long long)(u & 0x7fffffffffffffffull))
           : __longlong_as_double((long long)~u);
}
__device__ __forceinline__ double dmin_(double a, double b) { return b < a ? b : a; }

// recover_internal_energy (default_physics.h:126-145)
template<int D>
__device__ __forceinline__ double recover_u(const Particles & P,
  const PhysParams & pp, int i, DevStatus * st) {
  double vv = 0;
  for(int d = 0; d < D; ++d)
    vv += P.f[F_VX + d][i] * P.f[F_VX + d][i];
  double ekin = .5 * vv;
  double eint = P.f[F_E][i] - ekin - ext_potential_of<D>(pp, P.f, i);
  if(!(eint > 0))
    raise_status(st, FSPH_ERR_NEG_ENERGY, i);
  return eint;
}

template<int D>
__global__ void __launch_bounds__(ELEM_THREADS) k_elem(Particles P,
  PhysParams pp, int op, const DevTime * tm, DevStatus * st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  double ** f = P.f;
  const double dt = tm->dt;
  switch(op) {
    case OP_EOS_INIT:  // eos_t<>::init (eos.h:67-92, 157-159, 240-243, 345-364)
      if(pp.eos == FSPH_EOS_WD)
        f[F_U][i] = wd_internal_energy(f[F_RHO][i], f[F_YE][i]);
      else if(pp.eos == FSPH_EOS_PPT) {
        const double rho = f[F_RHO][i], P_ = f[F_P][i], thr = pp.rho_thr;
        double K1 = 0.0;
        if(rho < thr)
          K1 = P_ / pow(rho, pp.gamma);
        else {
          double K2 = P_ / pow(rho, pp.gamma2);
          K1 = K2 * pow(thr, pp.gamma2 - pp.gamma);
        }
        f[F_K][i] = K1;
      }
      else if(pp.eos != FSPH_EOS_NO_EOS)
        f[F_K][i] = f[F_P][i] / pow(f[F_RHO][i], pp.gamma);
      break;
    case OP_SET_TOTAL_ENERGY: {  // default_physics.h:327-335
      double vv = 0;
      for(int d = 0; d < D; ++d)
        vv += f[F_VX + d][i] * f[F_VX + d][i];
      double ekin = .5 * vv;
      f[F_E][i] = ekin + f[F_U][i] + ext_potential_of<D>(pp, f, i);
      break;
    }
    case OP_SAVE_VHALF:  // integration.h:52-55
      for(int d = 0; d < D; ++d)
        f[F_VHX + d][i] = f[F_VX + d][i];
      break;
    case OP_KICK_V: {  // integration.h:65-70
      const double s = 0.5 * dt;
      for(int d = 0; d < D; ++d)
        f[F_VX + d][i] = f[F_VX + d][i] + (f[F_AX + d][i] + f[F_GAX + d][i]) * s;
      break;
    }
    case OP_KICK_U:  // integration.h:80-84
      f[F_U][i] = f[F_U][i] + 0.5 * dt * f[F_DUDT][i];
      break;
    case OP_KICK_E:  // integration.h:94-98
      f[F_E][i] = f[F_E][i] + 0.5 * dt * f[F_DEDT][i];
      break;
    case OP_DRIFT:  // integration.h:106-110
      for(int d = 0; d < D; ++d)
        f[F_X + d][i] = f[F_X + d][i] + f[F_VX + d][i] * dt;
      break;
    case OP_KICK_DRIFT_E:
    case OP_KICK_DRIFT_U:
    case OP_KICK_DRIFT_NONE: {
      // the start of a leapfrog step, hydro/main_driver.cc:176-188:
      // kick e (or u), kick v, save v_half, drift
      if(op == OP_KICK_DRIFT_E)
        f[F_E][i] = f[F_E][i] + 0.5 * dt * f[F_DEDT][i];
      else if(op == OP_KICK_DRIFT_U)
        f[F_U][i] = f[F_U][i] + 0.5 * dt * f[F_DUDT][i];
      const double s = 0.5 * dt;
      for(int d = 0; d < D; ++d) {
        double v = f[F_VX + d][i] + (f[F_AX + d][i] + f[F_GAX + d][i]) * s;
        f[F_VX + d][i] = v;
        f[F_VHX + d][i] = v;
        f[F_X + d][i] = f[F_X + d][i] + v * dt;
      }
      break;
    }
    case OP_RECOMPUTE:
    case OP_RECOMPUTE_KICK_U: {  // default_physics.h:153-161 (+ kick_u)
      double uint = f[F_U][i];
      double P_, cs;
      eos_p_cs(pp, f[F_RHO][i], uint + 0.5 * dt * f[F_DUDT][i], f[F_K][i],
        f[F_YE][i], f[F_P][i], f[F_CS][i], P_, cs);
      f[F_P][i] = P_;
      f[F_CS][i] = cs;
      if(op == OP_RECOMPUTE_KICK_U)
        f[F_U][i] = uint + 0.5 * dt * f[F_DUDT][i];
      break;
    }
    case OP_RECOMPUTE_THERMO:
    case OP_RECOMPUTE_KICK_E: {  // default_physics.h:169-182 (+ kick_e)
      double eint = recover_u<D>(P, pp, i, st);
      f[F_U][i] = eint;
      double vda = 0;
      for(int d = 0; d < D; ++d)
        vda += f[F_VX + d][i] * f[F_AX + d][i];
      double P_, cs;
      eos_p_cs(pp, f[F_RHO][i], eint + 0.5 * dt * (f[F_DEDT][i] - vda),
        f[F_K][i], f[F_YE][i], f[F_P][i], f[F_CS][i], P_, cs);
      f[F_P][i] = P_;
      f[F_CS][i] = cs;
      if(op == OP_RECOMPUTE_KICK_E)
        f[F_E][i] = f[F_E][i] + 0.5 * dt * f[F_DEDT][i];
      break;
    }
    case OP_SMOOTHING_LENGTH: {  // default_physics.h:825-848
      double q = f[F_M][i] / f[F_RHO][i];
      double r = D == 3 ? cbrt(q) : sqrt(q);
      f[F_H][i] = r * pp.eta * pp.kw;
      break;
    }
    case OP_INIT_ALPHA:  // viscosity::initialize_alpha (viscosity.h:171-177)
      f[F_ALPHA][i] = pp.cullen ? 0.0 : pp.alpha;
      break;
    case OP_DRAG_ACC:    // add_drag_acceleration (default_physics.h:699-708)
    case OP_DRAG_DEDT:   // add_drag_dedt (:571-579)
    case OP_DRAG_DUDT: { // add_drag_dudt (:586-594)
      double vel[3] = {0.0, 0.0, 0.0}, drag[3];
      for(int d = 0; d < D; ++d)
        vel[d] = f[F_VX + d][i];
      drag_acceleration<D>(pp, vel, drag);
      if(op == OP_DRAG_ACC) {
        for(int d = 0; d < D; ++d)
          f[F_AX + d][i] = f[F_AX + d][i] + drag[d];
      }
      else {
        double v_dot_a = 0.0;
        for(int d = 0; d < D; ++d)
          v_dot_a += vel[d] * drag[d];
        const int F = op == OP_DRAG_DEDT ? F_DEDT : F_DUDT;
        f[F][i] = f[F][i] + v_dot_a;
      }
      break;
    }
    case OP_SET_H:  // second half of compute_average_smoothinglength
      f[F_H][i] = 1. / (double)P.n * tm->hsum;
      break;
    case OP_CHECK_NANS: {  // default_physics.h:918-945
      bool bad = false;
      for(int d = 0; d < D; ++d) {
        double q[5] = {f[F_X + d][i], f[F_VX + d][i], f[F_VHX + d][i],
          f[F_AX + d][i], f[F_GAX + d][i]};
        for(int k = 0; k < 5; ++k)
          bad |= q[k] != q[k];
      }
      const int sc[] = {F_M, F_GPOT, F_RHO, F_P, F_E, F_DEDT, F_DUDT, F_K, F_VSIG};
      for(int k = 0; k < 9; ++k)
        bad |= f[sc[k]][i] != f[sc[k]][i];
      if(pp.evolve_u)
        bad |= f[F_U][i] != f[F_U][i];
      if(bad)
        raise_status(st, FSPH_ERR_NAN, i);
      break;
    }
    case OP_CHECK_NEGATIVITY:  // default_physics.h:953-979
      if(f[F_RHO][i] < 0 || f[F_P][i] < 0 || (pp.evolve_u && f[F_U][i] < 0))
        raise_status(st, FSPH_ERR_NEGATIVITY, i);
      break;
  }
}

cudaError_t launch_elementwise(const Launch & L, const Particles & P,
  const PhysParams & pp, int op, DevTime * t, DevStatus * st) {
  const int nb = (P.n + ELEM_THREADS - 1) / ELEM_THREADS;
  if(pp.dim == 3)
    k_elem<3><<<nb, ELEM_THREADS, 0, L.stream>>>(P, pp, op, t, st);
  else
    k_elem<2><<<nb, ELEM_THREADS, 0, L.stream>>>(P, pp, op, t, st);
  *L.counter += 1;
  return cudaGetLastError();
}

// compute_dt (default_physics.h:602-695) per particle, then the minimum.
__global__ void k_dt_init(DevTime * t) { t->dtmin_bits = ord_enc_e(1e24); }

// NaN / negativity from the bit pattern: integer instructions instead of
// FP64 compares, which run on this part's narrow FP64 pipe.
__device__ __forceinline__ bool bits_nan(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) >
         0x7ff0000000000000ull;
}
__device__ __forceinline__ bool bits_negative(double x) {  // x < 0, not -0, not NaN
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) && (b & 0x7fffffffffffffffull) != 0 &&
         (b & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull;
}

// CHECKS folds check_nans and check_negativity (default_physics.h:918-979)
// into the same pass, as the driver runs them back to back before dt.
// F32 evaluates the per-particle estimate of compute_dt in single precision
// (mixed-precision runs); the global minimum and the adaptive rule stay FP64.
template<int D, bool CHECKS, bool F32>
__global__ void __launch_bounds__(ELEM_THREADS) k_compute_dt(Particles P,
  PhysParams pp, DevTime * tm, DevStatus * st) {
  // grid-stride: one atomic per block of a grid sized to the machine
  double dtmin = 1e24;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
      i += gridDim.x * blockDim.x) {
    double ** f = P.f;
    double dtp = 1e24;
    if(CHECKS) {
      bool bad = false;
      for(int d = 0; d < D; ++d)
        bad |= bits_nan(f[F_X + d][i]) | bits_nan(f[F_VX + d][i]) |
               bits_nan(f[F_VHX + d][i]) | bits_nan(f[F_AX + d][i]) |
               bits_nan(f[F_GAX + d][i]);
      const int sc[] = {F_M, F_GPOT, F_RHO, F_P, F_E, F_DEDT, F_DUDT, F_K, F_VSIG};
      for(int k = 0; k < 9; ++k)
        bad |= bits_nan(f[sc[k]][i]);
      if(pp.evolve_u)
        bad |= bits_nan(f[F_U][i]);
      if(bad)
        raise_status(st, FSPH_ERR_NAN, i);
      if(bits_negative(f[F_RHO][i]) || bits_negative(f[F_P][i]) ||
         (pp.evolve_u && bits_negative(f[F_U][i])))
        raise_status(st, FSPH_ERR_NEGATIVITY, i);
    }
    if(F32) {
      const float tiny = 1e-24f;
      const float dx = (float)f[F_H][i] / (float)(pp.eta * pp.kw);
      float vn = 0.f, acc = 0.f;
      for(int d = 0; d < D; ++d) {
        const float v = (float)f[F_VX + d][i];
        const float a = (float)(f[F_AX + d][i] + f[F_GAX + d][i]);
        vn += v * v;
        acc += a * a;
      }
      const float dt_v = dx / (sqrtf(vn) + tiny);
      const float dt_a = sqrtf(dx / (sqrtf(acc) + tiny));
      const float dt_c = dx / (tiny + (float)f[F_VSIG][i] * (1.f + 0.6f * (float)pp.alpha));
      dtp = (double)((float)pp.cfl * fminf(fminf(dt_v, dt_a), dt_c));
    }
    else {
      const double tiny = 1e-24, mc = 0.6;
      const double dx = f[F_H][i] / (pp.eta * pp.kw);
      double vn = 0;
      for(int d = 0; d < D; ++d)
        vn += f[F_VX + d][i] * f[F_VX + d][i];
      vn = sqrt(vn);
      const double dt_v = dx / (vn + tiny);
      double acc = 0;
      for(int d = 0; d < D; ++d) {
        double ad = f[F_AX + d][i] + f[F_GAX + d][i];
        acc += ad * ad;
      }
      acc = sqrt(acc);
      const double dt_a = sqrt(dx / (acc + tiny));
      const double dt_c = dx / (tiny + f[F_VSIG][i] * (1 + mc * pp.alpha));
      dtp = pp.cfl * dmin_(dmin_(dt_v, dt_a), dt_c);
    }
    if(pp.evolve_u && pp.thermokinetic) {
      const double eint = f[F_U][i];
      if(!(eint > 0))
        raise_status(st, FSPH_ERR_NEG_ENERGY, i);
      double gdv = 0;
      for(int d = 0; d < D; ++d)
        gdv += f[F_VX + d][i] * f[F_GAX + d][i];
      // with no external potential and v . g = 0, the first test passes
      if(gdv != 0.0 || pp.n_eforce > 0) {
        const double pos[3] = {f[F_X][i], f[F_Y][i], D == 3 ? f[F_Z][i] : 0.0};
        const double epot = ext_potential<D>(pp, pos);
        int it;
        for(it = 0; it < 20; ++it) {
          double p1[3] = {0.0, 0.0, 0.0};
          for(int d = 0; d < D; ++d)
            p1[d] = pos[d] + dtp * f[F_VX + d][i];
          double delta_epot = ext_potential<D>(pp, p1) - epot;
          double delta_egrv = -dtp * gdv;
          if(delta_epot + delta_egrv < eint * 0.5)
            break;
          dtp *= 0.25;
        }
        if(it >= 20)
          raise_status(st, FSPH_ERR_DT, i);
      }
    }
    f[F_DT][i] = dtp;
    dtmin = dmin_(dtmin, dtp);
  }
  // block minimum first, then one atomic per block
  __shared__ double wmin[ELEM_THREADS / 32];
  for(int o = 16; o; o >>= 1)
    dtmin = dmin_(dtmin, __shfl_xor_sync(0xffffffffu, dtmin, o));
  if((threadIdx.x & 31) == 0)
    wmin[threadIdx.x >> 5] = dtmin;
  __syncthreads();
  if(threadIdx.x == 0) {
    double m = wmin[0];
    for(int k = 1; k < ELEM_THREADS / 32; ++k)
      m = dmin_(m, wmin[k]);
    atomicMin(&tm->dtmin_bits, ord_enc_e(m));
  }
}

cudaError_t launch_compute_dt(const Launch & L, const Particles & P,
  const PhysParams & pp, DevTime * t, DevStatus * st, int with_checks,
  int f32) {
  k_dt_init<<<1, 1, 0, L.stream>>>(t);
  // a few blocks per SM: the per-block minima meet in one atomic each
  int nb = (P.n + ELEM_THREADS - 1) / ELEM_THREADS;
  if(nb > 152 * 8)
    nb = 152 * 8;
#define DT_LAUNCH(D, C, F) \
  k_compute_dt<D, C, F><<<nb, ELEM_THREADS, 0, L.stream>>>(P, pp, t, st)
  if(pp.dim == 3) {
    if(with_checks) { if(f32) DT_LAUNCH(3, true, true); else DT_LAUNCH(3, true, false); }
    else { if(f32) DT_LAUNCH(3, false, true); else DT_LAUNCH(3, false, false); }
  }
  else {
    if(with_checks) { if(f32) DT_LAUNCH(2, true, true); else DT_LAUNCH(2, true, false); }
    else { if(f32) DT_LAUNCH(2, false, true); else DT_LAUNCH(2, false, false); }
  }
#undef DT_LAUNCH
  *L.counter += 2;
  return cudaGetLastError();
}

// set_adaptive_timestep (default_physics.h:761-823), one thread.
__global__ void k_set_adaptive(PhysParams pp, DevTime * t) {
  double dtmin = ord_dec_e(t->dtmin_bits);
  double dt = t->dt;
  if(dtmin < dt)
    dt = dmin_(dtmin, dt / 2.0);
  if(dtmin > 2.0 * dt)
    dt = dt * 2.0;
  double tt = t->totaltime;
  double next = tt + dt;
  if(pp.out_screen_dt > 0) {
    if(tt == t->t_screen) {
      if(t->dt_saved > 0) dt = t->dt_saved;
      t->t_screen += pp.out_screen_dt;
    }
    if(tt + dt > t->t_screen - 0.1 * pp.out_screen_dt) {
      t->dt_saved = dt;
      next = t->t_screen;
    }
  }
  if(pp.out_scalar_dt > 0) {
    if(tt == t->t_scalar) {
      if(t->dt_saved > 0) dt = t->dt_saved;
      t->t_scalar += pp.out_scalar_dt;
    }
    if(tt + dt > t->t_scalar - 0.1 * pp.out_scalar_dt) {
      t->dt_saved = dt;
      next = dmin_(next, t->t_scalar);
    }
  }
  if(pp.out_h5data_dt > 0) {
    if(tt == t->t_h5) {
      if(t->dt_saved > 0) dt = t->dt_saved;
      t->t_h5 += pp.out_h5data_dt;
    }
    if(tt + dt > t->t_h5 - 0.1 * pp.out_h5data_dt) {
      t->dt_saved = dt;
      next = dmin_(next, t->t_h5);
    }
  }
  t->totaltime_next = next;
  t->dt = next - tt;
}

cudaError_t launch_set_adaptive_timestep(const Launch & L,
  const PhysParams & pp, DevTime * t) {
  k_set_adaptive<<<1, 1, 0, L.stream>>>(pp, t);
  *L.counter += 1;
  return cudaGetLastError();
}

// advance_time (default_physics.h:853-860)
__global__ void k_advance(PhysParams pp, DevTime * t) {
  t->iteration++;
  if(pp.adaptive)
    t->totaltime = t->totaltime_next;
  else
    t->totaltime = t->totaltime + t->dt;
}

cudaError_t launch_advance_time(const Launch & L, const PhysParams & pp,
  DevTime * t) {
  k_advance<<<1, 1, 0, L.stream>>>(pp, t);
  *L.counter += 1;
  return cudaGetLastError();
}

// Deterministic sum of h (fixed two-level order) for the averaged h.
__global__ void __launch_bounds__(1024) k_hsum(Particles P, DevTime * t) {
  __shared__ double part[1024];
  double s = 0;
  for(int i = threadIdx.x; i < P.n; i += 1024)
    s += P.f[F_H][i];
  part[threadIdx.x] = s;
  __syncthreads();
  for(int o = 512; o; o >>= 1) {
    if(threadIdx.x < o)
      part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0)
    t->hsum = part[0];
}

cudaError_t launch_hsum(const Launch & L, const Particles & P, DevTime * t) {
  k_hsum<<<1, 1024, 0, L.stream>>>(P, t);
  *L.counter += 1;
  return cudaGetLastError();
}

// Conserved totals (analysis.h:56-214): mass, energy, momentum (3),
// angular momentum (3).  Two passes in a fixed order (deterministic):
// CONS_BLOCKS block partials, then one block adds them up.
__global__ void __launch_bounds__(256) k_conserved_part(Particles P,
  PhysParams pp, double * part_out, long long nreal) {
  __shared__ double part[8][256];
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int D = pp.dim;
  for(int i = blockIdx.x * 256 + threadIdx.x; i < P.n; i += gridDim.x * 256) {
    if(P.id[i] >= nreal)  // periodic copies (WALL) are not counted
      continue;
    double m = P.f[F_M][i];
    double x[3] = {P.f[F_X][i], P.f[F_Y][i], D == 3 ? P.f[F_Z][i] : 0.0};
    double v[3] = {P.f[F_VX][i], P.f[F_VY][i], D == 3 ? P.f[F_VZ][i] : 0.0};
    s[0] += m;
    if(pp.thermokinetic)
      s[1] += m * P.f[F_E][i];
    else {
      const double epot = D == 3 ? ext_potential<3>(pp, x) : ext_potential<2>(pp, x);
      s[1] += m * (.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + P.f[F_U][i] + epot);
    }
    s[1] += .5 * m * P.f[F_GPOT][i];
    for(int d = 0; d < 3; ++d)
      s[2 + d] += m * v[d];
    s[5] += m * (x[1] * v[2] - x[2] * v[1]);
    s[6] += m * (x[2] * v[0] - x[0] * v[2]);
    s[7] += m * (x[0] * v[1] - x[1] * v[0]);
  }
  for(int k = 0; k < 8; ++k)
    part[k][threadIdx.x] = s[k];
  __syncthreads();
  for(int o = 128; o; o >>= 1) {
    if(threadIdx.x < o)
      for(int k = 0; k < 8; ++k)
        part[k][threadIdx.x] += part[k][threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x < 8)
    part_out[8 + 8 * blockIdx.x + threadIdx.x] = part[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) k_conserved_final(double * buf, int nb) {
  __shared__ double part[8][256];
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for(int b = threadIdx.x; b < nb; b += 256)
    for(int k = 0; k < 8; ++k)
      s[k] += buf[8 + 8 * b + k];
  for(int k = 0; k < 8; ++k)
    part[k][threadIdx.x] = s[k];
  __syncthreads();
  for(int o = 128; o; o >>= 1) {
    if(threadIdx.x < o)
      for(int k = 0; k < 8; ++k)
        part[k][threadIdx.x] += part[k][threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x < 8)
    buf[threadIdx.x] = part[threadIdx.x][0];
}

cudaError_t launch_conserved(const Launch & L, const Particles & P,
  const PhysParams & pp, double * out8, long long nreal) {
  // out8 holds 8 totals followed by 8 * CONS_BLOCKS partials
  const int nb = P.n < 256 * CONS_BLOCKS ? (P.n + 255) / 256 : CONS_BLOCKS;
  k_conserved_part<<<nb > 0 ? nb : 1, 256, 0, L.stream>>>(P, pp, out8, nreal);
  k_conserved_final<<<1, 256, 0, L.stream>>>(out8, nb > 0 ? nb : 1);
  *L.counter += 2;
  return cudaGetLastError();
}

}  // namespace fsph
