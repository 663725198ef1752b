// fsph_internal.cuh -- device-side types shared by the translation units of
// libfsph_gb300.so.  Not part of the public ABI (that is include/fsph.h).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <stdint.h>

#include "../../include/fsph.h"

namespace fsph {

// Particle fields held on the device, one FP64 array each (SoA).  Order is
// free; the names follow body_u (include/physics/body.h:221-251).
enum Field {
  F_X, F_Y, F_Z, F_VX, F_VY, F_VZ, F_VHX, F_VHY, F_VHZ, F_AX, F_AY, F_AZ,
  F_GAX, F_GAY, F_GAZ, F_GPOT, F_M, F_H, F_RHO, F_P, F_CS, F_U, F_E, F_DUDT,
  F_DEDT, F_K, F_ALPHA, F_VSIG, F_DT, F_DIVV, F_DDIVVDT, F_YE, NF
};

// physics:: time globals of the reference (default_physics.h:32-39), kept in
// device memory so a whole step runs without a host round trip.
struct DevTime {
  double dt, dt_saved, totaltime, totaltime_next;
  double t_screen, t_scalar, t_h5;
  long long iteration;
  // global reductions written by kernels
  unsigned long long dtmin_bits;  // ordered encoding of min particle dt
  double hsum;                    // sum of h (average smoothing length)
};

// First device-side error: code (fsph_status) and the particle it concerns.
struct DevStatus {
  int code;
  int flags;  // reserved
  long long index;
};

struct Particles {
  double * f[NF];
  long long * id;
  unsigned long long * key;
  int n;
};

struct PhysParams {
  int dim, kernel, eos, thermokinetic, evolve_u, adaptive;
  int cullen;  // sph_viscosity == visc_cullen
  double gamma, eta, kw, alpha, beta, eps, cfl;
  double alpha_max, visc_l, visc_delta;  // visc_cullen parameters
  double sinc_index, sinc_sigma[3];       // sinc kernel power and norms
  double gamma2, rho_thr;                 // eos_ppt upper segment
  double ppt_k2;                          // rho_thr^(gamma - gamma2)
  double out_screen_dt, out_scalar_dt, out_h5data_dt;
  double G;
  // external forces (eforce.h) in the order external_force::select lists
  // them, with the parameters their functions read
  int n_eforce, eforce[8];
  int has_eacc;                // a term with an acceleration (all but poison)
  int dprof;                   // density profile of the density support
  double ew_n, ew_a;           // extforce_wall_powerindex, _steepness
  double box_half[3];          // .5 * box_length, _width, _height
  double sphere_r, grav_acc, poison;
  double orb_a, orb_mns, orb_mwd;
  double af_size, af_thick, af_camber, af_x, af_y, af_alpha;  // alpha in radians
  double ds_K0, ds_rho0, rho_init, mesa_q, mesa_rho0;         // density support
  // particle relaxation (default_physics.h:571-599,699-753)
  double relax_beta, relax_gamma, rep_radius, rep_gamma;
  long long relax_steps;       // relaxation_steps
};

// Binary radix tree over the sorted keys (n-1 internal nodes, node 0 is the
// root).  Child encoding: >= 0 internal node, < 0 leaf ~index.
struct NodeBox {   // 64 bytes: two aligned double4 loads
  double lo[3];
  double hmax;
  double hi[3];
  double pad;
};

struct Tree {
  int * left;
  int * right;
  int * parent;       // internal node -> parent (-1 for the root)
  int * leaf_parent;  // particle -> parent internal node
  int * first;
  int * last;
  int4 * qbox;             // per node: {lo.xyz, float bits of h_max}, {hi.xyz, 0}
                           // in the fixed-point position space of Packed::qpos
  NodeBox * box2;          // reference node box: union of [x - h/2, x + h/2]
  float4 * fbox2;          // the same box in FP32 relative to the range's
                           // lower corner, rounded outwards (lo, hi pairs)
  int * opar;              // particle -> binary node standing for its octree parent
  int * gref;              // particle -> its reference traversal group
  unsigned * counter;
  unsigned char * edepth;  // reference octree depth of each particle
  int * group_first;
  int * group_last;
  int * group_start;       // per group: the node its mixed walk starts from
  int * ngroups;           // device scalar
  double * gmom;           // with gravity only (else null): per node the raw
                           // moments of mass about the range centre,
                           // {m, m y_xyz, m y_x^2, m y_y^2, m y_z^2,
                           //  m y_x y_y, m y_x y_z, m y_y y_z}
};

// Packed FP32 records of the mixed-precision path (rebuilt every step).
// Positions are 31-bit fixed point over the step's range: differences are
// exact integers, so separations keep ~1e-9 of the range.
struct Packed {
  int4 * qpos;      // {qx, qy, qz, float bits of h}
  float4 * vhm;     // {vh_x, vh_y, vh_z, m}
  float4 * vel;     // {v_x, v_y, v_z, c_s before the density pass}
  float4 * thermo;  // {rho, P/rho^2, c_s (new), c_s (previous)}
  float * mass;     // m alone, for the density pass (4 B per pair instead of 16)
  float4 * velp;    // de/dt pass: {v_x, v_y, v_z, P/rho^2}
  // Records of the float-float acceleration pass and of the energy passes
  // that carry v_half's low words (v - (float)v): a velocity difference
  // taken as (high - high) + (low - low) keeps ~2^-24 of itself however
  // large v is beside it (in a shear flow v_a - v_b is ~1e-3 of v, where
  // FP32 records alone leave ~1e-5 of it).  v itself is v_half + (v -
  // v_half), the second term in FP32: it is the step's kick, small beside
  // v.  Filled four floats a record: the acceleration pass reads six
  // 16-byte records a pair (fph, fpl, fmA, fv1, fv2, vel), the energy passes
  // four (qpos, fv1, fv2, fdv).
  float4 * fv1;     // {vh_x, vh_y, vh_z high words, rho}
  float4 * fv2;     // {vh_x, vh_y, vh_z low words, c_s (of the density pass)}
  float4 * fdv;     // energy passes: {v - v_half (FP32), m}
  float2 * rc;      // de/dt pass: {rho, c_s} (56 B per pair with qpos, vhm, velp)
  float2 * visc;    // Cullen & Dehnen: {c_s, sign(div v)} in the alpha pass,
                    // {alpha, 0} in the pair passes
  float * qscale;   // device [3]: one fixed-point step per axis, E / 2^31 (E: the largest range extent enlarged by 2^-19)
  // Float-float records of the density and acceleration passes (Wendland
  // kernels).  Positions are X = 1 + (x - lo) / E with E the largest range
  // extent (slightly enlarged), so every X lies in [1, 2): the high words
  // of two positions share one exponent and their difference is exact;
  // h is in the same units.
  float4 * fph;     // {X_h, Y_h, Z_h, h_h}
  float4 * fpl;     // {X_l, Y_l, Z_l, h_l}
  float4 * fmA;     // {m_h, m_l, (P/rho^2)_h, (P/rho^2)_l}: m packed with the
                    // positions, P/rho^2 by the density pass (two 8-byte halves)
  double * fscale;  // device [3]: E, 1 / E, 1 if every h is equal (else 0)
  // pressure-only hydro acceleration of the float-float pass,
  // -sum_b m_b (P_a/rho_a^2 + P_b/rho_b^2) grad W, as three FP64 arrays of
  // stride n: the de/dt pass rewrites its pressure terms with it while
  // positions, P/rho^2, v_half and alpha are unchanged
  double * ahyd;
};

// Multipole of a radix-tree node (FP64): mass, centre of mass, traceless
// quadrupole {xx, yy, zz, xy, xz, yz} about it, bounding radius.
struct GravNode {
  double m;
  double c[3];
  double q[6];
  double rmax;
  double pad;
};

// Device buffers of the gravity pass.  gnf holds every node again in FP32
// for the walk: {c_hi, rmax (rounded up)}, {m, c_lo}, {q0..q3}, {q4, q5},
// c_hi + c_lo being the centre of mass relative to the range's lower corner
// as an unevaluated FP32 sum; gpk holds every particle as {x_hi, m},
// {x_lo} in the same frame.
struct GravBuffers {
  GravNode * gn;       // n nodes
  float4 * gnf;        // 4 n
  float4 * gpk;        // 2 n
};

// Neighbour lists, interleaved by warp in chunks of four slots:
// [(i>>5)][slot/4][i&31][slot%4], so a lane reads four slots with one
// 16-byte load and a warp reads 512 contiguous bytes.  maxnb is a multiple
// of 4; the slots past a list's end in its last chunk hold the particle
// itself (a zero-weight pair for every pass but the density, which masks
// them).
struct Lists {
  int * idx;
  int * cnt;
  int maxnb;
};

__host__ __device__ inline size_t list_slot(int i, int j, int maxnb) {
  return ((size_t)(i >> 5) * (size_t)maxnb + (size_t)(j & ~3)) * 32u +
         (size_t)(i & 31) * 4u + (size_t)(j & 3);
}

// offset of slot j from slot 0 of the same particle
__host__ __device__ inline int slot_off(int j) { return ((j & ~3) << 5) | (j & 3); }

// Kernel launch helpers (host).  Each translation unit exports plain host
// functions; the API layer strings them together on the context stream.
struct Launch {
  cudaStream_t stream;
  long long * counter;  // launches issued
};

// Kernel attributes (cudaFuncSetAttribute) belong to a device.  Runs
// `apply` (returning a cudaError_t) once for the current device, bit d of
// *mask recording device d, so a process with contexts on several devices
// sets them once on each (devices past 64 apply every time).  Contexts on
// different host threads may share a device: the bit is set only after
// `apply` has succeeded, under a process-wide lock, so no thread sees the
// device marked and launches before the attributes are in place.
inline std::mutex & attr_mutex() {
  static std::mutex m;
  return m;
}

template<class F>
inline cudaError_t once_per_device(std::atomic<unsigned long long> * mask, F apply) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if(e != cudaSuccess)
    return e;
  if(dev < 0 || dev >= 64)
    return apply();
  const unsigned long long bit = 1ull << dev;
  if(mask->load(std::memory_order_acquire) & bit)
    return cudaSuccess;
  std::lock_guard<std::mutex> lock(attr_mutex());
  if(mask->load(std::memory_order_acquire) & bit)
    return cudaSuccess;
  e = apply();
  if(e == cudaSuccess)
    mask->fetch_or(bit, std::memory_order_release);
  return e;
}

// ---- fsph_tree.cu ----
cudaError_t launch_range_keys(const Launch & L, const Particles & P,
  const PhysParams & pp, double * d_range, unsigned long long * keys_out,
  int * idx_out);
cudaError_t radix_sort_pairs(const Launch & L, unsigned long long * keys,
  int * vals, unsigned long long * keys_tmp, int * vals_tmp, int n,
  unsigned * hist, int nblocks_cap);
size_t radix_hist_entries(int n);
cudaError_t launch_check_duplicates(const Launch & L,
  const unsigned long long * keys, int n, DevStatus * st);
cudaError_t launch_permute(const Launch & L, const Particles & src,
  const Particles & dst, const int * perm, const unsigned long long * keys,
  unsigned skip, float4 * vel = nullptr, int dim = 3);
struct Packed;
cudaError_t launch_build_tree(const Launch & L, const Particles & P,
  const PhysParams & pp, Tree & T, int group_max,
  const unsigned long long * rbits, const int4 * qpos, const float * qscale, int ordered);
cudaError_t launch_neighbors(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, Lists & Ls, DevStatus * st, int nsm,
  const unsigned long long * rbits, const Packed & K, int ordered);

// ---- fsph_mixed.cu ----
cudaError_t launch_pack_positions(const Launch & L, const Particles & P,
  const PhysParams & pp, const unsigned long long * rbits, const Packed & K);
cudaError_t launch_density_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, double * cs_new,
  DevStatus * st, const DevTime * tm, int vel_current);
cudaError_t launch_alpha_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t);
cudaError_t launch_vsig_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K);
// fv_current / fdv_current: the fv1/fv2 (fdv) records already hold the
// current state (the caller tracks it), so the pass does not repack them.
cudaError_t launch_accel_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int kick,
  const DevTime * t, int fused_vsig, int fv_current);
cudaError_t launch_dudt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, const DevTime * t,
  int then_op, int fv_current, int fdv_current);
cudaError_t launch_dedt_mixed(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const Packed & K, int then_op,
  const DevTime * t, DevStatus * st, int use_ahyd, int fdv_current);

// ---- fsph_gravity.cu ----
cudaError_t launch_let_export(const Launch & L, const Particles & P, int dim,
  const Tree & T, const GravBuffers & G, const double * blo, const double * bhi,
  double theta, int order, double * cells, long long cap,
  unsigned long long * count, DevStatus * st);
cudaError_t launch_let_apply(const Launch & L, const Particles & P, int dim,
  const double * cells, long long ncell, double Gc, int mixed);
cudaError_t launch_gravity(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, const GravBuffers & G,
  const unsigned long long * rbits, double theta, int order, int mixed,
  DevStatus * st, int nsm);

// ---- fsph_periodic.cu ----
struct PeriodicScratch {
  int * flag;     // cap: real flags, then copy counts
  int * pos;      // cap: exclusive scan
  int * perm;     // cap: compaction gather
  int * tiles;    // scan_tiles(cap)
  int * total;    // 1
  unsigned long long * hbits;  // 1: max h of the real particles (bits)
};
int scan_tiles(int n);
cudaError_t launch_exclusive_scan(const Launch & L, const int * in, int * out,
  int n, int * tile_sums, int * total);
// Drops the copies (ids >= nreal) keeping the order of the rest, teleports
// and appends the new copies; P.n / Palt.n become the new total (also in
// *n_out).  If cap is too small nothing is appended and *why says so.
cudaError_t launch_periodic(const Launch & L, Particles & P, Particles & Palt,
  const PhysParams & pp, const double * box_len, const int * periodic,
  long long nreal, int cap, PeriodicScratch & S, int * n_out,
  const char ** why, unsigned skip);

// ---- fsph_fp64.cu ----
cudaError_t launch_density_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, double * cs_new, DevStatus * st,
  const DevTime * t);
cudaError_t launch_alpha_cullen(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const DevTime * t);
cudaError_t launch_vsig_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const double * cs_new);
cudaError_t launch_repulsion(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls);
cudaError_t launch_accel_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, int kick, const DevTime * t);
cudaError_t launch_dudt_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls, const DevTime * t);
cudaError_t launch_dedt_fp64(const Launch & L, const Particles & P,
  const PhysParams & pp, const Lists & Ls);

// ---- fsph_elementwise.cu ----
enum ElemOp {
  OP_EOS_INIT, OP_SET_TOTAL_ENERGY, OP_SAVE_VHALF, OP_KICK_V, OP_KICK_U,
  OP_KICK_E, OP_DRIFT, OP_RECOMPUTE, OP_RECOMPUTE_THERMO, OP_SMOOTHING_LENGTH,
  OP_CHECK_NANS, OP_CHECK_NEGATIVITY, OP_KICK_DRIFT_E, OP_KICK_DRIFT_U,
  OP_KICK_DRIFT_NONE, OP_SET_H, OP_RECOMPUTE_KICK_E, OP_RECOMPUTE_KICK_U,
  OP_INIT_ALPHA, OP_DRAG_ACC, OP_DRAG_DEDT, OP_DRAG_DUDT
};
cudaError_t launch_elementwise(const Launch & L, const Particles & P,
  const PhysParams & pp, int op, DevTime * t, DevStatus * st);
cudaError_t launch_compute_dt(const Launch & L, const Particles & P,
  const PhysParams & pp, DevTime * t, DevStatus * st, int with_checks,
  int f32);
cudaError_t launch_set_adaptive_timestep(const Launch & L,
  const PhysParams & pp, DevTime * t);
cudaError_t launch_advance_time(const Launch & L, const PhysParams & pp,
  DevTime * t);
cudaError_t launch_hsum(const Launch & L, const Particles & P, DevTime * t);
#define CONS_BLOCKS 1024
// out8: 8 * (1 + CONS_BLOCKS) doubles; the totals land in the first 8
cudaError_t launch_conserved(const Launch & L, const Particles & P,
  const PhysParams & pp, double * out8, long long nreal);

}  // namespace fsph
