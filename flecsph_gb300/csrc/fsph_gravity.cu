// fsph_gravity.cu -- self-gravity over the radix tree: an upward multipole
// pass and a group walk with particle-cell and particle-particle terms.
//
// Replaces body_system::gravitation_fmm (mpisph/bodies_system.h:282-288),
// i.e. tree_topology::traversal_fmm (tree_topology.h:448-795) with the
// kernels of include/physics/fmm.h.  The reference expands cells to first
// order around their centre of mass (monopole field plus its gradient
// applied through fmm_c2p, fmm.h:91-119) in a dual-tree walk; this build
// expands every accepted cell to quadrupole order (order 1 = monopole only)
// and walks the tree once per particle group:
//   multipoles (FP64, k_grav_nodes): mass, centre of mass, traceless
//     quadrupole Q_ij = sum m (3 x_i x_j - r^2 delta_ij) about it and the
//     radius of the bounding box seen from it, from raw mass moments that
//     the tree's bottom-up pass sums (children add);
//   walk (k_gravity_walk): one warp per group of <= 32 particles; a cell is
//     accepted when r_max < theta * d_min, d_min being the distance from
//     its centre of mass to the group's box (so the test holds for every
//     member); accepted cells go to a shared-memory multipole list, leaves
//     of opened cells to a particle list; each lane then sums both lists
//     for its particle.  The walk itself (acceptance test, list building)
//     runs in FP32 on copies of the nodes and particles made by the up
//     pass, in both precisions, so both evaluate the same interaction
//     lists; positions there are relative to the range's lower corner and
//     split into FP32 hi + lo words, so that a difference of two of them
//     keeps FP32 relative accuracy however close the pair.
// The pair kernel is the reference's unsoftened Newtonian one
// (fmm.h:37-46): phi += -G m / r, a += -G m (x_a - x_b) / r^3, skipping the
// particle itself (fmm.h:136-137).  Results are added to g-acceleration
// and potential (the acceleration pass zeroes them first, as
// default_physics.h:406-407 does).  FP64 mode evaluates the lists in FP64
// from the FP64 nodes and positions; the mixed path evaluates them in FP32
// with Kahan sums (multipoles accumulated in FP64, stored in FP32).
#include <cuda_runtime.h>

#include <type_traits>

#include "fsph_internal.cuh"

namespace fsph {

#define GW_WARPS 8
#define GW_STACK 1024
#define GW_MCAP 64
#define GW_PCAP 128
#define GFULL 0xffffffffu

__device__ __forceinline__ unsigned lanemask_lt_g() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------- up pass -----
__device__ __forceinline__ double ord_dec_g(unsigned long long u) {
  return (u & 0x8000000000000000ull)
           ? __longlong_as_double((long long)(u & 0x7fffffffffffffffull))
           : __longlong_as_double((long long)~u);
}

__device__ __forceinline__ void split_hi_lo(double v, float & hi, float & lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Multipoles from the raw moments the tree's bottom-up pass summed
// (Tree::gmom, about the range centre r_c), one thread per node, no
// dependency between nodes:
//   M = S_0, C = r_c + S_1 / M,
//   sum m y'_i y'_j = S_ij - M c_i c_j   (c = C - r_c, y' = x - C),
//   Q_ij = 3 sum m y'_i y'_j - delta_ij sum m |y'|^2   (traceless).
// The cancellation in S_ij - M c_i c_j costs ~1e-16 (|y| / node size)^2
// relative, ~1e-10 for the smallest nodes of a 4M-particle set.  r_max is
// the distance from C to the farthest corner of the node's position box
// (the fixed-point box of the tree, widened by one quantisation step).
// Every particle also gets its FP32 walk record here.
__global__ void k_grav_nodes(Particles P, int dim, Tree T, GravBuffers G,
  const unsigned long long * rbits, int order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = P.n;
  if(i >= n)
    return;
  double r0[3] = {0.0, 0.0, 0.0}, rc[3] = {0.0, 0.0, 0.0}, step[3] = {0.0, 0.0, 0.0};
  // one step of the tree's fixed point, E / 2^31 on every axis (E: the
  // largest range extent enlarged by 2^-19, as the positions were packed)
  double E = 0.0;
  for(int d = 0; d < dim; ++d) {
    const double lo = ord_dec_g(rbits[d]), hi = ord_dec_g(rbits[3 + d]);
    r0[d] = lo;
    rc[d] = 0.5 * (lo + hi);
    E = fmax(E, hi - lo);
  }
  for(int d = 0; d < dim; ++d)
    step[d] = E * (1.0 + 0x1p-19) * 0x1p-31;
  {
    // this particle for the walk: position relative to the corner, hi + lo
    float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
    for(int d = 0; d < dim; ++d)
      split_hi_lo(P.f[F_X + d][i] - r0[d], h[d], l[d]);
    G.gpk[2 * i] = make_float4(h[0], h[1], h[2], (float)P.f[F_M][i]);
    G.gpk[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
  if(i >= n - 1)
    return;
  const double * S = T.gmom + 10 * (size_t)i;
  double Sv[10];
  for(int k = 0; k < 10; ++k)
    Sv[k] = S[k];
  const double M = Sv[0];
  const double iM = 1.0 / M;
  const double c[3] = {Sv[1] * iM, Sv[2] * iM, Sv[3] * iM};
  double Q[6] = {0, 0, 0, 0, 0, 0};
  if(order >= 2) {
    const double sxx = Sv[4] - M * c[0] * c[0], syy = Sv[5] - M * c[1] * c[1];
    const double szz = Sv[6] - M * c[2] * c[2];
    const double tr = sxx + syy + szz;
    Q[0] = 3.0 * sxx - tr;
    Q[1] = 3.0 * syy - tr;
    Q[2] = 3.0 * szz - tr;
    Q[3] = 3.0 * (Sv[7] - M * c[0] * c[1]);
    Q[4] = 3.0 * (Sv[8] - M * c[0] * c[2]);
    Q[5] = 3.0 * (Sv[9] - M * c[1] * c[2]);
  }
  GravNode out;
  out.m = M;
  double cr[3];  // centre relative to the corner
  const int4 qlo = T.qbox[2 * i], qhi = T.qbox[2 * i + 1];
  const int ql[3] = {qlo.x, qlo.y, qlo.z}, qh[3] = {qhi.x, qhi.y, qhi.z};
  double rmax2 = 0.0;
  for(int d = 0; d < 3; ++d) {
    out.c[d] = d < dim ? rc[d] + c[d] : 0.0;
    cr[d] = d < dim ? out.c[d] - r0[d] : 0.0;
    if(d < dim) {
      const double e = fmax((double)qh[d] * step[d] - cr[d], cr[d] - (double)ql[d] * step[d]) +
                       step[d];
      rmax2 += e * e;
    }
  }
  for(int k = 0; k < 6; ++k)
    out.q[k] = Q[k];
  out.rmax = sqrt(rmax2);
  out.pad = 0;
  G.gn[i] = out;
  float ch_[3] = {0.f, 0.f, 0.f}, cl_[3] = {0.f, 0.f, 0.f};
  for(int d = 0; d < dim; ++d)
    split_hi_lo(cr[d], ch_[d], cl_[d]);
  // the acceptance radius rounded up, a hair wider for the FP32 tests
  const float rf = __double2float_ru(out.rmax * (1.0 + 1e-6));
  G.gnf[4 * i] = make_float4(ch_[0], ch_[1], ch_[2], rf);
  G.gnf[4 * i + 1] = make_float4((float)M, cl_[0], cl_[1], cl_[2]);
  G.gnf[4 * i + 2] = make_float4((float)Q[0], (float)Q[1], (float)Q[2], (float)Q[3]);
  G.gnf[4 * i + 3] = make_float4((float)Q[4], (float)Q[5], 0.f, 0.f);
}

// ------------------------------------------------------------ the walk --
template<class R>
__device__ __forceinline__ void kahan_g(R & s, R & c, R t) {
  R y = t - c;
  R u = s + y;
  c = (u - s) - y;
  s = u;
}

// Terms of a flush are summed plainly in blocks of GW_SUB and each block is
// added to the compensated total: a plain sum over a whole flush (up to 128
// terms) let its rounding, a fraction of the sum of |terms|, dominate where
// the terms cancel (at the centre of a self-gravitating body).
#define GW_SUB 8
template<class R>
__device__ __forceinline__ void fold_g(R & s, R & c, R & part) {
  kahan_g(s, c, part);
  part = (R)0;
}

// Shared-memory list records, one broadcast 16-byte load per quarter:
//   mixed cell     {m, c - g} {q0..q3} {q4, q5, -, -}             48 B
//                  (g: the group's reference point, see the walk)
//   mixed particle {x_hi, m} {x_lo, index}                        32 B
//   FP64 cell      {m, c} {q0..q5}  as five double2              80 B
//   FP64 particle  {x, m} as two double2, index beside            32 B + 4
template<bool MIXED>
__host__ __device__ constexpr size_t gw_cell_bytes() { return MIXED ? 48 : 80; }

template<bool MIXED>
__host__ __device__ constexpr size_t gw_warp_bytes() {
  return (size_t)GW_STACK * 4 + (size_t)GW_MCAP * gw_cell_bytes<MIXED>() +
         (size_t)GW_PCAP * 32 + (MIXED ? 0 : (size_t)GW_PCAP * 4);
}

template<bool MIXED>
__global__ void __launch_bounds__(GW_WARPS * 32) k_gravity_walk(Particles P,
  Tree T, GravBuffers G, float theta, double Gc, int order, int dim,
  DevStatus * st) {
  typedef typename std::conditional<MIXED, float, double>::type R;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char * base = gsm + gw_warp_bytes<MIXED>() * w;
  int * stack = (int *)base;
  unsigned char * mrec = base + (size_t)GW_STACK * 4;
  unsigned char * prec = mrec + (size_t)GW_MCAP * gw_cell_bytes<MIXED>();
  int * pidx = (int *)(prec + (size_t)GW_PCAP * 32);  // FP64 only
  float4 * mf = (float4 *)mrec;
  float4 * pf = (float4 *)prec;
  double2 * md = (double2 *)mrec;
  double2 * pd = (double2 *)prec;
  const unsigned lt = lanemask_lt_g();
  const int ngroups = *T.ngroups;
  const float th2 = theta * theta;
  for(int g = blockIdx.x * GW_WARPS + w; g < ngroups; g += gridDim.x * GW_WARPS) {
    const int gf = T.group_first[g], gl = T.group_last[g];
    const bool mem = lane <= gl - gf;
    const int a = gf + lane;
    float4 ah = make_float4(0.f, 0.f, 0.f, 0.f), al = ah;
    if(mem) {
      ah = G.gpk[2 * a];
      al = G.gpk[2 * a + 1];
    }
    // the group's box (FP32, relative frame) for the acceptance test
    float lo[3] = {mem ? ah.x : 3e38f, mem ? ah.y : 3e38f, mem ? ah.z : 3e38f};
    float hi[3] = {mem ? ah.x : -3e38f, mem ? ah.y : -3e38f, mem ? ah.z : -3e38f};
    for(int d = 0; d < 3; ++d)
      for(int o = 16; o; o >>= 1) {
        lo[d] = fminf(lo[d], __shfl_xor_sync(GFULL, lo[d], o));
        hi[d] = fmaxf(hi[d], __shfl_xor_sync(GFULL, hi[d], o));
      }
    // mixed: positions relative to the first member (the group's reference
    // point), from the hi + lo words; cells entering the list get the same
    // frame once per group, so a cell term needs one subtraction per axis
    const float rh[3] = {__shfl_sync(GFULL, ah.x, 0), __shfl_sync(GFULL, ah.y, 0),
      __shfl_sync(GFULL, ah.z, 0)};
    const float rl[3] = {__shfl_sync(GFULL, al.x, 0), __shfl_sync(GFULL, al.y, 0),
      __shfl_sync(GFULL, al.z, 0)};
    const float rx = (ah.x - rh[0]) + (al.x - rl[0]);
    const float ry = (ah.y - rh[1]) + (al.y - rl[1]);
    const float rz = (ah.z - rh[2]) + (al.z - rl[2]);
    double xa = 0.0, ya = 0.0, za = 0.0;
    if(!MIXED && mem) {
      xa = P.f[F_X][a];
      ya = P.f[F_Y][a];
      za = dim == 3 ? P.f[F_Z][a] : 0.0;
    }
    R sx = 0, sy = 0, sz = 0, sp = 0, cx = 0, cy = 0, cz = 0, cp = 0;
    int sptr = 1, nm = 0, np = 0;
    if(lane == 0)
      stack[0] = 0;
    __syncwarp();
    while(true) {
      const bool done = sptr == 0;
      if(!done) {
        const int k = sptr < 32 ? sptr : 32;
        const bool act = lane < k;
        const int node = act ? stack[sptr - 1 - lane] : 0;
        __syncwarp();
        sptr -= k;
        bool acc = false, open = false, leaf = false;
        int code = 0;
        if(act) {
          if(node < 0)
            leaf = true;
          else {
            const float4 c0 = G.gnf[4 * node];
            code = T.qbox[2 * node + 1].w;
            const float ex = fmaxf(0.f, fmaxf(lo[0] - c0.x, c0.x - hi[0]));
            const float ey = fmaxf(0.f, fmaxf(lo[1] - c0.y, c0.y - hi[1]));
            const float ez = fmaxf(0.f, fmaxf(lo[2] - c0.z, c0.z - hi[2]));
            const float dd = ex * ex + ey * ey + ez * ez;
            acc = dd > 0.f && c0.w * c0.w < th2 * dd;
            open = !acc;
          }
        }
        const unsigned bo = __ballot_sync(GFULL, open);
        const unsigned ba = __ballot_sync(GFULL, acc);
        const unsigned bl = __ballot_sync(GFULL, leaf);
        const int npush = 2 * __popc(bo);
        if(sptr + npush > GW_STACK) {
          if(lane == 0 && atomicCAS(&st->code, 0, (int)FSPH_ERR_STACK_OVERFLOW) == 0)
            st->index = gf;
          break;
        }
        if(open) {
          const int pos = sptr + 2 * __popc(bo & lt);
          const int split = code >> 2;
          stack[pos] = (code & 1) ? ~(split + 1) : split + 1;
          stack[pos + 1] = (code & 2) ? ~split : split;
        }
        sptr += npush;
        if(acc) {
          const int pos = nm + __popc(ba & lt);
          if(MIXED) {
            // gnf: {c_hi, rmax} {m, c_lo} {q0..q3} {q4, q5}; stored as
            // {m, centre - group reference} {q0..q3} {q4, q5}
            const float4 c0 = G.gnf[4 * node], c1 = G.gnf[4 * node + 1];
            const float4 q0 = G.gnf[4 * node + 2], q1 = G.gnf[4 * node + 3];
            mf[3 * pos] = make_float4(c1.x, (c0.x - rh[0]) + (c1.y - rl[0]),
              (c0.y - rh[1]) + (c1.z - rl[1]), (c0.z - rh[2]) + (c1.w - rl[2]));
            mf[3 * pos + 1] = q0;
            mf[3 * pos + 2] = make_float4(q1.x, q1.y, 0.f, 0.f);
          }
          else {
            const GravNode & gnd = G.gn[node];
            md[5 * pos] = make_double2(gnd.m, gnd.c[0]);
            md[5 * pos + 1] = make_double2(gnd.c[1], gnd.c[2]);
            md[5 * pos + 2] = make_double2(gnd.q[0], gnd.q[1]);
            md[5 * pos + 3] = make_double2(gnd.q[2], gnd.q[3]);
            md[5 * pos + 4] = make_double2(gnd.q[4], gnd.q[5]);
          }
        }
        nm += __popc(ba);
        if(leaf) {
          const int j = ~node;
          const int pos = np + __popc(bl & lt);
          if(MIXED) {
            const float4 h = G.gpk[2 * j], l = G.gpk[2 * j + 1];
            pf[2 * pos] = h;
            pf[2 * pos + 1] = make_float4(l.x, l.y, l.z, __int_as_float(j));
          }
          else {
            pd[2 * pos] = make_double2(P.f[F_X][j], P.f[F_Y][j]);
            pd[2 * pos + 1] = make_double2(dim == 3 ? P.f[F_Z][j] : 0.0, P.f[F_M][j]);
            pidx[pos] = j;
          }
        }
        np += __popc(bl);
        __syncwarp();
      }
      const bool flush_m = nm > GW_MCAP - 32 || (done && nm > 0);
      const bool flush_p = np > GW_PCAP - 32 || (done && np > 0);
      // n terms summed plainly in blocks of GW_SUB, each block folded into
      // the compensated totals: unrolled whole in the FP32 walk; the FP64
      // walk, whose terms take twice the registers, keeps one loop
      auto sum_terms = [&](int n, auto term) {
        R px = 0, py = 0, pz = 0, pp = 0;
        if constexpr(MIXED) {
          int k = 0;
          for(; k + GW_SUB <= n; k += GW_SUB) {
#pragma unroll
            for(int u = 0; u < GW_SUB; ++u)
              term(k + u, px, py, pz, pp);
            fold_g(sx, cx, px);
            fold_g(sy, cy, py);
            fold_g(sz, cz, pz);
            fold_g(sp, cp, pp);
          }
          for(; k < n; ++k)
            term(k, px, py, pz, pp);
        }
        else {
          for(int k = 0; k < n; ++k) {
            term(k, px, py, pz, pp);
            if((k & (GW_SUB - 1)) == GW_SUB - 1) {
              fold_g(sx, cx, px);
              fold_g(sy, cy, py);
              fold_g(sz, cz, pz);
              fold_g(sp, cp, pp);
            }
          }
        }
        fold_g(sx, cx, px);
        fold_g(sy, cy, py);
        fold_g(sz, cz, pz);
        fold_g(sp, cp, pp);
      };
      if(mem && flush_m) {
        // one cell's potential and acceleration (monopole + quadrupole)
        auto cell = [&](int k, R & px, R & py, R & pz, R & pp) {
          R m, dx, dy, dz, qxx, qyy, qzz, qxy, qxz, qyz;
          if(MIXED) {
            const float4 r0 = mf[3 * k];
            m = r0.x;
            dx = rx - r0.y;
            dy = ry - r0.z;
            dz = rz - r0.w;
            if(order >= 2) {
              const float4 r1 = mf[3 * k + 1], r2 = mf[3 * k + 2];
              qxx = r1.x; qyy = r1.y; qzz = r1.z; qxy = r1.w; qxz = r2.x; qyz = r2.y;
            }
          }
          else {
            const double2 r0 = md[5 * k], r1 = md[5 * k + 1];
            m = r0.x;
            dx = xa - r0.y;
            dy = ya - r1.x;
            dz = za - r1.y;
            if(order >= 2) {
              const double2 r2 = md[5 * k + 2], r3 = md[5 * k + 3], r4 = md[5 * k + 4];
              qxx = r2.x; qyy = r2.y; qzz = r3.x; qxy = r3.y; qxz = r4.x; qyz = r4.y;
            }
          }
          const R r2 = dx * dx + dy * dy + dz * dz;
          const R ir = MIXED ? (R)rsqrtf((float)r2) : (R)rsqrt((double)r2);
          const R ir2 = ir * ir;
          const R ir3 = ir * ir2;
          R phi = -m * ir;
          R fx = -m * ir3 * dx, fy = -m * ir3 * dy, fz = -m * ir3 * dz;
          if(order >= 2) {
            // phi_Q = -(1/2) d.Q.d / r^5,  a_Q = Q.d / r^5 - (5/2) (d.Q.d) d / r^7
            const R qdx = qxx * dx + qxy * dy + qxz * dz;
            const R qdy = qxy * dx + qyy * dy + qyz * dz;
            const R qdz = qxz * dx + qyz * dy + qzz * dz;
            const R dqd = dx * qdx + dy * qdy + dz * qdz;
            const R ir5 = ir3 * ir2;
            const R ir7 = ir5 * ir2;
            phi += (R)-0.5 * dqd * ir5;
            fx += qdx * ir5 - (R)2.5 * dqd * ir7 * dx;
            fy += qdy * ir5 - (R)2.5 * dqd * ir7 * dy;
            fz += qdz * ir5 - (R)2.5 * dqd * ir7 * dz;
          }
          px += fx;
          py += fy;
          pz += fz;
          pp += phi;
        };
        sum_terms(nm, cell);
      }
      if(mem && flush_p) {
        // one particle's potential and acceleration; the particle itself
        // drops out (fmm.h:136-137)
        auto part = [&](int k, R & px, R & py, R & pz, R & pp) {
          int j;
          R m, dx, dy, dz;
          if(MIXED) {
            const float4 h = pf[2 * k], l = pf[2 * k + 1];
            j = __float_as_int(l.w);
            m = h.w;
            dx = (ah.x - h.x) + (al.x - l.x);
            dy = (ah.y - h.y) + (al.y - l.y);
            dz = (ah.z - h.z) + (al.z - l.z);
          }
          else {
            const double2 p0 = pd[2 * k], p1 = pd[2 * k + 1];
            j = pidx[k];
            m = p1.y;
            dx = xa - p0.x;
            dy = ya - p0.y;
            dz = za - p1.x;
          }
          const R r2 = dx * dx + dy * dy + dz * dz;
          const R ir = j == a ? (R)0
                              : (MIXED ? (R)rsqrtf((float)r2) : (R)rsqrt((double)r2));
          const R w = m * ir;
          const R w3 = w * ir * ir;
          px -= w3 * dx;
          py -= w3 * dy;
          pz -= w3 * dz;
          pp -= w;
        };
        sum_terms(np, part);
      }
      __syncwarp();
      if(flush_m)
        nm = 0;
      if(flush_p)
        np = 0;
      if(done)
        break;
    }
    if(mem) {
      const double fx = ((double)sx - (double)cx) * Gc;
      const double fy = ((double)sy - (double)cy) * Gc;
      const double fz = ((double)sz - (double)cz) * Gc;
      P.f[F_GAX][a] += fx;
      P.f[F_GAY][a] += fy;
      if(dim == 3)
        P.f[F_GAZ][a] += fz;
      P.f[F_GPOT][a] += ((double)sp - (double)cp) * Gc;
    }
  }
}

// ------------------------------------------- multi-rank gravity (LET) --
// A locally essential tree for a run decomposed over ranks.  The reference
// shares top-tree branches and fetches remote subtrees during its FMM walk
// (tree_topology.h:1142-1542,1550-1744); here a rank exports, for every
// other rank's bounding box, the cells of its own tree that are far enough
// for that whole box (r_max < theta * d(centre of mass, box), the test the
// walk applies to a group's box) as multipoles, and the particles of the
// cells that are not, as point masses; the receiving rank adds their field
// to its particles (k_let_apply) after its own tree walk.  Cell record, 10
// doubles: {m, c_x, c_y, c_z, Q_xx, Q_yy, Q_zz, Q_xy, Q_xz, Q_yz} (Q
// traceless about c; zero for a point mass).
#define LET_REC 10

// One warp walks the tree (k_grav_nodes must have filled G.gn since the
// last tree build) against the box [blo, bhi], in FP64.
__global__ void k_let_export(Particles P, int dim, Tree T, GravBuffers G,
  double3 blo, double3 bhi, double th2, int order, double * cells,
  long long cap, unsigned long long * count, DevStatus * st) {
  __shared__ int stack[GW_STACK];
  const int lane = threadIdx.x;
  const unsigned lt = lanemask_lt_g();
  const double lo[3] = {blo.x, blo.y, blo.z}, hi[3] = {bhi.x, bhi.y, bhi.z};
  int sptr = 1;
  if(lane == 0)
    stack[0] = 0;
  __syncwarp();
  while(sptr > 0) {
    const int k = sptr < 32 ? sptr : 32;
    const bool act = lane < k;
    const int node = act ? stack[sptr - 1 - lane] : 0;
    __syncwarp();
    sptr -= k;
    bool acc = false, open = false, leaf = false;
    int code = 0;
    if(act) {
      if(node < 0)
        leaf = true;
      else {
        const GravNode & g = G.gn[node];
        double dd = 0.0;
        for(int d = 0; d < dim; ++d) {
          const double e = fmax(0.0, fmax(lo[d] - g.c[d], g.c[d] - hi[d]));
          dd += e * e;
        }
        acc = dd > 0.0 && g.rmax * g.rmax < th2 * dd;
        open = !acc;
        code = T.qbox[2 * node + 1].w;
      }
    }
    const unsigned bo = __ballot_sync(GFULL, open);
    const int npush = 2 * __popc(bo);
    if(sptr + npush > GW_STACK) {
      if(lane == 0 && atomicCAS(&st->code, 0, (int)FSPH_ERR_STACK_OVERFLOW) == 0)
        st->index = -1;
      return;
    }
    if(open) {
      const int pos = sptr + 2 * __popc(bo & lt);
      const int split = code >> 2;
      stack[pos] = (code & 1) ? ~(split + 1) : split + 1;
      stack[pos + 1] = (code & 2) ? ~split : split;
    }
    sptr += npush;
    if(acc || leaf) {
      const unsigned long long slot = atomicAdd(count, 1ull);
      if(slot < (unsigned long long)cap) {
        double * r = cells + LET_REC * slot;
        if(acc) {
          const GravNode & g = G.gn[node];
          r[0] = g.m;
          for(int d = 0; d < 3; ++d)
            r[1 + d] = g.c[d];
          for(int q = 0; q < 6; ++q)
            r[4 + q] = order >= 2 ? g.q[q] : 0.0;
        }
        else {
          const int j = ~node;
          r[0] = P.f[F_M][j];
          r[1] = P.f[F_X][j];
          r[2] = P.f[F_Y][j];
          r[3] = dim == 3 ? P.f[F_Z][j] : 0.0;
          for(int q = 0; q < 6; ++q)
            r[4 + q] = 0.0;
        }
      }
    }
    __syncwarp();
  }
}

// Field of ncell cells on every particle, added to g-acceleration and
// potential: the multipole terms of the walk (monopole + traceless
// quadrupole), staged through shared memory in chunks.  FP64 mode in FP64;
// the mixed path in FP32 relative to a reference point per block (the
// block's first particle), with Kahan sums.  A cell at a particle's own
// position (distance 0) adds nothing.
#define LET_CHUNK 128
template<bool MIXED>
__global__ void __launch_bounds__(256) k_let_apply(Particles P, int dim,
  const double * cells, long long ncell, double Gc) {
  typedef typename std::conditional<MIXED, float, double>::type R;
  __shared__ R sc[LET_CHUNK][LET_REC];
  __shared__ double sref[3];
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = P.n;
  if(threadIdx.x == 0) {
    const int r = blockIdx.x * blockDim.x;
    for(int d = 0; d < 3; ++d)
      sref[d] = (MIXED && d < dim) ? P.f[F_X + d][r] : 0.0;
  }
  __syncthreads();
  R xa[3] = {0, 0, 0};
  if(a < n)
    for(int d = 0; d < dim; ++d)
      xa[d] = (R)(P.f[F_X + d][a] - sref[d]);
  R s[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
  for(long long c0 = 0; c0 < ncell; c0 += LET_CHUNK) {
    const int m = (int)(ncell - c0 < LET_CHUNK ? ncell - c0 : LET_CHUNK);
    __syncthreads();
    for(int t = threadIdx.x; t < m * LET_REC; t += blockDim.x) {
      const int k = t / LET_REC, f = t % LET_REC;
      double v = cells[LET_REC * (c0 + k) + f];
      if(f >= 1 && f <= 3)
        v -= sref[f - 1];
      sc[k][f] = (R)v;
    }
    __syncthreads();
    if(a >= n)
      continue;
    R p[4] = {0, 0, 0, 0};
    for(int k = 0; k < m; ++k) {
      const R mm = sc[k][0];
      const R dx = xa[0] - sc[k][1], dy = xa[1] - sc[k][2];
      const R dz = dim == 3 ? xa[2] - sc[k][3] : (R)0;
      const R r2 = dx * dx + dy * dy + dz * dz;
      if(!(r2 > (R)0))
        continue;
      const R ir = MIXED ? (R)rsqrtf((float)r2) : (R)rsqrt((double)r2);
      const R ir2 = ir * ir, ir3 = ir * ir2;
      R phi = -mm * ir;
      R fx = -mm * ir3 * dx, fy = -mm * ir3 * dy, fz = -mm * ir3 * dz;
      const R qxx = sc[k][4], qyy = sc[k][5], qzz = sc[k][6];
      const R qxy = sc[k][7], qxz = sc[k][8], qyz = sc[k][9];
      const R qdx = qxx * dx + qxy * dy + qxz * dz;
      const R qdy = qxy * dx + qyy * dy + qyz * dz;
      const R qdz = qxz * dx + qyz * dy + qzz * dz;
      const R dqd = dx * qdx + dy * qdy + dz * qdz;
      const R ir5 = ir3 * ir2, ir7 = ir5 * ir2;
      phi += (R)-0.5 * dqd * ir5;
      fx += qdx * ir5 - (R)2.5 * dqd * ir7 * dx;
      fy += qdy * ir5 - (R)2.5 * dqd * ir7 * dy;
      fz += qdz * ir5 - (R)2.5 * dqd * ir7 * dz;
      p[0] += fx;
      p[1] += fy;
      p[2] += fz;
      p[3] += phi;
    }
    for(int q = 0; q < 4; ++q)
      kahan_g(s[q], c[q], p[q]);
  }
  if(a >= n)
    return;
  for(int d = 0; d < dim; ++d)
    P.f[F_GAX + d][a] += ((double)s[d] - (double)c[d]) * Gc;
  P.f[F_GPOT][a] += ((double)s[3] - (double)c[3]) * Gc;
}

cudaError_t launch_let_export(const Launch & L, const Particles & P, int dim,
  const Tree & T, const GravBuffers & G, const double * blo, const double * bhi,
  double theta, int order, double * cells, long long cap,
  unsigned long long * count, DevStatus * st) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), L.stream);
  if(e != cudaSuccess)
    return e;
  const double3 lo = make_double3(blo[0], blo[1], dim == 3 ? blo[2] : 0.0);
  const double3 hi = make_double3(bhi[0], bhi[1], dim == 3 ? bhi[2] : 0.0);
  k_let_export<<<1, 32, 0, L.stream>>>(P, dim, T, G, lo, hi, theta * theta, order,
    cells, cap, count, st);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_let_apply(const Launch & L, const Particles & P, int dim,
  const double * cells, long long ncell, double Gc, int mixed) {
  if(P.n < 1 || ncell < 1)
    return cudaSuccess;
  const int nb = (P.n + 255) / 256;
  if(mixed)
    k_let_apply<true><<<nb, 256, 0, L.stream>>>(P, dim, cells, ncell, Gc);
  else
    k_let_apply<false><<<nb, 256, 0, L.stream>>>(P, dim, cells, ncell, Gc);
  *L.counter += 1;
  return cudaGetLastError();
}

cudaError_t launch_gravity(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, const GravBuffers & G,
  const unsigned long long * rbits, double theta, int order, int mixed,
  DevStatus * st, int nsm) {
  const int n = P.n;
  if(n < 2)  // a lone particle feels no force
    return cudaSuccess;
  k_grav_nodes<<<(n + 255) / 256, 256, 0, L.stream>>>(P, pp.dim, T, G, rbits, order);
  const size_t smem = (mixed ? gw_warp_bytes<true>() : gw_warp_bytes<false>()) * GW_WARPS;
  static std::atomic<unsigned long long> attr_devices{0};
  cudaError_t ae = once_per_device(&attr_devices, [&]() {
    cudaError_t e = cudaFuncSetAttribute(k_gravity_walk<true>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(gw_warp_bytes<true>() * GW_WARPS));
    if(e == cudaSuccess)
      e = cudaFuncSetAttribute(k_gravity_walk<false>,
        cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)(gw_warp_bytes<false>() * GW_WARPS));
    return e;
  });
  if(ae != cudaSuccess)
    return ae;
  int blocks = nsm * 4;
  const int maxb = (n + GW_WARPS * 32 - 1) / (GW_WARPS * 32) * 4;
  if(blocks > maxb)
    blocks = maxb > 0 ? maxb : 1;
  if(mixed)
    k_gravity_walk<true><<<blocks, GW_WARPS * 32, smem, L.stream>>>(P, T, G,
      (float)theta, pp.G, order, pp.dim, st);
  else
    k_gravity_walk<false><<<blocks, GW_WARPS * 32, smem, L.stream>>>(P, T, G,
      (float)theta, pp.G, order, pp.dim, st);
  *L.counter += 2;
  return cudaGetLastError();
}

}  // namespace fsph
