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
//   upward pass (FP64, k_multipoles): mass, centre of mass, traceless
//     quadrupole Q_ij = sum m (3 x_i x_j - r^2 delta_ij) about it and the
//     radius of the bounding box seen from it, children combined bottom-up;
//   walk (k_gravity_walk): one warp per group of <= 32 particles; a cell is
//     accepted when r_max < theta * d_min, d_min being the distance from
//     its centre of mass to the group's box (so the test holds for every
//     member); accepted cells go to a shared-memory multipole list, leaves
//     of opened cells to a particle list; each lane then sums both lists
//     for its particle.
// The pair kernel is the reference's unsoftened Newtonian one
// (fmm.h:37-46): phi += -G m / r, a += -G m (x_a - x_b) / r^3, skipping the
// particle itself (fmm.h:136-137).  Results are added to g-acceleration
// and potential (the acceleration pass zeroes them first, as
// default_physics.h:406-407 does).  FP64 mode evaluates in FP64; the mixed
// path evaluates in FP32 relative to the group centre with Kahan sums while
// the multipoles stay FP64.
#include <cuda_runtime.h>

#include <type_traits>

#include "fsph_internal.cuh"

namespace fsph {

#define GW_WARPS 4
#define GW_STACK 1024
#define GW_MCAP 128
#define GW_PCAP 256
#define GFULL 0xffffffffu

__device__ __forceinline__ unsigned lanemask_lt_g() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------- up pass -----
__global__ void k_multipoles(Particles P, int dim, Tree T, GravNode * gn,
  double * gbox, unsigned * counter, int order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  int p = T.leaf_parent[i];
  while(p >= 0) {
    __threadfence();
    if(atomicAdd(&counter[p], 1u) == 0)
      return;
    double M = 0, C[3] = {0, 0, 0}, lo[3] = {1e308, 1e308, 1e308},
           hi[3] = {-1e308, -1e308, -1e308};
    double cm[2], cc[2][3], cq[2][6];
    const int ch[2] = {T.left[p], T.right[p]};
    for(int c = 0; c < 2; ++c) {
      if(ch[c] < 0) {
        const int j = ~ch[c];
        cm[c] = P.f[F_M][j];
        for(int d = 0; d < 3; ++d) {
          cc[c][d] = d < dim ? P.f[F_X + d][j] : 0.0;
          lo[d] = fmin(lo[d], cc[c][d]);
          hi[d] = fmax(hi[d], cc[c][d]);
        }
        for(int k = 0; k < 6; ++k)
          cq[c][k] = 0.0;
      }
      else {
        const GravNode * g = &gn[ch[c]];
        cm[c] = __ldcg(&g->m);
        for(int d = 0; d < 3; ++d) {
          cc[c][d] = __ldcg(&g->c[d]);
          lo[d] = fmin(lo[d], __ldcg(&gbox[6 * ch[c] + d]));
          hi[d] = fmax(hi[d], __ldcg(&gbox[6 * ch[c] + 3 + d]));
        }
        for(int k = 0; k < 6; ++k)
          cq[c][k] = __ldcg(&g->q[k]);
      }
      M += cm[c];
    }
    for(int d = 0; d < 3; ++d)
      C[d] = (cm[0] * cc[0][d] + cm[1] * cc[1][d]) / M;
    double Q[6] = {0, 0, 0, 0, 0, 0};
    if(order >= 2)
      for(int c = 0; c < 2; ++c) {
        // parallel-axis shift of the child's quadrupole to the new centre
        const double dx = cc[c][0] - C[0], dy = cc[c][1] - C[1], dz = cc[c][2] - C[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double m = cm[c];
        Q[0] += cq[c][0] + m * (3 * dx * dx - r2);
        Q[1] += cq[c][1] + m * (3 * dy * dy - r2);
        Q[2] += cq[c][2] + m * (3 * dz * dz - r2);
        Q[3] += cq[c][3] + m * 3 * dx * dy;
        Q[4] += cq[c][4] + m * 3 * dx * dz;
        Q[5] += cq[c][5] + m * 3 * dy * dz;
      }
    double rmax2 = 0;
    for(int k = 0; k < 8; ++k) {
      const double ex = ((k & 1) ? hi[0] : lo[0]) - C[0];
      const double ey = ((k & 2) ? hi[1] : lo[1]) - C[1];
      const double ez = ((k & 4) ? hi[2] : lo[2]) - C[2];
      rmax2 = fmax(rmax2, ex * ex + ey * ey + ez * ez);
    }
    GravNode out;
    out.m = M;
    for(int d = 0; d < 3; ++d)
      out.c[d] = C[d];
    for(int k = 0; k < 6; ++k)
      out.q[k] = Q[k];
    out.rmax = sqrt(rmax2);
    out.pad = 0;
    gn[p] = out;
    for(int d = 0; d < 3; ++d) {
      gbox[6 * p + d] = lo[d];
      gbox[6 * p + 3 + d] = hi[d];
    }
    __threadfence();
    p = T.parent[p];
  }
}

// ------------------------------------------------------------ the walk --
template<class R>
__device__ __forceinline__ void kahan_g(R & s, R & c, R t) {
  R y = t - c;
  R u = s + y;
  c = (u - s) - y;
  s = u;
}

template<bool MIXED>
__global__ void __launch_bounds__(GW_WARPS * 32) k_gravity_walk(Particles P,
  Tree T, const GravNode * gn, double theta, double G, int order, int dim,
  DevStatus * st) {
  typedef typename std::conditional<MIXED, float, double>::type R;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // particle rows: x, y, z, m (+ the low words of x, y, z in FP32)
  constexpr int PROWS = MIXED ? 7 : 4;
  const size_t per_warp = (size_t)GW_STACK * 4 + (size_t)GW_MCAP * 10 * sizeof(R) +
                          (size_t)GW_PCAP * PROWS * sizeof(R) + (size_t)GW_PCAP * 4;
  unsigned char * base = gsm + per_warp * w;
  int * stack = (int *)base;
  R * mm = (R *)(base + (size_t)GW_STACK * 4);
  R * pl = mm + GW_MCAP * 10;
  int * pidx = (int *)(pl + GW_PCAP * PROWS);
  const unsigned lt = lanemask_lt_g();
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * Mm = P.f[F_M];
  const int ngroups = *T.ngroups;
  const double th2 = theta * theta;
  for(int g = blockIdx.x * GW_WARPS + w; g < ngroups; g += gridDim.x * GW_WARPS) {
    const int gf = T.group_first[g], gl = T.group_last[g];
    const bool mem = lane <= gl - gf;
    const int a = gf + lane;
    double xa = mem ? X[a] : 0.0, ya = mem ? Y[a] : 0.0;
    double za = (mem && dim == 3) ? Z[a] : 0.0;
    double lo[3] = {mem ? xa : 1e308, mem ? ya : 1e308, mem ? za : 1e308};
    double hi[3] = {mem ? xa : -1e308, mem ? ya : -1e308, mem ? za : -1e308};
    for(int d = 0; d < 3; ++d)
      for(int o = 16; o; o >>= 1) {
        lo[d] = fmin(lo[d], __shfl_xor_sync(GFULL, lo[d], o));
        hi[d] = fmax(hi[d], __shfl_xor_sync(GFULL, hi[d], o));
      }
    const double gc[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]),
      0.5 * (lo[2] + hi[2])};
    // this particle relative to the group centre; in FP32 as a hi + lo pair
    // so that the separation of a close pair keeps its relative accuracy
    // (the FP32 rounding of each end alone would leave an absolute error of
    // the group's size times 2^-24 in it)
    const R ax = (R)(xa - gc[0]), ay = (R)(ya - gc[1]), az = (R)(za - gc[2]);
    const R axl = (R)((xa - gc[0]) - (double)ax), ayl = (R)((ya - gc[1]) - (double)ay);
    const R azl = (R)((za - gc[2]) - (double)az);
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
        GravNode gnd;
        if(act) {
          if(node < 0)
            leaf = true;
          else {
            gnd = gn[node];
            code = T.qbox[2 * node + 1].w;
            double dd = 0;
            for(int d = 0; d < 3; ++d) {
              const double e = fmax(0.0, fmax(lo[d] - gnd.c[d], gnd.c[d] - hi[d]));
              dd += e * e;
            }
            acc = dd > 0.0 && gnd.rmax * gnd.rmax < th2 * dd;
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
          mm[0 * GW_MCAP + pos] = (R)gnd.m;
          mm[1 * GW_MCAP + pos] = (R)(gnd.c[0] - gc[0]);
          mm[2 * GW_MCAP + pos] = (R)(gnd.c[1] - gc[1]);
          mm[3 * GW_MCAP + pos] = (R)(gnd.c[2] - gc[2]);
          for(int q = 0; q < 6; ++q)
            mm[(4 + q) * GW_MCAP + pos] = (R)gnd.q[q];
        }
        nm += __popc(ba);
        if(leaf) {
          const int j = ~node;
          const int pos = np + __popc(bl & lt);
          const double ex = X[j] - gc[0], ey = Y[j] - gc[1];
          const double ez = (dim == 3 ? Z[j] : 0.0) - gc[2];
          pl[0 * GW_PCAP + pos] = (R)ex;
          pl[1 * GW_PCAP + pos] = (R)ey;
          pl[2 * GW_PCAP + pos] = (R)ez;
          pl[3 * GW_PCAP + pos] = (R)Mm[j];
          if(MIXED) {
            pl[4 * GW_PCAP + pos] = (R)(ex - (double)(R)ex);
            pl[5 * GW_PCAP + pos] = (R)(ey - (double)(R)ey);
            pl[6 * GW_PCAP + pos] = (R)(ez - (double)(R)ez);
          }
          pidx[pos] = j;
        }
        np += __popc(bl);
        __syncwarp();
      }
      const bool flush_m = nm > GW_MCAP - 32 || (done && nm > 0);
      const bool flush_p = np > GW_PCAP - 32 || (done && np > 0);
      if(mem && flush_m) {
        for(int k = 0; k < nm; ++k) {
          const R m = mm[k], dx = ax - mm[GW_MCAP + k], dy = ay - mm[2 * GW_MCAP + k];
          const R dz = az - mm[3 * GW_MCAP + k];
          const R r2 = dx * dx + dy * dy + dz * dz;
          const R ir = MIXED ? (R)rsqrtf((float)r2) : (R)rsqrt((double)r2);
          const R ir2 = ir * ir;
          const R ir3 = ir * ir2;
          R phi = -m * ir;
          R fx = -m * ir3 * dx, fy = -m * ir3 * dy, fz = -m * ir3 * dz;
          if(order >= 2) {
            // phi_Q = -(1/2) d.Q.d / r^5,  a_Q = Q.d / r^5 - (5/2) (d.Q.d) d / r^7
            const R qxx = mm[4 * GW_MCAP + k], qyy = mm[5 * GW_MCAP + k];
            const R qzz = mm[6 * GW_MCAP + k], qxy = mm[7 * GW_MCAP + k];
            const R qxz = mm[8 * GW_MCAP + k], qyz = mm[9 * GW_MCAP + k];
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
          kahan_g(sx, cx, fx);
          kahan_g(sy, cy, fy);
          kahan_g(sz, cz, fz);
          kahan_g(sp, cp, phi);
        }
      }
      if(mem && flush_p) {
        for(int k = 0; k < np; ++k) {
          const int j = pidx[k];
          R dx = ax - pl[k], dy = ay - pl[GW_PCAP + k], dz = az - pl[2 * GW_PCAP + k];
          if(MIXED) {
            dx += axl - pl[4 * GW_PCAP + k];
            dy += ayl - pl[5 * GW_PCAP + k];
            dz += azl - pl[6 * GW_PCAP + k];
          }
          const R m = pl[3 * GW_PCAP + k];
          const R r2 = dx * dx + dy * dy + dz * dz;
          // the particle itself drops out (fmm.h:136-137)
          const R ir = j == a ? (R)0
                              : (MIXED ? (R)rsqrtf((float)r2) : (R)rsqrt((double)r2));
          const R w = m * ir;
          const R w3 = w * ir * ir;
          kahan_g(sx, cx, -w3 * dx);
          kahan_g(sy, cy, -w3 * dy);
          kahan_g(sz, cz, -w3 * dz);
          kahan_g(sp, cp, -w);
        }
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
      const double fx = ((double)sx - (double)cx) * G;
      const double fy = ((double)sy - (double)cy) * G;
      const double fz = ((double)sz - (double)cz) * G;
      P.f[F_GAX][a] += fx;
      P.f[F_GAY][a] += fy;
      if(dim == 3)
        P.f[F_GAZ][a] += fz;
      P.f[F_GPOT][a] += ((double)sp - (double)cp) * G;
    }
  }
}

cudaError_t launch_gravity(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, GravNode * gn, double * gbox,
  unsigned * counter, double theta, int order, int mixed, DevStatus * st,
  int nsm) {
  const int n = P.n;
  if(n < 2)  // a lone particle feels no force
    return cudaSuccess;
  cudaMemsetAsync(counter, 0, sizeof(unsigned) * (size_t)n, L.stream);
  k_multipoles<<<(n + 255) / 256, 256, 0, L.stream>>>(P, pp.dim, T, gn, gbox,
    counter, order);
  auto smem_of = [](size_t rs, int prows) {
    return ((size_t)GW_STACK * 4 + (size_t)GW_MCAP * 10 * rs +
            (size_t)GW_PCAP * prows * rs + (size_t)GW_PCAP * 4) * GW_WARPS;
  };
  const size_t smem = mixed ? smem_of(sizeof(float), 7) : smem_of(sizeof(double), 4);
  static bool attr = false;
  if(!attr) {
    cudaFuncSetAttribute(k_gravity_walk<true>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_of(sizeof(float), 7));
    cudaFuncSetAttribute(k_gravity_walk<false>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_of(sizeof(double), 4));
    attr = true;
  }
  const int blocks = nsm * 4;
  if(mixed)
    k_gravity_walk<true><<<blocks, GW_WARPS * 32, smem, L.stream>>>(P, T, gn,
      theta, pp.G, order, pp.dim, st);
  else
    k_gravity_walk<false><<<blocks, GW_WARPS * 32, smem, L.stream>>>(P, T, gn,
      theta, pp.G, order, pp.dim, st);
  *L.counter += 2;
  return cudaGetLastError();
}

}  // namespace fsph
