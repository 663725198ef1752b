// fsph_tree.cu -- range, Morton keys, radix sort, permutation, binary radix
// tree, particle groups and neighbour lists.
//
// Compiled with -fmad=false: the range, the key quantisation and the
// neighbour predicate must round exactly like the reference's FP64 code
// (no fused multiply-add), so keys, sort order and neighbour sets are
// bit-identical to the CPU reference.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "fsph_internal.cuh"

namespace fsph {

#define FULL 0xffffffffu

__device__ __forceinline__ unsigned long long ord_enc(double x) {
  long long b = __double_as_longlong(x);
  return b < 0 ? ~(unsigned long long)b
               : ((unsigned long long)b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dec(unsigned long long u) {
  return (u & 0x8000000000000000ull)
           ? __longlong_as_double((long long)(u & 0x7fffffffffffffffull))
           : __longlong_as_double((long long)~u);
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------- range --
// body_system::mpi_compute_range (mpisph/bodies_system.h:231-268): the
// bounding box of [x - h, x + h] over all particles, initialised from the
// last particle's coordinates.  min/max are exact in any order.
__global__ void k_range_init(Particles P, int dim, unsigned long long * bits) {
  int d = threadIdx.x;
  if(d < dim) {
    double x = P.f[F_X + d][P.n - 1];
    bits[d] = ord_enc(x);
    bits[3 + d] = ord_enc(x);
  }
  if(d == 0) {
    bits[6] = ord_enc(1e308);
    bits[7] = ord_enc(-1e308);
  }
}

__global__ void k_range_reduce(Particles P, int dim, unsigned long long * bits) {
  double lo[3] = {1e308, 1e308, 1e308}, hi[3] = {-1e308, -1e308, -1e308};
  double hmn = 1e308, hmx = -1e308;
  const double * H = P.f[F_H];
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
      i += gridDim.x * blockDim.x) {
    double h = H[i];
    hmn = fmin(hmn, h);
    hmx = fmax(hmx, h);
    for(int d = 0; d < dim; ++d) {
      double x = P.f[F_X + d][i];
      double a = x + h, b = x - h;
      hi[d] = a > hi[d] ? a : hi[d];
      lo[d] = b < lo[d] ? b : lo[d];
    }
  }
  for(int d = 0; d < dim; ++d) {
    for(int o = 16; o; o >>= 1) {
      double l2 = __shfl_xor_sync(FULL, lo[d], o);
      double h2 = __shfl_xor_sync(FULL, hi[d], o);
      lo[d] = l2 < lo[d] ? l2 : lo[d];
      hi[d] = h2 > hi[d] ? h2 : hi[d];
    }
    if((threadIdx.x & 31) == 0) {
      atomicMin(&bits[d], ord_enc(lo[d]));
      atomicMax(&bits[3 + d], ord_enc(hi[d]));
    }
  }
  for(int o = 16; o; o >>= 1) {
    hmn = fmin(hmn, __shfl_xor_sync(FULL, hmn, o));
    hmx = fmax(hmx, __shfl_xor_sync(FULL, hmx, o));
  }
  if((threadIdx.x & 31) == 0) {
    atomicMin(&bits[6], ord_enc(hmn));
    atomicMax(&bits[7], ord_enc(hmx));
  }
}

// Morton key, morton_curve_u(range, p) (filling_curve.h:503-525): bit i of
// the quantised coordinate j goes to bit D*i + j, above them the depth
// marker bit at D*max_depth.
__device__ __forceinline__ unsigned long long spread3(unsigned long long x) {
  x &= 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
__device__ __forceinline__ unsigned long long spread2(unsigned long long x) {
  x &= 0x7fffffffull;
  x = (x | x << 16) & 0x0000ffff0000ffffull;
  x = (x | x << 8) & 0x00ff00ff00ff00ffull;
  x = (x | x << 4) & 0x0f0f0f0f0f0f0f0full;
  x = (x | x << 2) & 0x3333333333333333ull;
  x = (x | x << 1) & 0x5555555555555555ull;
  return x;
}

__global__ void k_keys(Particles P, int dim, const unsigned long long * bits,
  unsigned long long * keys, int * idx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  const int md = 63 / dim;
  const unsigned long long maxv = (1ull << md) - 1;
  const double mult = (double)(1ull << md);
  unsigned long long c[3] = {0, 0, 0};
  for(int d = 0; d < dim; ++d) {
    double mn = ord_dec(bits[d]);
    double mx = ord_dec(bits[3 + d]);
    double scale = mx - mn;
    double q = (P.f[F_X + d][i] - mn) / scale * mult;
    unsigned long long u = q > 0.0 ? __double2ull_rz(q) : 0ull;
    c[d] = u < maxv ? u : maxv;
  }
  unsigned long long k;
  if(dim == 3)
    k = (1ull << 63) | spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
  else
    k = (1ull << 62) | spread2(c[0]) | (spread2(c[1]) << 1);
  keys[i] = k;
  idx[i] = i;
}

cudaError_t launch_range_keys(const Launch & L, const Particles & P,
  const PhysParams & pp, double * d_range, unsigned long long * keys_out,
  int * idx_out) {
  unsigned long long * bits = (unsigned long long *)d_range;
  k_range_init<<<1, 32, 0, L.stream>>>(P, pp.dim, bits);
  int nb = (P.n + 255) / 256;
  if(nb > 152 * 8)
    nb = 152 * 8;
  k_range_reduce<<<nb, 256, 0, L.stream>>>(P, pp.dim, bits);
  k_keys<<<(P.n + 255) / 256, 256, 0, L.stream>>>(P, pp.dim, bits, keys_out,
    idx_out);
  *L.counter += 3;
  return cudaGetLastError();
}

// ---------------------------------------------------------- radix sort --
// LSD radix sort of (key, value) pairs, 8-bit digits.  Tiles of 4096 keys:
// histogram per tile, one exclusive scan over [digit][tile], then a stable
// scatter in which each tile ranks its keys with warp match/ballot.
#define RS_THREADS 256
#define RS_ITEMS 16
#define RS_TILE (RS_THREADS * RS_ITEMS)

size_t radix_hist_entries(int n) {
  size_t nb = ((size_t)n + RS_TILE - 1) / RS_TILE;
  return 256 * nb;
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(
  const unsigned long long * keys, int n, int shift, unsigned * hist) {
  __shared__ unsigned sh[256];
  sh[threadIdx.x] = 0;
  __syncthreads();
  int base = blockIdx.x * RS_TILE;
  for(int r = 0; r < RS_ITEMS; ++r) {
    int i = base + r * RS_THREADS + threadIdx.x;
    if(i < n)
      atomicAdd(&sh[(keys[i] >> shift) & 255], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = sh[threadIdx.x];
}

// Exclusive scan of `m` counters by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_excl(unsigned * a, int m) {
  __shared__ unsigned part[1024];
  int per = (m + 1023) / 1024;
  int b0 = threadIdx.x * per;
  unsigned s = 0;
  for(int k = 0; k < per; ++k)
    if(b0 + k < m)
      s += a[b0 + k];
  part[threadIdx.x] = s;
  __syncthreads();
  for(int o = 1; o < 1024; o <<= 1) {
    unsigned v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = part[threadIdx.x] - s;
  for(int k = 0; k < per; ++k)
    if(b0 + k < m) {
      unsigned v = a[b0 + k];
      a[b0 + k] = run;
      run += v;
    }
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(
  const unsigned long long * kin, const int * vin, unsigned long long * kout,
  int * vout, int n, int shift, const unsigned * offs) {
  __shared__ unsigned base[256];
  __shared__ unsigned running[256];
  __shared__ unsigned wcnt[RS_THREADS / 32][256];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  base[t] = offs[t * gridDim.x + blockIdx.x];
  running[t] = 0;
  for(int k = 0; k < RS_THREADS / 32; ++k)
    wcnt[k][t] = 0;
  __syncthreads();
  const unsigned lt = lanemask_lt();
  const int tile = blockIdx.x * RS_TILE;
  for(int r = 0; r < RS_ITEMS; ++r) {
    int i = tile + r * RS_THREADS + t;
    bool valid = i < n;
    unsigned long long key = valid ? kin[i] : 0ull;
    int digit = valid ? (int)((key >> shift) & 255) : 256;
    unsigned mask = __match_any_sync(FULL, digit);
    int rank = __popc(mask & lt);
    bool leader = (__ffs(mask) - 1) == lane;
    if(valid && leader)
      wcnt[w][digit] = __popc(mask);
    __syncthreads();
    if(valid) {
      unsigned pre = running[digit];
      for(int k = 0; k < w; ++k)
        pre += wcnt[k][digit];
      unsigned pos = base[digit] + pre + rank;
      kout[pos] = key;
      vout[pos] = vin[i];
    }
    __syncthreads();
    unsigned s = 0;
    for(int k = 0; k < RS_THREADS / 32; ++k) {
      s += wcnt[k][t];
      wcnt[k][t] = 0;
    }
    running[t] += s;
    __syncthreads();
  }
}

cudaError_t radix_sort_pairs(const Launch & L, unsigned long long * keys,
  int * vals, unsigned long long * keys_tmp, int * vals_tmp, int n,
  unsigned * hist, int) {
  int nb = (n + RS_TILE - 1) / RS_TILE;
  unsigned long long *ka = keys, *kb = keys_tmp;
  int *va = vals, *vb = vals_tmp;
  for(int shift = 0; shift < 64; shift += 8) {
    k_radix_hist<<<nb, RS_THREADS, 0, L.stream>>>(ka, n, shift, hist);
    k_scan_excl<<<1, 1024, 0, L.stream>>>(hist, 256 * nb);
    k_radix_scatter<<<nb, RS_THREADS, 0, L.stream>>>(ka, va, kb, vb, n, shift,
      hist);
    *L.counter += 3;
    unsigned long long * tk = ka;
    ka = kb;
    kb = tk;
    int * tv = va;
    va = vb;
    vb = tv;
  }
  // eight passes: the result is back in (keys, vals)
  return cudaGetLastError();
}

// Two particles with one full key make the reference's build_tree loop run
// past depth 0 (tree_topology.h:957-971); report it instead.
__global__ void k_check_dups(const unsigned long long * keys, int n,
  DevStatus * st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i + 1 < n && keys[i] == keys[i + 1]) {
    if(atomicCAS(&st->code, 0, (int)FSPH_ERR_DUPLICATE_KEY) == 0)
      st->index = i;
  }
}

cudaError_t launch_check_duplicates(const Launch & L,
  const unsigned long long * keys, int n, DevStatus * st) {
  k_check_dups<<<(n + 255) / 256, 256, 0, L.stream>>>(keys, n, st);
  *L.counter += 1;
  return cudaGetLastError();
}

__global__ void k_permute(Particles src, Particles dst, const int * perm,
  const unsigned long long * keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= src.n)
    return;
  int p = perm[i];
#pragma unroll
  for(int k = 0; k < NF; ++k)
    dst.f[k][i] = src.f[k][p];
  dst.id[i] = src.id[p];
  dst.key[i] = keys[i];
}

cudaError_t launch_permute(const Launch & L, const Particles & src,
  const Particles & dst, const int * perm, const unsigned long long * keys) {
  k_permute<<<(src.n + 255) / 256, 256, 0, L.stream>>>(src, dst, perm, keys);
  *L.counter += 1;
  return cudaGetLastError();
}

// ------------------------------------------------------- radix tree -----
// Karras (2012) binary radix tree over the sorted, distinct keys.
// Equal keys (reported as FSPH_ERR_DUPLICATE_KEY) are ordered by index so
// the tree stays a valid binary tree and every walk over it terminates.
__device__ __forceinline__ int kdelta(const unsigned long long * k, int n,
  int i, int j) {
  if(j < 0 || j >= n)
    return -1;
  unsigned long long x = k[i] ^ k[j];
  return x ? __clzll(x) : 64 + __clz((unsigned)(i ^ j));
}

__global__ void k_karras(const unsigned long long * K, int n, Tree T) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n - 1)
    return;
  int d = (kdelta(K, n, i, i + 1) - kdelta(K, n, i, i - 1)) > 0 ? 1 : -1;
  int dmin = kdelta(K, n, i, i - d);
  int lmax = 2;
  while(kdelta(K, n, i, i + lmax * d) > dmin)
    lmax <<= 1;
  int l = 0;
  for(int t = lmax >> 1; t >= 1; t >>= 1)
    if(kdelta(K, n, i, i + (l + t) * d) > dmin)
      l += t;
  int j = i + l * d;
  int dnode = kdelta(K, n, i, j);
  int s = 0, t = l;
  while(true) {
    t = (t + 1) >> 1;
    if(kdelta(K, n, i, i + (s + t) * d) > dnode)
      s += t;
    if(t == 1)
      break;
  }
  int gamma = i + s * d + (d < 0 ? -1 : 0);
  int first = min(i, j), last = max(i, j);
  int left = (first == gamma) ? ~gamma : gamma;
  int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  T.left[i] = left;
  T.right[i] = right;
  T.first[i] = first;
  T.last[i] = last;
  if(left < 0)
    T.leaf_parent[gamma] = i;
  else
    T.parent[gamma] = i;
  if(right < 0)
    T.leaf_parent[gamma + 1] = i;
  else
    T.parent[gamma + 1] = i;
  if(i == 0)
    T.parent[0] = -1;
}

// Depth of each particle in the reference's octree: one level below its
// deepest shared prefix with a key neighbour (tree_topology.h:957-986).
__global__ void k_edepth(const unsigned long long * K, int n, int dim,
  unsigned char * ed) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  const int md = 63 / dim;
  const int lead = 64 - md * dim;
  int best = 0;
  if(i > 0)
    best = max(best, (__clzll(K[i] ^ K[i - 1]) - lead) / dim);
  if(i + 1 < n)
    best = max(best, (__clzll(K[i] ^ K[i + 1]) - lead) / dim);
  ed[i] = (unsigned char)(best + 1);
}

// Bottom-up bounding boxes of positions and the largest h per node.
__global__ void k_bounds(Particles P, int dim, Tree T) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  int p = T.leaf_parent[i];
  while(p >= 0) {
    __threadfence();
    if(atomicAdd(&T.counter[p], 1u) == 0)
      return;  // the sibling subtree is not finished yet
    NodeBox nb, n2;
    nb.hmax = 0;
    nb.pad = 0;
    n2.hmax = 0;
    n2.pad = 0;
    for(int d = 0; d < 3; ++d) {
      nb.lo[d] = n2.lo[d] = 1e308;
      nb.hi[d] = n2.hi[d] = -1e308;
    }
    int ch[2] = {T.left[p], T.right[p]};
    for(int c = 0; c < 2; ++c) {
      if(ch[c] < 0) {
        int j = ~ch[c];
        const double hj = P.f[F_H][j];
        for(int d = 0; d < dim; ++d) {
          double x = P.f[F_X + d][j];
          nb.lo[d] = fmin(nb.lo[d], x);
          nb.hi[d] = fmax(nb.hi[d], x);
          // compute_cofm's bmin/bmax (default_physics.h:79-82)
          n2.lo[d] = fmin(n2.lo[d], x - hj / 2.);
          n2.hi[d] = fmax(n2.hi[d], x + hj / 2.);
        }
        nb.hmax = fmax(nb.hmax, hj);
      }
      else {
        const double * cb = (const double *)&T.box[ch[c]];
        const double * cb2 = (const double *)&T.box2[ch[c]];
        for(int d = 0; d < dim; ++d) {
          nb.lo[d] = fmin(nb.lo[d], __ldcg(cb + d));
          nb.hi[d] = fmax(nb.hi[d], __ldcg(cb + 4 + d));
          n2.lo[d] = fmin(n2.lo[d], __ldcg(cb2 + d));
          n2.hi[d] = fmax(n2.hi[d], __ldcg(cb2 + 4 + d));
        }
        nb.hmax = fmax(nb.hmax, __ldcg(cb + 3));
      }
    }
    if(dim == 2) {
      nb.lo[2] = nb.hi[2] = 0;
      n2.lo[2] = n2.hi[2] = 0;
    }
    T.box[p] = nb;
    T.box2[p] = n2;
    __threadfence();
    p = T.parent[p];
  }
}

// Groups: maximal subtrees with at most `gmax` particles.
__global__ void k_groups(int n, Tree T, int gmax) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  int g = ~i;
  int p = T.leaf_parent[i];
  while(p >= 0 && T.last[p] - T.first[p] + 1 <= gmax) {
    g = p;
    p = T.parent[p];
  }
  int f = g < 0 ? i : T.first[g];
  int l = g < 0 ? i : T.last[g];
  if(f == i) {
    int slot = atomicAdd(T.ngroups, 1);
    T.group_first[slot] = f;
    T.group_last[slot] = l;
  }
}

// Level of a binary node in the reference's octree: the number of whole
// D-bit digits its keys share.
__device__ __forceinline__ int node_level(const unsigned long long * K,
  const Tree & T, int v, int dim, int lead) {
  return (__clzll(K[T.first[v]] ^ K[T.last[v]]) - lead) / dim;
}

// For each particle: the binary node whose range is its octree parent in
// the reference tree (the topmost binary ancestor of the same level), and
// the reference traversal group containing it -- the octree child of the
// first octree ancestor holding more than 128 particles
// (tree_topology.h:220-235, sub_entities_ = 128 at :2121).
__global__ void k_refgroups(const unsigned long long * K, int n, int dim,
  Tree T) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  const int lead = 64 - (63 / dim) * dim;
  int p = T.leaf_parent[i];
  int lp = node_level(K, T, p, dim, lead);
  int q = p;
  while(T.parent[q] >= 0 && node_level(K, T, T.parent[q], dim, lead) == lp)
    q = T.parent[q];
  T.opar[i] = q;
  int g = ~i;
  int u = p;
  while(u >= 0) {
    int up = T.parent[u];
    bool octree = up < 0 || node_level(K, T, u, dim, lead) > node_level(K, T, up, dim, lead);
    if(octree) {
      if(T.last[u] - T.first[u] + 1 > 128)
        break;
      g = u;
    }
    u = up;
  }
  T.gref[i] = g;
}

cudaError_t launch_build_tree(const Launch & L, const Particles & P,
  const PhysParams & pp, Tree & T, int group_max) {
  const int n = P.n;
  cudaMemsetAsync(T.counter, 0, sizeof(unsigned) * (size_t)n, L.stream);
  cudaMemsetAsync(T.ngroups, 0, sizeof(int), L.stream);
  k_karras<<<(n + 254) / 256, 256, 0, L.stream>>>(P.key, n, T);
  k_edepth<<<(n + 255) / 256, 256, 0, L.stream>>>(P.key, n, pp.dim, T.edepth);
  k_bounds<<<(n + 255) / 256, 256, 0, L.stream>>>(P, pp.dim, T);
  k_groups<<<(n + 255) / 256, 256, 0, L.stream>>>(n, T, group_max);
  k_refgroups<<<(n + 255) / 256, 256, 0, L.stream>>>(P.key, n, pp.dim, T);
  *L.counter += 5;
  return cudaGetLastError();
}

// ---------------------------------------------------- neighbour lists --
// One warp per group (<= 32 particles, lane = member).  The warp walks the
// radix tree with a shared-memory stack, up to 32 nodes per round (one per
// lane), pruning a node when its position box lies farther from the group's
// box than max(h_max(group), h_max(node)) -- a conservative bound, so no
// pair with d <= max(h_a, h_b) is lost.  Surviving particles are staged as
// candidates in shared memory, sorted by (reference octree depth, index)
// and then filtered by every member with the reference predicate
// (tree_geometry.h:265-276, as applied at tree_topology.h:372-379):
//     (dx*dx + dy*dy) + dz*dz <= max(h_a, h_b)^2   in FP64, no FMA.
// The candidate order makes each list come out in the order in which the
// reference's breadth-first walk appends neighbours (by depth, then key).
#define NB_WARPS 4
#define NB_STACK 1024
#define NB_CAND 2048

__device__ __forceinline__ void warp_bitonic(unsigned long long * a, int m,
  int lane) {
  int S = 32;
  while(S < m)
    S <<= 1;
  for(int i = m + lane; i < S; i += 32)
    a[i] = ~0ull;
  __syncwarp();
  for(int k = 2; k <= S; k <<= 1)
    for(int j = k >> 1; j > 0; j >>= 1) {
      for(int i = lane; i < S; i += 32) {
        int l = i ^ j;
        if(l > i) {
          unsigned long long x = a[i], y = a[l];
          bool up = (i & k) == 0;
          if((x > y) == up) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncwarp();
    }
}

// intersects_sphere_box (tree_geometry.h:329-341 in 3D, :219-227 in 2D)
__device__ __forceinline__ bool sphere_box(const double * b2, double c0,
  double c1, double c2, double r, int dim) {
  if(dim == 3) {
    double x0 = c0 < b2[4] ? c0 : b2[4];
    double x1 = c1 < b2[5] ? c1 : b2[5];
    double x2 = c2 < b2[6] ? c2 : b2[6];
    x0 = x0 < b2[0] ? b2[0] : x0;
    x1 = x1 < b2[1] ? b2[1] : x1;
    x2 = x2 < b2[2] ? b2[2] : x2;
    double dist = (x0 - c0) * (x0 - c0) + (x1 - c1) * (x1 - c1) +
                  (x2 - c2) * (x2 - c2);
    return dist <= r * r;
  }
  double y0 = b2[4] < c0 ? b2[4] : c0;
  double y1 = b2[5] < c1 ? b2[5] : c1;
  double x0 = b2[0] < y0 ? y0 : b2[0];
  double x1 = b2[1] < y1 ? y1 : b2[1];
  double sum = 0;
  sum += (x0 - c0) * (x0 - c0);
  sum += (x1 - c1) * (x1 - c1);
  return sqrt(sum) - r <= 2.220446049250313e-16 * 10.;
}

// intersects_box_box (tree_geometry.h:306-314, :201-207)
__device__ __forceinline__ bool box_box(const double * a, const double * b,
  int dim) {
  bool sep = a[4] < b[0] || a[5] < b[1] || b[4] < a[0] || b[5] < a[1];
  if(dim == 3)
    sep = sep || a[6] < b[2] || b[6] < a[2];
  return !sep;
}

// With varying h the reference's walk drops a candidate b of particle a
// unless the box of b's octree parent passes both node tests against a's
// traversal group G (tree_topology.h:323-355): box-box with G's box when G
// is a node, and sphere-box with at least one member of G.  Neither test
// can fail for a pair passing the predicate when every h is equal.
__device__ bool ref_node_tests(const Tree & T, const double * X,
  const double * Y, const double * Z, const double * H, int dim, int b,
  int a, double xa, double ya, double za, double ha, int gnode,
  const double * g2) {
  const double * b2 = (const double *)&T.box2[T.opar[b]];
  double bb[8];
  for(int k = 0; k < 8; ++k)
    bb[k] = b2[k];
  if(gnode >= 0 && !box_box(bb, g2, dim))
    return false;
  if(sphere_box(bb, xa, ya, za, ha, dim))
    return true;
  if(gnode < 0)
    return false;
  for(int k = T.first[gnode]; k <= T.last[gnode]; ++k) {
    if(k == a)
      continue;
    if(sphere_box(bb, X[k], Y[k], dim == 3 ? Z[k] : 0.0, H[k], dim))
      return true;
  }
  return false;
}

__global__ void __launch_bounds__(NB_WARPS * 32) k_neighbors(Particles P,
  Tree T, Lists Ls, DevStatus * st, int dim, const unsigned long long * rbits) {
  extern __shared__ unsigned long long smem_u64[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long * cand = smem_u64 + (size_t)w * NB_CAND;
  int * stack = (int *)(smem_u64 + (size_t)NB_WARPS * NB_CAND) + w * NB_STACK;
  const unsigned lt = lanemask_lt();
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const int ngroups = *T.ngroups;
  const int maxnb = Ls.maxnb;
  const bool nonuni = rbits[6] != rbits[7];
  for(int g = blockIdx.x * NB_WARPS + w; g < ngroups;
      g += gridDim.x * NB_WARPS) {
    const int gf = T.group_first[g], gl = T.group_last[g];
    const bool mem = lane <= gl - gf;
    const int a = gf + lane;
    double xa = 0, ya = 0, za = 0, ha = 0;
    if(mem) {
      xa = X[a];
      ya = Y[a];
      za = dim == 3 ? Z[a] : 0.0;
      ha = H[a];
    }
    int gnode = -1;
    double g2[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if(mem && nonuni) {
      gnode = T.gref[a];
      if(gnode >= 0) {
        const double * gp = (const double *)&T.box2[gnode];
        for(int k = 0; k < 8; ++k)
          g2[k] = gp[k];
      }
    }
    double lo0 = mem ? xa : 1e308, lo1 = mem ? ya : 1e308, lo2 = mem ? za : 1e308;
    double hi0 = mem ? xa : -1e308, hi1 = mem ? ya : -1e308,
           hi2 = mem ? za : -1e308;
    double hg = ha;
    for(int o = 16; o; o >>= 1) {
      lo0 = fmin(lo0, __shfl_xor_sync(FULL, lo0, o));
      lo1 = fmin(lo1, __shfl_xor_sync(FULL, lo1, o));
      lo2 = fmin(lo2, __shfl_xor_sync(FULL, lo2, o));
      hi0 = fmax(hi0, __shfl_xor_sync(FULL, hi0, o));
      hi1 = fmax(hi1, __shfl_xor_sync(FULL, hi1, o));
      hi2 = fmax(hi2, __shfl_xor_sync(FULL, hi2, o));
      hg = fmax(hg, __shfl_xor_sync(FULL, hg, o));
    }
    int cnt = 0;
    int sp = 1;
    int ncand = 0;
    bool chunked = false;
    if(lane == 0)
      stack[0] = 0;
    __syncwarp();
    while(sp > 0) {
      const int k = sp < 32 ? sp : 32;
      const bool act = lane < k;
      int node = act ? stack[sp - 1 - lane] : 0;
      __syncwarp();
      sp -= k;
      bool acc = false;
      const bool leaf = node < 0;
      if(act) {
        double blo0, blo1, blo2, bhi0, bhi1, bhi2, bh;
        if(!leaf) {
          const double4 * bp = (const double4 *)&T.box[node];
          double4 q0 = bp[0], q1 = bp[1];
          blo0 = q0.x; blo1 = q0.y; blo2 = q0.z; bh = q0.w;
          bhi0 = q1.x; bhi1 = q1.y; bhi2 = q1.z;
        }
        else {
          int j = ~node;
          blo0 = bhi0 = X[j];
          blo1 = bhi1 = Y[j];
          blo2 = bhi2 = dim == 3 ? Z[j] : 0.0;
          bh = H[j];
        }
        double s0 = fmax(0.0, fmax(blo0 - hi0, lo0 - bhi0));
        double s1 = fmax(0.0, fmax(blo1 - hi1, lo1 - bhi1));
        double s2 = fmax(0.0, fmax(blo2 - hi2, lo2 - bhi2));
        double R = fmax(hg, bh);
        double d2 = s0 * s0 + s1 * s1 + s2 * s2;
        acc = d2 <= R * R * (1.0 + 1e-10);
      }
      const unsigned bi = __ballot_sync(FULL, acc && !leaf);
      const unsigned bl = __ballot_sync(FULL, acc && leaf);
      const int npush = 2 * __popc(bi);
      if(sp + npush > NB_STACK) {
        if(lane == 0 && atomicCAS(&st->code, 0, (int)FSPH_ERR_STACK_OVERFLOW) == 0)
          st->index = gf;
        break;
      }
      if(acc && !leaf) {
        int pos = sp + 2 * __popc(bi & lt);
        stack[pos] = T.right[node];
        stack[pos + 1] = T.left[node];
      }
      sp += npush;
      if(acc && leaf) {
        int j = ~node;
        int pos = ncand + __popc(bl & lt);
        cand[pos] = ((unsigned long long)T.edepth[j] << 32) | (unsigned)j;
      }
      ncand += __popc(bl);
      __syncwarp();
      const bool last = (sp == 0);
      if(ncand > NB_CAND - 32 || (last && ncand > 0)) {
        if(!last)
          chunked = true;
        warp_bitonic(cand, ncand, lane);
        for(int c = 0; c < ncand; ++c) {
          const int b = (int)(cand[c] & 0xffffffffu);
          const double xb = X[b], yb = Y[b], hb = H[b];
          const double zb = dim == 3 ? Z[b] : 0.0;
          if(mem) {
            double dx = xa - xb, dy = ya - yb, dz = za - zb;
            double d2 = dx * dx + dy * dy;
            if(dim == 3)
              d2 = d2 + dz * dz;
            double r = ha < hb ? hb : ha;
            if(d2 <= r * r &&
               (!nonuni || ref_node_tests(T, X, Y, Z, H, dim, b, a, xa, ya, za,
                             ha, gnode, g2))) {
              if(cnt < maxnb)
                Ls.idx[list_slot(a, cnt, maxnb)] = b;
              ++cnt;
            }
          }
        }
        __syncwarp();
        ncand = 0;
      }
    }
    if(mem) {
      if(cnt > maxnb) {
        if(atomicCAS(&st->code, 0, (int)FSPH_ERR_LIST_OVERFLOW) == 0)
          st->index = a;
        cnt = maxnb;
      }
      Ls.cnt[a] = cnt;
    }
    if(chunked && lane == 0)
      atomicOr(&st->flags, FLAG_LIST_ORDER_CHUNKED);
  }
}

cudaError_t launch_neighbors(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, Lists & Ls, DevStatus * st, int nsm,
  const unsigned long long * rbits) {
  size_t smem = (size_t)NB_WARPS * NB_CAND * 8 + (size_t)NB_WARPS * NB_STACK * 4;
  static bool attr_set = false;
  if(!attr_set) {
    cudaFuncSetAttribute(k_neighbors, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
    attr_set = true;
  }
  int blocks = nsm * 4;
  int maxb = (P.n + NB_WARPS * 32 - 1) / (NB_WARPS * 32) * 8;
  if(blocks > maxb)
    blocks = maxb > 0 ? maxb : 1;
  k_neighbors<<<blocks, NB_WARPS * 32, smem, L.stream>>>(P, T, Ls, st,
    pp.dim, rbits);
  *L.counter += 1;
  return cudaGetLastError();
}

}  // namespace fsph

// ------------------------------------------- allocation-free key sort --
// Range, Morton keys and the radix sort of fsph_update_iteration for
// callers that must not allocate device memory themselves -- for example a
// host application whose device memory is owned by its own pool allocator,
// or a time-critical loop in which cudaMalloc/cudaFree (which may
// synchronise the device) are not acceptable.  Its scratch (range words,
// ping-pong keys and indices, digit histogram) is this file-scope array,
// sized for FSPH_NOALLOC_SORT_MAX particles: 12,845,312 bytes that every
// GPU loading the library holds until the process exits.
#define FSPH_NOALLOC_SORT_MAX (1 << 20)
#define NOALLOC_RANGE_BYTES 256
#define NOALLOC_KEYS_BYTES ((size_t)FSPH_NOALLOC_SORT_MAX * 8)
#define NOALLOC_VALS_BYTES ((size_t)FSPH_NOALLOC_SORT_MAX * 4)
#define NOALLOC_HIST_BYTES ((size_t)256 * (FSPH_NOALLOC_SORT_MAX / RS_TILE) * 4)
#define NOALLOC_TOTAL \
  (NOALLOC_RANGE_BYTES + NOALLOC_KEYS_BYTES + NOALLOC_VALS_BYTES + NOALLOC_HIST_BYTES)

namespace fsph {
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_TOTAL];
}  // namespace fsph

namespace {
// Device address of g_noalloc_scratch per device.  In host code the symbol
// names a host-side shadow, not device memory, so the address must come
// from cudaGetSymbolAddress, taken once per device with that device current.
std::mutex g_noalloc_mu;
void * g_noalloc_addr[64] = {};
}  // namespace

extern "C" fsph_status fsph_sort_keys_noalloc(const double * x,
  const double * y, const double * z, const double * h, int64_t n,
  int32_t dimension, uint64_t * keys_out, int32_t * perm_out, void * stream) {
  using namespace fsph;
  if(n < 2 || n > FSPH_NOALLOC_SORT_MAX || (dimension != 2 && dimension != 3) ||
     !x || !y || (dimension == 3 && !z) || !h || !keys_out || !perm_out)
    return FSPH_ERR_ARG;
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return FSPH_ERR_NO_DEVICE;
  void * base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if(!g_noalloc_addr[dev]) {
      void * ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if(e != cudaSuccess || !ptr)
        return FSPH_ERR_CUDA;
      g_noalloc_addr[dev] = ptr;
    }
    base = g_noalloc_addr[dev];
  }
  unsigned char * b = (unsigned char *)base;
  double * range = (double *)b;
  unsigned long long * ktmp = (unsigned long long *)(b + NOALLOC_RANGE_BYTES);
  int * vtmp = (int *)(b + NOALLOC_RANGE_BYTES + NOALLOC_KEYS_BYTES);
  unsigned * hist =
    (unsigned *)(b + NOALLOC_RANGE_BYTES + NOALLOC_KEYS_BYTES + NOALLOC_VALS_BYTES);
  Particles P{};
  P.f[F_X] = const_cast<double *>(x);
  P.f[F_Y] = const_cast<double *>(y);
  P.f[F_Z] = const_cast<double *>(z ? z : y);
  P.f[F_H] = const_cast<double *>(h);
  P.n = (int)n;
  PhysParams pp{};
  pp.dim = dimension;
  long long launches = 0;
  Launch L{(cudaStream_t)stream, &launches};
  // every scratch word that is read is first written by these launches: the
  // range words by k_range_init, the histogram by k_radix_hist per pass
  if(launch_range_keys(L, P, pp, range, (unsigned long long *)keys_out,
       perm_out) != cudaSuccess)
    return FSPH_ERR_CUDA;
  if(radix_sort_pairs(L, (unsigned long long *)keys_out, perm_out, ktmp, vtmp,
       (int)n, hist, 0) != cudaSuccess)
    return FSPH_ERR_CUDA;
  return FSPH_OK;
}

