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

__device__ __forceinline__ unsigned long long umin64(unsigned long long a,
  unsigned long long b) {
  return b < a ? b : a;
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

// The comparisons run on the ordered integer encodings (the integer pipe);
// only x + h and x - h use the FP64 pipe, which is the bound of this
// kernel on a part with GB300's FP64 rate.
__global__ void __launch_bounds__(256) k_range_reduce(Particles P, int dim,
  unsigned long long * bits) {
  // v[k]: minima of the encodings of lo[0..2], h and of the complemented
  // encodings of hi[0..2], h (so that every slot is a minimum)
  unsigned long long v[8];
  for(int k = 0; k < 8; ++k)
    v[k] = ~0ull;
  const double * H = P.f[F_H];
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n;
      i += gridDim.x * blockDim.x) {
    const double h = H[i];
    const unsigned long long eh = ord_enc(h);
    v[6] = umin64(v[6], eh);
    v[7] = umin64(v[7], ~eh);
    for(int d = 0; d < dim; ++d) {
      const double x = P.f[F_X + d][i];
      v[d] = umin64(v[d], ord_enc(x - h));
      v[3 + d] = umin64(v[3 + d], ~ord_enc(x + h));
    }
  }
  // warp, then block, then one atomic per block and quantity
  __shared__ unsigned long long red[8][8];
  for(int k = 0; k < 8; ++k)
    for(int o = 16; o; o >>= 1)
      v[k] = umin64(v[k], __shfl_xor_sync(FULL, v[k], o));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if(lane == 0)
    for(int k = 0; k < 8; ++k)
      red[w][k] = v[k];
  __syncthreads();
  if(threadIdx.x < 8) {
    const int k = threadIdx.x;
    unsigned long long m = red[0][k];
    for(int q = 1; q < (int)(blockDim.x >> 5); ++q)
      m = umin64(m, red[q][k]);
    if(k < 3) {
      if(k < dim) atomicMin(&bits[k], m);
    }
    else if(k < 6) {
      if(k - 3 < dim) atomicMax(&bits[k], ~m);
    }
    else if(k == 6)
      atomicMin(&bits[6], m);
    else
      atomicMax(&bits[7], ~m);
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
  // the range and its reciprocal scaled by 2^md, once per block (FP64
  // division is costly at this part's FP64 rate)
  __shared__ double s_mn[3], s_scale[3], s_rs[3];
  const int md = 63 / dim;
  const double mult = (double)(1ull << md);
  if(threadIdx.x < dim) {
    const int d = threadIdx.x;
    const double mn = ord_dec(bits[d]);
    const double scale = ord_dec(bits[3 + d]) - mn;
    s_mn[d] = mn;
    s_scale[d] = scale;
    s_rs[d] = (1.0 / scale) * mult;
  }
  __syncthreads();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  const unsigned long long maxv = (1ull << md) - 1;
  unsigned long long c[3] = {0, 0, 0};
  for(int d = 0; d < dim; ++d) {
    const double mn = s_mn[d];
    const double scale = s_scale[d];
    const double t = P.f[F_X + d][i] - mn;
    // The reference quantises fl(t / scale) * 2^md (a power of two, exact).
    // t * (1 / scale) can differ from fl(t / scale) by an ulp, which moves
    // the integer part only when the scaled value lies within ~7e-7 of an
    // integer (2D: 2^31 scale); there the correctly rounded division decides.
    // Scaling by 2^md commutes with rounding, so t * ((1 / scale) * 2^md)
    // equals fl(t * (1 / scale)) * 2^md.
    double q = t * s_rs[d];
    const double fq = floor(q);
    if(q - fq < 1e-5 || q - fq > 1.0 - 1e-5)
      q = t / scale * mult;
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
#ifndef RS_ITEMS
#define RS_ITEMS 18
#endif
#define RS_TILE (RS_THREADS * RS_ITEMS)
// resident scatter blocks per SM (each holds its tile, 12 B a key, in
// shared memory)
#ifndef RS_SCATTER_BLOCKS
#define RS_SCATTER_BLOCKS 3
#endif

size_t radix_hist_entries(int n) {
  size_t nb = ((size_t)n + RS_TILE - 1) / RS_TILE;
  return 256 * nb + 256;  // [digit][tile] counts, then the 256 digit totals
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(
  const unsigned long long * keys, int n, int shift, unsigned * hist) {
  __shared__ unsigned sh[256];
  sh[threadIdx.x] = 0;
  __syncthreads();
  int base = blockIdx.x * RS_TILE;
  unsigned long long kreg[RS_ITEMS];
#pragma unroll
  for(int r = 0; r < RS_ITEMS; ++r) {
    const int i = base + r * RS_THREADS + threadIdx.x;
    kreg[r] = i < n ? keys[i] : 0ull;
  }
#pragma unroll
  for(int r = 0; r < RS_ITEMS; ++r) {
    const int i = base + r * RS_THREADS + threadIdx.x;
    if(i < n)
      atomicAdd(&sh[(kreg[r] >> shift) & 255], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = sh[threadIdx.x];
}

// Per digit: exclusive scan of its row of tile counts (coalesced, one
// block per digit) and the row total in tot[digit].
__global__ void __launch_bounds__(1024) k_scan_rows(unsigned * hist, int nb,
  unsigned * tot) {
  __shared__ unsigned wsum[32];
  const int d = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned * row = hist + (size_t)d * nb;
  unsigned run = 0;
  for(int base = 0; base < nb; base += 1024) {
    const int i = base + t;
    const unsigned v = i < nb ? row[i] : 0u;
    unsigned x = v;
    for(int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(FULL, x, o);
      if(lane >= o)
        x += y;
    }
    if(lane == 31)
      wsum[w] = x;
    __syncthreads();
    if(w == 0) {
      unsigned s2 = wsum[lane];
      for(int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(FULL, s2, o);
        if(lane >= o)
          s2 += y;
      }
      wsum[lane] = s2;
    }
    __syncthreads();
    const unsigned excl = run + (w ? wsum[w - 1] : 0u) + x - v;
    if(i < nb)
      row[i] = excl;
    run += wsum[31];
    __syncthreads();
  }
  if(t == 0)
    tot[d] = run;
}

// Stable scatter of one tile.  Warp w owns the tile's items
// [w * 32 * RS_ITEMS, (w + 1) * 32 * RS_ITEMS) and ranks them within their
// digits with a warp-private count per digit (match/ballot per round of 32
// keys, no block barrier); one scan per digit over the warps then gives
// every key its place in the tile sorted by digit (tile order kept), the
// tile is placed there in shared memory and written out in that order, so
// the keys of one digit leave the tile as one run of consecutive addresses.
#define RS_DYN_SMEM ((size_t)RS_TILE * 12)
__global__ void __launch_bounds__(RS_THREADS, RS_SCATTER_BLOCKS) k_radix_scatter(
  const unsigned long long * kin, const int * vin, unsigned long long * kout,
  int * vout, int n, int shift, const unsigned * offs) {
  extern __shared__ __align__(16) unsigned char rs_dyn[];
  unsigned long long * skey = (unsigned long long *)rs_dyn;
  int * sval = (int *)(rs_dyn + (size_t)RS_TILE * 8);
  __shared__ unsigned base[256];   // where the tile's run of each digit goes
  __shared__ unsigned toff[256];   // where each digit starts in the sorted tile
  __shared__ unsigned wcnt[RS_THREADS / 32][256];
  __shared__ unsigned wtot[RS_THREADS / 32];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  // exclusive block scan of one value per thread (256 threads)
  auto block_scan = [&](unsigned v) {
    unsigned x = v;
    for(int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(FULL, x, o);
      if(lane >= o)
        x += y;
    }
    if(lane == 31)
      wtot[w] = x;
    __syncthreads();
    unsigned pre = 0;
    for(int k = 0; k < w; ++k)
      pre += wtot[k];
    __syncthreads();
    return pre + x - v;
  };
  // digit base = sum of the totals of smaller digits + this tile's offset
  // within its digit row
  base[t] = block_scan(offs[256 * gridDim.x + t]) + offs[t * gridDim.x + blockIdx.x];
  for(int k = 0; k < RS_THREADS / 32; ++k)
    wcnt[k][t] = 0;
  // this warp's keys into registers first: all loads in flight (the
  // values follow when the keys are placed)
  const int tile = blockIdx.x * RS_TILE;
  const int wbase = tile + w * 32 * RS_ITEMS;
  unsigned long long kreg[RS_ITEMS];
#pragma unroll
  for(int r = 0; r < RS_ITEMS; ++r) {
    const int i = wbase + r * 32 + lane;
    kreg[r] = i < n ? kin[i] : 0ull;
  }
  __syncthreads();
  const unsigned lt = lanemask_lt();
  unsigned * cnt = wcnt[w];
  unsigned rk[RS_ITEMS];  // digit << 16 | rank within the digit in this warp
#pragma unroll
  for(int r = 0; r < RS_ITEMS; ++r) {
    const bool valid = wbase + r * 32 + lane < n;
    const int digit = valid ? (int)((kreg[r] >> shift) & 255) : 256;
    const unsigned mask = __match_any_sync(FULL, digit);
    const unsigned before = valid ? cnt[digit] : 0u;
    __syncwarp();
    if(valid && (__ffs(mask) - 1) == lane)
      cnt[digit] = before + __popc(mask);
    __syncwarp();
    rk[r] = ((unsigned)(valid ? digit : 0) << 16) | (before + __popc(mask & lt));
  }
  __syncthreads();
  // per digit (thread t): exclusive prefix over the warps, then the start of
  // the digit in the sorted tile
  unsigned run = 0;
  for(int k = 0; k < RS_THREADS / 32; ++k) {
    const unsigned c = wcnt[k][t];
    wcnt[k][t] = run;
    run += c;
  }
  toff[t] = block_scan(run);
  __syncthreads();
#pragma unroll
  for(int r = 0; r < RS_ITEMS; ++r) {
    const int i = wbase + r * 32 + lane;
    if(i < n) {
      const unsigned d = rk[r] >> 16;
      const unsigned l = toff[d] + cnt[d] + (rk[r] & 0xffffu);
      skey[l] = kreg[r];
      sval[l] = vin[i];
    }
  }
  __syncthreads();
  const int ntile = n - tile < RS_TILE ? n - tile : RS_TILE;
  for(int l = t; l < ntile; l += RS_THREADS) {
    const unsigned long long key = skey[l];
    const int d = (int)((key >> shift) & 255);
    const unsigned pos = base[d] + ((unsigned)l - toff[d]);
    kout[pos] = key;
    vout[pos] = sval[l];
  }
}

cudaError_t radix_sort_pairs(const Launch & L, unsigned long long * keys,
  int * vals, unsigned long long * keys_tmp, int * vals_tmp, int n,
  unsigned * hist, int) {
  static std::atomic<unsigned long long> attr_devices{0};
  cudaError_t ae = once_per_device(&attr_devices, []() {
    return cudaFuncSetAttribute(k_radix_scatter,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_DYN_SMEM);
  });
  if(ae != cudaSuccess)
    return ae;
  int nb = (n + RS_TILE - 1) / RS_TILE;
  unsigned long long *ka = keys, *kb = keys_tmp;
  int *va = vals, *vb = vals_tmp;
  for(int shift = 0; shift < 64; shift += 8) {
    k_radix_hist<<<nb, RS_THREADS, 0, L.stream>>>(ka, n, shift, hist);
    k_scan_rows<<<256, 1024, 0, L.stream>>>(hist, nb, hist + (size_t)256 * nb);
    k_radix_scatter<<<nb, RS_THREADS, RS_DYN_SMEM, L.stream>>>(ka, va, kb, vb, n,
      shift, hist);
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

// Fields whose bit is set in `skip` are left behind: the caller overwrites
// them before anything reads them.  With `vel`, the mixed path's
// {v, c_s} record of the new order is written on the way (what the density
// pass would otherwise pack).
__global__ void k_permute(Particles src, Particles dst, const int * perm,
  const unsigned long long * keys, unsigned skip, float4 * vel, int dim) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= src.n)
    return;
  int p = perm[i];
#pragma unroll
  for(int k = 0; k < NF; ++k)
    if(!((skip >> k) & 1u))
      dst.f[k][i] = src.f[k][p];
  dst.id[i] = src.id[p];
  dst.key[i] = keys[i];
  if(vel)
    vel[i] = make_float4((float)src.f[F_VX][p], (float)src.f[F_VY][p],
      dim == 3 ? (float)src.f[F_VZ][p] : 0.f, (float)src.f[F_CS][p]);
}

cudaError_t launch_permute(const Launch & L, const Particles & src,
  const Particles & dst, const int * perm, const unsigned long long * keys,
  unsigned skip, float4 * vel, int dim) {
  k_permute<<<(src.n + 255) / 256, 256, 0, L.stream>>>(src, dst, perm, keys, skip, vel,
    dim);
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

// Bottom-up node data: the fixed-point position box and the largest h of
// every node (what the neighbour walk prunes with); only when h varies, the
// reference's FP64 box of x -/+ h/2 (compute_cofm, default_physics.h:
// 79-82,90-93) used by the reference node tests; only with gravity, the
// node's raw mass moments (ten FP64 sums: children add, so every level
// costs ten additions whatever the order of the multipoles built from
// them).
// refboxes: also the reference's x +- h/2 node boxes (box2, fbox2), which
// the walk's node tests read: with varying h, or in the ordered (FP64) mode
// where equal-h ties take them too.
// Shared-memory layout of one k_bounds_* block (dynamic): the node data of the
// internal nodes whose leaf range lies inside the block's own leaves (slot =
// node index - first leaf of the block: such a node's index is one end of
// its range), their arrival counters, two work queues and the list of the
// block's topmost nodes (and leaves) whose parents lie outside it.
#define BOUNDS_THREADS 256
__host__ __device__ constexpr size_t bounds_smem(bool gmom) {
  return (size_t)BOUNDS_THREADS * (2 * sizeof(int4) + 6 * sizeof(double) + sizeof(unsigned) +
                                   3 * sizeof(int) + (gmom ? 10 * sizeof(double) : 0)) +
         4 * sizeof(int);
}

struct BoundsShared {
  int4 * sq;        // lo, hi per slot
  double * sb;      // box2 lo xyz, hi xyz per slot
  unsigned * scnt;  // arrival counts per slot
  int * queue;      // 2 x 256: nodes whose two children are done (current pass, next pass)
  int * exits;      // nodes (~leaf for a leaf) whose parent is outside the block
  int * counts;     // queue lengths [2], exit count
  double * sg;      // ten moments per slot (gravity)
};

// Node p's data from its two children, written to device memory and, for a
// node inside the block (local), to its shared-memory slot.  A local node's
// inner children are local too and are read from shared memory; the
// children of other nodes from device memory through L2.  Children combine
// in a fixed order (left, then right), so the sums do not depend on which
// thread or path combined a node.
template<int dim>
__device__ __forceinline__ void bounds_node(const Particles & P, const Tree & T, const int4 * qpos,
  const BoundsShared & S, int p, bool local, int b0, bool nonuni, const double * rc,
  const double * r0) {
  const int cg[2] = {T.left[p], T.right[p]};
  if(T.gmom) {
    double M[10];
    for(int c = 0; c < 2; ++c) {
      double C[10];
      if(cg[c] < 0) {
        const int j = ~cg[c];
        const double m = P.f[F_M][j];
        double y[3] = {0.0, 0.0, 0.0};
        for(int d = 0; d < dim; ++d)
          y[d] = P.f[F_X + d][j] - rc[d];
        const double my[3] = {m * y[0], m * y[1], m * y[2]};
        C[0] = m;
        C[1] = my[0];
        C[2] = my[1];
        C[3] = my[2];
        C[4] = my[0] * y[0];
        C[5] = my[1] * y[1];
        C[6] = my[2] * y[2];
        C[7] = my[0] * y[1];
        C[8] = my[0] * y[2];
        C[9] = my[1] * y[2];
      }
      else if(local) {
        const double * cs = S.sg + (cg[c] - b0);
        for(int k = 0; k < 10; ++k)
          C[k] = cs[k * BOUNDS_THREADS];
      }
      else {
        const double * cs = T.gmom + 10 * (size_t)cg[c];
        for(int k = 0; k < 10; ++k)
          C[k] = __ldcg(cs + k);
      }
      for(int k = 0; k < 10; ++k)
        M[k] = c == 0 ? C[k] : M[k] + C[k];
    }
    double * out = T.gmom + 10 * (size_t)p;
    for(int k = 0; k < 10; ++k)
      out[k] = M[k];
    if(local)
      for(int k = 0; k < 10; ++k)
        S.sg[k * BOUNDS_THREADS + (p - b0)] = M[k];
  }
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff};
  int hi[3] = {-1, -1, -1};
  float hm = 0.f;
  double blo[3] = {1e308, 1e308, 1e308}, bhi[3] = {-1e308, -1e308, -1e308};
  for(int c = 0; c < 2; ++c) {
    if(cg[c] < 0) {
      const int j = ~cg[c];
      const int4 q = qpos[j];
      lo[0] = min(lo[0], q.x); hi[0] = max(hi[0], q.x);
      lo[1] = min(lo[1], q.y); hi[1] = max(hi[1], q.y);
      lo[2] = min(lo[2], q.z); hi[2] = max(hi[2], q.z);
      hm = fmaxf(hm, __int_as_float(q.w));
      if(nonuni) {
        const double hj = P.f[F_H][j];
        for(int d = 0; d < dim; ++d) {
          double x = P.f[F_X + d][j];
          blo[d] = fmin(blo[d], x - hj / 2.);
          bhi[d] = fmax(bhi[d], x + hj / 2.);
        }
      }
    }
    else {
      int4 a, b;
      if(local) {
        a = S.sq[2 * (cg[c] - b0)];
        b = S.sq[2 * (cg[c] - b0) + 1];
      }
      else {
        const int4 * cq = &T.qbox[2 * cg[c]];
        a = __ldcg(cq);
        b = __ldcg(cq + 1);
      }
      lo[0] = min(lo[0], a.x); lo[1] = min(lo[1], a.y); lo[2] = min(lo[2], a.z);
      hi[0] = max(hi[0], b.x); hi[1] = max(hi[1], b.y); hi[2] = max(hi[2], b.z);
      hm = fmaxf(hm, __int_as_float(a.w));
      if(nonuni) {
        if(local) {
          const double * cb2 = S.sb + (cg[c] - b0);
          for(int d = 0; d < dim; ++d) {
            blo[d] = fmin(blo[d], cb2[d * BOUNDS_THREADS]);
            bhi[d] = fmax(bhi[d], cb2[(3 + d) * BOUNDS_THREADS]);
          }
        }
        else {
          const double * cb2 = (const double *)&T.box2[cg[c]];
          for(int d = 0; d < dim; ++d) {
            blo[d] = fmin(blo[d], __ldcg(cb2 + d));
            bhi[d] = fmax(bhi[d], __ldcg(cb2 + 4 + d));
          }
        }
      }
    }
  }
  // children of a radix-tree node are always (split, split + 1): store
  // split and the two leaf flags with the box, so the walk needs one load
  const int l = cg[0], r = cg[1];
  const int split = l < 0 ? ~l : l;
  const int code = (split << 2) | ((l < 0) << 1) | (r < 0);
  const int4 qlo = make_int4(lo[0], lo[1], lo[2], __float_as_int(hm));
  const int4 qhi = make_int4(hi[0], hi[1], hi[2], code);
  T.qbox[2 * p] = qlo;
  T.qbox[2 * p + 1] = qhi;
  if(local) {
    S.sq[2 * (p - b0)] = qlo;
    S.sq[2 * (p - b0) + 1] = qhi;
  }
  if(nonuni) {
    if(dim == 2)
      blo[2] = bhi[2] = 0;
    // NodeBox: lo xyz, hmax (0), hi xyz, pad (0)
    double4 * bx = (double4 *)&T.box2[p];
    bx[0] = make_double4(blo[0], blo[1], blo[2], 0.0);
    bx[1] = make_double4(bhi[0], bhi[1], bhi[2], 0.0);
    if(local)
      for(int d = 0; d < 3; ++d) {
        S.sb[d * BOUNDS_THREADS + (p - b0)] = blo[d];
        S.sb[(3 + d) * BOUNDS_THREADS + (p - b0)] = bhi[d];
      }
    float fl[3] = {0.f, 0.f, 0.f}, fh[3] = {0.f, 0.f, 0.f};
    for(int d = 0; d < dim; ++d) {
      fl[d] = __double2float_rd(blo[d] - r0[d]);
      fh[d] = __double2float_ru(bhi[d] - r0[d]);
    }
    T.fbox2[2 * p] = make_float4(fl[0], fl[1], fl[2], 0.f);
    T.fbox2[2 * p + 1] = make_float4(fh[0], fh[1], fh[2], 0.f);
  }
}

__device__ __forceinline__ BoundsShared bounds_shared(unsigned char * bsm) {
  BoundsShared S;
  S.sq = (int4 *)bsm;
  S.sb = (double *)(S.sq + 2 * BOUNDS_THREADS);
  S.scnt = (unsigned *)(S.sb + 6 * BOUNDS_THREADS);
  S.queue = (int *)(S.scnt + BOUNDS_THREADS);
  S.exits = S.queue + 2 * BOUNDS_THREADS;
  S.counts = S.exits + BOUNDS_THREADS;
  S.sg = (double *)(S.counts + 4);
  return S;
}

// The bottom-up pass comes in two variants; both are launched and the one
// the run does not select returns at once.
//
// With gravity or varying h (FP64 moments and x +- h/2 boxes per node):
// inside a block (its 256 leaves), rounds separated by block barriers, each
// combining the nodes whose two children finished in earlier rounds, taken
// from a compacted queue so that whole warps do the FP64 node arithmetic (a
// thread per leaf climbing the tree keeps ~1/3 of its lanes busy, and the
// FP64 pipe, not the lanes, is what the node arithmetic waits on); a
// shared-memory count per node finds the round in which its second child
// finishes.  Above the block -- nodes whose range straddles a block
// boundary, a few per block -- the classic chain: the thread arriving second
// at a node (a device-scope acquire-release count) combines it and climbs
// on.  4M polytrope: 5.03 -> 2.84 ms per tree phase.  One block per 256
// leaves: a smaller grid striding over the leaf blocks (so that equal-h runs
// skip the variant in one wave) measured 4.30 ms, as each block's climb
// above its leaves then holds back its next leaves.
//
// Equal h without gravity (integer boxes only): the chain from every leaf,
// with the counts and node data of the nodes inside the block in shared
// memory (block-scope fences order them); there the barriers of the round
// variant cost more than the idle lanes (Sedov 128^3 tree phase 0.48 ms
// against 0.58).
template<int dim>
__global__ void __launch_bounds__(BOUNDS_THREADS) k_bounds_chain(Particles P, Tree T,
  const int4 * qpos, const unsigned long long * rbits, int refboxes) {
  if(T.gmom || refboxes || rbits[6] != rbits[7])
    return;  // the round variant's run
  extern __shared__ __align__(16) unsigned char bsm[];
  const BoundsShared S = bounds_shared(bsm);
  const int b0 = blockIdx.x * BOUNDS_THREADS;
  const int b1 = min(b0 + BOUNDS_THREADS, P.n) - 1;
  S.scnt[threadIdx.x] = 0u;
  __syncthreads();
  const int i = b0 + threadIdx.x;
  if(i >= P.n)
    return;
  const double rc[3] = {0.0, 0.0, 0.0}, r0[3] = {0.0, 0.0, 0.0};
  int p = T.leaf_parent[i];
  while(p >= 0) {
    const bool local = T.first[p] >= b0 && T.last[p] <= b1;
    unsigned prior;
    if(local) {
      // shared-memory count at block scope: the fences order this thread's
      // node data before the count (release) and the sibling's after it
      // (acquire)
      __threadfence_block();
      prior = atomicAdd(&S.scnt[p - b0], 1u);
      __threadfence_block();
    }
    else {
      // device-scope acquire-release count: publishes this thread's node
      // data (release) to the sibling's thread, which reads it after its
      // own arrival (acquire; the reads go through L2 with __ldcg)
      asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], 1;"
                   : "=r"(prior) : "l"(T.counter + p) : "memory");
    }
    if(prior == 0)
      return;  // the sibling subtree is not finished yet
    bounds_node<dim>(P, T, qpos, S, p, local, b0, false, rc, r0);
    p = T.parent[p];
  }
}

template<int dim>
__global__ void __launch_bounds__(BOUNDS_THREADS) k_bounds_rounds(Particles P, Tree T,
  const int4 * qpos, const unsigned long long * rbits, int refboxes) {
  const bool nonuni = refboxes || rbits[6] != rbits[7];
  if(!T.gmom && !nonuni)
    return;  // the chain variant's run
  extern __shared__ __align__(16) unsigned char bsm[];
  const BoundsShared S = bounds_shared(bsm);
  const int t = threadIdx.x;
  const int b0 = blockIdx.x * BOUNDS_THREADS;
  const int b1 = min(b0 + BOUNDS_THREADS, P.n) - 1;
  S.scnt[t] = 0u;
  if(t < 4)
    S.counts[t] = 0;
  double rc[3] = {0.0, 0.0, 0.0}, r0[3] = {0.0, 0.0, 0.0};
  for(int d = 0; d < dim; ++d) {
    r0[d] = ord_dec(rbits[d]);
    if(T.gmom)
      rc[d] = 0.5 * (r0[d] + ord_dec(rbits[3 + d]));
  }
  auto is_local = [&](int v) { return T.first[v] >= b0 && T.last[v] <= b1; };
  // a node (or ~leaf) whose data are final: count its arrival at the parent
  auto arrive = [&](int v, int next) {
    const int p = v < 0 ? T.leaf_parent[~v] : T.parent[v];
    if(p < 0)
      return;
    if(is_local(p)) {
      if(atomicAdd(&S.scnt[p - b0], 1u) == 1u)
        S.queue[next * BOUNDS_THREADS + atomicAdd(&S.counts[next], 1)] = p;
    }
    else
      S.exits[atomicAdd(&S.counts[2], 1)] = v;
  };
  __syncthreads();
  if(b0 + t <= b1)
    arrive(~(b0 + t), 0);
  __syncthreads();
  for(int cur = 0;; cur ^= 1) {
    const int len = S.counts[cur];
    if(len == 0)
      break;
    __syncthreads();  // every thread has read len
    if(t == 0)
      S.counts[cur] = 0;  // the queue after next reuses this one
    if(t < len) {
      const int p = S.queue[cur * BOUNDS_THREADS + t];
      bounds_node<dim>(P, T, qpos, S, p, true, b0, nonuni, rc, r0);
      arrive(p, cur ^ 1);
    }
    __syncthreads();
  }
  const int nex = S.counts[2];
  if(nex == 0)
    return;
  // the exits' data (written by any thread of the block before the last
  // barrier) become visible device-wide before this thread's counts
  __threadfence();
  for(int e = t; e < nex; e += BOUNDS_THREADS) {
    const int v = S.exits[e];
    int p = v < 0 ? T.leaf_parent[~v] : T.parent[v];
    while(p >= 0) {
      unsigned prior;
      asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], 1;"
                   : "=r"(prior) : "l"(T.counter + p) : "memory");
      if(prior == 0)
        break;  // the sibling subtree is not finished yet
      bounds_node<dim>(P, T, qpos, S, p, false, b0, nonuni, rc, r0);
      p = T.parent[p];
    }
  }
}

// Groups: maximal subtrees with at most `gmax` particles.  Each group also
// gets the node its mixed walk starts from: the lowest ancestor whose
// fixed-point box, less one step on every side, holds the group's box grown
// by the largest reach (max h, with the walk's 1e-5 slack and two steps for
// the quantisation).  A radix-tree node holds every particle whose key
// shares its prefix, so its particles' box lies in that Morton cell; a
// particle within reach lies in the grown box, hence a step inside the
// node's box, hence in the cell and in the subtree: the walk below that
// node finds every candidate the walk from the root finds.
__global__ void k_groups(int n, Tree T, int gmax, int dim, const float * qscale,
  const unsigned long long * rbits) {
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
    // (a one-particle group walks from the root)
    int v = 0;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if(g >= 0) {
      const int4 glo = T.qbox[2 * g], ghi = T.qbox[2 * g + 1];
      const int gl[3] = {glo.x, glo.y, glo.z}, gh[3] = {ghi.x, ghi.y, ghi.z};
      const float R = (float)ord_dec(rbits[7]) * 1.00001f;
      for(int d = 0; d < dim; ++d) {
        const int r = (int)ceilf(R / qscale[d]) + 2;
        lo[d] = gl[d] - r;
        hi[d] = gh[d] + r;
      }
      v = T.parent[g];
    }
    while(v > 0) {
      const int4 a = T.qbox[2 * v], b = T.qbox[2 * v + 1];
      const int al[3] = {a.x, a.y, a.z}, bh[3] = {b.x, b.y, b.z};
      bool in = true;
      for(int d = 0; d < dim; ++d)
        in = in && al[d] + 1 <= lo[d] && bh[d] - 1 >= hi[d];
      if(in)
        break;
      v = T.parent[v];
    }
    T.group_start[slot] = v < 0 ? 0 : v;
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
  Tree T, const unsigned long long * rbits, int refboxes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  // read only when h varies, or for ties in the ordered mode
  if(i >= n || (!refboxes && rbits[6] == rbits[7]))
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
  const PhysParams & pp, Tree & T, int group_max,
  const unsigned long long * rbits, const int4 * qpos, const float * qscale,
  int ordered) {
  const int n = P.n;
  cudaMemsetAsync(T.counter, 0, sizeof(unsigned) * (size_t)n, L.stream);
  cudaMemsetAsync(T.ngroups, 0, sizeof(int), L.stream);
  k_karras<<<(n + 254) / 256, 256, 0, L.stream>>>(P.key, n, T);
  if(ordered)  // reference octree depths order the FP64 lists
    k_edepth<<<(n + 255) / 256, 256, 0, L.stream>>>(P.key, n, pp.dim, T.edepth);
  const int nbb = (n + BOUNDS_THREADS - 1) / BOUNDS_THREADS;
  const size_t bsm = bounds_smem(T.gmom != nullptr);
  if(pp.dim == 3) {
    k_bounds_chain<3><<<nbb, BOUNDS_THREADS, bsm, L.stream>>>(P, T, qpos, rbits, ordered);
    k_bounds_rounds<3><<<nbb, BOUNDS_THREADS, bsm, L.stream>>>(P, T, qpos, rbits, ordered);
  }
  else {
    k_bounds_chain<2><<<nbb, BOUNDS_THREADS, bsm, L.stream>>>(P, T, qpos, rbits, ordered);
    k_bounds_rounds<2><<<nbb, BOUNDS_THREADS, bsm, L.stream>>>(P, T, qpos, rbits, ordered);
  }
  k_groups<<<(n + 255) / 256, 256, 0, L.stream>>>(n, T, group_max, pp.dim, qscale,
    rbits);
  k_refgroups<<<(n + 255) / 256, 256, 0, L.stream>>>(P.key, n, pp.dim, T, rbits,
    ordered);
  *L.counter += ordered ? 6 : 5;
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
// Launch shape: one-warp blocks, 20 resident per SM (96 registers, a few
// bytes of spills; 9 KB of shared memory each: 256 candidates and a
// 1,024-entry stack).  Two eight-warp blocks at 122 registers hold 16 warps
// per SM; the 20 here hide more of the walk's fixed-latency stalls and run
// the Sedov 128^3 walk 11 % faster.  At 80 registers (24 warps) the spills
// make it slower.  The FP64 (ordered) walk keeps its larger candidate buffer
// and runs eight blocks per SM.
#ifndef NB_WARPS
#define NB_WARPS 1
#endif
#ifndef NB_STACK
#define NB_STACK 1024
#endif
#define NB_CAND_ORDERED 2048
#ifndef NB_CAND
#define NB_CAND 256
#endif
#ifndef NB_BLOCKS_PER_SM
#define NB_BLOCKS_PER_SM 20
#endif
#define NB_ORDERED_BLOCKS_PER_SM 8
// The mixed walk comes in two variants, one for runs in which every h is
// equal and one for varying h; both are launched and each returns at once
// unless the device's range words select it.  The equal-h variant keeps
// none of the reference node-test state (FP64 group box, reference group,
// FP32 centre) and no candidate h, so it fits more warps per SM.
#ifndef NB_UNI_BLOCKS_PER_SM
#define NB_UNI_BLOCKS_PER_SM 24
#endif
#ifndef NB_UNI_CAND
#define NB_UNI_CAND 256
#endif
enum { NB_MODE_UNI = 0, NB_MODE_VAR = 1, NB_MODE_ORDERED = 2 };

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

// FP32 versions of the two node tests, for answers that are certain.  Boxes
// are the outward-rounded FP32 copies (fbox2) relative to the range's lower
// corner and points are FP32 roundings of the same relative coordinates, so
// every FP32 box face and point lies within `tol` (a few FP32 ulps of the
// range's extent) of its FP64 value; an answer that a perturbation of that
// size could flip returns -1 and the caller runs the FP64 test.
__device__ __forceinline__ int box_box_f(const float4 & alo, const float4 & ahi,
  const float4 & blo, const float4 & bhi, int dim, float tol) {
  float g = fmaxf(fmaxf(blo.x - ahi.x, alo.x - bhi.x),
    fmaxf(blo.y - ahi.y, alo.y - bhi.y));
  if(dim == 3)
    g = fmaxf(g, fmaxf(blo.z - ahi.z, alo.z - bhi.z));
  if(g > 0.f)  // outer boxes apart: the exact boxes are apart
    return 0;
  if(g < -2.f * tol)  // overlap by more than both roundings on every axis
    return 1;
  return -1;
}

__device__ __forceinline__ int sphere_box_f(const float4 & lo,
  const float4 & hi, float cx, float cy, float cz, float r, int dim,
  float tol) {
  const float dx = fmaxf(0.f, fmaxf(lo.x - cx, cx - hi.x));
  const float dy = fmaxf(0.f, fmaxf(lo.y - cy, cy - hi.y));
  const float dz = dim == 3 ? fmaxf(0.f, fmaxf(lo.z - cz, cz - hi.z)) : 0.f;
  const float d = sqrtf(dx * dx + dy * dy + dz * dz);
  // box faces and the point each within tol per axis; 1e-6 relative covers
  // the FP32 rounding of the distance and of r
  const float slack = 3.5f * tol + 1e-6f * (d + r) + 3e-15f;
  if(d + slack < r)
    return 1;
  if(d - slack > r)
    return 0;
  return -1;
}

// With varying h the reference's walk drops a candidate b of particle a
// unless the box of b's octree parent passes both node tests against a's
// traversal group G (tree_topology.h:323-355): box-box with G's box when G
// is a node, and sphere-box with at least one member of G.  When every h
// is equal only the box-box test can fail, and only for a pair whose
// separation along an axis ties with h to rounding.  Each
// test is decided in FP32 first and in FP64 (box_box, sphere_box) only when
// the FP32 answer is not certain, so the answers are the FP64 ones.
__device__ bool ref_node_tests_mixed(const Tree & T, const double * X,
  const double * Y, const double * Z, const double * H, int dim, int b, int a,
  double xa, double ya, double za, double ha, float cax, float cay, float caz,
  float haf, int gnode, const double * g2, const float4 & glo,
  const float4 & ghi, const double * rlo, float tol) {
  const int ob = T.opar[b];
  const float4 blo = T.fbox2[2 * ob], bhi = T.fbox2[2 * ob + 1];
  const double * b2 = (const double *)&T.box2[ob];
  if(gnode >= 0) {
    const int r = box_box_f(blo, bhi, glo, ghi, dim, tol);
    if(r == 0)
      return false;
    if(r < 0) {
      double bb[8];
      for(int k = 0; k < 8; ++k)
        bb[k] = b2[k];
      if(!box_box(bb, g2, dim))
        return false;
    }
  }
  const int s = sphere_box_f(blo, bhi, cax, cay, caz, haf, dim, tol);
  if(s == 1)
    return true;
  if(s < 0) {
    double bb[8];
    for(int k = 0; k < 8; ++k)
      bb[k] = b2[k];
    if(sphere_box(bb, xa, ya, za, ha, dim))
      return true;
  }
  if(gnode < 0)
    return false;
  for(int k = T.first[gnode]; k <= T.last[gnode]; ++k) {
    if(k == a)
      continue;
    const double xk = X[k], yk = Y[k], zk = dim == 3 ? Z[k] : 0.0, hk = H[k];
    const int t = sphere_box_f(blo, bhi, (float)(xk - rlo[0]), (float)(yk - rlo[1]),
      dim == 3 ? (float)(zk - rlo[2]) : 0.f, (float)hk, dim, tol);
    if(t == 1)
      return true;
    if(t < 0) {
      double bb[8];
      for(int q = 0; q < 8; ++q)
        bb[q] = b2[q];
      if(sphere_box(bb, xk, yk, zk, hk, dim))
        return true;
    }
  }
  return false;
}

// Conservative pruning test in the fixed-point space: the separation of
// two boxes per axis, less one quantisation step (each coordinate is
// within half a step of the true one), against max(h) with 1e-5 slack.
__device__ __forceinline__ bool box_near(int4 glo, int4 ghi, float hg,
  int4 lo, int4 hi, float hn, float s0, float s1, float s2) {
  int sx = max(0, max(lo.x - ghi.x, glo.x - hi.x) - 1);
  int sy = max(0, max(lo.y - ghi.y, glo.y - hi.y) - 1);
  int sz = max(0, max(lo.z - ghi.z, glo.z - hi.z) - 1);
  float fx = (float)sx * s0, fy = (float)sy * s1, fz = (float)sz * s2;
  float R = fmaxf(hg, hn);
  return fx * fx + fy * fy + fz * fz <= R * R * 1.00001f;
}

// One warp per group (<= 32 particles, lane = member).  The warp walks the
// radix tree with a shared-memory stack, up to 32 nodes per round (one per
// lane), pruning a node when its box lies farther from the group's box than
// max(h_max(group), h_max(node)) -- conservative, so no pair with
// d <= max(h_a, h_b) is lost.  Surviving particles are staged as candidates
// in shared memory and filtered by every member with the reference
// predicate (tree_geometry.h:265-276, as applied at tree_topology.h:372-379),
//     (dx*dx + dy*dy) + dz*dz <= max(h_a, h_b)^2   in FP64, no FMA,
// decided first in FP32 from the fixed-point positions with a margin well
// above that estimate's error; only pairs inside the margin pay the FP64
// test.  ORDERED (the FP64 path) sorts the candidates by (reference octree
// depth, index) before filtering, so each list comes out in the order in
// which the reference's breadth-first walk appends neighbours; when the
// candidates of a group did not fit one chunk, every member's list is
// sorted by the same key at the end.
template<int MODE>
__global__ void __launch_bounds__(NB_WARPS * 32,
  MODE == NB_MODE_ORDERED ? NB_ORDERED_BLOCKS_PER_SM
  : MODE == NB_MODE_UNI ? NB_UNI_BLOCKS_PER_SM : NB_BLOCKS_PER_SM) k_neighbors(
  Particles P, Tree T, Lists Ls, DevStatus * st, int dim,
  const unsigned long long * rbits, Packed K) {
  constexpr bool ORDERED = MODE == NB_MODE_ORDERED;
  constexpr bool UNI = MODE == NB_MODE_UNI;
  if(!ORDERED && UNI != (rbits[6] == rbits[7]))
    return;  // the other variant's run
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int CAND = ORDERED ? NB_CAND_ORDERED : UNI ? NB_UNI_CAND : NB_CAND;
  const int cap = CAND;
  unsigned long long * ckey = nullptr;
  float * cxs = nullptr;  // candidates as SoA: minus their position relative
  float * cys = nullptr;  // to the group box corner, h and particle index,
  float * czs = nullptr;  // so the filter reads consecutive pairs as float2
  float * chs = nullptr;
  int * cidx = nullptr;
  int * stack;
  if(ORDERED) {
    ckey = (unsigned long long *)smem + (size_t)w * NB_CAND_ORDERED;
    stack = (int *)(smem + (size_t)NB_WARPS * NB_CAND_ORDERED * 8) + w * NB_STACK;
  }
  else {
    constexpr int NA = UNI ? 4 : 5;  // arrays per candidate (no h with UNI)
    float * base = (float *)smem + (size_t)w * NA * CAND;
    cxs = base;
    cys = base + CAND;
    czs = base + 2 * CAND;
    chs = UNI ? nullptr : base + 3 * CAND;
    cidx = (int *)(base + (NA - 1) * CAND);
    stack = (int *)(smem + (size_t)NB_WARPS * CAND * NA * 4) + w * NB_STACK;
  }
  const unsigned lt = lanemask_lt();
  const double * X = P.f[F_X];
  const double * Y = P.f[F_Y];
  const double * Z = P.f[F_Z];
  const double * H = P.f[F_H];
  const int ngroups = *T.ngroups;
  const int maxnb = Ls.maxnb;
  const bool nonuni = !UNI && rbits[6] != rbits[7];
  const float qs0 = K.qscale[0], qs1 = K.qscale[1], qs2 = dim == 3 ? K.qscale[2] : 0.f;
  const float qmax = fmaxf(qs0, fmaxf(qs1, qs2));
  const float hglob = (float)ord_dec(rbits[7]);
  double rlo[3] = {0.0, 0.0, 0.0};
  float ext = 0.f;
  for(int d = 0; d < dim; ++d) {
    rlo[d] = ord_dec(rbits[d]);
    ext = fmaxf(ext, (float)(ord_dec(rbits[3 + d]) - rlo[d]));
  }
  // FP32 boxes and points lie within a few ulps of the range's extent of
  // their FP64 values (outward rounding of the boxes, nearest of points)
  const float ftol = 4e-7f * ext;
  for(int g = blockIdx.x * NB_WARPS + w; g < ngroups;
      g += gridDim.x * NB_WARPS) {
    const int gf = T.group_first[g], gl = T.group_last[g];
    const bool mem = lane <= gl - gf;
    const int a = gf + lane;
    int4 qa = make_int4(0, 0, 0, 0);
    if(mem)
      qa = K.qpos[a];
    const float haf = __int_as_float(qa.w);
    int gnode = -1;
    double g2[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float4 fglo = make_float4(0.f, 0.f, 0.f, 0.f), fghi = fglo;
    float cax = 0.f, cay = 0.f, caz = 0.f;
    // the reference's group and boxes exist with varying h, and in the
    // ordered mode (k_bounds_rounds, k_refgroups)
    if(mem && (nonuni || ORDERED)) {
      gnode = T.gref[a];
      if(gnode >= 0) {
        const double * gp = (const double *)&T.box2[gnode];
        for(int k = 0; k < 8; ++k)
          g2[k] = gp[k];
        fglo = T.fbox2[2 * gnode];
        fghi = T.fbox2[2 * gnode + 1];
      }
      cax = (float)(X[a] - rlo[0]);
      cay = (float)(Y[a] - rlo[1]);
      caz = dim == 3 ? (float)(Z[a] - rlo[2]) : 0.f;
    }
    int4 glo = mem ? qa : make_int4(0x7fffffff, 0x7fffffff, 0x7fffffff, 0);
    int4 ghi = mem ? qa : make_int4(-1, -1, -1, 0);
    float hg = haf;
    for(int o = 16; o; o >>= 1) {
      glo.x = min(glo.x, __shfl_xor_sync(FULL, glo.x, o));
      glo.y = min(glo.y, __shfl_xor_sync(FULL, glo.y, o));
      glo.z = min(glo.z, __shfl_xor_sync(FULL, glo.z, o));
      ghi.x = max(ghi.x, __shfl_xor_sync(FULL, ghi.x, o));
      ghi.y = max(ghi.y, __shfl_xor_sync(FULL, ghi.y, o));
      ghi.z = max(ghi.z, __shfl_xor_sync(FULL, ghi.z, o));
      hg = fmaxf(hg, __shfl_xor_sync(FULL, hg, o));
    }
    int cnt = 0;
    int sp = 1;
    int ncand = 0;
    bool chunked = false;
    bool refdone = false;  // varying h: this lane's list is already filtered
    if(lane == 0)
      stack[0] = ORDERED ? 0 : T.qbox[2 * T.group_start[g] + 1].w;
    __syncwarp();
    while(sp > 0) {
      const int k = sp < 32 ? sp : 32;
      const bool act = lane < k;
      int node = act ? stack[sp - 1 - lane] : 0;
      __syncwarp();
      sp -= k;
      if(!ORDERED) {
        // The stack holds the split codes of accepted nodes (split << 2 |
        // left leaf << 1 | right leaf, as qbox's .w keeps them); a round
        // tests both children of each -- nodes split and split + 1, whose
        // boxes are adjacent in qbox, or a leaf's position -- pushes the
        // accepted inner children's codes and stages the accepted leaves, so
        // every level of the descent costs one round instead of two.
        int4 cl[2], chh[2];
        bool lf[2] = {false, false}, ca[2] = {false, false};
        int split = 0;
        if(act) {
          const int code = node;
          split = code >> 2;
          lf[0] = (code & 2) != 0;
          lf[1] = (code & 1) != 0;
          for(int c = 0; c < 2; ++c) {
            if(lf[c]) {
              cl[c] = chh[c] = K.qpos[split + c];
            }
            else {
              cl[c] = T.qbox[2 * (split + c)];
              chh[c] = T.qbox[2 * (split + c) + 1];
            }
          }
          for(int c = 0; c < 2; ++c)
            ca[c] = box_near(glo, ghi, hg, cl[c], chh[c], __int_as_float(cl[c].w), qs0,
              qs1, qs2);
        }
        const int cc[2] = {lf[0] ? ~split : chh[0].w, lf[1] ? ~(split + 1) : chh[1].w};
        const unsigned bi0 = __ballot_sync(FULL, ca[0] && !lf[0]);
        const unsigned bi1 = __ballot_sync(FULL, ca[1] && !lf[1]);
        const unsigned bl0 = __ballot_sync(FULL, ca[0] && lf[0]);
        const unsigned bl1 = __ballot_sync(FULL, ca[1] && lf[1]);
        const int npush = __popc(bi0) + __popc(bi1);
        if(sp + npush > NB_STACK) {
          if(lane == 0 && atomicCAS(&st->code, 0, (int)FSPH_ERR_STACK_OVERFLOW) == 0)
            st->index = gf;
          break;
        }
        if(ca[0] && !lf[0])
          stack[sp + __popc(bi0 & lt)] = cc[0];
        if(ca[1] && !lf[1])
          stack[sp + __popc(bi0) + __popc(bi1 & lt)] = cc[1];
        sp += npush;
        // a node's two leaves go side by side (lane order, left first): the
        // lists keep the tree's index order, which the pair passes' gathers
        // share between the lanes of a group
        const int lfirst = ncand + __popc(bl0 & lt) + __popc(bl1 & lt);
        for(int c = 0; c < 2; ++c) {
          if(ca[c] && lf[c]) {
            const int pos = lfirst + (c && ca[0] && lf[0] ? 1 : 0);
            const int4 ql = cl[c];
            // minus the position relative to the group box corner, in FP32
            cxs[pos] = -((float)(ql.x - glo.x) * qs0);
            cys[pos] = -((float)(ql.y - glo.y) * qs1);
            czs[pos] = -((float)(ql.z - glo.z) * qs2);
            if(!UNI)
              chs[pos] = __int_as_float(ql.w);
            cidx[pos] = ~cc[c];
          }
        }
        ncand += __popc(bl0) + __popc(bl1);
      }
      else {
      bool acc = false;
      const bool leaf = node < 0;
      int4 ql = make_int4(0, 0, 0, 0);
      int code = 0;
      if(act) {
        if(!leaf) {
          const int4 lo = T.qbox[2 * node], hi = T.qbox[2 * node + 1];
          code = hi.w;
          acc = box_near(glo, ghi, hg, lo, hi, __int_as_float(lo.w), qs0, qs1, qs2);
        }
        else {
          ql = K.qpos[~node];
          acc = box_near(glo, ghi, hg, ql, ql, __int_as_float(ql.w), qs0, qs1, qs2);
        }
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
        const int pos = sp + 2 * __popc(bi & lt);
        const int split = code >> 2;
        stack[pos] = (code & 1) ? ~(split + 1) : split + 1;
        stack[pos + 1] = (code & 2) ? ~split : split;
      }
      sp += npush;
      if(acc && leaf) {
        const int j = ~node;
        const int pos = ncand + __popc(bl & lt);
        ckey[pos] = ((unsigned long long)T.edepth[j] << 32) | (unsigned)j;
      }
      ncand += __popc(bl);
      }
      __syncwarp();
      const bool last = (sp == 0);
      if(ncand > cap - (ORDERED ? 33 : 65) || (last && ncand > 0)) {
        if(!last)
          chunked = true;
        if(ORDERED)
          warp_bitonic(ckey, ncand, lane);
        if(!ORDERED && (ncand & 1)) {
          // pad to an even count with a candidate that can never pass
          if(lane == 0) {
            cxs[ncand] = 1e30f;
            cys[ncand] = 1e30f;
            czs[ncand] = 1e30f;
            if(!UNI)
              chs[ncand] = 0.f;
            cidx[ncand] = -1;
          }
          __syncwarp();
        }
        if(mem) {
          const double xa = X[a], ya = Y[a], za = dim == 3 ? Z[a] : 0.0, ha = H[a];
          int * out = Ls.idx + list_slot(a, 0, maxnb);
          // this member relative to the same corner
          const float ax = (float)(qa.x - glo.x) * qs0;
          const float ay = (float)(qa.y - glo.y) * qs1;
          const float az = (float)(qa.z - glo.z) * qs2;
          // largest extent of the group box: with the walk radius it bounds
          // the magnitude of every relative coordinate below
          const float lg = fmaxf((float)(ghi.x - glo.x) * qs0,
            fmaxf((float)(ghi.y - glo.y) * qs1, (float)(ghi.z - glo.z) * qs2));
          // The FP32 estimate t = d^2 - r^2 decides a pair only when |t|
          // exceeds a margin well above its error bound: fixed-point
          // quantisation (one step per axis), two roundings of each relative
          // coordinate (|value| <= lg + max h, as the walk accepted the
          // candidate), the squares and the sum (~2e-6 r^2).  Inside the
          // margin the exact FP64 predicate decides.
          const float kq = 16.f * qmax + 4e-6f * (lg + fmaxf(hg, hglob));
          auto decide = [&](float t, float mg, int b) -> bool {
            if(fabsf(t) > mg)
              return t < 0.f;
            const double xb = X[b], yb = Y[b], hbd = H[b];
            const double zb = dim == 3 ? Z[b] : 0.0;
            double dx = xa - xb, dy = ya - yb, dz = za - zb;
            double d2 = dx * dx + dy * dy;
            if(dim == 3)
              d2 = d2 + dz * dz;
            double r = ha < hbd ? hbd : ha;
            return d2 <= r * r;
          };
          // The reference's node tests (varying h) run after the walk over
          // each lane's whole list, where every lane of the warp has work;
          // a list that fills up before then is filtered on the spot and
          // the lane tests the rest as they come, so the capacity counts the
          // same pairs as the reference's list.
          auto refok = [&](int b) {
            return ref_node_tests_mixed(T, X, Y, Z, H, dim, b, a, xa, ya, za, ha,
              cax, cay, caz, haf, gnode, g2, fglo, fghi, rlo, ftol);
          };
          // Equal h: the node tests can only drop a pair whose separation
          // along some axis ties with h, where the rounding of x +- h/2 in
          // the boxes decides (box-box, tree_topology.h:326-330).  In the
          // ordered mode such pairs (none off a lattice) take the tests,
          // decided exactly; the mixed path keeps them (W(h) = 0 for the
          // compactly supported kernels).
          auto tie = [&](float fx, float fy, float fz, float rf) {
            return fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) >= rf - kq;
          };
          auto append = [&](int b) {
            if(nonuni && !refdone && cnt == maxnb) {
              int kept = 0;
              for(int j = 0; j < cnt; ++j) {
                const int e = out[slot_off(j)];
                if(refok(e)) {
                  out[slot_off(kept)] = e;
                  ++kept;
                }
              }
              cnt = kept;
              refdone = true;
            }
            if(nonuni && refdone && !refok(b))
              return;
            if(cnt < maxnb)
              out[slot_off(cnt)] = b;
            ++cnt;
          };
          if(ORDERED) {
            for(int c = 0; c < ncand; ++c) {
              const int b = (int)(ckey[c] & 0xffffffffu);
              const int4 qb = K.qpos[b];
              const float fx = (float)(qa.x - qb.x) * qs0;
              const float fy = (float)(qa.y - qb.y) * qs1;
              const float fz = (float)(qa.z - qb.z) * qs2;
              const float d2f = fx * fx + fy * fy + fz * fz;
              const float rf = fmaxf(haf, __int_as_float(qb.w));
              const float t = d2f - rf * rf;
              const float mg = rf * (4e-5f * rf + kq);
              if(decide(t, mg, b) && (nonuni || !tie(fx, fy, fz, rf) || refok(b)))
                append(b);
            }
          }
          else if(UNI) {
            // every h is equal: r and the margin are constants of the group
            // and the predicate decides (ties included, see tie)
            const float2 ax2 = make_float2(ax, ax), ay2 = make_float2(ay, ay);
            const float2 az2 = make_float2(az, az);
            const float r2 = haf * haf;
            const float2 nr2 = make_float2(-r2, -r2);
            const float mg = haf * (4e-5f * haf + kq);
            for(int c = 0; c < ncand; c += 2) {
              const float2 nx = *(const float2 *)&cxs[c];
              const float2 ny = *(const float2 *)&cys[c];
              const float2 nz = *(const float2 *)&czs[c];
              const int2 id = *(const int2 *)&cidx[c];
              const float2 dx = __fadd2_rn(ax2, nx);
              const float2 dy = __fadd2_rn(ay2, ny);
              const float2 dz = __fadd2_rn(az2, nz);
              float2 d2 = __fmul2_rn(dx, dx);
              d2 = __ffma2_rn(dy, dy, d2);
              d2 = __ffma2_rn(dz, dz, d2);
              const float2 t = __fadd2_rn(d2, nr2);
              bool in0 = t.x < 0.f, in1 = t.y < 0.f;
              if(fabsf(t.x) <= mg)
                in0 = decide(t.x, mg, id.x);
              if(fabsf(t.y) <= mg && id.y >= 0)
                in1 = decide(t.y, mg, id.y);
              if(in0) {
                if(cnt < maxnb)
                  out[slot_off(cnt)] = id.x;
                ++cnt;
              }
              if(in1) {
                if(cnt < maxnb)
                  out[slot_off(cnt)] = id.y;
                ++cnt;
              }
            }
          }
          else if(!UNI) {
            // two candidates per iteration with Blackwell's packed FP32x2
            // arithmetic
            const float2 ax2 = make_float2(ax, ax), ay2 = make_float2(ay, ay);
            const float2 az2 = make_float2(az, az);
            const float2 eps2 = make_float2(4e-5f, 4e-5f), kq2 = make_float2(kq, kq);
            for(int c = 0; c < ncand; c += 2) {
              const float2 nx = *(const float2 *)&cxs[c];
              const float2 ny = *(const float2 *)&cys[c];
              const float2 nz = *(const float2 *)&czs[c];
              const float2 hb = *(const float2 *)&chs[c];
              const int2 id = *(const int2 *)&cidx[c];
              const float2 dx = __fadd2_rn(ax2, nx);
              const float2 dy = __fadd2_rn(ay2, ny);
              const float2 dz = __fadd2_rn(az2, nz);
              float2 d2 = __fmul2_rn(dx, dx);
              d2 = __ffma2_rn(dy, dy, d2);
              d2 = __ffma2_rn(dz, dz, d2);
              const float2 rf = make_float2(fmaxf(haf, hb.x), fmaxf(haf, hb.y));
              const float2 nrf = make_float2(-rf.x, -rf.y);
              const float2 t = __ffma2_rn(rf, nrf, d2);
              const float2 mg = __fmul2_rn(rf, __ffma2_rn(rf, eps2, kq2));
              if(id.x >= 0 && decide(t.x, mg.x, id.x))
                append(id.x);
              if(id.y >= 0 && decide(t.y, mg.y, id.y))
                append(id.y);
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
      if(nonuni && !refdone) {
        // drop the pairs the reference's node tests drop; the list keeps
        // its order
        const double xa = X[a], ya = Y[a], za = dim == 3 ? Z[a] : 0.0, ha = H[a];
        int * o = Ls.idx + list_slot(a, 0, maxnb);
        int kept = 0;
        for(int j = 0; j < cnt; ++j) {
          const int b = o[slot_off(j)];
          if(ref_node_tests_mixed(T, X, Y, Z, H, dim, b, a, xa, ya, za, ha, cax,
               cay, caz, haf, gnode, g2, fglo, fghi, rlo, ftol)) {
            o[slot_off(kept)] = b;
            ++kept;
          }
        }
        cnt = kept;
      }
      Ls.cnt[a] = cnt;
      {
        // pad the last chunk of four with the particle itself
        int * o = Ls.idx + list_slot(a, 0, maxnb);
        for(int k = cnt; k < ((cnt + 3) & ~3); ++k)
          o[slot_off(k)] = a;
      }
      if(ORDERED && chunked) {
        // the candidates came in several sorted chunks: put the whole list
        // in (reference octree depth, index) order (Shell sort, Ciura gaps)
        int * out = Ls.idx + list_slot(a, 0, maxnb);
        auto key = [&](int b) {
          return ((unsigned long long)T.edepth[b] << 32) | (unsigned)b;
        };
        const int gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
        for(int gi = 0; gi < 8; ++gi) {
          const int gap = gaps[gi];
          for(int i = gap; i < cnt; ++i) {
            const int v = out[slot_off(i)];
            const unsigned long long kv = key(v);
            int j = i;
            while(j >= gap && key(out[slot_off(j - gap)]) > kv) {
              out[slot_off(j)] = out[slot_off(j - gap)];
              j -= gap;
            }
            out[slot_off(j)] = v;
          }
        }
      }
    }
  }
}

cudaError_t launch_neighbors(const Launch & L, const Particles & P,
  const PhysParams & pp, const Tree & T, Lists & Ls, DevStatus * st, int nsm,
  const unsigned long long * rbits, const Packed & K, int ordered) {
  const size_t smem_o = (size_t)NB_WARPS * NB_CAND_ORDERED * 8 +
                        (size_t)NB_WARPS * NB_STACK * 4;
  const size_t smem_v = (size_t)NB_WARPS * NB_CAND * 20 +
                        (size_t)NB_WARPS * NB_STACK * 4;
  const size_t smem_u = (size_t)NB_WARPS * NB_UNI_CAND * 16 +
                        (size_t)NB_WARPS * NB_STACK * 4;
  static std::atomic<unsigned long long> attr_devices{0};
  cudaError_t ae = once_per_device(&attr_devices, [&]() {
    cudaError_t e = cudaFuncSetAttribute(k_neighbors<NB_MODE_ORDERED>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_o);
    if(e == cudaSuccess)
      e = cudaFuncSetAttribute(k_neighbors<NB_MODE_VAR>,
        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_v);
    if(e == cudaSuccess)
      e = cudaFuncSetAttribute(k_neighbors<NB_MODE_UNI>,
        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_u);
    return e;
  });
  if(ae != cudaSuccess)
    return ae;
  const int maxb0 = (P.n + NB_WARPS * 32 - 1) / (NB_WARPS * 32) * 8;
  const int maxb = maxb0 > 0 ? maxb0 : 1;
  auto grid = [&](int per_sm) { return nsm * per_sm < maxb ? nsm * per_sm : maxb; };
  if(ordered) {
    k_neighbors<NB_MODE_ORDERED><<<grid(NB_ORDERED_BLOCKS_PER_SM), NB_WARPS * 32,
      smem_o, L.stream>>>(P, T, Ls, st, pp.dim, rbits, K);
    *L.counter += 1;
  }
  else {
    // both variants; the one the range words do not select returns at once
    k_neighbors<NB_MODE_UNI><<<grid(NB_UNI_BLOCKS_PER_SM), NB_WARPS * 32, smem_u,
      L.stream>>>(P, T, Ls, st, pp.dim, rbits, K);
    k_neighbors<NB_MODE_VAR><<<grid(NB_BLOCKS_PER_SM), NB_WARPS * 32, smem_v,
      L.stream>>>(P, T, Ls, st, pp.dim, rbits, K);
    *L.counter += 2;
  }
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
// sized for FSPH_NOALLOC_SORT_MAX particles: 12,846,336 bytes that every
// GPU loading the library holds until the process exits.
#define FSPH_NOALLOC_SORT_MAX (1 << 20)
#define NOALLOC_RANGE_BYTES 256
#define NOALLOC_KEYS_BYTES ((size_t)FSPH_NOALLOC_SORT_MAX * 8)
#define NOALLOC_VALS_BYTES ((size_t)FSPH_NOALLOC_SORT_MAX * 4)
#define NOALLOC_HIST_BYTES \
  ((size_t)(256 * ((FSPH_NOALLOC_SORT_MAX + RS_TILE - 1) / RS_TILE) + 256) * 4)
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

