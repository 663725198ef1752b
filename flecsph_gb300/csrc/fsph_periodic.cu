// fsph_periodic.cu -- periodic boundaries by ghost copies, regenerated at
// every update_iteration.
//
// Replaces boundary::pboundary_clean / pboundary_generate
// (include/physics/boundary.h:45-248) as called from
// body_system::update_iteration (mpisph/bodies_system.h:160-169):
//   1. clean: drop the previous iteration's WALL copies and keep the real
//      particles in their current order (std::stable_partition);
//   2. halo = 2.5 * max h over the real particles (getSmoothinglength,
//      bodies_system.h:112-124);
//   3. teleport every real particle that left the box [-L/2, L/2] along a
//      periodic axis (x > max: x -= L; x <= min: x += L);
//   4. for every real particle, in order, append a copy shifted by one box
//      length for each periodic axis whose face lies within the halo, then
//      one for each pair (xy, xz, zy) and the triple of such axes; copies
//      get ids n_real, n_real + 1, ... in the order they are made.
// The WALL type of the reference is carried by the id: real particles hold
// the ids 0 .. n_real - 1 (the reference asserts this through its id-sum
// check, boundary.h:241-246) and copies the ids above.
//
// The physics treats copies like real particles, as the reference does
// (no physics module tests the type); only the conserved sums skip them.
//
// Device-wide order is kept with exclusive scans: one for the compaction,
// one for the copy offsets, so the layout is the reference's exactly.
#include <cuda_runtime.h>

#include "fsph_internal.cuh"

namespace fsph {

#define SCAN_THREADS 1024
#define SCAN_ITEMS 4
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

// ------------------------------------------------------ exclusive scan --
__device__ __forceinline__ int block_exclusive_scan(int v, int * warp_sums,
  int * total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
  for(int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if(lane >= o)
      incl += t;
  }
  if(lane == 31)
    warp_sums[w] = incl;
  __syncthreads();
  if(w == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
    int si = s;
    for(int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, si, o);
      if(lane >= o)
        si += t;
    }
    warp_sums[lane] = si - s;
    if(lane == 31)
      warp_sums[32] = si;
  }
  __syncthreads();
  const int r = warp_sums[w] + incl - v;
  *total = warp_sums[32];
  __syncthreads();
  return r;
}

// per tile: exclusive scan of its elements and the tile's total
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const int * in,
  int * out, int n, int * tile_sums) {
  __shared__ int ws[33];
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS], s = 0;
#pragma unroll
  for(int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int run = block_exclusive_scan(s, ws, &total);
#pragma unroll
  for(int k = 0; k < SCAN_ITEMS; ++k) {
    if(base + k < n)
      out[base + k] = run;
    run += v[k];
  }
  if(threadIdx.x == 0)
    tile_sums[blockIdx.x] = total;
}

// one block: exclusive scan over the tile sums, in chunks of SCAN_TILE
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_sums(int * sums,
  int ntiles, int * grand_total) {
  __shared__ int ws[33];
  int carry = 0;
  for(int c0 = 0; c0 < ntiles; c0 += SCAN_TILE) {
    const int base = c0 + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS], s = 0;
#pragma unroll
    for(int k = 0; k < SCAN_ITEMS; ++k) {
      v[k] = base + k < ntiles ? sums[base + k] : 0;
      s += v[k];
    }
    int total;
    int run = carry + block_exclusive_scan(s, ws, &total);
#pragma unroll
    for(int k = 0; k < SCAN_ITEMS; ++k) {
      if(base + k < ntiles)
        sums[base + k] = run;
      run += v[k];
    }
    carry += total;
  }
  if(threadIdx.x == 0)
    *grand_total = carry;
}

__global__ void k_scan_add(int * out, int n, const int * tile_offsets) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n)
    out[i] += tile_offsets[i / SCAN_TILE];
}

int scan_tiles(int n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// out[i] = sum of in[0 .. i-1]; *total = sum of all.  tile_sums holds
// scan_tiles(n) ints.
cudaError_t launch_exclusive_scan(const Launch & L, const int * in, int * out,
  int n, int * tile_sums, int * total) {
  const int nt = scan_tiles(n);
  if(nt == 0)
    return cudaMemsetAsync(total, 0, sizeof(int), L.stream);
  k_scan_tiles<<<nt, SCAN_THREADS, 0, L.stream>>>(in, out, n, tile_sums);
  k_scan_tile_sums<<<1, SCAN_THREADS, 0, L.stream>>>(tile_sums, nt, total);
  k_scan_add<<<(n + 255) / 256, 256, 0, L.stream>>>(out, n, tile_sums);
  *L.counter += 3;
  return cudaGetLastError();
}

// ---------------------------------------------------------- clean -------
__global__ void k_flag_real(const long long * id, int n, long long nreal,
  int * flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n)
    flag[i] = id[i] < nreal ? 1 : 0;
}

__global__ void k_compact_perm(const int * flag, const int * pos, int n,
  int * perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && flag[i])
    perm[pos[i]] = i;
}

// ----------------------------------------------------- halo and copies --
__global__ void k_hmax_real(const double * h, int n, unsigned long long * out) {
  __shared__ unsigned long long part[8];
  unsigned long long m = 0;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += gridDim.x * blockDim.x) {
    // h >= 0: the bit pattern orders like the value
    const double v = h[i];
    const unsigned long long b = v > 0 ? (unsigned long long)__double_as_longlong(v) : 0ull;
    m = b > m ? b : m;
  }
  for(int o = 16; o; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if((threadIdx.x & 31) == 0)
    part[threadIdx.x >> 5] = m;
  __syncthreads();
  if(threadIdx.x == 0) {
    for(int w = 1; w < (int)(blockDim.x >> 5); ++w)
      m = part[w] > m ? part[w] : m;
    atomicMax(out, m);
  }
}

struct PBox {
  double lo[3], hi[3];
  int per[3];
  int dim;
};

// Copies made for one particle, in the reference's order: faces by axis,
// then the pairs (0,1), (0,2), (2,1) and the triple (3D) or the pair (0,1)
// (2D).  on_edge bit d set <=> the axis-d face lies within the halo.
__device__ __forceinline__ int edge_mask(const PBox & B, const double * x,
  double halo) {
  int m = 0;
  for(int d = 0; d < B.dim; ++d)
    if(B.per[d] && (x[d] + halo > B.hi[d] || x[d] - halo <= B.lo[d]))
      m |= 1 << d;
  return m;
}

__device__ __forceinline__ int copies_of(int m, int dim) {
  int c = __popc(m);
  if(dim == 2)
    c += (m & 3) == 3;
  else if(dim == 3) {
    c += (m & 3) == 3;
    c += (m & 5) == 5;
    c += (m & 6) == 6;
    c += m == 7;
  }
  return c;
}

__global__ void k_teleport_count(Particles P, PBox B,
  const unsigned long long * hbits, int * count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= P.n)
    return;
  const double halo = 2.5 * __longlong_as_double((long long)*hbits);
  double x[3] = {0, 0, 0};
  for(int d = 0; d < B.dim; ++d) {
    double v = P.f[F_X + d][i];
    if(B.per[d]) {
      if(v > B.hi[d])
        v -= B.hi[d] - B.lo[d];
      else if(v <= B.lo[d])
        v += B.hi[d] - B.lo[d];
      P.f[F_X + d][i] = v;
    }
    x[d] = v;
  }
  count[i] = copies_of(edge_mask(B, x, halo), B.dim);
}

// coordinate of a face copy along axis d
__device__ __forceinline__ double face_shift(const PBox & B, double v, int d,
  double halo) {
  return v + halo > B.hi[d] ? v - (B.hi[d] - B.lo[d]) : v + (B.hi[d] - B.lo[d]);
}

// coordinate of a pair / triple copy along axis d (boundary.h:80-86)
__device__ __forceinline__ double corner_shift(const PBox & B, double v, int d,
  double halo) {
  return v + halo > B.hi[d] ? B.lo[d] - fabs(v + B.lo[d])
                            : B.hi[d] + fabs(v + B.hi[d]);
}

__global__ void k_write_copies(Particles P, int nreal, PBox B,
  const unsigned long long * hbits, const int * offset) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= nreal)
    return;
  const double halo = 2.5 * __longlong_as_double((long long)*hbits);
  double x[3] = {0, 0, 0};
  for(int d = 0; d < B.dim; ++d)
    x[d] = P.f[F_X + d][i];
  const int m = edge_mask(B, x, halo);
  if(!m)
    return;
  int slot = nreal + offset[i];
  auto emit = [&](const double * c) {
#pragma unroll
    for(int k = 0; k < NF; ++k)
      P.f[k][slot] = P.f[k][i];
    for(int d = 0; d < B.dim; ++d)
      P.f[F_X + d][slot] = c[d];
    P.id[slot] = slot;
    ++slot;
  };
  for(int d = 0; d < B.dim; ++d)
    if(m >> d & 1) {
      double c[3] = {x[0], x[1], x[2]};
      c[d] = face_shift(B, x[d], d, halo);
      emit(c);
    }
  auto pair = [&](int a, int b) {
    if((m >> a & 1) && (m >> b & 1)) {
      double c[3] = {x[0], x[1], x[2]};
      c[a] = corner_shift(B, x[a], a, halo);
      c[b] = corner_shift(B, x[b], b, halo);
      emit(c);
    }
  };
  pair(0, 1);
  if(B.dim == 3) {
    pair(0, 2);
    pair(2, 1);
    if(m == 7) {
      double c[3];
      for(int d = 0; d < 3; ++d)
        c[d] = corner_shift(B, x[d], d, halo);
      emit(c);
    }
  }
}

// ------------------------------------------------------------- driver ---
cudaError_t launch_periodic(const Launch & L, Particles & P, Particles & Palt,
  const PhysParams & pp, const double * box_len, const int * periodic,
  long long nreal, int cap, PeriodicScratch & S, int * n_out,
  const char ** why, unsigned skip) {
  cudaError_t e;
  const int n = P.n;
  *why = nullptr;
  // 1. clean: stable compaction of the real particles
  if(n > nreal) {
    k_flag_real<<<(n + 255) / 256, 256, 0, L.stream>>>(P.id, n, nreal, S.flag);
    *L.counter += 1;
    if((e = launch_exclusive_scan(L, S.flag, S.pos, n, S.tiles, S.total)))
      return e;
    k_compact_perm<<<(n + 255) / 256, 256, 0, L.stream>>>(S.flag, S.pos, n, S.perm);
    *L.counter += 1;
    Particles src = P;
    src.n = (int)nreal;
    Particles dst = Palt;
    dst.n = (int)nreal;
    if((e = launch_permute(L, src, dst, S.perm, P.key, skip)))
      return e;
    Particles t = P;
    P = Palt;
    Palt = t;
  }
  const int nr = (int)nreal;
  P.n = Palt.n = nr;
  // 2. halo from the real particles' largest h
  if((e = cudaMemsetAsync(S.hbits, 0, sizeof(unsigned long long), L.stream)))
    return e;
  k_hmax_real<<<304, 256, 0, L.stream>>>(P.f[F_H], nr, S.hbits);
  *L.counter += 1;
  // 3. teleport and count the copies, 4. place them
  PBox B;
  B.dim = pp.dim;
  for(int d = 0; d < 3; ++d) {
    B.lo[d] = -0.5 * box_len[d];
    B.hi[d] = 0.5 * box_len[d];
    B.per[d] = periodic[d];
  }
  k_teleport_count<<<(nr + 255) / 256, 256, 0, L.stream>>>(P, B, S.hbits, S.flag);
  *L.counter += 1;
  if((e = launch_exclusive_scan(L, S.flag, S.pos, nr, S.tiles, S.total)))
    return e;
  int ncopies = 0;
  if((e = cudaMemcpyAsync(&ncopies, S.total, sizeof(int), cudaMemcpyDeviceToHost,
        L.stream)))
    return e;
  if((e = cudaStreamSynchronize(L.stream)))
    return e;
  if((long long)nr + ncopies > cap) {
    *why = "capacity too small for the periodic copies";
    *n_out = nr + ncopies;
    return cudaSuccess;
  }
  k_write_copies<<<(nr + 255) / 256, 256, 0, L.stream>>>(P, nr, B, S.hbits, S.pos);
  *L.counter += 1;
  P.n = Palt.n = nr + ncopies;
  *n_out = nr + ncopies;
  return cudaGetLastError();
}

}  // namespace fsph
