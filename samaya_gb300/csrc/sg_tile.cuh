// Load-balanced, deterministic CSR tile kernel core with fused per-row epilogues.
//
// A CTA processes one tile at a time (persistent loop over tiles):
//   phase A  streams the tile's nonzeros [k0, k1) with coalesced loads and stages the NV
//            products prod(v, val, col) in shared memory;
//   phase B  reduces each row's products inside the tile: `team` lanes per row (chosen from the
//            tile's mean row length), lanes step by `team`, then a fixed shuffle tree;
//   phase C  calls epi.row(row, sums) with one thread per row, so the epilogue's vector accesses
//            (iterates, bounds, averages) are coalesced across the CTA.
// A row longer than the tile capacity is cut into consecutive segment tiles; each segment's
// block sum goes to TileSet::seg_part and the last segment to arrive (counter) adds the segments
// in tile order (the whole CTA, fixed tree) and runs epi.long_row. Every sum is taken in a fixed
// order, so results do not depend on scheduling and a re-run is bit-identical.
//
// Shared memory (dynamic): red[kMaxSums * 8] doubles | prod[NV][cap_nnz] ACC | rows[NV][cap_rows].
#pragma once

#include "sg_common.cuh"

namespace sg {

constexpr int kRedDoubles = kMaxSums * (kBlock / 32);

__host__ __device__ constexpr size_t tile_smem_size(int nv, size_t acc_bytes, int cap_nnz,
                                                    int cap_rows) {
  return sizeof(double) * kRedDoubles + acc_bytes * nv * (static_cast<size_t>(cap_nnz) + cap_rows);
}

template <typename ACC, int NV>
struct TileSmem {
  double* red;
  ACC* prod;  // [NV][cap_nnz]
  ACC* rows;  // [NV][cap_rows]
  int cap_nnz, cap_rows;
  __device__ __forceinline__ ACC& p(int v, int q) { return prod[v * cap_nnz + q]; }
  __device__ __forceinline__ ACC& r(int v, int q) { return rows[v * cap_rows + q]; }
};

template <typename ACC, int NV>
__device__ __forceinline__ TileSmem<ACC, NV> tile_smem(const TileSet& ts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<ACC, NV> s;
  s.red = reinterpret_cast<double*>(smem_raw);
  s.prod = reinterpret_cast<ACC*>(smem_raw + sizeof(double) * kRedDoubles);
  s.rows = s.prod + NV * ts.cap_nnz;
  s.cap_nnz = ts.cap_nnz;
  s.cap_rows = ts.cap_rows;
  return s;
}

// Iterates over tiles. Prod: ACC operator()(int v, T val, int col) const.
// Epi: void row(int r, const ACC (&s)[NV]) for rows of kind-0 tiles (called by one thread),
//      void long_row(int lrow, int r, const ACC (&s)[NV]) for a split row (thread 0 of the CTA
//      that completes it).
__device__ __forceinline__ double* smem_red() {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  return reinterpret_cast<double*>(smem_raw);
}

template <bool MAXRED, typename ACC>
__device__ __forceinline__ ACC combine(ACC a, ACC b) {
  if constexpr (MAXRED) {
    return a > b ? a : b;
  } else {
    return a + b;
  }
}

// MAXRED: each row's products are combined by max instead of + (norm statistics).
template <typename T, typename ACC, int NV, typename Prod, typename Epi, bool MAXRED = false>
__device__ __forceinline__ void run_tiles(const TileSet& ts, const int* __restrict__ ptr,
                                          const int* __restrict__ idx,
                                          const T* __restrict__ val, const Prod& prod, Epi& epi) {
  TileSmem<ACC, NV> sm = tile_smem<ACC, NV>(ts);
  const int tid = threadIdx.x;
  __shared__ bool last_seg;
  for (int ti = blockIdx.x; ti < ts.ntiles; ti += gridDim.x) {
    const Tile tile = ts.tiles[ti];
    const int k0 = tile.k0;
    const int len = tile.k1 - k0;
    // Phase A: coalesced stream of the tile's nonzeros (4 independent loads in flight per
    // thread).
    {
      int q = tid;
      for (; q + 3 * kBlock < len; q += 4 * kBlock) {
        const T a0 = ldg(val + k0 + q);
        const T a1 = ldg(val + k0 + q + kBlock);
        const T a2 = ldg(val + k0 + q + 2 * kBlock);
        const T a3 = ldg(val + k0 + q + 3 * kBlock);
        const int j0 = ldg(idx + k0 + q);
        const int j1 = ldg(idx + k0 + q + kBlock);
        const int j2 = ldg(idx + k0 + q + 2 * kBlock);
        const int j3 = ldg(idx + k0 + q + 3 * kBlock);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          sm.p(v, q) = prod(v, a0, j0);
          sm.p(v, q + kBlock) = prod(v, a1, j1);
          sm.p(v, q + 2 * kBlock) = prod(v, a2, j2);
          sm.p(v, q + 3 * kBlock) = prod(v, a3, j3);
        }
      }
      for (; q < len; q += kBlock) {
        const T a = ldg(val + k0 + q);
        const int j = ldg(idx + k0 + q);
#pragma unroll
        for (int v = 0; v < NV; ++v) sm.p(v, q) = prod(v, a, j);
      }
    }
    __syncthreads();
    if (tile.kind == 0) {
      // Phase B: team-per-row reduction in shared memory.
      const int team = tile.team;
      const int nteams = kBlock / team;
      const int my_team = tid / team;
      const int lane = tid % team;
      const int nrows = tile.r1 - tile.r0;
      const int rounds = (nrows + nteams - 1) / nteams;
      for (int rr = 0; rr < rounds; ++rr) {
        const int lr = rr * nteams + my_team;
        ACC s[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) s[v] = ACC(0);
        if (lr < nrows) {
          const int b = ldg(ptr + tile.r0 + lr) - k0;
          const int e = ldg(ptr + tile.r0 + lr + 1) - k0;
          for (int q = b + lane; q < e; q += team) {
#pragma unroll
            for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], sm.p(v, q));
          }
        }
        for (int o = team / 2; o > 0; o >>= 1) {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            s[v] = combine<MAXRED>(s[v], __shfl_down_sync(0xffffffffu, s[v], o, team));
          }
        }
        if (lane == 0 && lr < nrows) {
#pragma unroll
          for (int v = 0; v < NV; ++v) sm.r(v, lr) = s[v];
        }
      }
      __syncthreads();
      // Phase C: epilogue, one thread per row.
      for (int lr = tid; lr < nrows; lr += kBlock) {
        ACC s[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) s[v] = sm.r(v, lr);
        epi.row(tile.r0 + lr, s);
      }
    } else {
      // A segment of a long row: block sum in a fixed order.
      double part[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        ACC s = ACC(0);
        for (int q = tid; q < len; q += kBlock) s = combine<MAXRED>(s, sm.p(v, q));
        part[v] = static_cast<double>(s);
      }
      double tot[NV];
      block_reduce<NV, MAXRED ? 0xFFu : 0u>(part, sm.red, tot);
      if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) ts.seg_part[ti * kMaxVec + v] = tot[v];
        __threadfence();
        const unsigned prev = atomicAdd(ts.lcount + tile.lrow, 1u);
        last_seg = (prev == static_cast<unsigned>(tile.nseg - 1));
      }
      __syncthreads();
      if (last_seg) {
        // The whole CTA adds the row's segments: thread t takes segments t, t + 256, ... in
        // order, then the fixed block tree.
        __threadfence();
        const int first = ti - tile.seg;
        double acc[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double a = 0.0;
          for (int g = tid; g < tile.nseg; g += kBlock) {
            a = combine<MAXRED>(a, __ldcg(ts.seg_part + (first + g) * kMaxVec + v));
          }
          acc[v] = a;
        }
        double sum[NV];
        block_reduce<NV, MAXRED ? 0xFFu : 0u>(acc, sm.red, sum);
        if (tid == 0) {
          ACC s[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = static_cast<ACC>(sum[v]);
          ts.lcount[tile.lrow] = 0u;
          epi.long_row(tile.lrow, tile.r0, s);
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace sg
