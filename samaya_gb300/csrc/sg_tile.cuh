// Load-balanced, deterministic CSR tile kernel core with fused per-row epilogues.
//
// The rows of an operator are cut into tiles of bounded nonzeros and rows (host, once). A CTA
// processes tiles in a persistent loop:
//   kind 0 (short rows, at most 128 nonzeros): one thread per row, which sums the row and runs
//     epi.row(row, sums) — the fused update of the row's entries; a row longer than 32
//     nonzeros is taken over by its whole warp (ballot queue, fixed shuffle tree).
//   kind 2 (up to 8 rows of medium length, 128 < nonzeros <= the tile capacity): one warp per
//     row, or a team of 2-8 warps for the longer rows of a skewed operator, 16-byte loads of
//     four nonzeros per lane, a fixed shuffle tree (then the team's partials in warp order),
//     and epi.row(row, sums). A CTA per row would spend most of its time on the block tree.
//   kind 1 (a segment of a row longer than the tile capacity): the CTA sums the segment
//     (strided, then the fixed block tree) into TileSet::seg_part; the last segment to arrive
//     (counter) adds the row's segments in tile order and runs epi.long_row.
//   kind 3 (dual step kernels, GROUPS): up to 32 consecutive rows whose k-th nonzeros lie in
//     neighbouring columns (the demand rows of a transportation LP: the k-th nonzero of row j
//     is column k D + j). Each warp stages 16 nonzero positions of every row in shared memory
//     (row-wise, coalesced loads) and then lane l sums row l's staged positions, so one
//     gather instruction reads neighbouring entries of the gathered vector instead of 32
//     separate sectors. The warps take alternate 16-position blocks; their sums are added in
//     warp order, the segments of a group in segment order (TileSet::grp_part, counter), and
//     lane l runs epi.row for row l.
// Every sum is taken in a fixed order, so results do not depend on scheduling and a re-run is
// bit-identical.
#pragma once

#include <type_traits>

#include "sg_common.cuh"

namespace sg {

constexpr int kRedDoubles = kMaxSums * (kBlock / 32);

// Dynamic shared memory of a tile kernel: the block-reduction scratch only.
__host__ __device__ constexpr size_t tile_smem_size(int, size_t, int, int) {
  return sizeof(double) * kRedDoubles;
}

// Staged kind-1 segments: two chunks of kSegChunk indices and values (double buffer).
template <typename T>
__host__ __device__ constexpr size_t staged_smem_size() {
  return sizeof(double) * kRedDoubles + 2 * kSegChunk * (sizeof(int) + sizeof(T));
}

// mbarrier and bulk-copy primitives (PTX ISA: mbarrier, cp.async.bulk).
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes,
                                              unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// A bounded wait: gives up after kWaitTries polls (each poll may suspend the thread for a
// while), far beyond any copy's completion time.
constexpr int kWaitTries = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  for (int k = 0; k < kWaitTries; ++k) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

// Kind-3 staging: per warp kGroupRows x (kGroupPos + 1) indices and values (the extra column
// keeps lane l's reads of row l conflict-free), then the warps' row sums.
constexpr int kGroupStride = kGroupPos + 1;
template <typename T, typename ACC>
__host__ __device__ constexpr size_t group_smem_size() {
  return sizeof(double) * kRedDoubles +
         (kBlock / 32) * (kGroupRows * kGroupStride * (sizeof(int) + sizeof(T)) +
                          kGroupRows * sizeof(ACC));
}

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

// Epilogues that declare `struct Pre` split the row update into `Pre load(r)` (the row's own
// vector entries, independent of the dot product) and `row(r, s, pre)`: the loads are issued
// before the dot product so their latency overlaps it.
template <typename E, typename = void>
struct has_pre : std::false_type {};
template <typename E>
struct has_pre<E, std::void_t<typename E::Pre>> : std::true_type {};

// 16-byte loads of four consecutive nonzeros (values and indices) at a 4-aligned position.
template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  __device__ __forceinline__ static void load(const float* v, int q, float (&out)[4]) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(v + q));
    out[0] = a.x;
    out[1] = a.y;
    out[2] = a.z;
    out[3] = a.w;
  }
};
template <>
struct Vec4<double> {
  __device__ __forceinline__ static void load(const double* v, int q, double (&out)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(v + q));
    const double2 b = __ldg(reinterpret_cast<const double2*>(v + q + 2));
    out[0] = a.x;
    out[1] = a.y;
    out[2] = b.x;
    out[3] = b.y;
  }
};

// Deterministic block reduction of K values in the accumulation type (fixed shuffle tree, then
// the warps in order by thread 0, which receives the totals).
template <typename ACC, int K, bool MAXRED>
__device__ __forceinline__ void block_reduce_acc(ACC (&v)[K], ACC* scratch, ACC (&out)[K]) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = kBlock / 32;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    ACC s = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = combine<MAXRED>(s, __shfl_down_sync(0xffffffffu, s, o));
    if (lane == 0) scratch[q * kWarps + warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      ACC s = scratch[q * kWarps];
      for (int w = 1; w < kWarps; ++w) s = combine<MAXRED>(s, scratch[q * kWarps + w]);
      out[q] = s;
    }
  }
  __syncthreads();
}

// Two consecutive nonzeros (values and indices) at an even position, in one load each.
template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  __device__ __forceinline__ static float2 load(const float* v, int q) {
    return __ldg(reinterpret_cast<const float2*>(v + q));
  }
};
template <>
struct Vec2<double> {
  __device__ __forceinline__ static double2 load(const double* v, int q) {
    return __ldg(reinterpret_cast<const double2*>(v + q));
  }
};

// s += the products of a short row's nonzeros [b, e), in order: an odd first position alone,
// then pairs at even positions read with one load for two indices and one for two values (a
// column of a transportation LP is one pair), then a last single nonzero.
template <typename T, int NV, bool MAXRED, typename Prod, typename ACC>
__device__ __forceinline__ void short_row_sum(int b, int e, const int* __restrict__ idx,
                                              const T* __restrict__ val, const Prod& prod,
                                              ACC (&s)[NV]) {
  int q = b;
  if ((q & 1) != 0 && q < e) {
    const T a = ldg(val + q);
    const int j = ldg(idx + q);
#pragma unroll
    for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
    ++q;
  }
#pragma unroll 2
  for (; q + 1 < e; q += 2) {
    const int2 j = __ldg(reinterpret_cast<const int2*>(idx + q));
    const auto a = Vec2<T>::load(val, q);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      s[v] = combine<MAXRED>(s[v], prod(v, a.x, j.x));
      s[v] = combine<MAXRED>(s[v], prod(v, a.y, j.y));
    }
  }
  if (q < e) {
    const T a = ldg(val + q);
    const int j = ldg(idx + q);
#pragma unroll
    for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
  }
}

// A kind-3 tile (see the file comment). Barriers: uniform over the CTA (every thread of the CTA
// runs the same tile).
template <typename T, typename ACC, typename Prod, typename Epi>
__device__ __forceinline__ void group_tile(const TileSet& ts, const Tile& tile, int ti,
                                           const int* __restrict__ ptr,
                                           const int* __restrict__ idx,
                                           const T* __restrict__ val, const Prod& prod, Epi& epi,
                                           double* red) {
  constexpr int kWarps = kBlock / 32;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nr = tile.r1 - tile.r0;  // 1..32 rows
  // Lane l: row l's start and length.
  int my_row = 0, my_b = 0, my_len = 0;
  if (lane < nr) {
    my_row = tile_row(ts, tile.r0 + lane);
    my_b = ldg(ptr + my_row);
    my_len = ldg(ptr + my_row + 1) - my_b;
  }
  unsigned char* base = reinterpret_cast<unsigned char*>(red + kRedDoubles);
  int* sidx = reinterpret_cast<int*>(base) + warp * kGroupRows * kGroupStride;
  T* sval = reinterpret_cast<T*>(base + kWarps * kGroupRows * kGroupStride * sizeof(int)) +
            warp * kGroupRows * kGroupStride;
  ACC* wsum = reinterpret_cast<ACC*>(base + kWarps * kGroupRows * kGroupStride *
                                                (sizeof(int) + sizeof(T)));
  const int half = lane >> 4;  // staging: lanes 0-15 take row i, lanes 16-31 row i + 1
  const int col = lane & 15;
  ACC s = ACC(0);
  for (int pb = tile.k0 + warp * kGroupPos; pb < tile.k1; pb += kWarps * kGroupPos) {
    const int pos = pb + col;
#pragma unroll
    for (int i2 = 0; i2 < kGroupRows; i2 += 2) {
      const int i = i2 + half;
      const int bi = __shfl_sync(0xffffffffu, my_b, i);
      const int li = __shfl_sync(0xffffffffu, my_len, i);
      int j = 0;
      T a = T(0);
      if (i < nr && pos < li && pos < tile.k1) {
        j = ldg(idx + bi + pos);
        a = ldg(val + bi + pos);
      }
      sidx[i * kGroupStride + col] = j;
      sval[i * kGroupStride + col] = a;
    }
    __syncwarp();
    if (lane < nr) {
#pragma unroll
      for (int t = 0; t < kGroupPos; ++t) {
        if (pb + t < my_len && pb + t < tile.k1) {
          const ACC p[1] = {prod(0, sval[lane * kGroupStride + t], sidx[lane * kGroupStride + t])};
          s += p[0];
        }
      }
    }
    __syncwarp();
  }
  wsum[warp * kGroupRows + lane] = s;
  __syncthreads();
  ACC tot = ACC(0);
  if (warp == 0) {
    tot = wsum[lane];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) tot += wsum[w * kGroupRows + lane];
  }
  __syncthreads();
  if (warp != 0) return;
  if (tile.nseg == 1) {
    if (lane < nr) {
      const ACC out[1] = {tot};
      epi.row(my_row, out);
    }
    return;
  }
  ts.grp_part[ti * kGroupRows + lane] = static_cast<double>(tot);
  __threadfence();
  __syncwarp();
  unsigned prev = 0;
  if (lane == 0) prev = atomicAdd(ts.lcount + tile.lrow, 1u);
  prev = __shfl_sync(0xffffffffu, prev, 0);
  if (prev != static_cast<unsigned>(tile.nseg - 1)) return;
  // The last segment to arrive adds the group's segments in order.
  __threadfence();
  const int first = ti - tile.seg;
  double acc = 0.0;
  for (int g = 0; g < tile.nseg; ++g) acc += __ldcg(ts.grp_part + (first + g) * kGroupRows + lane);
  if (lane == 0) ts.lcount[tile.lrow] = 0u;
  if (lane < nr) {
    const ACC out[1] = {static_cast<ACC>(acc)};
    epi.row(my_row, out);
  }
}

// Prod: ACC operator()(int v, T val, int col) const — the v-th product of a nonzero.
// Epi: void row(int r, const ACC (&s)[NV]) for rows of kind-0 tiles (lane 0 of the row's team),
//      void long_row(int lrow, int r, const ACC (&s)[NV]) for a split row (thread 0 of the CTA
//      that completes it).
// MAXRED: each row's products are combined by max instead of + (norm statistics).
// WIDE: unroll the warp-per-row loop 8 deep (4 otherwise) and the segment loop 4 deep (2).
template <typename T, typename ACC, int NV, typename Prod, typename Epi, bool MAXRED = false,
          bool WIDE = false, bool GROUPS = false>
__device__ __forceinline__ void run_tiles(const TileSet& ts, const int* __restrict__ ptr,
                                          const int* __restrict__ idx,
                                          const T* __restrict__ val, const Prod& prod, Epi& epi) {
  const int tid = threadIdx.x;
  __shared__ bool last_seg;
  double* red = smem_red();
  // Staged segments (GROUPS kernels of a set with ts.staged): two chunk buffers after the
  // reduction scratch, their completion barriers and expected parities (uniform over the CTA).
  __shared__ __align__(8) unsigned long long seg_bar[2];
  __shared__ int seg_fail;
  unsigned seg_parity = 0u;
  if constexpr (GROUPS) {
    if (ts.staged) {
      if (tid == 0) {
        mbar_init(&seg_bar[0], 1);
        mbar_init(&seg_bar[1], 1);
        seg_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      }
      __syncthreads();
    }
  }
  for (int ti = blockIdx.x; ti < ts.ntiles; ti += gridDim.x) {
    const Tile tile = ts.tiles[ti];
    if constexpr (GROUPS) {
      static_assert(NV == 1 && !MAXRED, "kind-3 tiles carry one plain sum per row");
      if (tile.kind == 3) {
        group_tile<T, ACC>(ts, tile, ti, ptr, idx, val, prod, epi, red);
        continue;
      }
    }
    if (tile.kind == 0) {
      // One thread per row; a row longer than a warp is taken over by its whole warp (ballot
      // queue), so skewed row lengths inside a tile cost no serial tail.
      const int lane = tid & 31;
      const int nrows = tile.r1 - tile.r0;
      const int rounds = (nrows + kBlock - 1) / kBlock;
      for (int rr = 0; rr < rounds; ++rr) {
        const int lr = rr * kBlock + tid;
        const bool valid = lr < nrows;
        int b = 0, e = 0, row = 0;
        if (valid) {
          row = tile_row(ts, tile.r0 + lr);
          if (ts.uniform_len > 0) {
            b = row * ts.uniform_len;
            e = b + ts.uniform_len;
          } else {
            b = ldg(ptr + row);
            e = ldg(ptr + row + 1);
          }
        }
        const bool shortrow = valid && e - b <= 32;
        if constexpr (has_pre<Epi>::value) {
          typename Epi::Pre pre;
          if (shortrow) pre = epi.load(row);
          if (shortrow) {
            ACC s[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) s[v] = ACC(0);
            short_row_sum<T, NV, MAXRED>(b, e, idx, val, prod, s);
            epi.row(row, s, pre);
          }
        } else {
          if (shortrow) {
            ACC s[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) s[v] = ACC(0);
            short_row_sum<T, NV, MAXRED>(b, e, idx, val, prod, s);
            epi.row(row, s);
          }
        }
        unsigned pending = __ballot_sync(0xffffffffu, valid && !shortrow);
        while (pending != 0u) {
          const int src = __ffs(pending) - 1;
          pending &= pending - 1u;
          const int rb = __shfl_sync(0xffffffffu, b, src);
          const int re = __shfl_sync(0xffffffffu, e, src);
          const int rrow = __shfl_sync(0xffffffffu, row, src);
          ACC s[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = ACC(0);
#pragma unroll 4
          for (int q = rb + lane; q < re; q += 32) {
            const T a = ldg(val + q);
            const int j = ldg(idx + q);
#pragma unroll
            for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              s[v] = combine<MAXRED>(s[v], __shfl_down_sync(0xffffffffu, s[v], o));
            }
          }
          if (lane == 0) epi.row(rrow, s);
        }
      }
    } else if (tile.kind == 2) {
      // Rows of medium length, `team` warps each (1, 2, 4 or 8; the CTA holds 8 / team rows):
      // head up to a 4-aligned position, 16-byte loads of four nonzeros per lane (the team's
      // warps take every team-th block of 128 nonzeros), tail, then the fixed shuffle tree;
      // the team's partial sums are added in warp order and lane 0 of its first warp updates
      // the row.
      const int lane = tid & 31;
      const int warp = tid >> 5;
      const int team = tile.team;
      const int part = warp & (team - 1);
      const int rv = tile.r0 + warp / team;
      const int r = rv < tile.r1 ? tile_row(ts, rv) : 0;
      ACC s[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) s[v] = ACC(0);
      if (rv < tile.r1) {
        const int b = ldg(ptr + r);
        const int e = ldg(ptr + r + 1);
        const int a0 = min(e, (b + 3) & ~3);
        const int a1 = max(a0, e & ~3);
        if (part == 0 && b + lane < a0) {
          const int q = b + lane;
          const T a = ldg(val + q);
          const int j = ldg(idx + q);
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
        }
        auto quad = [&](int q) {
          T a[4];
          Vec4<T>::load(val, q, a);
          const int4 j = __ldg(reinterpret_cast<const int4*>(idx + q));
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            s[v] = combine<MAXRED>(s[v], prod(v, a[0], j.x));
            s[v] = combine<MAXRED>(s[v], prod(v, a[1], j.y));
            s[v] = combine<MAXRED>(s[v], prod(v, a[2], j.z));
            s[v] = combine<MAXRED>(s[v], prod(v, a[3], j.w));
          }
        };
        // A warp per row keeps its own loop (a compile-time stride unrolls deeper).
        const int step = 128 * team;
        if constexpr (WIDE) {
          if (team == 1) {
#pragma unroll 8
            for (int q = a0 + 4 * lane; q < a1; q += 128) quad(q);
          } else {
#pragma unroll 8
            for (int q = a0 + 4 * lane + 128 * part; q < a1; q += step) quad(q);
          }
        } else {
          if (team == 1) {
#pragma unroll 4
            for (int q = a0 + 4 * lane; q < a1; q += 128) quad(q);
          } else {
#pragma unroll 4
            for (int q = a0 + 4 * lane + 128 * part; q < a1; q += step) quad(q);
          }
        }
        if (part == 0 && a1 + lane < e) {
          const int q = a1 + lane;
          const T a = ldg(val + q);
          const int j = ldg(idx + q);
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            s[v] = combine<MAXRED>(s[v], __shfl_down_sync(0xffffffffu, s[v], o));
          }
        }
        if (team == 1 && lane == 0) epi.row(r, s);
      }
      if (team > 1) {
        // team is uniform over the tile, so every thread of the CTA reaches both barriers.
        ACC* partial = reinterpret_cast<ACC*>(red);
        if (lane == 0) {
#pragma unroll
          for (int v = 0; v < NV; ++v) partial[warp * NV + v] = s[v];
        }
        __syncthreads();
        if (part == 0 && lane == 0 && rv < tile.r1) {
          ACC tot[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            ACC a = partial[warp * NV + v];
            for (int w = 1; w < team; ++w) a = combine<MAXRED>(a, partial[(warp + w) * NV + v]);
            tot[v] = a;
          }
          epi.row(r, tot);
        }
        __syncthreads();
      }
    } else {
      // A segment of a long row: strided sums, then the fixed block tree (in the accumulation
      // type: FP32 kernels keep off GB300's small FP64 pipe).
      ACC s[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) s[v] = ACC(0);
      bool staged_done = false;
      if constexpr (GROUPS) {
        if (ts.staged) {
          // The segment [k0, k1) streamed through shared memory: chunks of kSegChunk nonzeros
          // from the 4-aligned position below k0 to the one above k1 (16-byte aligned copies
          // of a multiple of 16 bytes; the arrays carry kSegPad elements of padding), two in
          // flight, completing on an mbarrier each. Thread t sums the in-segment elements at
          // 4 t .. 4 t + 3 and 4 t + 1024 .. of every chunk, in chunk order.
          int* cidx = reinterpret_cast<int*>(red + kRedDoubles);
          T* cval = reinterpret_cast<T*>(cidx + 2 * kSegChunk);
          const int k0 = tile.k0;
          const int k1 = tile.k1;
          const int base = k0 & ~3;
          const int end = (k1 + 3) & ~3;
          const int nch = (end - base + kSegChunk - 1) / kSegChunk;
          auto issue = [&](int c) {
            const int st = c & 1;
            const int from = base + c * kSegChunk;
            const int len = min(kSegChunk, end - from);
            const unsigned bi = static_cast<unsigned>(len) * sizeof(int);
            const unsigned bv = static_cast<unsigned>(len) * sizeof(T);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(&seg_bar[st], bi + bv);
            bulk_copy_g2s(cidx + st * kSegChunk, idx + from, bi, &seg_bar[st]);
            bulk_copy_g2s(cval + st * kSegChunk, val + from, bv, &seg_bar[st]);
          };
          auto wait = [&](int c) {
            const int st = c & 1;
            if (!mbar_wait_bounded(&seg_bar[st], (seg_parity >> st) & 1u)) seg_fail = 1;
            seg_parity ^= 1u << st;
          };
          if (tid == 0) {
            issue(0);
            if (nch > 1) issue(1);
          }
          wait(0);
          __syncthreads();
          for (int c = 0; c < nch && !seg_fail; ++c) {
            const int st = c & 1;
            const int from = base + c * kSegChunk;
#pragma unroll
            for (int u = 0; u < kSegChunk / (4 * kBlock); ++u) {
              const int e = 4 * tid + u * 4 * kBlock;
              const int4 j = *reinterpret_cast<const int4*>(cidx + st * kSegChunk + e);
              const T* vp = cval + st * kSegChunk + e;
              const int p = from + e;
              const int jj[4] = {j.x, j.y, j.z, j.w};
#pragma unroll
              for (int w = 0; w < 4; ++w) {
                if (p + w >= k0 && p + w < k1) {
#pragma unroll
                  for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, vp[w], jj[w]));
                }
              }
            }
            if (c + 1 < nch) wait(c + 1);
            __syncthreads();
            if (tid == 0 && c + 2 < nch && !seg_fail) issue(c + 2);
          }
          if (seg_fail) {
            // A copy never completed: report it and leave the tile loop (the solve then fails
            // on the flag; the sums of this launch are not used).
            if (tid == 0) atomicExch(ts.wait_error, 1);
            return;
          }
          staged_done = true;
        }
      }
      if (!staged_done) {
        // Head up to a 4-aligned position, then 16-byte loads of four nonzeros per thread,
        // then the tail (scalar).
        const int k0 = tile.k0;
        const int k1 = tile.k1;
        const int a0 = min(k1, (k0 + 3) & ~3);
        const int a1 = max(a0, k1 & ~3);
        if (k0 + tid < a0) {
          const int q = k0 + tid;
          const T a = ldg(val + q);
          const int j = ldg(idx + q);
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
        }
        auto quad = [&](int q) {
          T a[4];
          Vec4<T>::load(val, q, a);
          const int4 j = __ldg(reinterpret_cast<const int4*>(idx + q));
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            s[v] = combine<MAXRED>(s[v], prod(v, a[0], j.x));
            s[v] = combine<MAXRED>(s[v], prod(v, a[1], j.y));
            s[v] = combine<MAXRED>(s[v], prod(v, a[2], j.z));
            s[v] = combine<MAXRED>(s[v], prod(v, a[3], j.w));
          }
        };
        if constexpr (WIDE) {
#pragma unroll 4
          for (int q = a0 + 4 * tid; q < a1; q += 4 * kBlock) quad(q);
        } else {
#pragma unroll 2
          for (int q = a0 + 4 * tid; q < a1; q += 4 * kBlock) quad(q);
        }
        for (int q = a1 + tid; q < k1; q += kBlock) {
          const T a = ldg(val + q);
          const int j = ldg(idx + q);
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = combine<MAXRED>(s[v], prod(v, a, j));
        }
      }
      ACC tot[NV];
      block_reduce_acc<ACC, NV, MAXRED>(s, reinterpret_cast<ACC*>(red), tot);
      if (tile.nseg == 1) {
        // The whole row in one tile: no partials to combine.
        if (tid == 0) epi.long_row(tile.lrow, tile_row(ts, tile.r0), tot);
        continue;
      }
      if (tid == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) ts.seg_part[ti * kMaxVec + v] = static_cast<double>(tot[v]);
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
        block_reduce<NV, MAXRED ? 0xFFu : 0u>(acc, red, sum);
        if (tid == 0) {
          ACC s[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) s[v] = static_cast<ACC>(sum[v]);
          ts.lcount[tile.lrow] = 0u;
          epi.long_row(tile.lrow, tile_row(ts, tile.r0), s);
        }
      }
      __syncthreads();
    }
  }
}

}  // namespace sg
