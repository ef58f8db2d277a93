// GPU breadth-first construction of the additive pattern databases, layout
// conversions, and the batched heuristic kernel.
//
// The reference loads two 6-tile tables from files it does not ship
// (src/24puzzle_block_parallel_with_pdb.cu:164-230).  Their contents are
// defined here by the abstraction that reproduces the reference's golden
// node counts (benchmarks/pdb_expand_nodes.csv, all 50 rows):
//   * an abstract state is the pattern tiles' cells plus the connected region
//     of non-pattern cells that holds the blank (other tiles move for free
//     inside a region);
//   * one abstract move slides a pattern tile into a neighbouring cell of the
//     blank's region, cost 1;
//   * the goal is the pattern tiles on their goal cells with the blank in the
//     region of its home cell 0;
//   * a table entry is the distance to the goal, minimised over the blank's
//     regions (the reference's index holds no blank position).
// The search runs level-synchronously over a [placement rank][region]
// byte array (placement rank = lexicographic rank of the k-permutation of
// cells, the byte order of the reference's table files), one thread per
// placement row per level.  Rows are 16 or 32 bytes (one byte per possible
// lowest cell of a region) so a row is read with one or two 16-byte loads.
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>

#include "sp_defs.h"
#include "sp_device.cuh"
#include "sp_kernels.h"

namespace sp {

namespace {

struct Geo {
  int w, n, k;
  uint32_t full, not_col0, not_collast;
  int base[6];
};

Geo make_geo(int w, int table_id) {
  Geo g{};
  g.w = w;
  g.n = w * w;
  PatternSet ps = pattern_set(w);
  g.k = ps.k;
  g.full = (1u << g.n) - 1u;
  uint32_t c0 = 0, cl = 0;
  for (int r = 0; r < w; ++r) {
    c0 |= 1u << (r * w);
    cl |= 1u << (r * w + w - 1);
  }
  g.not_col0 = g.full & ~c0;
  g.not_collast = g.full & ~cl;
  for (int j = 0; j < g.k; ++j) g.base[j] = ps.table_tiles[table_id][j];
  return g;
}

__host__ __device__ __forceinline__ uint32_t flood(const Geo &g, uint32_t free_cells, int c) {
  uint32_t r = 1u << c, prev;
  do {
    prev = r;
    r = (r | ((r << 1) & g.not_col0) | ((r >> 1) & g.not_collast) | (r << g.w) | (r >> g.w)) &
        free_cells;
  } while (r != prev);
  return r;
}

__host__ __device__ __forceinline__ int neighbour(const Geo &g, int cell, int d) {
  int r = cell / g.w, c = cell - r * g.w;
  switch (d) {
    case 0: return r == 0 ? -1 : cell - g.w;
    case 1: return c == g.w - 1 ? -1 : cell + 1;
    case 2: return c == 0 ? -1 : cell - 1;
    default: return r == g.w - 1 ? -1 : cell + g.w;
  }
}

__host__ __device__ __forceinline__ uint64_t rank_k(int n, int k, const int *pos) {
  uint64_t r = 0;
  uint32_t used = 0;
  for (int i = 0; i < k; ++i) {
#ifdef __CUDA_ARCH__
    int less = __popc(used & ((1u << pos[i]) - 1u));
#else
    int less = __builtin_popcount(used & ((1u << pos[i]) - 1u));
#endif
    r = r * (uint64_t)(n - i) + (uint64_t)(pos[i] - less);
    used |= 1u << pos[i];
  }
  return r;
}

__device__ __forceinline__ void unrank_k(int n, int k, uint64_t r, int *pos) {
  int digit[6];
  for (int i = k - 1; i >= 0; --i) {
    uint64_t q = r / (uint64_t)(n - i);
    digit[i] = (int)(r - q * (uint64_t)(n - i));
    r = q;
  }
  uint32_t unused = (1u << n) - 1u;
  for (int i = 0; i < k; ++i) {
    // position of the (digit+1)-th set bit of `unused`
    uint32_t m = unused;
    for (int s = 0; s < digit[i]; ++s) m &= m - 1u;
    int c = __ffs(m) - 1;
    pos[i] = c;
    unused &= ~(1u << c);
  }
}

__device__ __forceinline__ uint32_t lookup_index(int n, int k, const int *pos) {
  uint32_t x = 0;
  for (int j = 0; j < k; ++j) x = x * (uint32_t)n + (uint32_t)pos[j];
  return x;
}

constexpr uint8_t kUnseen = 0xFF;

template <int STRIDE>
__global__ void bfs_level_kernel(uint8_t *dist, uint64_t T, Geo g, int d,
                                 unsigned long long *produced) {
  unsigned long long local = 0;
  const uint32_t dd = 0x01010101u * (uint32_t)d;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < T;
       r += (uint64_t)gridDim.x * blockDim.x) {
    uint8_t *row = dist + r * STRIDE;
    uint4 v[STRIDE / 16];
#pragma unroll
    for (int q = 0; q < STRIDE / 16; ++q) v[q] = *(const uint4 *)(row + 16 * q);
    uint32_t hit = 0;
#pragma unroll
    for (int q = 0; q < STRIDE / 16; ++q)
      hit |= __vcmpeq4(v[q].x, dd) | __vcmpeq4(v[q].y, dd) | __vcmpeq4(v[q].z, dd) |
             __vcmpeq4(v[q].w, dd);
    if (!hit) continue;
    const uint8_t *rb = (const uint8_t *)v;
    int pos[6] = {0, 0, 0, 0, 0, 0};
    unrank_k(g.n, g.k, r, pos);
    uint32_t occ = 0;
    for (int j = 0; j < g.k; ++j) occ |= 1u << pos[j];
    const uint32_t free_cells = g.full & ~occ;
    for (int m = 0; m < g.n; ++m) {
      if (rb[m] != d) continue;
      const uint32_t reg = flood(g, free_cells, m);
      for (int j = 0; j < g.k; ++j) {
        for (int dir = 0; dir < 4; ++dir) {
          const int c = neighbour(g, pos[j], dir);
          if (c < 0 || !((reg >> c) & 1u)) continue;
          int q[6];
          for (int a = 0; a < 6; ++a) q[a] = pos[a];
          q[j] = c;
          const uint32_t free2 = (free_cells & ~(1u << c)) | (1u << pos[j]);
          const uint32_t reg2 = flood(g, free2, pos[j]);
          const uint64_t r2 = rank_k(g.n, g.k, q);
          uint8_t *e = dist + r2 * STRIDE + (__ffs(reg2) - 1);
          if (*e == kUnseen) {
            *e = (uint8_t)(d + 1);
            ++local;
          }
        }
      }
    }
  }
  if (local) atomicAdd(produced, local);
}

template <int STRIDE>
__global__ void region_min_kernel(const uint8_t *dist, uint64_t T, int n, uint8_t *compact) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < T;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t *row = dist + r * STRIDE;
    uint8_t best = kUnseen;
    for (int m = 0; m < n; ++m) best = min(best, row[m]);
    compact[r] = best;
  }
}

__global__ void compact_lookup_kernel(int n, int k, uint64_t T, const uint8_t *src, uint8_t *dst,
                                      int to_lookup) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < T;
       r += (uint64_t)gridDim.x * blockDim.x) {
    int pos[6] = {0, 0, 0, 0, 0, 0};
    unrank_k(n, k, r, pos);
    const uint32_t x = lookup_index(n, k, pos);
    if (to_lookup) dst[x] = src[r];
    else dst[r] = src[x];
  }
}

template <int W, bool PDB>
__global__ void heuristic_kernel(const uint8_t *boards, int n, int32_t *hout, const HeurTables *ht,
                                 const uint8_t *tables) {
  constexpr int N = W * W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  hout[i] = board_h<W, PDB>(boards + (size_t)i * N, ht, tables);
}

int grid_for(uint64_t T, int block) {
  uint64_t g = (T + block - 1) / block;
  if (g > 152ull * 64ull) g = 152ull * 64ull;
  return (int)(g ? g : 1);
}

}  // namespace

uint64_t compact_table_size(int w) {
  PatternSet ps = pattern_set(w);
  uint64_t s = 1;
  for (int i = 0; i < ps.k; ++i) s *= (uint64_t)(w * w - i);
  return s;
}

uint64_t lookup_table_stride(int w) { return w == 4 ? (1ull << 20) : (1ull << 28); }

cudaError_t pdb_compact_to_lookup(int w, int table_id, const uint8_t *compact, uint8_t *lookup,
                                  cudaStream_t st) {
  PatternSet ps = pattern_set(w);
  const uint64_t T = compact_table_size(w);
  cudaError_t e = cudaMemsetAsync(lookup, 0, lookup_table_stride(w), st);
  if (e != cudaSuccess) return e;
  compact_lookup_kernel<<<grid_for(T, 256), 256, 0, st>>>(w * w, ps.k, T, compact, lookup, 1);
  note_launch();
  (void)table_id;
  return cudaGetLastError();
}

cudaError_t pdb_lookup_to_compact(int w, int table_id, const uint8_t *lookup, uint8_t *compact,
                                  cudaStream_t st) {
  PatternSet ps = pattern_set(w);
  const uint64_t T = compact_table_size(w);
  compact_lookup_kernel<<<grid_for(T, 256), 256, 0, st>>>(w * w, ps.k, T, lookup, compact, 0);
  note_launch();
  (void)table_id;
  return cudaGetLastError();
}

cudaError_t build_pdb_table(int w, int table_id, uint8_t *lookup, uint8_t *compact,
                            cudaStream_t st, int *levels_out, double *ms_out) {
  auto t0 = std::chrono::steady_clock::now();
  const Geo g = make_geo(w, table_id);
  const uint64_t T = compact_table_size(w);
  const int stride = g.n <= 16 ? 16 : 32;
  uint8_t *dist = nullptr, *cmp = nullptr;
  unsigned long long *produced = nullptr, *h_produced = nullptr;
  cudaError_t e = cudaMalloc(&dist, T * (uint64_t)stride);
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&cmp, T);
  if (e == cudaSuccess) e = cudaMalloc(&produced, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost(&h_produced, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(dist, 0xFF, T * (uint64_t)stride, st);
  if (e == cudaSuccess) {
    // goal: pattern tiles home, blank in the region of cell 0
    uint32_t occ = 0;
    for (int j = 0; j < g.k; ++j) occ |= 1u << g.base[j];
    const uint32_t reg = flood(g, g.full & ~occ, 0);
    const uint64_t r0 = rank_k(g.n, g.k, g.base);
    static const uint8_t zero = 0;
    e = cudaMemcpyAsync(dist + r0 * stride + (__builtin_ffs((int)reg) - 1), &zero, 1,
                        cudaMemcpyHostToDevice, st);
  }
  int levels = 0;
  for (int d = 0; e == cudaSuccess && d < 254; ++d) {
    e = cudaMemsetAsync(produced, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) break;
    if (stride == 16)
      bfs_level_kernel<16><<<grid_for(T, 256), 256, 0, st>>>(dist, T, g, d, produced);
    else
      bfs_level_kernel<32><<<grid_for(T, 256), 256, 0, st>>>(dist, T, g, d, produced);
    note_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_produced, produced, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    levels = d + 1;
    if (e != cudaSuccess || *h_produced == 0) break;
  }
  if (e == cudaSuccess) {
    if (stride == 16)
      region_min_kernel<16><<<grid_for(T, 256), 256, 0, st>>>(dist, T, g.n, cmp);
    else
      region_min_kernel<32><<<grid_for(T, 256), 256, 0, st>>>(dist, T, g.n, cmp);
    note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = pdb_compact_to_lookup(w, table_id, cmp, lookup, st);
  if (e == cudaSuccess && compact) e = cudaMemcpyAsync(compact, cmp, T, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(dist);
  cudaFree(cmp);
  cudaFree(produced);
  cudaFreeHost(h_produced);
  if (levels_out) *levels_out = levels;
  if (ms_out)
    *ms_out = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return e;
}

cudaError_t launch_heuristic(int w, bool pdb, const uint8_t *boards, int n, int32_t *h,
                             const HeurTables *ht, const uint8_t *tables, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (n + 127) / 128;
  if (w == 4) {
    if (pdb) heuristic_kernel<4, true><<<blocks, 128, 0, st>>>(boards, n, h, ht, tables);
    else heuristic_kernel<4, false><<<blocks, 128, 0, st>>>(boards, n, h, ht, tables);
  } else {
    if (pdb) heuristic_kernel<5, true><<<blocks, 128, 0, st>>>(boards, n, h, ht, tables);
    else heuristic_kernel<5, false><<<blocks, 128, 0, st>>>(boards, n, h, ht, tables);
  }
  note_launch();
  return cudaGetLastError();
}

}  // namespace sp
