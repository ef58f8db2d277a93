// Root set ("frontier") of a batch on the device.
//
// The root set of an instance is its search tree expanded to a uniform depth
// D with no pruning and no duplicate detection (the reference builds a root
// set of BLOCK_NUM nodes per instance, create_root_set in
// src/24puzzle_block_parallel_with_pdb.cu:454-490).  Without pruning the
// tree's shape -- which move sequences it holds, in breadth-first order --
// depends only on the cell of the blank, so the host builds one template per
// blank cell (moves from the root, parent, depth, children) and this kernel
// applies it to every instance at once: one block per instance replays each
// node's moves on the instance's board, computes h and the prefix maximum of
// g + h along the node's path, and writes
//   * the leaves (depth D) as SubRoot records sorted by that maximum, ties in
//     tree order (the active roots of a threshold round are then a prefix);
//   * per maximum value: the number of leaves, the children generated by
//     interior nodes, and the shallowest goal node (h == 0), which is what
//     the threshold loop needs to count the nodes above the roots.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/slide.h"
#include "sp_defs.h"
#include "sp_device.cuh"
#include "sp_kernels.h"

namespace sp {
namespace {

constexpr int kFrontThreads = 1024;
constexpr int kFrontWarps = kFrontThreads / 32;

template <int W>
__device__ __forceinline__ int replay(const uint8_t *root, int root_blank, uint64_t path, int depth, uint8_t *b) {
  constexpr int N = W * W;
  for (int c = 0; c < N; ++c) b[c] = root[c];
  int blank = root_blank;
  for (int j = 0; j < depth; ++j) {
    const int d = (int)((path >> (2 * j)) & 3u);
    const int src = blank + move_delta(W, d);
    b[blank] = b[src];
    b[src] = 0;
    blank = src;
  }
  return blank;
}

template <int W, bool PDB>
__global__ void __launch_bounds__(kFrontThreads) frontier_kernel(FrontArgs A) {
  constexpr int N = W * W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t li = blockIdx.x;
  const uint32_t inst = A.live[li];
  const uint32_t ti = A.live_tmpl[li];
  const FrontTmpl T = A.tmpl[ti];
  const uint32_t *lev = A.lev + (size_t)ti * kFrontLevStride;
  const uint64_t *path = A.path + T.node_off;
  const int32_t *parent = A.parent + T.node_off;
  const uint8_t *nchild = A.nchild + T.node_off;
  const uint8_t *depth = A.depth + T.node_off;
  int16_t *F = A.f + A.live_scratch[li];
  int16_t *M = A.maxf + A.live_scratch[li];

  __shared__ uint8_t s_root[32];
  __shared__ int s_blank, s_bad;
  __shared__ uint32_t s_leaf[kFrontBuckets], s_child[kFrontBuckets], s_goal[kFrontBuckets];
  __shared__ uint32_t s_wcnt[kFrontWarps][kFrontBuckets];

  if (tid < N) {
    const uint8_t v = A.tiles[(size_t)inst * N + tid];
    s_root[tid] = v;
    if (v == 0) s_blank = tid;
  }
  for (int b = tid; b < kFrontBuckets; b += kFrontThreads) {
    s_leaf[b] = 0;
    s_child[b] = 0;
    s_goal[b] = 0xFFFFFFFFu;
    for (int q = 0; q < kFrontWarps; ++q) s_wcnt[q][b] = 0;
  }
  if (tid == 0) s_bad = 0;
  __syncthreads();

  // 1. g + h of every node
  uint8_t bd[N];
  for (uint32_t x = tid; x < T.n_nodes; x += kFrontThreads) {
    const int dep = depth[x];
    replay<W>(s_root, s_blank, path[x], dep, bd);
    F[x] = (int16_t)(dep + board_h<W, PDB>(bd, A.ht, A.pdb));
  }
  __syncthreads();
  const int h0 = F[0];
  // 2. prefix maximum of g + h along each path, one level at a time (the
  //    parent of a level-d node is on level d - 1)
  for (uint32_t d = 0; d <= T.D; ++d) {
    for (uint32_t x = lev[d] + tid; x < lev[d + 1]; x += kFrontThreads)
      M[x] = d ? (int16_t)max((int)F[x], (int)M[parent[x]]) : F[x];
    __syncthreads();
  }
  // 3. per maximum (bucket = maxf - h0): leaves, interior children, goals
  for (uint32_t x = tid; x < T.n_nodes; x += kFrontThreads) {
    const int b = M[x] - h0;
    const int dep = depth[x];
    if (b < 0 || b >= kFrontBuckets) {
      s_bad = 1;
      continue;
    }
    if ((uint32_t)dep == T.D) atomicAdd(&s_leaf[b], 1u);
    else atomicAdd(&s_child[b], (uint32_t)nchild[x]);
    if (F[x] == dep) atomicMin(&s_goal[b], ((uint32_t)dep << 24) | x);
  }
  __syncthreads();
  if (s_bad) {  // h changed by more than the bucket range allows along a path
    if (tid == 0) atomicCAS(A.error, 0, (int32_t)SP_ERR_ARG);
    return;
  }
  if (tid == 0) {  // exclusive prefix of the leaf counts, kept in s_leaf
    uint32_t c = 0;
    for (int b = 0; b < kFrontBuckets; ++b) {
      const uint32_t v = s_leaf[b];
      s_leaf[b] = c;
      c += v;
    }
  }
  __syncthreads();
  // 4. the leaves in tree order, each to its bucket's next position (a
  //    stable counting sort: ranks within a warp from the match mask, then
  //    the counts of the lower warps of the same chunk)
  const uint32_t l0 = lev[T.D], l1 = lev[T.D + 1];
  const uint32_t base = A.live_base[li];
  for (uint32_t c0 = l0; c0 < l1; c0 += kFrontThreads) {
    const uint32_t x = c0 + tid;
    const bool valid = x < l1;
    const int b = valid ? M[x] - h0 : kFrontBuckets;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, b);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) s_wcnt[warp][b] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pos = s_leaf[b] + rank;
      for (int q = 0; q < warp; ++q) pos += s_wcnt[q][b];
      const uint32_t j = base + pos;
      SubRoot r{};
      const int blank = replay<W>(s_root, s_blank, path[x], (int)T.D, bd);
      for (int c = 0; c < N; ++c) r.board[c] = bd[c];
      r.blank = (uint8_t)blank;
      r.g = (uint8_t)T.D;
      r.pre = T.D ? (uint8_t)((path[x] >> (2 * (T.D - 1))) & 3u) : kNoPre;
      r.inst = inst;
      const uint4 *src = reinterpret_cast<const uint4 *>(&r);
      uint4 *dst = reinterpret_cast<uint4 *>(A.subs + j);
      dst[0] = src[0];
      dst[1] = src[1];
      A.leaf_maxf[j] = M[x];
      A.leaf_h[j] = (uint8_t)(F[x] - (int)T.D);
      A.leaf_node[j] = (int32_t)x;
    }
    __syncthreads();
    for (int bb = tid; bb < kFrontBuckets; bb += kFrontThreads) {
      uint32_t t = 0;
      for (int q = 0; q < kFrontWarps; ++q) {
        t += s_wcnt[q][bb];
        s_wcnt[q][bb] = 0;
      }
      s_leaf[bb] += t;
    }
    __syncthreads();
  }
  // 5. per-instance summary (s_leaf now holds inclusive counts)
  FrontInst *O = A.out + li;
  if (tid == 0) {
    O->h0 = h0;
    O->n_leaves = l1 - l0;
  }
  for (int b = tid; b < kFrontBuckets; b += kFrontThreads) {
    O->leaf_cum[b] = s_leaf[b];
    O->child[b] = s_child[b];
    O->goal[b] = s_goal[b];
  }
}

}  // namespace

cudaError_t launch_frontier(int w, bool pdb, int n_live, const FrontArgs &A, cudaStream_t st) {
  if (n_live <= 0) return cudaSuccess;
  if (w == 4) {
    if (pdb) frontier_kernel<4, true><<<n_live, kFrontThreads, 0, st>>>(A);
    else frontier_kernel<4, false><<<n_live, kFrontThreads, 0, st>>>(A);
  } else {
    if (pdb) frontier_kernel<5, true><<<n_live, kFrontThreads, 0, st>>>(A);
    else frontier_kernel<5, false><<<n_live, kFrontThreads, 0, st>>>(A);
  }
  note_launch();
  return cudaGetLastError();
}

}  // namespace sp
