// sp_idas_parallel: Horie's host-callable search (src_horie/idas_parallel_host.h:33-34,
// src_horie/idas_parallel.cu:239-244), the one C function of the reference
// that a host program can call.
//
// Semantics kept from the reference (src_horie/idas_parallel.cu:172-236):
// every root of the 15-puzzle is searched on its own, depth-first, moves
// tried in the order up, right, left, down, the reverse of the last move
// skipped (none at the root), a child entered only if its depth below the
// root + 1 + h <= f_limit, h updated by the caller's h-difference table
// (h_diff[tile][its cell][blank's move]; the reverse move on backtracking),
// moves allowed by the caller's movable table [cell][move]; the search of a
// root stops at its first goal, and the root's plan row is [len, moves...]
// or [-1].  The root's own depth is not counted: roots are searched as if at
// depth 0.  No node counts: the reference reports none on this path.  Two
// guards the reference lacks: a path never grows past the plan row (251
// moves), and a root searched for more than 30 s gives up with [-2].
//
// GPU shape: one thread per root, its board packed 4 bits per cell in a
// 64-bit register, its move stack 2 bits per level in shared memory
// ([word][thread]: every thread owns a bank), both tables copied into shared
// memory by each block (or, with null table pointers, built there from the
// Manhattan distance as the reference's init_mdist / init_movable_table do,
// src_horie/idas_parallel_host.c:88-129).  Allocates nothing; launches on the
// caller's stream and returns, like the reference.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/slide.h"
#include "sp_defs.h"
#include "sp_kernels.h"

namespace sp {
namespace {

constexpr int kW = 4, kN = 16;
constexpr int kFpBlock = 128;
constexpr int kFpWords = (SP_PLAN_STRIDE + 15) / 16;  // 2-bit moves per lane, 16 per word
constexpr unsigned long long kFpLimitNs = 30000000000ull;  // 30 s per root

__global__ void __launch_bounds__(kFpBlock) first_path_kernel(const uint8_t *input, int n, int8_t *plan,
                                                              int f_limit, const int8_t *hdiff_in,
                                                              const uint8_t *movable_in) {
  __shared__ int8_t s_hdiff[kN * kN * 4];  // [tile][cell][move], the reference's layout
  __shared__ uint8_t s_mov[kN * 4];        // [cell][move]
  __shared__ uint32_t s_stack[kFpWords][kFpBlock];
  for (int i = threadIdx.x; i < kN * kN * 4; i += kFpBlock) {
    if (hdiff_in) {
      s_hdiff[i] = hdiff_in[i];
    } else {
      // the tile at `cell` moves against the blank's move: one step closer to
      // or farther from its goal cell (the tile's number)
      const int t = i / (kN * 4), c = (i / 4) % kN, d = i % 4;
      const int gr = t / kW, gc = t % kW, r = c / kW, cc = c % kW;
      int v = 0;
      if (d == 0) v = gr > r ? -1 : 1;        // blank up: tile down
      else if (d == 1) v = gc < cc ? -1 : 1;  // blank right: tile left
      else if (d == 2) v = gc > cc ? -1 : 1;  // blank left: tile right
      else v = gr < r ? -1 : 1;               // blank down: tile up
      s_hdiff[i] = (int8_t)v;
    }
  }
  // a caller's movable table is also held to the board's edges, so that no
  // table can move the blank off the board
  for (int i = threadIdx.x; i < kN * 4; i += kFpBlock)
    s_mov[i] = (uint8_t)((legal_moves(kW, i / 4) >> (i % 4)) & 1u) & (movable_in ? (movable_in[i] ? 1 : 0) : 1);
  __syncthreads();

  const int id = blockIdx.x * kFpBlock + threadIdx.x;
  if (id >= n) return;
  const int tid = threadIdx.x;
  int8_t *row = plan + (size_t)id * SP_PLAN_STRIDE;
  uint64_t b = 0;
  int blank = 0, h = 0;
  for (int c = 0; c < kN; ++c) {
    const uint32_t t = input[(size_t)id * kN + c] & 15u;
    b |= (uint64_t)t << (4 * c);
    if (!t) blank = c;
    else h += abs(c / kW - (int)t / kW) + abs(c % kW - (int)t % kW);
  }
  auto tile_at = [&](int c) -> int { return (int)((b >> (4 * c)) & 15u); };
  // the blank moves by d: the tile at the blank's new cell slides into its old one
  auto apply = [&](int d) {
    const int to = blank + move_delta(kW, d);
    const int t = tile_at(to);
    h += s_hdiff[(t * kN + to) * 4 + d];
    b ^= ((uint64_t)t << (4 * to)) ^ ((uint64_t)t << (4 * blank));
    blank = to;
  };
  int depth = 0, dir = 0;
  // the stack word holding level depth - 1, the last move made (completed
  // words below it sit in shared memory)
  uint32_t top = 0;
  auto last = [&]() -> int { return (int)((top >> (2 * ((depth - 1) & 15))) & 3u); };
  // a root whose search outlives the time limit (only a caller table that
  // lets h fall without bound can make one run that long) gives up: -2
  unsigned long long t0 = 0;
  uint32_t spin = 0;
  for (;;) {
    if ((++spin & 4095u) == 0) {
      unsigned long long now;
      asm volatile("mov.u64 %0, %globaltimer;" : "=l"(now));
      if (!t0) t0 = now;
      else if (now - t0 > kFpLimitNs) {
        row[0] = -2;
        return;
      }
    }
    if (h == 0) {  // the first goal in depth-first order: its path is the plan
      row[0] = (int8_t)depth;
      for (int i = 0; i < depth; ++i) {
        const uint32_t w = (i >> 4) == ((depth - 1) >> 4) ? top : s_stack[i >> 4][tid];
        row[1 + i] = (int8_t)((w >> (2 * (i & 15))) & 3u);
      }
      return;
    }
    if ((depth == 0 || last() != 3 - dir) && s_mov[blank * 4 + dir]) {
      const int to = blank + move_delta(kW, dir);
      const int nh = h + s_hdiff[(tile_at(to) * kN + to) * 4 + dir];
      if (depth + 1 + nh <= f_limit && depth + 1 < SP_PLAN_STRIDE) {
        apply(dir);
        const int sh = 2 * (depth & 15);
        top = sh ? (top & ~(3u << sh)) | ((uint32_t)dir << sh) : (uint32_t)dir;  // sh 0: a new word
        if ((depth & 15) == 15) s_stack[depth >> 4][tid] = top;
        ++depth;
        dir = 0;
        continue;
      }
    }
    while (++dir == 4) {
      if (depth == 0) {
        row[0] = -1;
        return;
      }
      --depth;  // undo the move of level depth, held in top
      dir = (int)((top >> (2 * (depth & 15))) & 3u);
      if ((depth & 15) == 0 && depth > 0) top = s_stack[(depth >> 4) - 1][tid];
      apply(3 - dir);
    }
  }
}

}  // namespace
}  // namespace sp

extern "C" int sp_idas_parallel(const uint8_t *d_input, int n, int8_t *d_plan, int f_limit,
                                const int8_t *d_h_diff_table, const uint8_t *d_movable_table, void *stream) {
  if (n < 0 || (n > 0 && (!d_input || !d_plan)) || f_limit < 0 || f_limit > SP_PLAN_STRIDE - 1) return SP_ERR_ARG;
  if (n == 0) return SP_OK;
  // an error the caller left pending is the caller's: report it without clearing it
  if (cudaPeekAtLastError() != cudaSuccess) return SP_ERR_CUDA;
  const int grid = (n + sp::kFpBlock - 1) / sp::kFpBlock;
  sp::first_path_kernel<<<grid, sp::kFpBlock, 0, (cudaStream_t)stream>>>(d_input, n, d_plan, f_limit, d_h_diff_table,
                                                                         d_movable_table);
  sp::note_launch();
  return cudaGetLastError() == cudaSuccess ? SP_OK : SP_ERR_CUDA;
}
