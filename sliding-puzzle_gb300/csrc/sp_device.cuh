// Device helpers shared by the kernels of libslide.
#pragma once
#include <stdint.h>

#include "sp_defs.h"

namespace sp {

// Heuristic of a board from scratch: Manhattan distance, or the additive PDB
// value max(sum of regular-partition lookups, sum of reflected lookups) with
// tables at t << 20 (width 4) or t << 28 (width 5) in `tables`.
template <int W, bool PDB>
__device__ __forceinline__ int board_h(const uint8_t *b, const HeurTables *ht, const uint8_t *tables) {
  constexpr int N = W * W;
  if (!PDB) {
    int s = 0;
    for (int c = 0; c < N; ++c) {
      const int t = b[c];
      if (!t) continue;
      s += abs(c / W - t / W) + abs(c % W - t % W);
    }
    return s;
  }
  constexpr int NP = W == 5 ? 4 : 3;
  uint32_t idx[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  for (int c = 0; c < N; ++c) {
    const int t = b[c];
    if (!t) continue;
    for (int part = 0; part < 2; ++part) idx[part][ht->pat[part][t]] += ht->code[part][t * N + c];
  }
  int best = 0;
  for (int part = 0; part < 2; ++part) {
    int s = 0;
    for (int p = 0; p < NP; ++p) {
      const size_t off = (W == 4) ? ((size_t)p << 20) : (p ? ((size_t)1 << 28) : 0);
      s += __ldg(tables + off + idx[part][p]);
    }
    best = max(best, s);
  }
  return best;
}

}  // namespace sp
