// Shared host/device definitions of libslide: geometry, pattern partitions
// and the records exchanged between the host round loop and the kernels.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define SP_HD __host__ __device__ __forceinline__
#else
#define SP_HD inline
#endif

namespace sp {

constexpr int kMaxN = 25;
constexpr int kMaxIters = 96;                // threshold iterations per instance
constexpr int kPathWords = 10;               // 2-bit moves: 160 moves per record
constexpr int kMaxPath = kPathWords * 16;
constexpr uint8_t kNoPre = 0xFF;
// Per-instance device status (besides sp_status codes): the instance left the
// persistent loop for the host round loop after a completed iteration.
constexpr int32_t kStatusHandback = 1;

// Blank displacement of move d (0 up, 1 right, 2 left, 3 down).
SP_HD int move_delta(int w, int d) { return d == 0 ? -w : d == 1 ? 1 : d == 2 ? -1 : w; }

// Bit d set when move d keeps the blank on the board.
SP_HD uint32_t legal_moves(int w, int blank) {
  int r = blank / w, c = blank - r * w;
  return (r > 0 ? 1u : 0u) | (c < w - 1 ? 2u : 0u) | (c > 0 ? 4u : 0u) | (r < w - 1 ? 8u : 0u);
}

// Cell symmetries used by the pattern lookups.  The 24-puzzle set is the
// reference's rf / rot90 / rot180 / rot90rf / rot180rf
// (src/24puzzle_expand_with_pdb.cpp:33-46), written as formulas.
enum Sym { kId = 0, kRf, kRot180, kRot90, kRot90Rf, kRot180Rf };

SP_HD int sym_cell(int w, int s, int p) {
  int r = p / w, c = p % w, m = w - 1;
  switch (s) {
    case kRf: return c * w + r;
    case kRot180: return (m - r) * w + (m - c);
    case kRot90: return (m - c) * w + r;
    case kRot90Rf: return (m - r) * w + c;
    case kRot180Rf: return (m - c) * w + (m - r);
    default: return p;
  }
}

// Pattern partitions.  Width 5: the reference's 6-6-6-6 partition, two
// tables reused through symmetry, h = max(regular, reflected)
// (src/24puzzle_block_parallel_with_pdb.cu:349-429).  Width 4: this
// project's 5-5-5 partition (the reference has no 15-puzzle PDB), reflected
// through the main diagonal in the same way.
struct PatternSet {
  int n_tables, n_pat, k, radix;
  int table_tiles[3][6];   // goal cells of each table's pattern, digit order
  int pat_table[2][4];     // [partition][pattern] -> table
  int pat_sym[2][4];       // [partition][pattern] -> Sym
};

SP_HD PatternSet pattern_set(int w) {
  PatternSet p{};
  if (w == 5) {
    p.n_tables = 2; p.n_pat = 4; p.k = 6; p.radix = 25;
    const int t0[6] = {1, 2, 5, 6, 7, 12}, t1[6] = {3, 4, 8, 9, 13, 14};
    for (int j = 0; j < 6; ++j) { p.table_tiles[0][j] = t0[j]; p.table_tiles[1][j] = t1[j]; }
    const int tab[4] = {0, 1, 1, 1};
    const int sr[4] = {kId, kId, kRot180, kRot90}, sf[4] = {kRf, kRf, kRot180Rf, kRot90Rf};
    for (int q = 0; q < 4; ++q) {
      p.pat_table[0][q] = p.pat_table[1][q] = tab[q];
      p.pat_sym[0][q] = sr[q];
      p.pat_sym[1][q] = sf[q];
    }
  } else {
    p.n_tables = 3; p.n_pat = 3; p.k = 5; p.radix = 16;
    const int t[3][5] = {{1, 2, 3, 6, 7}, {4, 5, 8, 9, 12}, {10, 11, 13, 14, 15}};
    for (int a = 0; a < 3; ++a)
      for (int j = 0; j < 5; ++j) p.table_tiles[a][j] = t[a][j];
    for (int q = 0; q < 3; ++q) {
      p.pat_table[0][q] = p.pat_table[1][q] = q;
      p.pat_sym[0][q] = kId;
      p.pat_sym[1][q] = kRf;
    }
  }
  return p;
}

// Root subproblem of a round: a node of the host-built frontier.
struct SubRoot {
  uint8_t board[kMaxN];
  uint8_t blank;
  uint8_t g;
  uint8_t pre;     // incoming move or kNoPre
  uint32_t inst;   // instance slot in the batch
};
static_assert(sizeof(SubRoot) == 32, "SubRoot layout");

// Unit of work in the device task pool: the node reached from SubRoot `sub`
// by `plen` moves, restricted to the first-level moves in `mask`.
struct Task {
  uint32_t sub;
  uint16_t plen;
  uint8_t mask;
  uint8_t flags;
  uint32_t path[kPathWords];
};
static_assert(sizeof(Task) == 48, "Task layout");

// One goal per instance: moves below its SubRoot.  `best` is
// 0xFFFFFFFF - (shortest absolute goal depth seen), 0 when none, so that a
// zeroed record needs no further initialisation.
struct Solution {
  uint32_t flag;
  uint32_t sub;
  uint32_t len;
  uint32_t best;
  uint32_t path[kPathWords];
  uint32_t pad2[2];
};
static_assert(sizeof(Solution) == 64, "Solution layout");

// Pool control block (reset by pool_init_kernel each round).  Each hot word
// has its own 128-byte line so claims, publications, completions and error
// polls do not queue behind each other in one L2 slice.
struct PoolCtl {
  uint32_t head;          // next index to claim (may run ahead of tail)
  uint32_t pad0[31];
  uint32_t tail;          // indices reserved by producers
  uint32_t pad1[31];
  uint32_t outstanding;   // tasks queued or running
  uint32_t pad2[31];
  int32_t error;          // first device error (sp_status)
  uint32_t err_info[4];
  uint32_t pad3[27];
  unsigned long long donated;
  unsigned long long pad4[15];
  uint32_t heartbeat;     // bumped by searching warps: a long task is progress too
  uint32_t pad6[31];
  // efficiency counters, one atomic per warp at exit:
  // [0] step() calls (active lane-steps)  [1] warp step iterations x 32
  // [2] clock cycles warps spent with no active lane  [3] total warp cycles
  unsigned long long counters[16];  // [4] donation tries [5] slot never freed [6] hungry
                                    // polls [7] tasks done [8] polls with a donor found
};
static_assert(sizeof(PoolCtl) == 896, "PoolCtl layout");

// Heuristic lookup tables built once per solver.
struct HeurTables {
  uint32_t code[2][kMaxN * kMaxN];  // [part][tile*N+cell]: digit contribution to its pattern index
  uint8_t pat[2][kMaxN];            // [part][tile] -> pattern (0xFF for the blank)
  int8_t mdd[4 * kMaxN * kMaxN];    // [(d*N + cell)*N + tile]: MD change when the tile at
                                    // `cell` slides into the blank after the blank's move d
};

}  // namespace sp
