// Kernel interfaces of libslide (device side), used by the host round loop.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sp_defs.h"

namespace sp {

struct RoundParams {
  const SubRoot *subs;
  // Task pool: a ring of `cap` slots (a power of two).  Index i lives in slot
  // i & (cap-1); seq[slot] == i once the slot is free for index i, == i + 1
  // once index i is published, and becomes i + cap when its claimant copied it.
  Task *tasks;
  uint32_t *seq;
  uint32_t cap;
  uint32_t pad0;
  PoolCtl *ctl;
  const int32_t *inst_limit;
  unsigned long long *sub_nodes;
  Solution *sol;
  const HeurTables *ht;
  const uint8_t *pdb;       // device tables, table t at t << (w == 4 ? 20 : 28)
  int32_t min_slack;
  int32_t steps;
  int32_t donate;
  uint32_t reserve;   // donate while fewer than this many tasks are queued
  uint32_t spread;    // one extra donor per warp per `spread` missing tasks
  uint32_t pad1;
  unsigned long long timeout_ns;
  unsigned long long poll_ns;  // min interval of a block's global pool poll
  // multi-iteration mode: every instance runs its own threshold loop on the
  // device; inst_limit and sol then hold two entries per instance, indexed
  // 2 * instance + (iteration & 1), and inst_limit is written by the kernel
  // as well
  int32_t *inst_iter;                 // current iteration
  uint32_t *inst_out;                 // tasks of the current iteration not finished
  int32_t *inst_final;                // iteration that ended the search, -1 while running
  int32_t *inst_status;
  const uint32_t *inst_sub_base;      // the instance's roots: subs[base .. base+nsub),
  const uint32_t *inst_nsub;          //   sorted by sub_maxf
  const int32_t *sub_maxf;            // prefix max of g+h along the root's path
  const uint32_t *inter_off, *inter_len;  // per instance: (f, cumulative children) pairs
  const int32_t *inter_f;             //   of root-set interior nodes, sorted by f
  const unsigned long long *inter_cum;
  const int32_t *goal_maxf;           // smallest maxf of a root-set goal node (INT32_MAX: none)
  uint32_t *inst_pair;                // 1: iterations inst_iter and inst_iter + 1 run together
  unsigned long long pair_nodes;      // run the next two iterations together when the second is
                                      //   predicted below this many nodes (0: one at a time)
  unsigned long long *iter_nodes;     // [instance][kMaxIters] generated nodes
  unsigned long long *sub_loads;      // [2][n_subs] per-root loads of the last two iterations
  unsigned long long *inst_fin_ns;    // %globaltimer when the instance's answer became final
  unsigned long long *t_begin_ns;     // %globaltimer at the launch's first block start (atomicMin)
  uint32_t n_subs;
  int32_t static_split;
  unsigned long long handback_nodes;  // 0: never hand an instance back to the host
  // learned balancer (null otherwise): per root, kGrowthSlacks codes of its
  // predicted growth from slack j to j + 1 (factor 2^(code / 16)), slack
  // counted from the root's prefix-maximum f
  const uint8_t *sub_growth;
};
constexpr int kGrowthSlacks = 8;

// One threshold round: grid = num_sms * blocks_per_sm (0 = occupancy maximum).
cudaError_t launch_search_round(int w, bool pdb, int block, int blocks_per_sm, int num_sms,
                                const RoundParams &P, cudaStream_t st, int *grid_out);
// The whole threshold loop of a batch in one launch (multi-iteration mode).
cudaError_t launch_search_multi(int w, bool pdb, int block, int blocks_per_sm, int num_sms,
                                const RoundParams &P, cudaStream_t st, int *grid_out);
// Publish the round's tasks (split pieces first, then the direct tasks) and
// reset the pool control block.
// Multi-iteration mode passes subs and inst_iter: each direct task then
// carries its instance's iteration parity.
cudaError_t launch_pool_init(Task *tasks, const Task *emit, const uint32_t *n_emit, const uint32_t *direct,
                             uint32_t n_direct, uint32_t *seq, uint32_t cap, PoolCtl *ctl, const SubRoot *subs,
                             const int32_t *inst_iter, cudaStream_t st);

// Split pre-pass: one breadth-first level over `in` (count *n_in).
struct SplitArgs {
  const SubRoot *subs;
  const int32_t *inst_limit;
  const HeurTables *ht;
  const uint8_t *pdb;
  unsigned long long *sub_nodes;
  Solution *sol;
  const Task *in;
  const uint32_t *n_in;
  Task *next;
  uint32_t *n_next;
  Task *out;
  uint32_t *n_out;
  uint32_t cap_next, cap_out;
  int32_t *error;
};
cudaError_t launch_split_level(int w, bool pdb, int num_sms, const SplitArgs &A, cudaStream_t st);

// Root-set templates and the device root-set build (frontier.cu).  A
// template is the uniform-depth tree of one blank cell in breadth-first
// order; its nodes live at [node_off, node_off + n_nodes) of the template
// arrays and its level d at [lev[d], lev[d + 1]) (template-relative).
constexpr int kFrontMaxDepth = 32;                  // moves in a 64-bit path
constexpr int kFrontLevStride = kFrontMaxDepth + 2;
// maxf - h0 in [0, 256).  The PDB tables are not consistent: h moved by up
// to 5 per move over the root sets of the benchmark workloads (maxf - h0 at
// most 22 at D = 10); 256 leaves room for 6 D at the deepest template.  A
// larger spread is reported as SP_ERR_ARG.
constexpr int kFrontBuckets = 256;
struct FrontTmpl {
  uint32_t node_off, n_nodes, D, pad;
};
struct FrontInst {
  int32_t h0;
  uint32_t n_leaves;
  uint32_t leaf_cum[kFrontBuckets];  // leaves with maxf <= h0 + b
  uint32_t child[kFrontBuckets];     // children of interior nodes with maxf == h0 + b
  uint32_t goal[kFrontBuckets];      // min (depth << 24 | node) of goal nodes with maxf == h0 + b
};
struct FrontArgs {
  const uint8_t *tiles;          // [instance][N]
  const uint32_t *live;          // [block] instance of the block
  const uint32_t *live_tmpl;     // [block] its template
  const uint32_t *live_base;     // [block] SubRoot index of its first leaf
  const uint32_t *live_scratch;  // [block] offset of its nodes in f / maxf
  const FrontTmpl *tmpl;
  const uint32_t *lev;           // [template][kFrontLevStride]
  const uint64_t *path;          // moves from the root, 2 bits each, first move lowest
  const int32_t *parent;
  const uint8_t *nchild;
  const uint8_t *depth;
  const HeurTables *ht;
  const uint8_t *pdb;
  int16_t *f, *maxf;             // scratch, one entry per node
  SubRoot *subs;                 // leaves, sorted by maxf per instance
  int32_t *leaf_maxf;
  uint8_t *leaf_h;
  int32_t *leaf_node;            // template node of each SubRoot
  FrontInst *out;                // [block]
  int32_t *error;
};
cudaError_t launch_frontier(int w, bool pdb, int n_live, const FrontArgs &A, cudaStream_t st);

// h of n boards (n * N bytes) into h[n]; PDB tables as in RoundParams.
cudaError_t launch_heuristic(int w, bool pdb, const uint8_t *boards, int n, int32_t *h,
                             const HeurTables *ht, const uint8_t *tables, cudaStream_t st);

// Breadth-first build of table `table_id` of width w into the device lookup
// layout (mixed radix 16^5 or 25^6 bytes) at `lookup`; also writes the
// compact rank-order table to `compact` when non-null.  Scratch is allocated
// and freed inside.
cudaError_t build_pdb_table(int w, int table_id, uint8_t *lookup, uint8_t *compact,
                            cudaStream_t st, int *levels_out, double *ms_out);
// compact rank order <-> lookup layout
cudaError_t pdb_compact_to_lookup(int w, int table_id, const uint8_t *compact, uint8_t *lookup,
                                  cudaStream_t st);
cudaError_t pdb_lookup_to_compact(int w, int table_id, const uint8_t *lookup, uint8_t *compact,
                                  cudaStream_t st);

uint64_t compact_table_size(int w);
uint64_t lookup_table_stride(int w);

// launch counter shared by all translation units
void note_launch(int n = 1);

}  // namespace sp
