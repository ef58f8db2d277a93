/*
 * slide.h -- C ABI of the GB300 block-parallel IDA* solver (libslide.so).
 *
 * The reference has no library API; its de-facto interfaces are
 *   - per instance: input_table(file) + ida_star(), printing the optimal
 *     length (src/24puzzle_block_parallel_with_pdb.cu:433, :756, :832) and,
 *     for the serial solvers, `len node_num` (src/24puzzle_expand.cc:154);
 *   - per threshold round: dfs_kernel(limit, root_set, dev_flag, loop_set, pdb)
 *     over a host-built root set (src/24puzzle_block_parallel_with_pdb.cu:524,
 *     :815), and Horie's idas_kernel(Input*, search_stat*, f_limit, ...)
 *     (src_horie/idas_smem.cu:282-283);
 *   - the one host-callable C function
 *     idas_parallel_main(uchar *input, signed char *plan, int f_limit, ...)
 *     (src_horie/idas_parallel_host.h:33-34).
 * Each entry point below names the one it replaces.
 *
 * Conventions
 *   - Tiles: width*width bytes, row-major, 0 is the blank; the goal is
 *     0 1 2 ... N-1 (blank top-left), as in the reference's instance files.
 *   - Move codes are the blank's moves: 0 = up, 1 = right, 2 = left,
 *     3 = down; reverse(d) = 3 - d (src_horie/idas_smem.cu:18-24; the same
 *     expansion order as src/24puzzle_expand.cc:23-26).
 *   - Node count: generated children (inside the board, not the reverse of
 *     the parent's move), summed per threshold iteration; every iteration is
 *     searched completely, so counts equal the reference's serial
 *     all-solutions solvers (src/24puzzle_expand.cc:127, :146-164).
 *   - Every call returns an sp_status (0 = OK, negative = error); nothing
 *     exits the process or traps the GPU.  Output buffers are caller-owned.
 *   - A solver owns one CUDA stream and its device memory; it is not
 *     re-entrant: use one solver per host thread.
 *   - There is no CPU search path: without a usable GPU, sp_create fails
 *     with SP_ERR_CUDA.
 */
#ifndef SLIDE_H
#define SLIDE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SP_MAX_ITERS 96
#define SP_MAX_MOVES 240

typedef enum {
  SP_OK = 0,
  SP_ERR_ARG = -1,
  SP_ERR_NOT_PERMUTATION = -2,
  SP_ERR_UNSOLVABLE = -3,
  SP_ERR_LIMIT = -4,          /* no solution within SP_MAX_ITERS thresholds */
  SP_ERR_CUDA = -5,           /* a CUDA call failed (message: sp_last_error) */
  SP_ERR_NO_PDB = -6,         /* PDB heuristic selected but tables not built */
  SP_ERR_STACK_OVERFLOW = -7, /* a subtree deeper than the per-lane stack */
  SP_ERR_TIMEOUT = -8,        /* a device wait made no progress in time */
  SP_ERR_CAPACITY = -9,       /* a host-side table would exceed its limit */
  SP_ERR_PATH = -10           /* a solution path longer than SP_MAX_MOVES */
} sp_status;

typedef enum { SP_HEUR_MANHATTAN = 0, SP_HEUR_PDB = 1 } sp_heuristic_kind;

typedef enum {
  SP_LB_STEAL = 0,         /* dynamic donation through the device task pool */
  SP_LB_STATIC_STEAL = 1,  /* + reference-style static re-split from the
                              previous round's loads
                              (src/24puzzle_block_parallel_with_pdb.cu:839-897) */
  SP_LB_NONE = 2,          /* root set only: no re-split, no donation */
  SP_LB_LEARNED = 3        /* SP_LB_STATIC_STEAL, every root's next load predicted
                              by the learned model (sp_lbm_*): its measured load x
                              its own predicted growth, or the model's size estimate */
} sp_lb_mode;

typedef struct {
  int32_t frontier_target;   /* subproblems per instance (default 3072; the
                                reference's BLOCK_NUM is 2048);
                                a batch is capped near 8 per resident GPU lane
                                (at least 32 per instance) */
  int32_t threads_per_block; /* 128 or 256 */
  int32_t blocks_per_sm;     /* 0 = occupancy maximum */
  int32_t lb_mode;           /* sp_lb_mode */
  int32_t donate_min_slack;  /* donate a branch only if limit - depth >= this */
  int32_t steps_per_poll;    /* DFS steps between task-pool polls */
  int32_t timeout_ms;        /* device no-progress limit for pool waits */
  int32_t static_split_cap;  /* max levels a root is split by (static LB) */
  int32_t donate_reserve;    /* donate while fewer tasks than this are queued;
                                0 = resident lanes / 16, -1 = only when a lane waits */
  int32_t persistent;        /* 1: every instance's threshold loop runs on the device in
                                one launch; 0: one launch per threshold round */
  int32_t handback_nodes;    /* persistent mode: an instance whose next iteration is
                                predicted (last iteration's nodes below its roots x its
                                growth) at this many nodes or more leaves the device loop
                                and finishes in the round loop (0 = never) */
} sp_config;

/* One instance's answer: "state in, optimal move sequence and per-iteration
 * node counts out" (the reference's ida_star() prints only `len [nodes]`). */
typedef struct {
  int32_t status;
  int32_t len;               /* optimal solution length, -1 if none */
  int32_t n_iter;            /* completed threshold iterations */
  int32_t n_moves;           /* == len when solved */
  uint64_t nodes_total;
  int32_t f_limit[SP_MAX_ITERS];
  uint64_t nodes[SP_MAX_ITERS];
  uint8_t moves[SP_MAX_MOVES];
  double seconds;            /* from the call's start until this instance's answer
                                was final (the batch's wall time at most) */
} sp_result;

#define SP_MAX_ROUNDS 96

typedef struct {
  double frontier_ms;        /* root-set construction (host templates + one device launch) */
  double kernel_ms;          /* device time of the round kernels (events) */
  double wall_ms;            /* whole call */
  int32_t rounds;
  int32_t kernel_launches;   /* this library's kernels launched by the call */
  uint64_t tasks_initial;    /* root subproblems started, summed over rounds */
  uint64_t tasks_donated;    /* tasks created by in-kernel donation */
  uint64_t nodes;            /* generated nodes, all instances, all rounds */
  uint64_t h2d_bytes, d2h_bytes;
  /* per threshold round of the batch */
  int32_t round_instances[SP_MAX_ROUNDS];  /* unsolved instances searched */
  int32_t round_tasks[SP_MAX_ROUNDS];      /* root tasks published */
  float round_kernel_ms[SP_MAX_ROUNDS];
  float round_host_ms[SP_MAX_ROUNDS];      /* host work of the round */
  uint64_t round_nodes[SP_MAX_ROUNDS];
  uint64_t round_donated[SP_MAX_ROUNDS];
  /* search-kernel efficiency, summed over rounds */
  uint64_t dev_lane_steps;   /* DFS steps executed by lanes */
  uint64_t dev_lane_slots;   /* lane slots offered by warps' step loops */
  uint64_t dev_idle_cycles;  /* warp cycles with no lane searching */
  uint64_t dev_warp_cycles;  /* all warp cycles */
  uint64_t dev_donate_tries;    /* donation attempts by a warp's chosen lane */
  uint64_t dev_donate_notfree;  /* ... refused: the ring slot still occupied */
  uint64_t dev_donate_nowait;   /* ... refused: no lane waiting any more */
  uint64_t dev_tasks_done;      /* tasks finished */
} sp_stats;

typedef struct sp_solver sp_solver;

void sp_config_default(sp_config *cfg);

/* Create a solver for width 4 (15-puzzle) or 5 (24-puzzle).  cfg may be
 * NULL.  Replaces the reference's per-program globals and main() set-up
 * (src/24puzzle_block_parallel_with_pdb.cu:925-944). */
int sp_create(int width, int heuristic, const sp_config *cfg, sp_solver **out);
void sp_destroy(sp_solver *s);
int sp_set_config(sp_solver *s, const sp_config *cfg);

/* Build the additive pattern databases on the GPU by breadth-first search
 * (width 4: this project's 5-5-5 partition; width 5: the reference's 6-6-6-6
 * tables {1,2,5,6,7,12} and {3,4,8,9,13,14}).  Replaces reading the absent
 * pat24.*.tab files (src/24puzzle_block_parallel_with_pdb.cu:164-230). */
int sp_pdb_build(sp_solver *s);
uint64_t sp_pdb_table_size(int width);   /* n!/(n-k)! bytes per table */
int sp_pdb_num_tables(int width);
/* Tables in compact rank order: the byte order of the reference's table
 * files, read by src/24puzzle_block_parallel_with_pdb.cu:177-230. */
int sp_pdb_export(sp_solver *s, int table, uint8_t *dst, uint64_t size);
int sp_pdb_import(sp_solver *s, int table, const uint8_t *src, uint64_t size);

/* Heuristic value of n states (tiles n*width*width) into h[n]. */
int sp_heuristic(sp_solver *s, const uint8_t *tiles, int n, int32_t *h);

/* The root-set template the batch solve uses for a blank at cell `blank`:
 * the search tree expanded level by level (children in move order, no move
 * reversing its parent's) until a level holds at least `target` nodes --
 * the uniform-depth counterpart of create_root_set
 * (src/24puzzle_block_parallel_with_pdb.cu:454-490).  Writes the number of
 * nodes, the depth D (the leaves are the level-D nodes) and the number of
 * leaves, and the first min(cap, nodes) nodes in breadth-first order as
 * their moves from the root (2 bits per move, first move lowest).  Host
 * only, needs no GPU. */
int sp_root_set_template(int width, int blank, int target, uint64_t *paths, uint32_t cap, uint32_t *n_nodes,
                         uint32_t *depth, uint32_t *n_leaves);

/* Solve n instances, results[n].  Replaces input_table() + ida_star()
 * (src/24puzzle_block_parallel_with_pdb.cu:433-452, :756-922), batched: all
 * instances share each threshold round's kernel launch. */
int sp_solve_batch(sp_solver *s, const uint8_t *tiles, int n, sp_result *results);

/* The same with the instances already in device memory (d_tiles is a device
 * pointer to n*width*width bytes). */
int sp_solve_batch_device(sp_solver *s, const void *d_tiles, int n, sp_result *results);

/* One threshold round over a caller-built root set: the drop-in for
 * dfs_kernel<<<root_node_size, 32>>>(limit, root_set, dev_flag, loop_set, pdb)
 * (src/24puzzle_block_parallel_with_pdb.cu:524, :815-822).
 *   roots      n*width*width tiles        (root_set[i].puzzle)
 *   depth[i]   g of root i                 (root_set[i].depth)
 *   pre[i]     move that produced root i, -1 if none (root_set[i].pre)
 *   limit      f-limit of the round
 *   nodes[i]   out: generated children in root i's subtree, root included
 *              if depth+h <= limit (the reference's loop_set counts rounds
 *              of its block loop; this counts nodes)
 *   found      out: shortest goal depth seen, -1 if none (dev_flag) */
int sp_dfs_round(sp_solver *s, const uint8_t *roots, const int32_t *depth,
                 const int32_t *pre, int n, int limit, uint64_t *nodes,
                 int32_t *found);

/* sp_dfs_round for the Manhattan heuristic without allocating any memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- hosts whose framework owns the device allocator (a caching
 * pool that must account for every device byte, or a memory budget fixed at
 * start-up) and real-time loops that must not enter the driver's allocator,
 * whose latency is unbounded.  All pointers are device pointers owned by the
 * caller: d_roots n*width*width tiles, d_depth[n], d_pre[n] as in
 * sp_dfs_round, d_nodes[n] and d_found[1] receive its outputs; stream is a
 * cudaStream_t (NULL = default stream).  The call is synchronous: it copies
 * the device status back and returns after the stream has drained.  Scratch
 * lives in a fixed device array of about 7 MB that every GPU loading the
 * library keeps until exit; n above 16384 roots returns SP_ERR_CAPACITY
 * before anything is launched.  Calls share that array and each re-writes
 * what must start clean: calls overlapping on the GPU race, so serialise
 * them.  Every call takes the array's device address on the current device
 * (cudaGetSymbolAddress) and rebuilds its tables there.  A CUDA error the
 * caller left pending is returned as SP_ERR_CUDA without being cleared;
 * after any error return d_nodes and d_found are undefined. */
int sp_dfs_round_md_noalloc(int width, const uint8_t *d_roots, const int32_t *d_depth,
                            const int32_t *d_pre, int n, int limit, uint64_t *d_nodes,
                            int32_t *d_found, void *stream);

/* Horie's host-callable search, the reference's one C entry point
 * (idas_parallel_main, src_horie/idas_parallel_host.h:33-34,
 * src_horie/idas_parallel.cu:239-244), for the 15-puzzle: each of n roots
 * (d_input, n*16 tiles, device memory) is searched on its own, depth-first
 * to f_limit (0..251; a child is entered when its depth below the root + 1
 * + h <= f_limit, the root counting as depth 0), moves tried up, right,
 * left, down without undoing the last one, and stops at its first goal.
 * Row i of d_plan (device memory, n*SP_PLAN_STRIDE bytes) receives
 * [len, move_1 ... move_len] or [-1] when the root has no goal within the
 * limit ([-2]: the root's search ran past 30 s, which only a table that lets
 * h fall without bound can cause).  d_h_diff_table (16*16*4 signed bytes,
 * [tile][its cell][blank's move], the reference's init_mdist layout) and
 * d_movable_table (16*4 bytes, [cell][move]; a move off the board is never
 * made, whatever the table says) are device tables as the
 * reference takes them; NULL selects the Manhattan tables the reference
 * builds (src_horie/idas_parallel_host.c:88-129).  The initial h is the
 * Manhattan distance, as in the reference.  Launches on stream (a
 * cudaStream_t, NULL = default) and returns without waiting, like the
 * reference; allocates nothing.  Not part of the optimal-solve path: a
 * first goal in depth-first order need not be the shortest. */
#define SP_PLAN_STRIDE 252
int sp_idas_parallel(const uint8_t *d_input, int n, int8_t *d_plan, int f_limit, const int8_t *d_h_diff_table,
                     const uint8_t *d_movable_table, void *stream);

/* Learned load balancer (no reference counterpart; the reference balances
 * only from the previous round's measured loads,
 * src/24puzzle_block_parallel_with_pdb.cu:839-897).  An MLP
 * ((N-1)*N one-hot tile placement + slack -> 256 -> 256 -> 1, ReLU, BF16
 * weights and activations, FP32 accumulation, tcgen05 tensor cores) predicts
 * log2(1 + generated nodes) of a root's subtree at threshold
 * f(root) + 2*slack.  The model belongs to the solver. */
uint64_t sp_lbm_num_params(int width);  /* floats: W1[D][256] b1 W2[256][256] b2 w3 b3, D = (N-1)*N+1 */
int sp_lbm_init(sp_solver *s, uint64_t seed);                  /* He-normal, seeded */
int sp_lbm_import(sp_solver *s, const float *src, uint64_t n);
int sp_lbm_export(sp_solver *s, float *dst, uint64_t n);
/* out[i] = predicted log2(1 + nodes) for tiles i (n*N bytes) at slack[i]. */
int sp_lbm_predict(sp_solver *s, const uint8_t *tiles, const int32_t *slack, int n, float *out);
/* One Adam step (lr) on the mean squared error against target[i] =
 * log2(1 + nodes); n a multiple of 128.  loss may be NULL. */
int sp_lbm_train_step(sp_solver *s, const uint8_t *tiles, const int32_t *slack, const float *target, int n,
                      float lr, float *loss);
/* The gradient of that loss (sp_lbm_num_params floats) without a step. */
int sp_lbm_gradients(sp_solver *s, const uint8_t *tiles, const int32_t *slack, const float *target, int n,
                     float *grads, float *loss);
/* c[m][256] = a[m][k] . b[256][k]^T on the tensor cores (bf16 bit patterns
 * in, fp32 out, host arrays; m a multiple of 128, n = 256, k a multiple of
 * 64): the model's GEMM on its own, for testing. */
int sp_gemm_bf16_nt(const uint16_t *a, const uint16_t *b, float *c, int m, int n, int k);

/* Self-test of the bounded device waits (no counterpart in the reference,
 * whose kernels have no waits): runs the search kernel on a pool that
 * reports one queued task that is never published, so every lane waits for
 * it.  The kernel must give up after timeout_ms (100..60000) of no progress
 * and report SP_ERR_TIMEOUT in *device_status without faulting; the solver
 * stays usable.  Returns SP_OK when the launch itself worked. */
int sp_selftest_stall(sp_solver *s, int timeout_ms, int32_t *device_status);

/* Self-test of the tensor-core GEMM's bounded waits (no counterpart in the
 * reference): a 128 x 256 x 256 GEMM of the learned balancer whose K chunk
 * `starve_chunk` (0..3) is never copied into shared memory, so the wait for
 * it has nothing to wait for.  The kernel must give up after timeout_ms
 * (10..2000), wait for the copies it did issue, free its tensor memory and
 * report SP_ERR_TIMEOUT in *device_status without faulting; later GEMMs
 * work.  Returns SP_OK when the launch itself worked. */
int sp_selftest_gemm_stall(int32_t starve_chunk, int32_t timeout_ms, int32_t *device_status);

/* Measured 32-bit integer operation rate of the current device (lane
 * operations per second; no counterpart in the reference): the roofline
 * denominator of the Manhattan search, which is bound by integer issue.  One
 * wave of resident blocks runs independent add/xor chains of `iters`
 * (1..2^24) steps; the best of `reps` (1..100) timed launches is reported,
 * its duration in *best_ms (may be NULL).  SP_ERR_CUDA without a GPU. */
int sp_probe_int_issue(int32_t iters, int32_t reps, double *lane_ops_per_s, double *best_ms);

/* Measured rate of random one-byte reads from a device buffer of
 * working_set_bytes (4096 .. 2^32-1), one byte per lane at independent
 * addresses through the read-only path, as the pattern-database search reads
 * its tables (no counterpart in the reference): the roofline denominator of
 * the PDB search, which each read costs one 32-byte sector.  A working set
 * inside the 129 MB L2 (the 15-puzzle's 3 MB of tables) measures L2; one
 * beyond it (the 24-puzzle's 488 MB) mostly DRAM.  One wave of resident
 * blocks runs `iters` (1..2^20) rounds of 8 reads per thread; the best of
 * `reps` (1..100) timed launches is reported, its duration in *best_ms (may
 * be NULL).  Allocates and frees its buffer.  SP_ERR_CUDA without a GPU. */
int sp_probe_random_sectors(uint64_t working_set_bytes, int32_t iters, int32_t reps, double *reads_per_s,
                            double *best_ms);

int sp_last_stats(const sp_solver *s, sp_stats *out);
const char *sp_status_string(int status);
const char *sp_last_error(const sp_solver *s);
/* Device kernels this library launched since load (evidence counter). */
uint64_t sp_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
