/*
 * CPU oracle for the sliding-puzzle IDA* path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker for the GPU solver in sliding-puzzle_gb300/.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product library never links or calls it.
 *
 * It restates, in plain C, the reference's serial IDA* programs:
 *   src/24puzzle_expand.cc            (Manhattan, full final iteration)
 *   src/24puzzle_expand_with_pdb.cpp  (6-6-6-6 additive PDB, full final iteration)
 *   src/24puzzle.cc, src/24puzzle_with_pdb.cc (first-solution variants)
 *   src/15puzzle_expand.cc            (the same program with N=4)
 * with 64-bit node counters, per-iteration counts and a recorded solution path,
 * and a CPU breadth-first pattern-database builder (the reference ships neither
 * its tables nor their generator; the builder's semantics are pinned by
 * benchmarks/pdb_expand_nodes.csv).
 *
 * Move codes are the blank's moves in the reference's expansion order
 * (src/24puzzle_expand.cc:23-26, order {1,0,2,3} over dx/dy):
 *   0 = up, 1 = right, 2 = left, 3 = down;  reverse(d) = 3 - d
 * which is also Horie's DIR_UP/RIGHT/LEFT/DOWN numbering
 * (src_horie/idas_smem.cu:18-24).
 */
#ifndef SP_ORACLE_H
#define SP_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_ITERS 96
#define ORC_MAX_MOVES 240

enum { ORC_HEUR_MD = 0, ORC_HEUR_PDB = 1 };
enum { ORC_MODE_ALL = 0, ORC_MODE_FIRST = 1 };
/* PDB abstraction semantics for the builder */
enum { ORC_PDB_BLANK_FREE = 0, ORC_PDB_BLANK_ANY = 1, ORC_PDB_BLANK_HOME = 2 };

enum {
  ORC_OK = 0,
  ORC_ERR_ARG = -1,
  ORC_ERR_NOT_PERMUTATION = -2,
  ORC_ERR_UNSOLVABLE = -3,
  ORC_ERR_LIMIT = -4,      /* no solution below the threshold cap */
  ORC_ERR_NODE_BUDGET = -5 /* node budget exhausted (bounded CPU samples) */
};

typedef struct {
  int32_t status;
  int32_t len;            /* optimal length, -1 if none */
  int32_t n_iter;         /* completed threshold iterations */
  int32_t n_moves;        /* moves recorded in moves[] (== len when found) */
  uint64_t nodes_total;   /* sum of nodes[] */
  int32_t f_limit[ORC_MAX_ITERS];
  uint64_t nodes[ORC_MAX_ITERS];  /* generated children per iteration */
  uint8_t moves[ORC_MAX_MOVES];
  double seconds;
} orc_result;

/* Heuristic description.  tables[] are compact (k-permutation rank) tables as
 * produced by orc_pdb_build; width 5 uses 2 tables (6-6-6-6 with symmetry,
 * src/24puzzle_expand_with_pdb.cpp:114-194), width 4 uses 3 tables (5-5-5). */
typedef struct {
  int width;
  int heuristic;
  const uint8_t *tables[4];
} orc_heur;

/* Solve one instance.  tiles: width*width bytes, row-major, 0 = blank. */
int orc_solve(const orc_heur *h, const uint8_t *tiles, int mode,
              uint64_t node_budget, orc_result *out);

/* Solve n instances with `threads` POSIX threads, one instance per thread at
 * a time (the reference's CPU solvers run one instance per process). */
int orc_solve_batch(const orc_heur *h, const uint8_t *tiles, int n, int mode,
                    uint64_t node_budget, int threads, orc_result *out);

/* The same answers (status, length, per-iteration counts) with all `threads`
 * working on one instance at a time: per iteration the root is expanded
 * breadth-first to a uniform depth and the depth-first searches below that
 * frontier are shared out.  Only ORC_MODE_ALL; node_budget (0 = none) is
 * checked between iterations.  The CPU baseline's driver for batches whose
 * hardest instance would otherwise run on one core. */
int orc_solve_batch_split(const orc_heur *h, const uint8_t *tiles, int n, uint64_t node_budget,
                          int threads, orc_result *out);

/* Horie's per-root search (src_horie/idas_parallel.cu:172-236): the first
 * goal path of one 15-puzzle root in depth-first order within f_limit
 * (0..251), into row = [len, moves...] or [-1].  h_diff (16*16*4,
 * [tile][cell][blank's move]) and movable (16*4) may be NULL for the
 * reference's Manhattan tables (src_horie/idas_parallel_host.c:88-129). */
int orc_first_path(const uint8_t *tiles, int f_limit, const int8_t *h_diff, const uint8_t *movable,
                   int8_t *row);

/* Heuristic value of one state (for tests of the frontier / h kernels). */
int orc_heuristic(const orc_heur *h, const uint8_t *tiles);

/* Pattern descriptions shared with the GPU solver.  For partition `part`
 * (0 = regular, 1 = reflected) and pattern `p`, fills tiles[k] (tile ids in
 * index-digit order, most significant first), sym[n] (cell map applied to
 * positions before indexing) and returns the table id; -1 if out of range. */
int orc_pattern(int width, int part, int p, int *tiles, int *sym);
int orc_num_patterns(int width);     /* patterns per partition */
int orc_pattern_k(int width);        /* tiles per pattern      */
int orc_num_tables(int width);

/* Compact table size: n!/(n-k)! */
uint64_t orc_table_size(int width);
uint64_t orc_rank(int n, int k, const int *pos);
void orc_unrank(int n, int k, uint64_t r, int *pos);

/* Breadth-first build of table `table_id` for `width` with the given
 * abstraction semantics; out must hold orc_table_size(width) bytes.
 * threads <= 0 means all cores.  Returns 0 or an error code. */
int orc_pdb_build(int width, int table_id, int semantics, int threads,
                  uint8_t *out);
/* Base pattern (goal cells) of table `table_id`. */
int orc_table_tiles(int width, int table_id, int *tiles);

#ifdef __cplusplus
}
#endif
#endif
