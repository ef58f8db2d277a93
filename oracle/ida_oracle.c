/*
 * CPU oracle: serial IDA* for the 15- and 24-puzzle -- TEST INFRASTRUCTURE.
 *
 * Restates the reference's serial solvers so the GPU solver can be checked
 * node-for-node.  Nothing in the product library links this file.
 *
 *  - Threshold loop: limit starts at h(root) and grows by 2
 *    (src/24puzzle_expand.cc:146-164, src/24puzzle_expand_with_pdb.cpp:269-289).
 *  - Node count: one per generated child that is inside the board and is not
 *    the reverse of the move that produced the parent, counted before the
 *    child's own f-test (src/24puzzle_expand.cc:119-127).  Counters are 64-bit
 *    (the reference's `int node_num`, src/24puzzle_expand.cc:45, overflows on
 *    the golden totals of benchmarks/manhattan_expand_nodes.csv).
 *  - Goal handling, ORC_MODE_ALL: a node with h == 0 records the answer and the
 *    search goes on, so the final iteration is searched completely
 *    (src/24puzzle_expand.cc:111-116).  ORC_MODE_FIRST returns at the first
 *    goal, before the f-test (src/24puzzle.cc:111-116).
 *  - Manhattan distance is updated incrementally per move
 *    (src/24puzzle_expand.cc:129-131); the PDB value is recomputed from all
 *    pattern lookups per node, max of the regular and the reflected partition
 *    (src/24puzzle_expand_with_pdb.cpp:191-194, :256).
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ */
/* geometry and pattern descriptions                                   */
/* ------------------------------------------------------------------ */

enum { SYM_ID, SYM_RF, SYM_ROT180, SYM_ROT90, SYM_ROT90RF, SYM_ROT180RF };

static int sym_cell(int w, int s, int p) {
  int r = p / w, c = p % w, m = w - 1;
  switch (s) {
    case SYM_ID: return p;
    case SYM_RF: return c * w + r;                 /* transpose            */
    case SYM_ROT180: return (m - r) * w + (m - c);
    case SYM_ROT90: return (m - c) * w + r;
    case SYM_ROT90RF: return (m - r) * w + c;      /* vertical flip        */
    case SYM_ROT180RF: return (m - c) * w + (m - r); /* anti-transpose     */
  }
  return -1;
}

/* Base patterns: the goal cells (= tile ids) of each table, in index-digit
 * order.  Width 5 follows the reference's two tables
 * (src/24puzzle_expand_with_pdb.cpp:78-83, :114-124); width 4 is this
 * project's own 5-5-5 partition (the reference has no 15-puzzle PDB). */
static const int base24[2][6] = {{1, 2, 5, 6, 7, 12}, {3, 4, 8, 9, 13, 14}};
static const int base15[3][5] = {{1, 2, 3, 6, 7}, {4, 5, 8, 9, 12}, {10, 11, 13, 14, 15}};

/* (table, symmetry) per pattern, regular then reflected partition.
 * Width 5: src/24puzzle_expand_with_pdb.cpp:114-189 -- hash0..3 use
 * id/id/rot180/rot90, hashref0..3 use rf/rf/rot180rf/rot90rf. */
static const int pat24[2][4][2] = {
    {{0, SYM_ID}, {1, SYM_ID}, {1, SYM_ROT180}, {1, SYM_ROT90}},
    {{0, SYM_RF}, {1, SYM_RF}, {1, SYM_ROT180RF}, {1, SYM_ROT90RF}}};
static const int pat15[2][3][2] = {{{0, SYM_ID}, {1, SYM_ID}, {2, SYM_ID}},
                                   {{0, SYM_RF}, {1, SYM_RF}, {2, SYM_RF}}};

int orc_num_patterns(int width) { return width == 5 ? 4 : width == 4 ? 3 : -1; }
int orc_pattern_k(int width) { return width == 5 ? 6 : width == 4 ? 5 : -1; }
int orc_num_tables(int width) { return width == 5 ? 2 : width == 4 ? 3 : -1; }

int orc_table_tiles(int width, int table_id, int *tiles) {
  int k = orc_pattern_k(width);
  if (k < 0 || table_id < 0 || table_id >= orc_num_tables(width)) return -1;
  for (int j = 0; j < k; ++j) tiles[j] = width == 5 ? base24[table_id][j] : base15[table_id][j];
  return k;
}

int orc_pattern(int width, int part, int p, int *tiles, int *sym) {
  int np = orc_num_patterns(width), k = orc_pattern_k(width), n = width * width;
  if (np < 0 || part < 0 || part > 1 || p < 0 || p >= np) return -1;
  int table = width == 5 ? pat24[part][p][0] : pat15[part][p][0];
  int s = width == 5 ? pat24[part][p][1] : pat15[part][p][1];
  int base[6];
  orc_table_tiles(width, table, base);
  for (int c = 0; c < n; ++c) sym[c] = sym_cell(width, s, c);
  /* the tile whose goal cell maps onto base[j] */
  for (int j = 0; j < k; ++j)
    for (int c = 0; c < n; ++c)
      if (sym[c] == base[j]) tiles[j] = c;
  return table;
}

uint64_t orc_table_size(int width) {
  int n = width * width, k = orc_pattern_k(width);
  if (k < 0) return 0;
  uint64_t s = 1;
  for (int i = 0; i < k; ++i) s *= (uint64_t)(n - i);
  return s;
}

/* Lexicographic rank among k-permutations of n cells: the reference's
 * on-disk table order (src/24puzzle_expand_with_pdb.cpp:87-112 reads bytes in
 * the order of its nested loops over distinct 6-tuples). */
uint64_t orc_rank(int n, int k, const int *pos) {
  uint64_t r = 0;
  uint32_t used = 0;
  for (int i = 0; i < k; ++i) {
    int less = __builtin_popcount(used & ((1u << pos[i]) - 1u));
    r = r * (uint64_t)(n - i) + (uint64_t)(pos[i] - less);
    used |= 1u << pos[i];
  }
  return r;
}

void orc_unrank(int n, int k, uint64_t r, int *pos) {
  int digit[8];
  for (int i = k - 1; i >= 0; --i) {
    digit[i] = (int)(r % (uint64_t)(n - i));
    r /= (uint64_t)(n - i);
  }
  uint32_t used = 0;
  for (int i = 0; i < k; ++i) {
    int d = digit[i], c = 0;
    for (;; ++c) {
      if (used & (1u << c)) continue;
      if (d-- == 0) break;
    }
    pos[i] = c;
    used |= 1u << c;
  }
}

/* ------------------------------------------------------------------ */
/* search                                                              */
/* ------------------------------------------------------------------ */

typedef struct {
  int w, n;
  int heuristic;
  int md[25][25];           /* md[cell][tile] */
  int np;                   /* patterns per partition */
  int k;
  int ptab[2][4];
  int ptiles[2][4][6];
  int psym[2][4][25];
  const uint8_t *tables[4];
} hctx;

static void hctx_init(hctx *c, const orc_heur *h) {
  memset(c, 0, sizeof(*c));
  c->w = h->width;
  c->n = h->width * h->width;
  c->heuristic = h->heuristic;
  for (int i = 0; i < c->n; ++i)
    for (int j = 0; j < c->n; ++j)
      c->md[i][j] = abs(i / c->w - j / c->w) + abs(i % c->w - j % c->w);
  if (h->heuristic == ORC_HEUR_PDB) {
    c->np = orc_num_patterns(c->w);
    c->k = orc_pattern_k(c->w);
    for (int part = 0; part < 2; ++part)
      for (int p = 0; p < c->np; ++p)
        c->ptab[part][p] = orc_pattern(c->w, part, p, c->ptiles[part][p], c->psym[part][p]);
    for (int t = 0; t < 4; ++t) c->tables[t] = h->tables[t];
  }
}

static int pdb_value(const hctx *c, const uint8_t *inv) {
  int best = 0;
  for (int part = 0; part < 2; ++part) {
    int sum = 0;
    for (int p = 0; p < c->np; ++p) {
      int pos[6];
      for (int j = 0; j < c->k; ++j) pos[j] = c->psym[part][p][inv[c->ptiles[part][p][j]]];
      sum += c->tables[c->ptab[part][p]][orc_rank(c->n, c->k, pos)];
    }
    if (sum > best) best = sum;
  }
  return best;
}

static int md_value(const hctx *c, const uint8_t *board) {
  int s = 0;
  for (int i = 0; i < c->n; ++i)
    if (board[i]) s += c->md[i][board[i]];
  return s;
}

typedef struct {
  const hctx *c;
  uint8_t board[25];
  uint8_t inv[25];
  int blank;
  int h;
  int limit;
  int mode;
  int ans;
  uint64_t nodes;        /* this iteration */
  uint64_t nodes_before; /* earlier iterations */
  uint64_t budget;
  int over_budget;
  uint8_t path[ORC_MAX_MOVES];
  uint8_t best_path[ORC_MAX_MOVES];
  int have_path;
} searcher;

/* blank displacement per move code: up, right, left, down */
static int legal_move(int w, int blank, int d, int *to) {
  int r = blank / w, cc = blank % w;
  switch (d) {
    case 0: if (r == 0) return 0; *to = blank - w; return 1;
    case 1: if (cc == w - 1) return 0; *to = blank + 1; return 1;
    case 2: if (cc == 0) return 0; *to = blank - 1; return 1;
    default: if (r == w - 1) return 0; *to = blank + w; return 1;
  }
}

static int dfs(searcher *s, int depth, int pre) {
  const hctx *c = s->c;
  if (s->h == 0) {
    if (s->ans < 0 || depth < s->ans) {
      s->ans = depth;
      if (!s->have_path && depth <= ORC_MAX_MOVES) {
        memcpy(s->best_path, s->path, (size_t)depth);
        s->have_path = 1;
      }
    }
    if (s->mode == ORC_MODE_FIRST) return 1;
  }
  if (depth + s->h > s->limit) return 0;
  if (s->budget && s->nodes + s->nodes_before > s->budget) {
    s->over_budget = 1;
    return 1;
  }
  for (int d = 0; d < 4; ++d) {
    int to;
    if (!legal_move(c->w, s->blank, d, &to)) continue;
    if (pre >= 0 && d == 3 - pre) continue;
    s->nodes++;
    int tile = s->board[to];
    int from = s->blank, old_h = s->h;
    /* move `tile` from `to` into the blank at `from` */
    s->board[from] = (uint8_t)tile;
    s->board[to] = 0;
    s->inv[tile] = (uint8_t)from;
    s->inv[0] = (uint8_t)to;
    s->blank = to;
    if (c->heuristic == ORC_HEUR_MD)
      s->h = old_h - c->md[to][tile] + c->md[from][tile];
    else
      s->h = pdb_value(c, s->inv);
    if (depth < ORC_MAX_MOVES) s->path[depth] = (uint8_t)d;
    int stop = dfs(s, depth + 1, d);
    if (stop) return 1;
    s->board[to] = (uint8_t)tile;
    s->board[from] = 0;
    s->inv[tile] = (uint8_t)to;
    s->inv[0] = (uint8_t)from;
    s->blank = from;
    s->h = old_h;
  }
  return 0;
}

static int check_instance(int w, const uint8_t *tiles) {
  int n = w * w;
  uint32_t seen = 0;
  for (int i = 0; i < n; ++i) {
    if (tiles[i] >= n || (seen >> tiles[i]) & 1u) return ORC_ERR_NOT_PERMUTATION;
    seen |= 1u << tiles[i];
  }
  int invs = 0, blank_row = 0;
  for (int i = 0; i < n; ++i) {
    if (!tiles[i]) { blank_row = i / w; continue; }
    for (int j = i + 1; j < n; ++j)
      if (tiles[j] && tiles[j] < tiles[i]) ++invs;
  }
  /* goal has the blank at cell 0: for odd widths the inversion parity is
   * invariant, for even widths inversions + blank row is */
  int parity = (w & 1) ? (invs & 1) : ((invs + blank_row) & 1);
  return parity ? ORC_ERR_UNSOLVABLE : ORC_OK;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int solve_ctx(const hctx *c, const uint8_t *tiles, int mode, uint64_t budget,
                     orc_result *out) {
  memset(out, 0, sizeof(*out));
  out->len = -1;
  double t0 = now_s();
  int st = check_instance(c->w, tiles);
  if (st != ORC_OK) { out->status = st; return st; }
  searcher *s = (searcher *)calloc(1, sizeof(searcher));
  s->c = c;
  s->mode = mode;
  s->budget = budget;
  for (int i = 0; i < c->n; ++i) {
    s->board[i] = tiles[i];
    s->inv[tiles[i]] = (uint8_t)i;
    if (!tiles[i]) s->blank = i;
  }
  int h0 = c->heuristic == ORC_HEUR_MD ? md_value(c, s->board) : pdb_value(c, s->inv);
  uint8_t board0[25], inv0[25];
  memcpy(board0, s->board, sizeof board0);
  memcpy(inv0, s->inv, sizeof inv0);
  int blank0 = s->blank;
  st = ORC_ERR_LIMIT;
  for (int it = 0; it < ORC_MAX_ITERS; ++it) {
    int limit = h0 + 2 * it;
    memcpy(s->board, board0, sizeof board0);
    memcpy(s->inv, inv0, sizeof inv0);
    s->blank = blank0;
    s->h = h0;
    s->limit = limit;
    s->ans = -1;
    s->nodes = 0;
    dfs(s, 0, -1);
    out->f_limit[it] = limit;
    out->nodes[it] = s->nodes;
    out->n_iter = it + 1;
    s->nodes_before += s->nodes;
    if (s->over_budget) { st = ORC_ERR_NODE_BUDGET; break; }
    if (s->ans >= 0) {
      out->len = s->ans;
      out->n_moves = s->have_path ? s->ans : 0;
      memcpy(out->moves, s->best_path, (size_t)out->n_moves);
      st = ORC_OK;
      break;
    }
  }
  out->nodes_total = s->nodes_before;
  out->status = st;
  out->seconds = now_s() - t0;
  free(s);
  return st;
}

int orc_solve(const orc_heur *h, const uint8_t *tiles, int mode, uint64_t node_budget,
              orc_result *out) {
  if (!h || !tiles || !out || (h->width != 4 && h->width != 5)) return ORC_ERR_ARG;
  if (h->heuristic == ORC_HEUR_PDB)
    for (int t = 0; t < orc_num_tables(h->width); ++t)
      if (!h->tables[t]) return ORC_ERR_ARG;
  hctx *c = (hctx *)malloc(sizeof(hctx));
  hctx_init(c, h);
  int st = solve_ctx(c, tiles, mode, node_budget, out);
  free(c);
  return st;
}

int orc_heuristic(const orc_heur *h, const uint8_t *tiles) {
  if (!h || !tiles || (h->width != 4 && h->width != 5)) return ORC_ERR_ARG;
  hctx *c = (hctx *)malloc(sizeof(hctx));
  hctx_init(c, h);
  uint8_t board[25], inv[25];
  for (int i = 0; i < c->n; ++i) { board[i] = tiles[i]; inv[tiles[i] % 25] = (uint8_t)i; }
  int v = c->heuristic == ORC_HEUR_MD ? md_value(c, board) : pdb_value(c, inv);
  free(c);
  return v;
}

typedef struct {
  const hctx *c;
  const uint8_t *tiles;
  int n, mode;
  uint64_t budget;
  orc_result *out;
  int next;
  pthread_mutex_t mu;
} batch_job;

static void *batch_worker(void *arg) {
  batch_job *job = (batch_job *)arg;
  for (;;) {
    pthread_mutex_lock(&job->mu);
    int i = job->next++;
    pthread_mutex_unlock(&job->mu);
    if (i >= job->n) break;
    solve_ctx(job->c, job->tiles + (size_t)i * (size_t)job->c->n, job->mode, job->budget,
              &job->out[i]);
  }
  return NULL;
}

int orc_solve_batch(const orc_heur *h, const uint8_t *tiles, int n, int mode,
                    uint64_t node_budget, int threads, orc_result *out) {
  if (!h || !tiles || !out || n < 0 || (h->width != 4 && h->width != 5)) return ORC_ERR_ARG;
  if (h->heuristic == ORC_HEUR_PDB)
    for (int t = 0; t < orc_num_tables(h->width); ++t)
      if (!h->tables[t]) return ORC_ERR_ARG;
  if (n == 0) return ORC_OK;
  hctx *c = (hctx *)malloc(sizeof(hctx));
  hctx_init(c, h);
  batch_job job;
  job.c = c;
  job.tiles = tiles;
  job.n = n;
  job.mode = mode;
  job.budget = node_budget;
  job.out = out;
  job.next = 0;
  pthread_mutex_init(&job.mu, NULL);
  if (threads < 1) threads = 1;
  if (threads > n) threads = n;
  pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, batch_worker, &job);
  for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
  free(tid);
  pthread_mutex_destroy(&job.mu);
  free(c);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* all host threads on one instance (CPU baseline of the benchmark)     */
/* ------------------------------------------------------------------ */

/* The same search with every host thread working on one instance at a time:
 * per threshold iteration the root is expanded breadth-first to a uniform
 * depth (no duplicate detection, children counted and goal-tested exactly as
 * dfs() counts and tests them), and the depth-first searches below the
 * frontier nodes that pass the f-test are shared out to the threads.  Every
 * node is generated by the same parent as in the serial search, so the
 * per-iteration counts and the optimal length are the serial ones; the
 * recorded path is that of the shortest goal in the first frontier subtree
 * holding one.  The reference's CPU solvers are serial; this only lets the
 * baseline use all host cores on batches whose hardest instance dominates. */

#define SPLIT_MAX_DEPTH 20

typedef struct {
  uint8_t board[25];
  uint8_t inv[25];
  uint8_t blank;
  int8_t pre;
  int h;
  uint8_t path[SPLIT_MAX_DEPTH];
} split_leaf;

typedef struct {
  uint64_t nodes;
  int ans;
  int ans_leaf;
  uint8_t path[ORC_MAX_MOVES];
} split_tres;

typedef struct {
  const hctx *c;
  int threads;
  pthread_barrier_t start, end;
  int quit;
  /* the current iteration's frontier */
  const split_leaf *leaves;
  int n_leaves, depth, limit;
  int next;
  split_tres *tres;
} split_job;

static void split_run(split_job *job, int tid, searcher *s) {
  split_tres *r = &job->tres[tid];
  r->nodes = 0;
  r->ans = -1;
  r->ans_leaf = -1;
  for (;;) {
    int i = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
    if (i >= job->n_leaves) break;
    const split_leaf *L = &job->leaves[i];
    memcpy(s->board, L->board, sizeof s->board);
    memcpy(s->inv, L->inv, sizeof s->inv);
    s->blank = L->blank;
    s->h = L->h;
    s->limit = job->limit;
    s->ans = -1;
    s->have_path = 0;
    s->nodes = 0;
    memcpy(s->path, L->path, (size_t)job->depth);
    dfs(s, job->depth, L->pre);
    r->nodes += s->nodes;
    if (s->ans >= 0 && (r->ans < 0 || s->ans < r->ans || (s->ans == r->ans && i < r->ans_leaf))) {
      r->ans = s->ans;
      r->ans_leaf = i;
      memcpy(r->path, s->best_path, (size_t)(s->ans <= ORC_MAX_MOVES ? s->ans : ORC_MAX_MOVES));
    }
  }
}

typedef struct {
  split_job *job;
  int tid;
} split_arg;

static void *split_worker(void *arg) {
  split_arg *a = (split_arg *)arg;
  searcher *s = (searcher *)calloc(1, sizeof(searcher));
  s->c = a->job->c;
  s->mode = ORC_MODE_ALL;
  for (;;) {
    pthread_barrier_wait(&a->job->start);
    if (a->job->quit) break;
    split_run(a->job, a->tid, s);
    pthread_barrier_wait(&a->job->end);
  }
  free(s);
  return NULL;
}

/* One instance, all threads.  node_budget (0 = none) is checked between
 * iterations. */
static int split_solve(split_job *job, searcher *s0, const uint8_t *tiles, uint64_t budget, orc_result *out) {
  const hctx *c = job->c;
  memset(out, 0, sizeof(*out));
  out->len = -1;
  double t0 = now_s();
  int st = check_instance(c->w, tiles);
  if (st != ORC_OK) { out->status = st; return st; }
  split_leaf root;
  memset(&root, 0, sizeof root);
  for (int i = 0; i < c->n; ++i) {
    root.board[i] = tiles[i];
    root.inv[tiles[i]] = (uint8_t)i;
    if (!tiles[i]) root.blank = (uint8_t)i;
  }
  root.pre = -1;
  root.h = c->heuristic == ORC_HEUR_MD ? md_value(c, root.board) : pdb_value(c, root.inv);
  const int target = 32 * job->threads;
  split_leaf *cur = NULL, *nxt = NULL;
  size_t cap_cur = 0, cap_nxt = 0;
  uint64_t before = 0;
  st = ORC_ERR_LIMIT;
  for (int it = 0; it < ORC_MAX_ITERS; ++it) {
    const int limit = root.h + 2 * it;
    if (budget && before > budget) { st = ORC_ERR_NODE_BUDGET; break; }
    /* breadth-first frontier */
    uint64_t interior = 0;
    int ans = -1;
    uint8_t ans_path[SPLIT_MAX_DEPTH + 1];
    size_t n_cur = 1;
    if (cap_cur < 1) { cap_cur = 1024; cur = (split_leaf *)realloc(cur, cap_cur * sizeof(split_leaf)); }
    cur[0] = root;
    if (root.h == 0) ans = 0;
    int depth = 0;
    while (n_cur > 0 && n_cur < (size_t)target && depth < SPLIT_MAX_DEPTH) {
      size_t n_nxt = 0;
      for (size_t q = 0; q < n_cur; ++q) {
        const split_leaf *P = &cur[q];
        for (int d = 0; d < 4; ++d) {
          int to;
          if (!legal_move(c->w, P->blank, d, &to)) continue;
          if (P->pre >= 0 && d == 3 - P->pre) continue;
          ++interior;
          split_leaf C = *P;
          const int tile = C.board[to], from = C.blank;
          C.board[from] = (uint8_t)tile;
          C.board[to] = 0;
          C.inv[tile] = (uint8_t)from;
          C.inv[0] = (uint8_t)to;
          C.blank = (uint8_t)to;
          C.pre = (int8_t)d;
          C.h = c->heuristic == ORC_HEUR_MD ? P->h - c->md[to][tile] + c->md[from][tile] : pdb_value(c, C.inv);
          C.path[depth] = (uint8_t)d;
          if (C.h == 0 && (ans < 0 || depth + 1 < ans)) {
            ans = depth + 1;
            memcpy(ans_path, C.path, (size_t)(depth + 1));
          }
          if (depth + 1 + C.h > limit) continue;  /* generated, not expanded */
          if (n_nxt == cap_nxt) {
            cap_nxt = cap_nxt ? 2 * cap_nxt : 1024;
            nxt = (split_leaf *)realloc(nxt, cap_nxt * sizeof(split_leaf));
          }
          nxt[n_nxt++] = C;
        }
      }
      split_leaf *tp = cur; cur = nxt; nxt = tp;
      size_t tc = cap_cur; cap_cur = cap_nxt; cap_nxt = tc;
      n_cur = n_nxt;
      ++depth;
    }
    /* depth-first below the frontier, on every thread */
    job->leaves = cur;
    job->n_leaves = (int)n_cur;
    job->depth = depth;
    job->limit = limit;
    job->next = 0;
    uint64_t nodes = interior;
    int leaf_ans = -1, leaf_at = -1, leaf_t = -1;
    if (n_cur > 0 && depth > 0) {
      pthread_barrier_wait(&job->start);
      split_run(job, 0, s0);
      pthread_barrier_wait(&job->end);
      for (int t = 0; t < job->threads; ++t) {
        const split_tres *r = &job->tres[t];
        nodes += r->nodes;
        if (r->ans >= 0 && (leaf_ans < 0 || r->ans < leaf_ans || (r->ans == leaf_ans && r->ans_leaf < leaf_at))) {
          leaf_ans = r->ans;
          leaf_at = r->ans_leaf;
          leaf_t = t;
        }
      }
    } else if (n_cur > 0) {
      /* the root alone passed the f-test and the frontier never grew: search it here */
      s0->limit = limit;
      memcpy(s0->board, root.board, sizeof s0->board);
      memcpy(s0->inv, root.inv, sizeof s0->inv);
      s0->blank = root.blank;
      s0->h = root.h;
      s0->ans = -1;
      s0->have_path = 0;
      s0->nodes = 0;
      dfs(s0, 0, -1);
      nodes = s0->nodes;
      if (s0->ans >= 0) {
        leaf_ans = s0->ans;
        leaf_t = -2;
      }
    }
    out->f_limit[it] = limit;
    out->nodes[it] = nodes;
    out->n_iter = it + 1;
    before += nodes;
    if (leaf_ans >= 0 && (ans < 0 || leaf_ans < ans)) {
      ans = leaf_ans;
      const uint8_t *p = leaf_t >= 0 ? job->tres[leaf_t].path : s0->best_path;
      out->n_moves = ans <= ORC_MAX_MOVES ? ans : 0;
      memcpy(out->moves, p, (size_t)out->n_moves);
    } else if (ans >= 0) {
      out->n_moves = ans;
      memcpy(out->moves, ans_path, (size_t)ans);
    }
    if (ans >= 0) {
      out->len = ans;
      st = ORC_OK;
      break;
    }
  }
  free(cur);
  free(nxt);
  out->nodes_total = before;
  out->status = st;
  out->seconds = now_s() - t0;
  return st;
}

int orc_solve_batch_split(const orc_heur *h, const uint8_t *tiles, int n, uint64_t node_budget, int threads,
                          orc_result *out) {
  if (!h || !tiles || !out || n < 0 || (h->width != 4 && h->width != 5)) return ORC_ERR_ARG;
  if (h->heuristic == ORC_HEUR_PDB)
    for (int t = 0; t < orc_num_tables(h->width); ++t)
      if (!h->tables[t]) return ORC_ERR_ARG;
  if (n == 0) return ORC_OK;
  if (threads < 1) threads = 1;
  hctx *c = (hctx *)malloc(sizeof(hctx));
  hctx_init(c, h);
  split_job job;
  memset(&job, 0, sizeof job);
  job.c = c;
  job.threads = threads;
  job.tres = (split_tres *)calloc((size_t)threads, sizeof(split_tres));
  pthread_barrier_init(&job.start, NULL, (unsigned)threads);
  pthread_barrier_init(&job.end, NULL, (unsigned)threads);
  pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  split_arg *args = (split_arg *)malloc(sizeof(split_arg) * (size_t)threads);
  for (int t = 1; t < threads; ++t) {
    args[t].job = &job;
    args[t].tid = t;
    pthread_create(&tid[t], NULL, split_worker, &args[t]);
  }
  searcher *s0 = (searcher *)calloc(1, sizeof(searcher));
  s0->c = c;
  s0->mode = ORC_MODE_ALL;
  for (int i = 0; i < n; ++i) split_solve(&job, s0, tiles + (size_t)i * (size_t)c->n, node_budget, &out[i]);
  job.quit = 1;
  pthread_barrier_wait(&job.start);
  for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
  pthread_barrier_destroy(&job.start);
  pthread_barrier_destroy(&job.end);
  free(s0);
  free(args);
  free(tid);
  free(job.tres);
  free(c);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Horie's per-root first-goal search (the reference's host-callable     */
/* entry point)                                                         */
/* ------------------------------------------------------------------ */

/* Restates the depth-first search of src_horie/idas_parallel.cu:172-197
 * (idas_internal) for one 15-puzzle root, recursively: moves in the order
 * up, right, left, down; the reverse of the last move skipped (none at the
 * root); a child entered when depth + 1 + h(child) <= f_limit, h updated by
 * the table hd[tile][tile's cell][blank's move] (undone by the reverse move's
 * entry, as state_move(dir_reverse(dir)) does); moves allowed by mov[cell]
 * [move]; the search returns at the first goal (h == 0, the root included).
 * Default tables: src_horie/idas_parallel_host.c:88-129.  The path is never
 * allowed past ORC_PLAN_STRIDE - 1 moves. */
#define ORC_PLAN_STRIDE 252

typedef struct {
  uint8_t board[16];
  int blank, h, limit;
  int8_t hd[16 * 16 * 4];
  uint8_t mov[16 * 4];
  uint8_t path[ORC_PLAN_STRIDE];
} fp_ctx;

static const int fp_delta[4] = {-4, 1, -1, 4};

static void fp_slide(fp_ctx *c, int d) {
  int to = c->blank + fp_delta[d], t = c->board[to];
  c->h += c->hd[(t * 16 + to) * 4 + d];
  c->board[c->blank] = (uint8_t)t;
  c->board[to] = 0;
  c->blank = to;
}

static int fp_dfs(fp_ctx *c, int depth, int last) {
  if (c->h == 0) return depth;
  for (int d = 0; d < 4; ++d) {
    if (depth > 0 && d == 3 - last) continue;
    if (!c->mov[c->blank * 4 + d]) continue;
    int to = c->blank + fp_delta[d];
    int nh = c->h + c->hd[(c->board[to] * 16 + to) * 4 + d];
    if (depth + 1 + nh > c->limit || depth + 1 >= ORC_PLAN_STRIDE) continue;
    fp_slide(c, d);
    c->path[depth] = (uint8_t)d;
    int r = fp_dfs(c, depth + 1, d);
    if (r >= 0) return r;
    fp_slide(c, 3 - d);
  }
  return -1;
}

int orc_first_path(const uint8_t *tiles, int f_limit, const int8_t *h_diff, const uint8_t *movable,
                   int8_t *row) {
  if (!tiles || !row || f_limit < 0 || f_limit > ORC_PLAN_STRIDE - 1) return ORC_ERR_ARG;
  fp_ctx *c = (fp_ctx *)calloc(1, sizeof(fp_ctx));
  c->limit = f_limit;
  for (int t = 0; t < 16; ++t)
    for (int i = 0; i < 16; ++i)
      for (int d = 0; d < 4; ++d) {
        int gx = t % 4, gy = t / 4, x = i % 4, y = i / 4, v;
        if (d == 0) v = gy > y ? -1 : 1;
        else if (d == 1) v = gx < x ? -1 : 1;
        else if (d == 2) v = gx > x ? -1 : 1;
        else v = gy < y ? -1 : 1;
        c->hd[(t * 16 + i) * 4 + d] = h_diff ? h_diff[(t * 16 + i) * 4 + d] : (int8_t)v;
      }
  for (int i = 0; i < 16; ++i)
    for (int d = 0; d < 4; ++d) {
      int x = i % 4, y = i / 4;
      int ok = d == 0 ? y > 0 : d == 1 ? x < 3 : d == 2 ? x > 0 : y < 3;
      c->mov[i * 4 + d] = (uint8_t)(ok && (!movable || movable[i * 4 + d] != 0));
    }
  for (int i = 0; i < 16; ++i) {
    c->board[i] = tiles[i] & 15u;
    if (!c->board[i]) c->blank = i;
    else c->h += abs(i % 4 - c->board[i] % 4) + abs(i / 4 - c->board[i] / 4);
  }
  int len = fp_dfs(c, 0, -1);
  row[0] = (int8_t)len;
  for (int i = 0; i < len; ++i) row[1 + i] = (int8_t)c->path[i];
  free(c);
  return ORC_OK;
}
