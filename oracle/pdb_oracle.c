/*
 * CPU oracle: breadth-first pattern-database builder -- TEST INFRASTRUCTURE.
 *
 * The reference reads two 6-tile tables for the 24-puzzle
 * (src/24puzzle_expand_with_pdb.cpp:77-112) but ships neither the tables nor
 * their generator.  This file builds them from first principles so that the
 * GPU builder's output can be checked byte-for-byte.  Three abstractions are
 * implemented; benchmarks/pdb_expand_nodes.csv (50 golden `len nodes` rows of
 * the reference's PDB solver) decides which one the reference's tables hold:
 *
 *   ORC_PDB_BLANK_FREE  a pattern tile may step onto any neighbouring cell not
 *                       held by another pattern tile; cost 1 per step.
 *   ORC_PDB_BLANK_ANY   the blank is modelled: an abstract state is the
 *                       pattern placement plus the connected region of
 *                       non-pattern cells holding the blank (moves of other
 *                       tiles are free inside a region); a pattern tile may
 *                       step into a neighbouring cell of the blank's region,
 *                       cost 1.  The goal is the goal placement with the
 *                       blank in any region; the stored value is the minimum
 *                       over the blank's regions.
 *   ORC_PDB_BLANK_HOME  as BLANK_ANY but the goal requires the blank in the
 *                       region of its home cell 0.
 *
 * Tables are stored in compact k-permutation rank order (orc_rank), which is
 * also the byte order of the reference's table files.
 */
#include "oracle.h"

#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define UNSEEN 0xFFu

typedef struct {
  int w, n, k;
  uint32_t full, not_col0, not_collast;
  int base[6];
} geo;

static void geo_init(geo *g, int width, int table_id) {
  g->w = width;
  g->n = width * width;
  g->k = orc_pattern_k(width);
  g->full = (g->n == 32) ? 0xFFFFFFFFu : ((1u << g->n) - 1u);
  uint32_t col0 = 0, coll = 0;
  for (int r = 0; r < width; ++r) {
    col0 |= 1u << (r * width);
    coll |= 1u << (r * width + width - 1);
  }
  g->not_col0 = g->full & ~col0;
  g->not_collast = g->full & ~coll;
  orc_table_tiles(width, table_id, g->base);
}

static inline uint32_t grow(const geo *g, uint32_t s) {
  return (((s << 1) & g->not_col0) | ((s >> 1) & g->not_collast) | (s << g->w) | (s >> g->w)) &
         g->full;
}

/* connected component of `free` containing cell c */
static inline uint32_t flood(const geo *g, uint32_t free_cells, int c) {
  uint32_t r = 1u << c, prev;
  do {
    prev = r;
    r = (r | grow(g, r)) & free_cells;
  } while (r != prev);
  return r;
}

static inline int neighbour(const geo *g, int cell, int d) {
  int r = cell / g->w, c = cell % g->w;
  switch (d) {
    case 0: return r == 0 ? -1 : cell - g->w;
    case 1: return c == g->w - 1 ? -1 : cell + 1;
    case 2: return c == 0 ? -1 : cell - 1;
    default: return r == g->w - 1 ? -1 : cell + g->w;
  }
}

static int build_blank_free(const geo *g, uint64_t T, uint8_t *dist, int threads) {
  memset(dist, UNSEEN, T);
  dist[orc_rank(g->n, g->k, g->base)] = 0;
  for (int d = 0; d < 254; ++d) {
    long long produced = 0;
#pragma omp parallel for schedule(dynamic, 65536) reduction(+ : produced) num_threads(threads)
    for (long long r = 0; r < (long long)T; ++r) {
      if (dist[r] != d) continue;
      int pos[6];
      orc_unrank(g->n, g->k, (uint64_t)r, pos);
      uint32_t occ = 0;
      for (int j = 0; j < g->k; ++j) occ |= 1u << pos[j];
      for (int j = 0; j < g->k; ++j)
        for (int dir = 0; dir < 4; ++dir) {
          int c = neighbour(g, pos[j], dir);
          if (c < 0 || ((occ >> c) & 1u)) continue;
          int q[6];
          memcpy(q, pos, sizeof q);
          q[j] = c;
          uint64_t r2 = orc_rank(g->n, g->k, q);
          if (dist[r2] == UNSEEN) {
            dist[r2] = (uint8_t)(d + 1);
            ++produced;
          }
        }
    }
    if (!produced) return 0;
  }
  return ORC_ERR_LIMIT;
}

/* rows of `stride` bytes: dist[r*stride + m], m = lowest cell of the
 * blank's region */
static int build_blank_region(const geo *g, uint64_t T, uint8_t *out, int semantics,
                              int threads) {
  const int stride = g->n <= 16 ? 16 : 32;
  uint8_t *dist = (uint8_t *)malloc((size_t)T * (size_t)stride);
  if (!dist) return ORC_ERR_ARG;
  memset(dist, UNSEEN, (size_t)T * (size_t)stride);
  {
    uint32_t occ = 0;
    for (int j = 0; j < g->k; ++j) occ |= 1u << g->base[j];
    uint32_t free_cells = g->full & ~occ;
    uint64_t r0 = orc_rank(g->n, g->k, g->base);
    for (int c = 0; c < g->n; ++c) {
      if (!((free_cells >> c) & 1u)) continue;
      uint32_t reg = flood(g, free_cells, c);
      if (semantics == ORC_PDB_BLANK_HOME && !(reg & 1u)) continue;
      dist[r0 * (uint64_t)stride + (uint64_t)__builtin_ctz(reg)] = 0;
    }
  }
  int st = ORC_ERR_LIMIT;
  for (int d = 0; d < 254; ++d) {
    long long produced = 0;
    const uint64_t pat = 0x0101010101010101ull * (uint64_t)d;
#pragma omp parallel for schedule(dynamic, 16384) reduction(+ : produced) num_threads(threads)
    for (long long r = 0; r < (long long)T; ++r) {
      const uint8_t *row = dist + (uint64_t)r * (uint64_t)stride;
      int any = 0;
      for (int wdx = 0; wdx < stride / 8; ++wdx) {
        uint64_t x;
        memcpy(&x, row + 8 * wdx, 8);
        x ^= pat;
        if ((x - 0x0101010101010101ull) & ~x & 0x8080808080808080ull) { any = 1; break; }
      }
      if (!any) continue;
      int pos[6];
      orc_unrank(g->n, g->k, (uint64_t)r, pos);
      uint32_t occ = 0;
      for (int j = 0; j < g->k; ++j) occ |= 1u << pos[j];
      uint32_t free_cells = g->full & ~occ;
      for (int m = 0; m < g->n; ++m) {
        if (row[m] != d) continue;
        uint32_t reg = flood(g, free_cells, m);
        for (int j = 0; j < g->k; ++j)
          for (int dir = 0; dir < 4; ++dir) {
            int c = neighbour(g, pos[j], dir);
            if (c < 0 || !((reg >> c) & 1u)) continue;
            int q[6];
            memcpy(q, pos, sizeof q);
            q[j] = c;
            uint32_t free2 = (free_cells & ~(1u << c)) | (1u << pos[j]);
            uint32_t reg2 = flood(g, free2, pos[j]);
            uint64_t r2 = orc_rank(g->n, g->k, q);
            uint8_t *e = dist + r2 * (uint64_t)stride + (uint64_t)__builtin_ctz(reg2);
            if (*e == UNSEEN) {
              *e = (uint8_t)(d + 1);
              ++produced;
            }
          }
      }
    }
    if (!produced) { st = 0; break; }
  }
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long r = 0; r < (long long)T; ++r) {
    const uint8_t *row = dist + (uint64_t)r * (uint64_t)stride;
    uint8_t best = UNSEEN;
    for (int m = 0; m < g->n; ++m)
      if (row[m] < best) best = row[m];
    out[r] = best;
  }
  free(dist);
  return st;
}

int orc_pdb_build(int width, int table_id, int semantics, int threads, uint8_t *out) {
  if ((width != 4 && width != 5) || !out) return ORC_ERR_ARG;
  if (table_id < 0 || table_id >= orc_num_tables(width)) return ORC_ERR_ARG;
  if (threads <= 0) threads = omp_get_num_procs();
  geo g;
  geo_init(&g, width, table_id);
  uint64_t T = orc_table_size(width);
  if (semantics == ORC_PDB_BLANK_FREE) return build_blank_free(&g, T, out, threads);
  if (semantics == ORC_PDB_BLANK_ANY || semantics == ORC_PDB_BLANK_HOME)
    return build_blank_region(&g, T, out, semantics, threads);
  return ORC_ERR_ARG;
}
