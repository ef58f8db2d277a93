/*
 * Command-line front end of the CPU oracle -- TEST INFRASTRUCTURE.
 *
 *   oracle_cli solve -w 5 -H md|pdb [-m all|first] [-t threads] [-p pdbdir] FILE...
 *       prints `FILE len nodes` per instance, the line format of the
 *       reference's CPU solvers (src/24puzzle_expand.cc:154, :190) and of the
 *       golden files benchmarks/{manhattan,pdb}_expand_nodes.csv.
 *   oracle_cli pdb -w 5 -s semantics -o DIR
 *       builds every table of the width and writes DIR/pdb<w>_<table>.bin in
 *       compact rank order (the byte order of the reference's table files).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "oracle.h"

static int read_instance(const char *path, int n, uint8_t *tiles) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  for (int i = 0; i < n; ++i) {
    int v;
    if (fscanf(f, "%d", &v) != 1) { fclose(f); return -1; }
    tiles[i] = (uint8_t)v;
  }
  fclose(f);
  return 0;
}

static uint8_t *load_table(const char *dir, int w, int t, uint64_t size) {
  char path[4096];
  snprintf(path, sizeof path, "%s/pdb%d_%d.bin", dir, w, t);
  FILE *f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", path); return NULL; }
  uint8_t *buf = (uint8_t *)malloc(size);
  if (fread(buf, 1, size, f) != size) { fprintf(stderr, "short %s\n", path); fclose(f); free(buf); return NULL; }
  fclose(f);
  return buf;
}

int main(int argc, char **argv) {
  if (argc < 2) { fprintf(stderr, "usage: oracle_cli solve|pdb ...\n"); return 2; }
  const char *cmd = argv[1];
  int w = 5, threads = 1, mode = ORC_MODE_ALL, heur = ORC_HEUR_MD, sem = ORC_PDB_BLANK_ANY;
  const char *dir = ".";
  int opt;
  optind = 2;
  while ((opt = getopt(argc, argv, "w:H:m:t:p:s:o:")) != -1) {
    switch (opt) {
      case 'w': w = atoi(optarg); break;
      case 'H': heur = strcmp(optarg, "pdb") == 0 ? ORC_HEUR_PDB : ORC_HEUR_MD; break;
      case 'm': mode = strcmp(optarg, "first") == 0 ? ORC_MODE_FIRST : ORC_MODE_ALL; break;
      case 't': threads = atoi(optarg); break;
      case 'p': case 'o': dir = optarg; break;
      case 's': sem = atoi(optarg); break;
      default: return 2;
    }
  }
  if (w != 4 && w != 5) { fprintf(stderr, "width must be 4 or 5\n"); return 2; }
  int n = w * w;
  uint64_t T = orc_table_size(w);
  if (strcmp(cmd, "pdb") == 0) {
    uint8_t *buf = (uint8_t *)malloc(T);
    for (int t = 0; t < orc_num_tables(w); ++t) {
      int st = orc_pdb_build(w, t, sem, threads <= 1 ? 0 : threads, buf);
      if (st) { fprintf(stderr, "build failed %d\n", st); return 1; }
      char path[4096];
      snprintf(path, sizeof path, "%s/pdb%d_%d.bin", dir, w, t);
      FILE *f = fopen(path, "wb");
      if (!f || fwrite(buf, 1, T, f) != T) { fprintf(stderr, "write %s failed\n", path); return 1; }
      fclose(f);
      fprintf(stderr, "wrote %s\n", path);
    }
    free(buf);
    return 0;
  }
  if (strcmp(cmd, "solve") != 0) { fprintf(stderr, "unknown command %s\n", cmd); return 2; }
  orc_heur h;
  memset(&h, 0, sizeof h);
  h.width = w;
  h.heuristic = heur;
  if (heur == ORC_HEUR_PDB)
    for (int t = 0; t < orc_num_tables(w); ++t)
      if (!(h.tables[t] = load_table(dir, w, t, T))) return 1;
  int count = argc - optind;
  uint8_t *tiles = (uint8_t *)malloc((size_t)(count > 0 ? count : 1) * (size_t)n);
  for (int i = 0; i < count; ++i)
    if (read_instance(argv[optind + i], n, tiles + (size_t)i * n)) {
      fprintf(stderr, "cannot read %s\n", argv[optind + i]);
      return 1;
    }
  orc_result *res = (orc_result *)calloc((size_t)(count > 0 ? count : 1), sizeof(orc_result));
  orc_solve_batch(&h, tiles, count, mode, 0, threads, res);
  for (int i = 0; i < count; ++i)
    printf("%s %d %llu\n", argv[optind + i], res[i].len, (unsigned long long)res[i].nodes_total);
  return 0;
}
