// Host side of libslide: the C ABI (include/slide.h), the root-set
// ("frontier") construction, the IDA* threshold-round loop and static load
// balancing.  Device work is in search.cu and pdb_build.cu.
//
// Reference counterparts:
//   create_root_set       src/24puzzle_block_parallel_with_pdb.cu:454-490
//   ida_star round loop   src/24puzzle_block_parallel_with_pdb.cu:756-922
//   divide_root_set       src/24puzzle_block_parallel_with_pdb.cu:652-747
//
// Differences that keep node counts exact (the reference's GPU solvers
// report lengths only):
//   * the root set is a tree expansion to a uniform depth with no duplicate
//     detection (Horie's A* distribution merges transpositions,
//     src_horie/idas_smem.cu:1083-1113, which changes counts);
//   * a goal met while building the root set does not end the search early
//     (src/24puzzle_block_parallel_with_pdb.cu:482-485 returns there);
//   * each round adds the children generated by root-set interior nodes
//     whose path stays within the limit (prefix maximum of g+h: the PDB
//     heuristic is not consistent, so f can drop along a path), and a root
//     becomes a device task only if the same holds for it;
//   * the static re-split of heavy roots (ceil(load/avg) pieces, as at
//     :839-897) refines the root-set tree, so the pieces' ancestors are
//     counted like any other interior node.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/slide.h"
#include "sp_defs.h"
#include "sp_kernels.h"

namespace sp {

static std::atomic<uint64_t> g_launches{0};
void note_launch(int n) { g_launches.fetch_add((uint64_t)n); }

namespace {

struct TreeNode {
  uint8_t board[kMaxN];
  uint8_t blank, g, pre, move;  // move: from parent (kNoPre for the root)
  int32_t parent;
  int32_t h;
  int32_t maxf;                 // max of g+h over the path root..this node
  uint8_t nchild;               // legal non-reverse children
  uint8_t leaf;                 // 1: root-set member (device task when active)
  uint8_t expanded;             // children present in the tree
  uint8_t pad;
  int32_t sub;                  // index into the batch's SubRoot array, -1 if none
};

struct Instance {
  int status = SP_OK;
  int h0 = 0;
  int iter = 0;
  bool done = false;
  std::vector<TreeNode> tree;
  std::vector<int32_t> leaves;      // tree indices of root-set members
  std::vector<uint64_t> last_load;  // per leaf, previous round
  uint64_t last_total = 0;          // device nodes of the previous round
  uint64_t prev_total = 0;          // and of the one before
  sp_result *out = nullptr;
};

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

int check_instance(int w, const uint8_t *t) {
  const int n = w * w;
  uint32_t seen = 0;
  for (int i = 0; i < n; ++i) {
    if (t[i] >= n || ((seen >> t[i]) & 1u)) return SP_ERR_NOT_PERMUTATION;
    seen |= 1u << t[i];
  }
  int inv = 0, brow = 0;
  for (int i = 0; i < n; ++i) {
    if (!t[i]) { brow = i / w; continue; }
    for (int j = i + 1; j < n; ++j)
      if (t[j] && t[j] < t[i]) ++inv;
  }
  // goal blank at cell 0: odd widths keep inversion parity; even widths keep
  // inversions + blank row
  const int par = (w & 1) ? (inv & 1) : ((inv + brow) & 1);
  return par ? SP_ERR_UNSOLVABLE : SP_OK;
}

}  // namespace
}  // namespace sp

using namespace sp;

struct sp_solver {
  int w = 4, n = 16, heur = SP_HEUR_MANHATTAN;
  sp_config cfg{};
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int num_sms = 0;
  HeurTables h_ht{};
  HeurTables *d_ht = nullptr;
  uint8_t *d_pdb = nullptr;
  bool pdb_ready = false;
  uint32_t import_mask = 0;
  double pdb_build_ms = 0;
  int last_lanes = 0;       // lanes of the last search launch
  uint32_t last_emitted = 0;
  // split pre-pass buffers
  uint32_t *d_cnt = nullptr;  // [level a, level b, emitted, error]
  Task *d_split_a = nullptr, *d_split_b = nullptr, *d_emit = nullptr;
  size_t split_cap_a = 0, split_cap_b = 0, emit_cap = 0;
  // device task pool
  Task *d_tasks = nullptr;
  uint32_t *d_seq = nullptr;
  uint32_t cap = 0;
  PoolCtl *d_ctl = nullptr;
  uint32_t stamp = 0;
  // per-batch buffers
  SubRoot *d_subs = nullptr;
  size_t subs_cap = 0;
  Task *d_init = nullptr;
  size_t init_cap = 0;
  unsigned long long *d_sub_nodes = nullptr;
  int32_t *d_limit = nullptr;
  Solution *d_sol = nullptr;
  size_t inst_cap = 0;
  uint8_t *d_boards = nullptr;
  int32_t *d_h = nullptr;
  size_t boards_cap = 0;
  size_t h_cap = 0;
  std::string err;
  sp_stats stats{};
};

namespace {

int fail_cuda(sp_solver *s, cudaError_t e, const char *what) {
  s->err = std::string(what) + ": " + cudaGetErrorString(e);
  return SP_ERR_CUDA;
}

#define SP_CUDA(s, call)                                      \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return fail_cuda((s), e_, #call); \
  } while (0)

template <typename T>
int ensure(sp_solver *s, T **p, size_t *cap, size_t need) {
  if (*cap >= need && *p) return SP_OK;
  size_t ncap = std::max(need, *cap * 2);
  if (ncap < 64) ncap = 64;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  SP_CUDA(s, cudaMalloc((void **)p, ncap * sizeof(T)));
  *cap = ncap;
  return SP_OK;
}

void build_heur_tables(int w, HeurTables *ht) {
  memset(ht, 0, sizeof(*ht));
  const int n = w * w;
  for (int d = 0; d < 4; ++d)
    for (int c = 0; c < n; ++c)
      for (int t = 0; t < n; ++t) {
        // the blank moved by d onto cell c; the tile t at c slides back to b
        const int b = c - move_delta(w, d);
        int v = 0;
        if (t && b >= 0 && b < n) {
          const int mb = abs(b / w - t / w) + abs(b % w - t % w);
          const int mc = abs(c / w - t / w) + abs(c % w - t % w);
          v = mb - mc;
        }
        ht->mdd[(d * n + c) * n + t] = (int8_t)v;
      }
  PatternSet ps = pattern_set(w);
  for (int part = 0; part < 2; ++part) {
    for (int t = 0; t < n; ++t) ht->pat[part][t] = 0xFF;
    for (int p = 0; p < ps.n_pat; ++p) {
      const int tab = ps.pat_table[part][p], sym = ps.pat_sym[part][p];
      for (int j = 0; j < ps.k; ++j) {
        // tile whose goal cell maps onto the table's j-th goal cell
        int tile = -1;
        for (int c = 0; c < n; ++c)
          if (sym_cell(w, sym, c) == ps.table_tiles[tab][j]) tile = c;
        uint32_t mul = 1;
        for (int q = j + 1; q < ps.k; ++q) mul *= (uint32_t)ps.radix;
        ht->pat[part][tile] = (uint8_t)p;
        for (int c = 0; c < n; ++c) ht->code[part][tile * n + c] = (uint32_t)sym_cell(w, sym, c) * mul;
      }
    }
  }
}

void make_root(int w, const uint8_t *tiles, TreeNode *r) {
  memset(r, 0, sizeof(*r));
  const int n = w * w;
  for (int i = 0; i < n; ++i) {
    r->board[i] = tiles[i];
    if (!tiles[i]) r->blank = (uint8_t)i;
  }
  r->g = 0;
  r->pre = kNoPre;
  r->move = kNoPre;
  r->parent = -1;
  r->sub = -1;
}

// Append the children of tree[idx]; returns how many.
int expand_node(int w, std::vector<TreeNode> &tree, int idx) {
  TreeNode p = tree[idx];
  uint32_t mv = legal_moves(w, p.blank);
  if (p.pre != kNoPre) mv &= ~(1u << (3 - p.pre));
  int cnt = 0;
  for (int d = 0; d < 4; ++d) {
    if (!((mv >> d) & 1u)) continue;
    TreeNode c = p;
    const int src = p.blank + move_delta(w, d);
    c.board[p.blank] = p.board[src];
    c.board[src] = 0;
    c.blank = (uint8_t)src;
    c.g = (uint8_t)(p.g + 1);
    c.pre = (uint8_t)d;
    c.move = (uint8_t)d;
    c.parent = idx;
    c.h = 0;
    c.maxf = 0;
    c.leaf = 1;
    c.expanded = 0;
    c.sub = -1;
    tree.push_back(c);
    ++cnt;
  }
  tree[idx].expanded = 1;
  tree[idx].leaf = 0;
  return cnt;
}

uint8_t count_children(int w, const TreeNode &t) {
  uint32_t mv = legal_moves(w, t.blank);
  if (t.pre != kNoPre) mv &= ~(1u << (3 - t.pre));
  return (uint8_t)__builtin_popcount(mv);
}

// h for tree nodes [from, tree.size()) of every instance, on the GPU.
int compute_tree_h(sp_solver *s, std::vector<Instance> &inst, const std::vector<size_t> &from) {
  size_t total = 0;
  for (size_t i = 0; i < inst.size(); ++i) total += inst[i].tree.size() - from[i];
  if (!total) return SP_OK;
  int rc = ensure(s, &s->d_boards, &s->boards_cap, total * (size_t)s->n);
  if (rc) return rc;
  rc = ensure(s, &s->d_h, &s->h_cap, total);
  if (rc) return rc;
  std::vector<uint8_t> boards(total * (size_t)s->n);
  size_t o = 0;
  for (size_t i = 0; i < inst.size(); ++i)
    for (size_t j = from[i]; j < inst[i].tree.size(); ++j, ++o)
      memcpy(&boards[o * s->n], inst[i].tree[j].board, (size_t)s->n);
  SP_CUDA(s, cudaMemcpyAsync(s->d_boards, boards.data(), boards.size(), cudaMemcpyHostToDevice, s->st));
  s->stats.h2d_bytes += boards.size();
  SP_CUDA(s, launch_heuristic(s->w, s->heur == SP_HEUR_PDB, s->d_boards, (int)total, s->d_h, s->d_ht,
                              s->d_pdb, s->st));
  std::vector<int32_t> hv(total);
  SP_CUDA(s, cudaMemcpyAsync(hv.data(), s->d_h, total * sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  s->stats.d2h_bytes += total * sizeof(int32_t);
  o = 0;
  for (size_t i = 0; i < inst.size(); ++i)
    for (size_t j = from[i]; j < inst[i].tree.size(); ++j, ++o) {
      TreeNode &t = inst[i].tree[j];
      t.h = hv[o];
      const int f = (int)t.g + t.h;
      t.maxf = t.parent < 0 ? f : std::max(inst[i].tree[t.parent].maxf, f);
      t.nchild = count_children(s->w, t);
    }
  return SP_OK;
}

void rebuild_leaves(Instance &I) {
  I.leaves.clear();
  for (size_t j = 0; j < I.tree.size(); ++j)
    if (I.tree[j].leaf) I.leaves.push_back((int32_t)j);
  I.last_load.assign(I.leaves.size(), 0);
}

bool replay_ok(int w, const uint8_t *tiles, const uint8_t *moves, int len) {
  const int n = w * w;
  uint8_t b[kMaxN];
  int blank = 0;
  for (int i = 0; i < n; ++i) {
    b[i] = tiles[i];
    if (!tiles[i]) blank = i;
  }
  for (int i = 0; i < len; ++i) {
    if (moves[i] > 3 || !((legal_moves(w, blank) >> moves[i]) & 1u)) return false;
    const int src = blank + move_delta(w, moves[i]);
    b[blank] = b[src];
    b[src] = 0;
    blank = src;
  }
  for (int i = 0; i < n; ++i)
    if (b[i] != i) return false;
  return true;
}

// Ring capacity: a power of two holding the round's root tasks plus room for
// a waiting claim from every resident lane.
int ensure_pool(sp_solver *s, size_t n_init) {
  size_t need = (size_t)1 << 20;
  while (need < n_init + ((size_t)1 << 19)) need <<= 1;
  if (need > ((size_t)1 << 30)) {
    s->err = "too many root tasks for the task pool";
    return SP_ERR_CAPACITY;
  }
  if (s->cap >= need) return SP_OK;
  if (s->d_tasks) cudaFree(s->d_tasks);
  if (s->d_seq) cudaFree(s->d_seq);
  s->d_tasks = nullptr;
  s->d_seq = nullptr;
  s->cap = 0;
  SP_CUDA(s, cudaMalloc(&s->d_tasks, need * sizeof(Task)));
  SP_CUDA(s, cudaMalloc(&s->d_seq, need * sizeof(uint32_t)));
  s->cap = (uint32_t)need;
  return SP_OK;
}

// The round's work: tasks started as they are, and roots expanded `flags`
// levels by the device split pre-pass first.
struct RoundPlan {
  std::vector<Task> direct;
  std::vector<Task> split;
  size_t level_bound = 0;  // nodes one split level can hold
  size_t emit_bound = 0;   // pieces the split pre-pass can emit
  int max_k = 0;
};

int launch_round(sp_solver *s, const RoundPlan &plan, float *ms, uint32_t *split_err) {
  const uint32_t n_direct = (uint32_t)plan.direct.size();
  int rc = ensure_pool(s, plan.direct.size() + plan.emit_bound);
  if (rc) return rc;
  rc = ensure(s, &s->d_init, &s->init_cap, std::max<size_t>(plan.direct.size(), 1));
  if (rc) return rc;
  if (!s->d_cnt) SP_CUDA(s, cudaMalloc(&s->d_cnt, 4 * sizeof(uint32_t)));
  if (n_direct) {
    SP_CUDA(s, cudaMemcpyAsync(s->d_init, plan.direct.data(), n_direct * sizeof(Task), cudaMemcpyHostToDevice, s->st));
    s->stats.h2d_bytes += n_direct * sizeof(Task);
  }
  uint32_t cnt0[4] = {(uint32_t)plan.split.size(), 0, 0, 0};
  SP_CUDA(s, cudaMemcpyAsync(s->d_cnt, cnt0, sizeof(cnt0), cudaMemcpyHostToDevice, s->st));
  if (!plan.split.empty()) {
    rc = ensure(s, &s->d_split_a, &s->split_cap_a, std::max(plan.level_bound, plan.split.size()));
    if (rc) return rc;
    rc = ensure(s, &s->d_split_b, &s->split_cap_b, std::max(plan.level_bound, plan.split.size()));
    if (rc) return rc;
    rc = ensure(s, &s->d_emit, &s->emit_cap, std::max<size_t>(plan.emit_bound, 1));
    if (rc) return rc;
    SP_CUDA(s, cudaMemcpyAsync(s->d_split_a, plan.split.data(), plan.split.size() * sizeof(Task),
                               cudaMemcpyHostToDevice, s->st));
    s->stats.h2d_bytes += plan.split.size() * sizeof(Task);
  }
  SP_CUDA(s, cudaEventRecord(s->ev0, s->st));
  for (int l = 0; l < plan.max_k; ++l) {
    const int cur = l & 1, nxt = cur ^ 1;
    SP_CUDA(s, cudaMemsetAsync(s->d_cnt + nxt, 0, sizeof(uint32_t), s->st));
    SplitArgs A{};
    A.subs = s->d_subs;
    A.inst_limit = s->d_limit;
    A.ht = s->d_ht;
    A.pdb = s->d_pdb;
    A.sub_nodes = s->d_sub_nodes;
    A.sol = s->d_sol;
    A.in = cur ? s->d_split_b : s->d_split_a;
    A.n_in = s->d_cnt + cur;
    A.next = nxt ? s->d_split_b : s->d_split_a;
    A.n_next = s->d_cnt + nxt;
    A.cap_next = (uint32_t)(nxt ? s->split_cap_b : s->split_cap_a);
    A.out = s->d_emit;
    A.n_out = s->d_cnt + 2;
    A.cap_out = (uint32_t)s->emit_cap;
    A.error = (int32_t *)(s->d_cnt + 3);
    SP_CUDA(s, launch_split_level(s->w, s->heur == SP_HEUR_PDB, s->num_sms, A, s->st));
    s->stats.kernel_launches += 1;
  }
  SP_CUDA(s, launch_pool_init(s->d_tasks, s->d_emit, plan.max_k ? s->d_cnt + 2 : nullptr, s->d_init, n_direct,
                              s->d_seq, s->cap, s->d_ctl, s->st));
  RoundParams P{};
  P.subs = s->d_subs;
  P.tasks = s->d_tasks;
  P.seq = s->d_seq;
  P.cap = s->cap;
  P.ctl = s->d_ctl;
  P.inst_limit = s->d_limit;
  P.sub_nodes = s->d_sub_nodes;
  P.sol = s->d_sol;
  P.ht = s->d_ht;
  P.pdb = s->d_pdb;
  P.min_slack = s->cfg.donate_min_slack;
  P.steps = s->cfg.steps_per_poll;
  P.donate = s->cfg.lb_mode == SP_LB_NONE ? 0 : 1;
  P.timeout_ns = (unsigned long long)s->cfg.timeout_ms * 1000000ull;
  P.poll_ns = 2000;
  const int block = s->cfg.threads_per_block == 128 ? 128 : 256;
  SP_CUDA(s, cudaEventRecord(s->ev0, s->st));
  int grid = 0;
  SP_CUDA(s, launch_search_round(s->w, s->heur == SP_HEUR_PDB, block, s->cfg.blocks_per_sm, s->num_sms, P,
                                 s->st, &grid));
  SP_CUDA(s, cudaEventRecord(s->ev1, s->st));
  uint32_t cnt[4] = {0, 0, 0, 0};
  SP_CUDA(s, cudaMemcpyAsync(cnt, s->d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaEventSynchronize(s->ev1));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  SP_CUDA(s, cudaEventElapsedTime(ms, s->ev0, s->ev1));
  *split_err = cnt[3];
  s->stats.kernel_launches += 2;
  s->last_lanes = grid * block;
  s->last_emitted = cnt[2];
  return SP_OK;
}

// Static load balancing for the next round: a root's work is predicted from
// its previous round (load x the instance's growth per threshold step); a
// root predicted above the round's piece size T is split ceil(log2(pred/T))
// levels by the device pre-pass -- the reference splits a root into
// ceil(load/avg) pieces (src/24puzzle_block_parallel_with_pdb.cu:839-897) --
// and direct tasks are published in decreasing predicted size.
void plan_static(sp_solver *s, std::vector<Instance> &inst, const std::vector<int32_t> &limits,
                 RoundPlan &plan) {
  struct Cand {
    double pred;
    Task t;
    int room;  // levels left below the root before the limit
  };
  std::vector<Cand> c;
  double total = 0;
  for (size_t i = 0; i < inst.size(); ++i) {
    Instance &I = inst[i];
    if (I.done) continue;
    double growth = 6.0;
    if (I.prev_total > 0 && I.last_total > 0) growth = std::min(30.0, std::max(2.0, (double)I.last_total / I.prev_total));
    for (size_t q = 0; q < I.leaves.size(); ++q) {
      const TreeNode &t = I.tree[(size_t)I.leaves[q]];
      if (t.maxf > limits[i]) continue;
      Cand x;
      x.pred = (double)I.last_load[q] * growth;
      x.t = Task{};
      x.t.sub = (uint32_t)t.sub;
      x.t.mask = 0xF;
      x.room = limits[i] - t.g;
      total += x.pred;
      c.push_back(x);
    }
  }
  const double lanes = s->last_lanes > 0 ? (double)s->last_lanes : (double)s->num_sms * 1024.0;
  const double T = total / (lanes * 4.0);
  size_t budget = (size_t)1 << 22;
  plan.max_k = 0;
  std::vector<int> k(c.size(), 0);
  if (T > 0 && s->cfg.lb_mode == SP_LB_STATIC_STEAL) {
    for (size_t j = 0; j < c.size(); ++j) {
      if (c[j].pred > T) {
        int kk = (int)std::ceil(std::log2(c[j].pred / T));
        kk = std::min(kk, std::min(10, std::max(0, c[j].room - 1)));
        k[j] = std::max(0, std::min(kk, std::max(1, s->cfg.static_split_cap)));
      }
    }
    auto bound = [&](int kk) { return kk ? (size_t)4 * (size_t)std::pow(3.0, kk - 1) : 0; };
    size_t need = 0;
    for (int kk : k) need += bound(kk);
    while (need > budget) {  // trim the deepest splits first
      int mk = 0;
      for (int kk : k) mk = std::max(mk, kk);
      if (!mk) break;
      for (auto &kk : k)
        if (kk == mk) { need -= bound(kk) - bound(kk - 1); --kk; }
    }
  }
  std::vector<size_t> order(c.size());
  for (size_t j = 0; j < c.size(); ++j) order[j] = j;
  if (s->cfg.lb_mode == SP_LB_STATIC_STEAL)
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return c[a].pred > c[b].pred; });
  std::vector<size_t> level(12, 0);
  for (size_t j : order) {
    if (k[j] > 0) {
      Task t = c[j].t;
      t.flags = (uint8_t)k[j];
      plan.split.push_back(t);
      plan.max_k = std::max(plan.max_k, k[j]);
      for (int l = 1; l <= k[j]; ++l) level[(size_t)l] += (size_t)4 * (size_t)std::pow(3.0, l - 1);
      plan.emit_bound += (size_t)4 * (size_t)std::pow(3.0, k[j] - 1);
    } else {
      plan.direct.push_back(c[j].t);
    }
  }
  for (size_t l = 1; l < level.size(); ++l) plan.level_bound = std::max(plan.level_bound, level[l]);
}

int solve_impl(sp_solver *s, const uint8_t *tiles, int nin, sp_result *res) {
  auto t_start = std::chrono::steady_clock::now();
  memset(&s->stats, 0, sizeof(s->stats));
  if (s->heur == SP_HEUR_PDB && !s->pdb_ready) {
    s->err = "PDB heuristic selected but sp_pdb_build/sp_pdb_import not done";
    return SP_ERR_NO_PDB;
  }
  const int w = s->w, n = s->n;
  std::vector<Instance> inst((size_t)nin);
  for (int i = 0; i < nin; ++i) {
    Instance &I = inst[(size_t)i];
    I.out = &res[i];
    memset(I.out, 0, sizeof(sp_result));
    I.out->len = -1;
    I.status = check_instance(w, tiles + (size_t)i * n);
    if (I.status != SP_OK) {
      I.done = true;
      I.out->status = I.status;
      continue;
    }
    TreeNode root;
    make_root(w, tiles + (size_t)i * n, &root);
    I.tree.push_back(root);
  }
  // root set: uniform-depth tree expansion to >= frontier_target leaves
  auto t_front = std::chrono::steady_clock::now();
  const int target = std::max(1, s->cfg.frontier_target);
  for (auto &I : inst) {
    if (I.done) continue;
    std::vector<int32_t> level{0};
    I.tree[0].leaf = 1;
    for (int dep = 0; dep < 40 && (int)level.size() < target; ++dep) {
      std::vector<int32_t> next;
      for (int32_t x : level) {
        size_t before = I.tree.size();
        expand_node(w, I.tree, x);
        for (size_t c = before; c < I.tree.size(); ++c) next.push_back((int32_t)c);
      }
      level.swap(next);
    }
  }
  std::vector<size_t> from(inst.size(), 0);
  int rc = compute_tree_h(s, inst, from);
  if (rc) return rc;
  for (auto &I : inst) {
    if (I.done) continue;
    I.h0 = I.tree[0].h;
    rebuild_leaves(I);
  }
  s->stats.frontier_ms += ms_since(t_front);

  std::vector<int32_t> sub_base(inst.size(), 0);
  std::vector<SubRoot> subs;
  std::vector<Task> init;
  std::vector<int32_t> limits(inst.size(), 0);
  std::vector<unsigned long long> sub_nodes;
  std::vector<Solution> sols(inst.size());
  bool subs_dirty = true;

  for (int round = 0; round < SP_MAX_ITERS; ++round) {
    int active = 0;
    for (auto &I : inst) active += !I.done;
    if (!active) break;
    const auto t_round = std::chrono::steady_clock::now();
    const int ri = std::min(round, SP_MAX_ROUNDS - 1);
    s->stats.round_instances[ri] = active;
    // (re)build the SubRoot array when the trees changed
    if (subs_dirty) {
      subs.clear();
      for (size_t i = 0; i < inst.size(); ++i) {
        sub_base[i] = (int32_t)subs.size();
        Instance &I = inst[i];
        if (I.done) continue;
        for (int32_t x : I.leaves) {
          TreeNode &t = I.tree[(size_t)x];
          t.sub = (int32_t)subs.size();
          SubRoot r{};
          memcpy(r.board, t.board, (size_t)n);
          r.blank = t.blank;
          r.g = t.g;
          r.pre = t.pre;
          r.inst = (uint32_t)i;
          subs.push_back(r);
        }
      }
      rc = ensure(s, &s->d_subs, &s->subs_cap, std::max<size_t>(subs.size(), 1));
      if (rc) return rc;
      if (!subs.empty()) {
        SP_CUDA(s, cudaMemcpyAsync(s->d_subs, subs.data(), subs.size() * sizeof(SubRoot),
                                   cudaMemcpyHostToDevice, s->st));
        s->stats.h2d_bytes += subs.size() * sizeof(SubRoot);
      }
      if (s->d_sub_nodes) cudaFree(s->d_sub_nodes);
      s->d_sub_nodes = nullptr;
      SP_CUDA(s, cudaMalloc(&s->d_sub_nodes, std::max<size_t>(subs.size(), 1) * sizeof(unsigned long long)));
      subs_dirty = false;
    }
    // per instance: interior counts, host-side goals, active roots
    std::vector<uint64_t> interior(inst.size(), 0);
    std::vector<int32_t> host_goal(inst.size(), -1);
    for (size_t i = 0; i < inst.size(); ++i) {
      Instance &I = inst[i];
      if (I.done) continue;
      const int L = I.h0 + 2 * I.iter;
      limits[i] = L;
      for (size_t j = 0; j < I.tree.size(); ++j) {
        const TreeNode &t = I.tree[j];
        if (t.maxf > L) continue;
        if (t.h == 0 && (host_goal[i] < 0 || t.g < I.tree[(size_t)host_goal[i]].g)) host_goal[i] = (int32_t)j;
        if (!t.leaf) interior[i] += t.nchild;
      }
    }
    RoundPlan plan;
    plan_static(s, inst, limits, plan);
    const size_t n_tasks = plan.direct.size() + plan.split.size();
    if (inst.size() > s->inst_cap || !s->d_limit) {
      if (s->d_limit) cudaFree(s->d_limit);
      if (s->d_sol) cudaFree(s->d_sol);
      s->d_limit = nullptr;
      s->d_sol = nullptr;
      size_t c = std::max<size_t>(inst.size(), 64);
      SP_CUDA(s, cudaMalloc(&s->d_limit, c * sizeof(int32_t)));
      SP_CUDA(s, cudaMalloc(&s->d_sol, c * sizeof(Solution)));
      s->inst_cap = c;
    }
    SP_CUDA(s, cudaMemcpyAsync(s->d_limit, limits.data(), inst.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s->st));
    SP_CUDA(s, cudaMemsetAsync(s->d_sol, 0, inst.size() * sizeof(Solution), s->st));
    SP_CUDA(s, cudaMemsetAsync(s->d_sub_nodes, 0, std::max<size_t>(subs.size(), 1) * sizeof(unsigned long long), s->st));
    s->stats.h2d_bytes += inst.size() * sizeof(int32_t);
    float ms = 0;
    if (n_tasks) {
      uint32_t split_err = 0;
      rc = launch_round(s, plan, &ms, &split_err);
      if (rc) return rc;
      s->stats.kernel_ms += ms;
      s->stats.tasks_initial += plan.direct.size() + s->last_emitted;
      PoolCtl ctl{};
      SP_CUDA(s, cudaMemcpyAsync(&ctl, s->d_ctl, sizeof(PoolCtl), cudaMemcpyDeviceToHost, s->st));
      sub_nodes.assign(subs.size(), 0);
      SP_CUDA(s, cudaMemcpyAsync(sub_nodes.data(), s->d_sub_nodes, subs.size() * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, s->st));
      SP_CUDA(s, cudaMemcpyAsync(sols.data(), s->d_sol, inst.size() * sizeof(Solution), cudaMemcpyDeviceToHost, s->st));
      SP_CUDA(s, cudaStreamSynchronize(s->st));
      s->stats.d2h_bytes += sizeof(PoolCtl) + subs.size() * 8 + inst.size() * sizeof(Solution);
      s->stats.tasks_donated += ctl.donated;
      s->stats.dev_lane_steps += ctl.counters[0];
      s->stats.dev_lane_slots += ctl.counters[1];
      s->stats.dev_idle_cycles += ctl.counters[2];
      s->stats.dev_warp_cycles += ctl.counters[3];
      s->stats.dev_donate_tries += ctl.counters[4];
      s->stats.dev_donate_notfree += ctl.counters[5];
      s->stats.dev_donate_nowait += ctl.counters[6];
      s->stats.dev_tasks_done += ctl.counters[7];
      s->stats.round_tasks[ri] = (int32_t)(plan.direct.size() + s->last_emitted);
      s->stats.round_kernel_ms[ri] = ms;
      s->stats.round_donated[ri] = ctl.donated;
      if (!ctl.error && split_err) ctl.error = (int32_t)split_err;
      if (ctl.error) {
        char buf[160];
        snprintf(buf, sizeof buf, "device error %d (info %u) in round %d", ctl.error, ctl.err_info[0], round);
        s->err = buf;
        for (auto &I : inst)
          if (!I.done) { I.out->status = ctl.error; I.done = true; }
        return ctl.error;
      }
    } else {
      sub_nodes.assign(subs.size(), 0);
      memset(sols.data(), 0, sols.size() * sizeof(Solution));
    }
    ++s->stats.rounds;
    // fold results
    for (size_t i = 0; i < inst.size(); ++i) {
      Instance &I = inst[i];
      if (I.done) continue;
      uint64_t nodes = interior[i], dev = 0;
      for (size_t q = 0; q < I.leaves.size(); ++q) {
        const uint64_t v = sub_nodes[(size_t)I.tree[(size_t)I.leaves[q]].sub];
        dev += v;
        I.last_load[q] = v;
      }
      nodes += dev;
      I.prev_total = I.last_total;
      I.last_total = dev;
      sp_result *R = I.out;
      R->f_limit[I.iter] = limits[i];
      R->nodes[I.iter] = nodes;
      R->nodes_total += nodes;
      R->n_iter = I.iter + 1;
      s->stats.nodes += nodes;
      s->stats.round_nodes[ri] += nodes;
      const bool dev_goal = sols[i].flag != 0;
      if (host_goal[i] >= 0 || dev_goal) {
        // path: root-set tree prefix, then the device's moves below its root
        std::vector<uint8_t> mv;
        int node = host_goal[i];
        uint32_t extra = 0;
        const uint32_t *pw = nullptr;
        if (node < 0) {
          const uint32_t sub = sols[i].sub;
          for (int32_t x : I.leaves)
            if (I.tree[(size_t)x].sub == (int32_t)sub) node = x;
          extra = sols[i].len;
          pw = sols[i].path;
        }
        for (int x = node; x > 0; x = I.tree[(size_t)x].parent) mv.push_back(I.tree[(size_t)x].move);
        std::reverse(mv.begin(), mv.end());
        for (uint32_t j = 0; j < extra; ++j) mv.push_back((uint8_t)((pw[j >> 4] >> (2 * (j & 15))) & 3u));
        R->len = (int32_t)mv.size();
        if (mv.size() > SP_MAX_MOVES) {
          R->status = SP_ERR_PATH;
        } else {
          R->n_moves = R->len;
          memcpy(R->moves, mv.data(), mv.size());
          R->status = replay_ok(w, tiles + i * (size_t)n, R->moves, R->n_moves) ? SP_OK : SP_ERR_PATH;
        }
        I.done = true;
        continue;
      }
      ++I.iter;
      if (I.iter >= SP_MAX_ITERS) {
        R->status = SP_ERR_LIMIT;
        I.done = true;
      }
    }
    s->stats.round_host_ms[ri] = (float)(ms_since(t_round) - s->stats.round_kernel_ms[ri]);
  }
  const double wall = ms_since(t_start);
  for (auto &I : inst) {
    I.out->seconds = wall / 1000.0;
    if (!I.done && I.out->status == SP_OK) I.out->status = SP_ERR_LIMIT;
  }
  s->stats.wall_ms = wall;
  return SP_OK;
}

bool config_ok(const sp_config *c) {
  return (c->threads_per_block == 128 || c->threads_per_block == 256) && c->frontier_target >= 1 &&
         c->frontier_target <= (1 << 20) && c->blocks_per_sm >= 0 && c->blocks_per_sm <= 16 &&
         c->lb_mode >= SP_LB_STEAL && c->lb_mode <= SP_LB_NONE && c->donate_min_slack >= 0 &&
         c->steps_per_poll >= 1 && c->steps_per_poll <= 4096 && c->timeout_ms >= 100 &&
         c->timeout_ms <= 600000 && c->static_split_cap >= 1;
}

}  // namespace

extern "C" {

void sp_config_default(sp_config *c) {
  if (!c) return;
  c->frontier_target = 2048;
  c->threads_per_block = 256;
  c->blocks_per_sm = 0;
  c->lb_mode = SP_LB_STEAL;
  c->donate_min_slack = 6;
  c->steps_per_poll = 32;
  c->timeout_ms = 20000;
  c->static_split_cap = 64;
}

int sp_create(int width, int heuristic, const sp_config *cfg, sp_solver **out) {
  if (!out || (width != 4 && width != 5) || (heuristic != SP_HEUR_MANHATTAN && heuristic != SP_HEUR_PDB))
    return SP_ERR_ARG;
  *out = nullptr;
  if (cfg && !config_ok(cfg)) return SP_ERR_ARG;
  std::unique_ptr<sp_solver> s(new sp_solver());
  s->w = width;
  s->n = width * width;
  s->heur = heuristic;
  sp_config_default(&s->cfg);
  if (cfg) s->cfg = *cfg;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_ht, sizeof(HeurTables));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_ctl, sizeof(PoolCtl));
  if (e == cudaSuccess) {
    build_heur_tables(width, &s->h_ht);
    e = cudaMemcpy(s->d_ht, &s->h_ht, sizeof(HeurTables), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess && heuristic == SP_HEUR_PDB) {
    const size_t bytes = (size_t)pattern_set(width).n_tables * lookup_table_stride(width);
    e = cudaMalloc(&s->d_pdb, bytes);
  }
  if (e != cudaSuccess) {
    sp_solver *raw = s.release();
    raw->err = cudaGetErrorString(e);
    sp_destroy(raw);
    return SP_ERR_CUDA;
  }
  *out = s.release();
  return SP_OK;
}

void sp_destroy(sp_solver *s) {
  if (!s) return;
  cudaFree(s->d_ht);
  cudaFree(s->d_pdb);
  cudaFree(s->d_tasks);
  cudaFree(s->d_seq);
  cudaFree(s->d_ctl);
  cudaFree(s->d_subs);
  cudaFree(s->d_init);
  cudaFree(s->d_sub_nodes);
  cudaFree(s->d_limit);
  cudaFree(s->d_sol);
  cudaFree(s->d_boards);
  cudaFree(s->d_h);
  cudaFree(s->d_cnt);
  cudaFree(s->d_split_a);
  cudaFree(s->d_split_b);
  cudaFree(s->d_emit);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

int sp_set_config(sp_solver *s, const sp_config *cfg) {
  if (!s || !cfg || !config_ok(cfg)) return SP_ERR_ARG;
  s->cfg = *cfg;
  return SP_OK;
}

uint64_t sp_pdb_table_size(int width) {
  if (width != 4 && width != 5) return 0;
  return compact_table_size(width);
}

int sp_pdb_num_tables(int width) {
  if (width != 4 && width != 5) return 0;
  return pattern_set(width).n_tables;
}

int sp_pdb_build(sp_solver *s) {
  if (!s) return SP_ERR_ARG;
  if (s->heur != SP_HEUR_PDB) return SP_ERR_ARG;
  const int nt = pattern_set(s->w).n_tables;
  double total = 0;
  for (int t = 0; t < nt; ++t) {
    int levels = 0;
    double ms = 0;
    cudaError_t e = build_pdb_table(s->w, t, s->d_pdb + (size_t)t * lookup_table_stride(s->w), nullptr,
                                    s->st, &levels, &ms);
    if (e != cudaSuccess) return fail_cuda(s, e, "build_pdb_table");
    total += ms;
  }
  s->pdb_build_ms = total;
  s->pdb_ready = true;
  return SP_OK;
}

int sp_pdb_export(sp_solver *s, int table, uint8_t *dst, uint64_t size) {
  if (!s || !dst || s->heur != SP_HEUR_PDB) return SP_ERR_ARG;
  if (table < 0 || table >= pattern_set(s->w).n_tables || size != compact_table_size(s->w)) return SP_ERR_ARG;
  if (!s->pdb_ready) return SP_ERR_NO_PDB;
  uint8_t *tmp = nullptr;
  SP_CUDA(s, cudaMalloc(&tmp, size));
  cudaError_t e = pdb_lookup_to_compact(s->w, table, s->d_pdb + (size_t)table * lookup_table_stride(s->w), tmp, s->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, tmp, size, cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail_cuda(s, e, "sp_pdb_export");
  return SP_OK;
}

int sp_pdb_import(sp_solver *s, int table, const uint8_t *src, uint64_t size) {
  if (!s || !src || s->heur != SP_HEUR_PDB) return SP_ERR_ARG;
  const int nt = pattern_set(s->w).n_tables;
  if (table < 0 || table >= nt || size != compact_table_size(s->w)) return SP_ERR_ARG;
  uint8_t *tmp = nullptr;
  SP_CUDA(s, cudaMalloc(&tmp, size));
  cudaError_t e = cudaMemcpyAsync(tmp, src, size, cudaMemcpyHostToDevice, s->st);
  if (e == cudaSuccess)
    e = pdb_compact_to_lookup(s->w, table, tmp, s->d_pdb + (size_t)table * lookup_table_stride(s->w), s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail_cuda(s, e, "sp_pdb_import");
  // tables become usable once every table has been imported or built
  s->import_mask |= 1u << table;
  if ((s->import_mask & ((1u << nt) - 1u)) == ((1u << nt) - 1u)) s->pdb_ready = true;
  return SP_OK;
}

int sp_heuristic(sp_solver *s, const uint8_t *tiles, int n, int32_t *h) {
  if (!s || (n > 0 && (!tiles || !h)) || n < 0) return SP_ERR_ARG;
  if (s->heur == SP_HEUR_PDB && !s->pdb_ready) return SP_ERR_NO_PDB;
  if (n == 0) return SP_OK;
  for (int i = 0; i < n; ++i) {
    int st = check_instance(s->w, tiles + (size_t)i * s->n);
    if (st == SP_ERR_NOT_PERMUTATION) return st;
  }
  int rc = ensure(s, &s->d_boards, &s->boards_cap, (size_t)n * s->n);
  if (rc) return rc;
  int32_t *dh = nullptr;
  SP_CUDA(s, cudaMalloc(&dh, (size_t)n * sizeof(int32_t)));
  cudaError_t e = cudaMemcpyAsync(s->d_boards, tiles, (size_t)n * s->n, cudaMemcpyHostToDevice, s->st);
  if (e == cudaSuccess) e = launch_heuristic(s->w, s->heur == SP_HEUR_PDB, s->d_boards, n, dh, s->d_ht, s->d_pdb, s->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, dh, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  cudaFree(dh);
  if (e != cudaSuccess) return fail_cuda(s, e, "sp_heuristic");
  return SP_OK;
}

int sp_solve_batch(sp_solver *s, const uint8_t *tiles, int n, sp_result *results) {
  if (!s || n < 0 || (n > 0 && (!tiles || !results))) return SP_ERR_ARG;
  if (n == 0) return SP_OK;
  return solve_impl(s, tiles, n, results);
}

int sp_solve_batch_device(sp_solver *s, const void *d_tiles, int n, sp_result *results) {
  if (!s || n < 0 || (n > 0 && (!d_tiles || !results))) return SP_ERR_ARG;
  if (n == 0) return SP_OK;
  std::vector<uint8_t> h((size_t)n * s->n);
  SP_CUDA(s, cudaMemcpyAsync(h.data(), d_tiles, h.size(), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  int rc = solve_impl(s, h.data(), n, results);
  s->stats.d2h_bytes += h.size();
  return rc;
}

int sp_dfs_round(sp_solver *s, const uint8_t *roots, const int32_t *depth, const int32_t *pre, int n,
                 int limit, uint64_t *nodes, int32_t *found) {
  if (!s || n < 0 || (n > 0 && (!roots || !depth || !pre || !nodes)) || !found) return SP_ERR_ARG;
  if (s->heur == SP_HEUR_PDB && !s->pdb_ready) return SP_ERR_NO_PDB;
  memset(&s->stats, 0, sizeof(s->stats));
  *found = -1;
  if (n == 0) return SP_OK;
  std::vector<SubRoot> subs((size_t)n);
  std::vector<Task> init((size_t)n);
  for (int i = 0; i < n; ++i) {
    const uint8_t *t = roots + (size_t)i * s->n;
    if (check_instance(s->w, t) == SP_ERR_NOT_PERMUTATION) return SP_ERR_NOT_PERMUTATION;
    if (depth[i] < 0 || depth[i] > 255 || pre[i] < -1 || pre[i] > 3) return SP_ERR_ARG;
    SubRoot r{};
    memcpy(r.board, t, (size_t)s->n);
    for (int c = 0; c < s->n; ++c)
      if (!t[c]) r.blank = (uint8_t)c;
    r.g = (uint8_t)depth[i];
    r.pre = pre[i] < 0 ? kNoPre : (uint8_t)pre[i];
    r.inst = 0;
    subs[(size_t)i] = r;
    init[(size_t)i].sub = (uint32_t)i;
    init[(size_t)i].plen = 0;
    init[(size_t)i].mask = 0xF;
  }
  // roots that are goals within the limit (the reference's dfs_kernel sets
  // dev_flag for them, :580-583)
  std::vector<int32_t> h((size_t)n);
  int rc = sp_heuristic(s, roots, n, h.data());
  if (rc) return rc;
  for (int i = 0; i < n; ++i)
    if (h[(size_t)i] == 0 && (*found < 0 || depth[i] < *found)) *found = depth[i];
  rc = ensure(s, &s->d_subs, &s->subs_cap, (size_t)n);
  if (rc) return rc;
  if (!s->d_limit || s->inst_cap < 1) {
    SP_CUDA(s, cudaMalloc(&s->d_limit, 64 * sizeof(int32_t)));
    SP_CUDA(s, cudaMalloc(&s->d_sol, 64 * sizeof(Solution)));
    s->inst_cap = 64;
  }
  if (s->d_sub_nodes) cudaFree(s->d_sub_nodes);
  s->d_sub_nodes = nullptr;
  SP_CUDA(s, cudaMalloc(&s->d_sub_nodes, (size_t)n * sizeof(unsigned long long)));
  SP_CUDA(s, cudaMemcpyAsync(s->d_subs, subs.data(), subs.size() * sizeof(SubRoot), cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemcpyAsync(s->d_limit, &limit, sizeof(int32_t), cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemsetAsync(s->d_sol, 0, sizeof(Solution), s->st));
  SP_CUDA(s, cudaMemsetAsync(s->d_sub_nodes, 0, (size_t)n * sizeof(unsigned long long), s->st));
  float ms = 0;
  RoundPlan plan;
  plan.direct = std::move(init);
  uint32_t split_err = 0;
  rc = launch_round(s, plan, &ms, &split_err);
  if (rc) return rc;
  PoolCtl ctl{};
  Solution sol{};
  SP_CUDA(s, cudaMemcpyAsync(&ctl, s->d_ctl, sizeof(PoolCtl), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(&sol, s->d_sol, sizeof(Solution), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(nodes, s->d_sub_nodes, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  s->stats.kernel_ms = ms;
  s->stats.rounds = 1;
  s->stats.tasks_initial = (uint64_t)n;
  s->stats.tasks_donated = ctl.donated;
  s->stats.dev_lane_steps = ctl.counters[0];
  s->stats.dev_lane_slots = ctl.counters[1];
  s->stats.dev_idle_cycles = ctl.counters[2];
  s->stats.dev_warp_cycles = ctl.counters[3];
  s->stats.dev_donate_tries = ctl.counters[4];
  s->stats.dev_donate_notfree = ctl.counters[5];
  s->stats.dev_donate_nowait = ctl.counters[6];
  s->stats.dev_tasks_done = ctl.counters[7];
  s->stats.round_tasks[0] = n;
  s->stats.round_kernel_ms[0] = ms;
  s->stats.round_donated[0] = ctl.donated;
  if (ctl.error) {
    char buf[320];
    snprintf(buf, sizeof buf,
             "device error %d (info %u) in sp_dfs_round: donated %llu tries %llu notfree %llu hungry-polls %llu "
             "donor-found %llu done %llu",
             ctl.error, ctl.err_info[0], (unsigned long long)ctl.donated, (unsigned long long)ctl.counters[4],
             (unsigned long long)ctl.counters[5], (unsigned long long)ctl.counters[6],
             (unsigned long long)ctl.counters[8], (unsigned long long)ctl.counters[7]);
    s->err = buf;
    return ctl.error;
  }
  if (sol.flag) {
    const int d = (int)subs[sol.sub].g + (int)sol.len;
    if (*found < 0 || d < *found) *found = d;
  }
  for (int i = 0; i < n; ++i) s->stats.nodes += nodes[i];
  return SP_OK;
}

int sp_last_stats(const sp_solver *s, sp_stats *out) {
  if (!s || !out) return SP_ERR_ARG;
  *out = s->stats;
  return SP_OK;
}

const char *sp_status_string(int st) {
  switch (st) {
    case SP_OK: return "ok";
    case SP_ERR_ARG: return "invalid argument";
    case SP_ERR_NOT_PERMUTATION: return "tiles are not a permutation";
    case SP_ERR_UNSOLVABLE: return "instance is unsolvable";
    case SP_ERR_LIMIT: return "no solution within the threshold cap";
    case SP_ERR_CUDA: return "CUDA error";
    case SP_ERR_NO_PDB: return "pattern databases not built";
    case SP_ERR_STACK_OVERFLOW: return "search deeper than the per-lane stack";
    case SP_ERR_TIMEOUT: return "device wait timed out";
    case SP_ERR_CAPACITY: return "capacity exceeded";
    case SP_ERR_PATH: return "solution path invalid or too long";
  }
  return "unknown status";
}

const char *sp_last_error(const sp_solver *s) { return s ? s->err.c_str() : "null solver"; }

uint64_t sp_kernel_launch_count(void) { return g_launches.load(); }

}  // extern "C"
