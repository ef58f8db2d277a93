// Host side of libslide: the C ABI (include/slide.h), the root-set
// ("frontier") templates, the IDA* threshold-round loop and static load
// balancing.  Device work is in search.cu, frontier.cu (the root sets
// themselves), pdb_build.cu and mlp.cu.
//
// A batch is solved in two phases by default: one persistent launch runs
// every instance's small iterations on the device (solve_multi); an instance
// whose next iteration is predicted large is handed back, with the per-root
// loads the device measured, to the round loop (solve_impl), which plans
// each round's static split on host worker threads (WorkPool) and launches
// the split pre-pass and the search.  `persistent = 0` runs only the round
// loop, `handback_nodes = 0` only the persistent launch.
//
// Reference counterparts:
//   create_root_set       src/24puzzle_block_parallel_with_pdb.cu:454-490
//   ida_star round loop   src/24puzzle_block_parallel_with_pdb.cu:756-922
//   static re-split       src/24puzzle_block_parallel_with_pdb.cu:839-897
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
//   * heavy roots are split by the device pre-pass (search.cu), which counts
//     the nodes it expands like the search would.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/slide.h"
#include "lbm.h"
#include "sp_defs.h"
#include "sp_kernels.h"

// Static split: a round's predicted work is cut into about this many pieces
// per resident lane (the piece size T of plan_round).  Measured: 1 beats 4,
// 16 and 64 (each piece costs a pre-pass expansion and a task start, and
// donation evens out the rest) and 0.5 or less (more donations).
#ifndef SP_SPLIT_PIECES_PER_LANE
#define SP_SPLIT_PIECES_PER_LANE 1.0
#endif

// Device loop: an instance's next two iterations run together (the instance
// advances once both are done) when the second is predicted below this many
// generated nodes -- in the hybrid loop, for batches of at most one instance
// per SP_PAIR_LANES resident lanes, where a chain of small iterations per
// instance leaves the GPU underused (measured: yama24_50_hard_new -5 %,
// the 15-puzzle batches of 100 -1 to -2 %; a 4096-instance batch, which
// fills the GPU anyway, +1.8 %, and the pure device loop much slower).
#ifndef SP_PAIR_NODES
#define SP_PAIR_NODES 300000
#endif
#ifndef SP_PAIR_LANES
#define SP_PAIR_LANES 256
#endif

// Shortest interval between two reads of the pool's control words by one
// block (ns); the block shares what it read.
#ifndef SP_POLL_NS
#define SP_POLL_NS 2000
#endif

namespace sp {

// Learned balancer: slacks above this are predicted as this one (the model
// is trained on slacks 0..7), and a root's predicted growth per threshold
// step is capped at 2^kLbmMaxStep.
constexpr int kLbmMaxSlack = 7;
constexpr double kLbmMaxStep = 6.0;

static std::atomic<uint64_t> g_launches{0};
void note_launch(int n) { g_launches.fetch_add((uint64_t)n); }

namespace {

// Root-set template of one blank cell: the tree expanded to a uniform depth
// D (every node of depth < D expanded, children in move order, no reverse
// moves), in breadth-first order.  Nodes are move sequences from the root;
// the device applies them to each instance's board (frontier.cu).
struct FrontTemplate {
  bool built = false;
  uint32_t D = 0;
  uint32_t node_off = 0;          // first node in the device template arrays
  std::vector<uint64_t> path;     // 2 bits per move, first move lowest
  std::vector<int32_t> parent;
  std::vector<uint8_t> nchild, depth;
  std::vector<uint32_t> lev;      // level d: nodes [lev[d], lev[d + 1])
};

struct Instance {
  int status = SP_OK;
  int h0 = 0;
  int iter = 0;
  bool done = false;
  // root set: the template of the instance's blank cell; its leaves are the
  // SubRoots [sub_base, sub_base + n_leaves), sorted by maxf (the prefix
  // maximum of g + h along the path), so a round's active roots are a prefix
  const FrontTemplate *tmpl = nullptr;
  uint32_t n_leaves = 0;
  std::vector<uint32_t> leaf_cum;    // [b]: leaves with maxf <= h0 + b
  std::vector<uint32_t> goal_key;    // [b]: min (depth << 24 | node) of goal nodes with maxf == h0 + b
  std::vector<std::pair<int32_t, uint64_t>> interior;  // (maxf, cumulative children), ascending
  std::vector<uint64_t> last_load;   // per leaf, previous round
  uint64_t last_total = 0, prev_total = 0;
  uint32_t sub_base = 0;             // SubRoot index of the first leaf
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

// Grow-only pinned host buffer.
template <typename T>
struct Pinned {
  T *p = nullptr;
  size_t cap = 0;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t reserve(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t c = std::max<size_t>({n, (size_t)1024, cap + cap / 2});  // geometric: pinned allocation is slow
    cudaError_t e = cudaMallocHost((void **)&p, c * sizeof(T));
    if (e == cudaSuccess) cap = c;
    return e;
  }
};

// Device tables of the multi-iteration mode (grow-only).
struct MultiBufs {
  int32_t *iter = nullptr, *fin = nullptr, *status = nullptr, *goal = nullptr, *ifv = nullptr;
  uint32_t *out = nullptr, *base = nullptr, *nsub = nullptr, *ioff = nullptr, *ilen = nullptr, *pair = nullptr;
  unsigned long long *icum = nullptr, *iter_nodes = nullptr, *loads = nullptr, *fin_ns = nullptr, *t0_ns = nullptr;
  uint8_t *growth = nullptr;  // learned balancer: [n_subs][kGrowthSlacks] growth codes
  size_t cap_iter = 0, cap_fin = 0, cap_status = 0, cap_goal = 0, cap_ifv = 0, cap_out = 0,
         cap_base = 0, cap_nsub = 0, cap_ioff = 0, cap_ilen = 0, cap_icum = 0, cap_iter_nodes = 0, cap_loads = 0, cap_pair = 0,
         cap_fin_ns = 0, cap_t0_ns = 0, cap_growth = 0;
  bool use_growth = false;  // the current launch has growth codes
  void release() {
    void *ptrs[] = {iter, fin,  status, goal, ifv,        out,   base,   nsub, pair,
                    ioff, ilen, icum,   iter_nodes, loads, fin_ns, t0_ns, growth};
    for (void *p : ptrs) cudaFree(p);
  }
};

// Device root set: the templates of the current target (one per blank cell,
// built on first use) and the per-batch outputs of frontier.cu.
struct FrontBufs {
  int target = -1;
  FrontTemplate t[kMaxN];
  bool dirty = false;  // a template was built since the last upload
  FrontTmpl *tmpl = nullptr;
  uint32_t *lev = nullptr;
  uint64_t *path = nullptr;
  int32_t *parent = nullptr;
  uint8_t *nchild = nullptr, *depth = nullptr;
  size_t cap_tmpl = 0, cap_lev = 0, cap_path = 0, cap_parent = 0, cap_nchild = 0, cap_depth = 0;
  uint8_t *in = nullptr;  // tiles, then the four per-block arrays
  int16_t *f = nullptr, *maxf = nullptr;
  int32_t *leaf_maxf = nullptr, *leaf_node = nullptr, *error = nullptr;
  uint8_t *leaf_h = nullptr;
  FrontInst *out = nullptr;
  size_t cap_in = 0, cap_f = 0, cap_maxf = 0, cap_leaf_maxf = 0, cap_leaf_node = 0, cap_error = 0, cap_leaf_h = 0,
         cap_out = 0;
  Pinned<uint8_t> h_in;
  Pinned<FrontInst> h_out;
  Pinned<int32_t> h_leaf_node;  // template node of each SubRoot
  Pinned<uint8_t> h_leaf_h;     // h of each SubRoot (learned balancer)
  Pinned<int32_t> h_error;
  void release() {
    void *ptrs[] = {tmpl, lev, path, parent, nchild, depth, in, f, maxf, leaf_maxf, leaf_node, error, leaf_h, out};
    for (void *p : ptrs) cudaFree(p);
  }
};

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
  // per-batch buffers
  SubRoot *d_subs = nullptr;
  size_t subs_cap = 0;
  uint32_t *d_direct = nullptr;
  size_t direct_cap = 0;
  unsigned long long *d_sub_nodes = nullptr;
  size_t sub_nodes_cap = 0;
  int32_t *d_limit = nullptr;
  Solution *d_sol = nullptr;
  size_t inst_cap = 0;
  uint8_t *d_boards = nullptr;  // sp_heuristic
  int32_t *d_h = nullptr;
  size_t boards_cap = 0, h_cap = 0;
  // pinned staging
  Pinned<uint32_t> h_direct;
  Pinned<Task> h_split;
  Pinned<unsigned long long> h_sub_nodes;
  Pinned<Solution> h_sols;
  Pinned<PoolCtl> h_ctl;
  Pinned<int32_t> h_limits;
  Pinned<uint32_t> h_cnt;
  Pinned<uint8_t> h_stage_up, h_stage_dn;  // solve_multi's tables and results
  Pinned<unsigned long long> h_loads;
  MultiBufs mb;
  FrontBufs fb;
  std::unique_ptr<lbm::Model> lbm;  // learned load balancer (SP_LB_LEARNED)
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

// Host worker threads, created once and kept for the process (never joined:
// a library must not block at exit on its own threads).  run(n, fn) calls
// fn(i) for i in [0, n) on the workers and the caller; one run at a time.
class WorkPool {
 public:
  static WorkPool &get() {
    static WorkPool *pool = new WorkPool(std::max(1u, std::min(16u, std::thread::hardware_concurrency())) - 1);
    return *pool;
  }
  // 0 in a forked child: it inherits this object but none of the threads
  unsigned workers() const { return getpid() == pid_ ? (unsigned)threads_.size() : 0u; }
  void run(size_t n, const std::function<void(size_t)> &fn) {
    std::lock_guard<std::mutex> one(run_m_);
    {
      std::lock_guard<std::mutex> l(m_);
      job_ = &fn;
      n_ = n;
      next_.store(0);
      active_ = (int)threads_.size();
      ++gen_;
    }
    cv_.notify_all();
    for (size_t i; (i = next_.fetch_add(1)) < n;) fn(i);
    std::unique_lock<std::mutex> l(m_);
    done_cv_.wait(l, [&] { return active_ == 0; });
  }

 private:
  explicit WorkPool(unsigned k) : pid_(getpid()) {
    for (unsigned t = 0; t < k; ++t) threads_.emplace_back([this] { loop(); });
    for (auto &t : threads_) t.detach();
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(size_t)> *job;
      size_t n;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return gen_ != seen; });
        seen = gen_;
        job = job_;
        n = n_;
      }
      for (size_t i; (i = next_.fetch_add(1)) < n;) (*job)(i);
      std::lock_guard<std::mutex> l(m_);
      if (--active_ == 0) done_cv_.notify_one();
    }
  }
  pid_t pid_;
  std::vector<std::thread> threads_;
  std::mutex run_m_, m_;
  std::condition_variable cv_, done_cv_;
  uint64_t gen_ = 0;
  size_t n_ = 0;
  std::atomic<size_t> next_{0};
  int active_ = 0;
  const std::function<void(size_t)> *job_ = nullptr;
};

// fn(i) for i in [0, n) on the host worker pool (instances are independent);
// small n, or little total work (`work` elements: waking the workers costs
// tens of microseconds), runs inline
constexpr size_t kInlineWork = 16384;
template <typename F>
void parallel_for(size_t n, F fn, size_t work = ~(size_t)0) {
  if (n < 8 || work < kInlineWork || WorkPool::get().workers() == 0) {
    for (size_t i = 0; i < n; ++i) fn(i);
    return;
  }
  const std::function<void(size_t)> f = fn;
  WorkPool::get().run(n, f);
}

// The template of blank cell `blank`: levels expanded while the last level
// holds fewer than `target` nodes.  Returns false if that needs more than
// kFrontMaxDepth levels (never for targets up to 2^20).
bool build_template(int w, int blank, int target, FrontTemplate &T) {
  T = FrontTemplate{};
  std::vector<uint8_t> cell{(uint8_t)blank}, pre{kNoPre};
  T.path.push_back(0);
  T.parent.push_back(-1);
  T.depth.push_back(0);
  T.lev.assign(kFrontLevStride, 0);
  uint32_t lo = 0, hi = 1, D = 0;
  while (hi - lo < (uint32_t)target) {
    if (D >= (uint32_t)kFrontMaxDepth) return false;
    for (uint32_t x = lo; x < hi; ++x) {
      uint32_t mv = legal_moves(w, cell[x]);
      if (pre[x] != kNoPre) mv &= ~(1u << (3 - pre[x]));
      for (int d = 0; d < 4; ++d) {
        if (!((mv >> d) & 1u)) continue;
        T.path.push_back(T.path[x] | ((uint64_t)d << (2 * D)));
        T.parent.push_back((int32_t)x);
        T.depth.push_back((uint8_t)(D + 1));
        cell.push_back((uint8_t)(cell[x] + move_delta(w, d)));
        pre.push_back((uint8_t)d);
      }
    }
    lo = hi;
    hi = (uint32_t)T.path.size();
    T.lev[++D] = lo;
  }
  T.lev[D + 1] = hi;
  T.D = D;
  T.nchild.resize(hi);
  for (uint32_t x = 0; x < hi; ++x) {
    uint32_t mv = legal_moves(w, cell[x]);
    if (pre[x] != kNoPre) mv &= ~(1u << (3 - pre[x]));
    T.nchild[x] = x < lo ? (uint8_t)__builtin_popcount(mv) : 0;
  }
  T.built = true;
  return hi < (1u << 24);  // node ids fit the goal keys
}

// Root sets of every live instance, built on the device (frontier.cu):
// templates for this target (built once per blank cell and uploaded when new),
// one upload of the tiles and the per-instance offsets, one launch, and the
// per-instance summaries back.  Sets h0, the leaf counts, interior counts and
// goals of each instance and returns the number of SubRoots.
int build_root_sets(sp_solver *s, const uint8_t *tiles, std::vector<Instance> &inst, int target,
                    size_t *n_subs_out) {
  FrontBufs &fb = s->fb;
  const int w = s->w, n = s->n;
  if (fb.target != target) {
    for (auto &t : fb.t) t = FrontTemplate{};
    fb.target = target;
    fb.dirty = true;
  }
  std::vector<uint32_t> live;
  for (size_t i = 0; i < inst.size(); ++i) {
    Instance &I = inst[i];
    if (I.done) continue;
    int blank = 0;
    for (int c = 0; c < n; ++c)
      if (!tiles[i * (size_t)n + c]) blank = c;
    FrontTemplate &T = fb.t[blank];
    if (!T.built) {
      if (!build_template(w, blank, target, T)) {
        s->err = "root-set template too deep or too large";
        return SP_ERR_CAPACITY;
      }
      fb.dirty = true;
    }
    I.tmpl = &T;
    live.push_back((uint32_t)i);
  }
  int rc = SP_OK;
  if (fb.dirty) {  // all built templates, concatenated
    size_t nodes = 0;
    for (auto &t : fb.t)
      if (t.built) t.node_off = (uint32_t)nodes, nodes += t.path.size();
    if ((rc = ensure(s, &fb.tmpl, &fb.cap_tmpl, (size_t)kMaxN)) ||
        (rc = ensure(s, &fb.lev, &fb.cap_lev, (size_t)kMaxN * kFrontLevStride)) ||
        (rc = ensure(s, &fb.path, &fb.cap_path, nodes)) || (rc = ensure(s, &fb.parent, &fb.cap_parent, nodes)) ||
        (rc = ensure(s, &fb.nchild, &fb.cap_nchild, nodes)) || (rc = ensure(s, &fb.depth, &fb.cap_depth, nodes)))
      return rc;
    std::vector<FrontTmpl> desc(kMaxN, FrontTmpl{});
    std::vector<uint32_t> lev((size_t)kMaxN * kFrontLevStride, 0);
    std::vector<uint64_t> path(nodes);
    std::vector<int32_t> parent(nodes);
    std::vector<uint8_t> nchild(nodes), depth(nodes);
    for (int b = 0; b < kMaxN; ++b) {
      const FrontTemplate &t = fb.t[b];
      if (!t.built) continue;
      desc[b] = FrontTmpl{t.node_off, (uint32_t)t.path.size(), t.D, 0};
      std::copy(t.lev.begin(), t.lev.end(), lev.begin() + (size_t)b * kFrontLevStride);
      std::copy(t.path.begin(), t.path.end(), path.begin() + t.node_off);
      std::copy(t.parent.begin(), t.parent.end(), parent.begin() + t.node_off);
      std::copy(t.nchild.begin(), t.nchild.end(), nchild.begin() + t.node_off);
      std::copy(t.depth.begin(), t.depth.end(), depth.begin() + t.node_off);
    }
    SP_CUDA(s, cudaMemcpy(fb.tmpl, desc.data(), desc.size() * sizeof(FrontTmpl), cudaMemcpyHostToDevice));
    SP_CUDA(s, cudaMemcpy(fb.lev, lev.data(), lev.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    SP_CUDA(s, cudaMemcpy(fb.path, path.data(), nodes * sizeof(uint64_t), cudaMemcpyHostToDevice));
    SP_CUDA(s, cudaMemcpy(fb.parent, parent.data(), nodes * sizeof(int32_t), cudaMemcpyHostToDevice));
    SP_CUDA(s, cudaMemcpy(fb.nchild, nchild.data(), nodes, cudaMemcpyHostToDevice));
    SP_CUDA(s, cudaMemcpy(fb.depth, depth.data(), nodes, cudaMemcpyHostToDevice));
    fb.dirty = false;
  }
  // per live instance: template, first SubRoot, first scratch node
  const size_t nl = live.size();
  size_t n_subs = 0, n_nodes = 0;
  std::vector<uint32_t> arr(4 * std::max<size_t>(nl, 1), 0);
  for (size_t k = 0; k < nl; ++k) {
    Instance &I = inst[live[k]];
    const FrontTemplate &T = *I.tmpl;
    I.sub_base = (uint32_t)n_subs;
    I.n_leaves = T.lev[T.D + 1] - T.lev[T.D];
    arr[k] = live[k];
    arr[nl + k] = (uint32_t)(&T - fb.t);
    arr[2 * nl + k] = (uint32_t)n_subs;
    arr[3 * nl + k] = (uint32_t)n_nodes;
    n_subs += I.n_leaves;
    n_nodes += T.path.size();
  }
  *n_subs_out = n_subs;
  if ((rc = ensure(s, &s->d_subs, &s->subs_cap, std::max<size_t>(n_subs, 1))) ||
      (rc = ensure(s, &s->d_sub_nodes, &s->sub_nodes_cap, std::max<size_t>(n_subs, 1))))
    return rc;
  if (!nl) return SP_OK;
  if (n_subs > 0xFFFFFFF0ull || n_nodes > 0xFFFFFFF0ull) {
    s->err = "root set too large";
    return SP_ERR_CAPACITY;
  }
  const size_t tiles_bytes = (inst.size() * (size_t)n + 15) & ~(size_t)15;
  const size_t in_bytes = tiles_bytes + 4 * nl * sizeof(uint32_t);
  if ((rc = ensure(s, &fb.in, &fb.cap_in, in_bytes)) || (rc = ensure(s, &fb.f, &fb.cap_f, n_nodes)) ||
      (rc = ensure(s, &fb.maxf, &fb.cap_maxf, n_nodes)) ||
      (rc = ensure(s, &fb.leaf_maxf, &fb.cap_leaf_maxf, n_subs)) ||
      (rc = ensure(s, &fb.leaf_node, &fb.cap_leaf_node, n_subs)) ||
      (rc = ensure(s, &fb.leaf_h, &fb.cap_leaf_h, n_subs)) || (rc = ensure(s, &fb.out, &fb.cap_out, nl)) ||
      (rc = ensure(s, &fb.error, &fb.cap_error, (size_t)1)))
    return rc;
  SP_CUDA(s, fb.h_in.reserve(in_bytes));
  SP_CUDA(s, fb.h_out.reserve(nl));
  SP_CUDA(s, fb.h_error.reserve(1));
  memcpy(fb.h_in.p, tiles, inst.size() * (size_t)n);
  memcpy(fb.h_in.p + tiles_bytes, arr.data(), 4 * nl * sizeof(uint32_t));
  SP_CUDA(s, cudaMemcpyAsync(fb.in, fb.h_in.p, in_bytes, cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemsetAsync(fb.error, 0, sizeof(int32_t), s->st));
  s->stats.h2d_bytes += in_bytes;
  const uint32_t *d_arr = reinterpret_cast<const uint32_t *>(fb.in + tiles_bytes);
  FrontArgs A{};
  A.tiles = fb.in;
  A.live = d_arr;
  A.live_tmpl = d_arr + nl;
  A.live_base = d_arr + 2 * nl;
  A.live_scratch = d_arr + 3 * nl;
  A.tmpl = fb.tmpl;
  A.lev = fb.lev;
  A.path = fb.path;
  A.parent = fb.parent;
  A.nchild = fb.nchild;
  A.depth = fb.depth;
  A.ht = s->d_ht;
  A.pdb = s->d_pdb;
  A.f = fb.f;
  A.maxf = fb.maxf;
  A.subs = s->d_subs;
  A.leaf_maxf = fb.leaf_maxf;
  A.leaf_h = fb.leaf_h;
  A.leaf_node = fb.leaf_node;
  A.out = fb.out;
  A.error = fb.error;
  SP_CUDA(s, launch_frontier(w, s->heur == SP_HEUR_PDB, (int)nl, A, s->st));
  s->stats.kernel_launches += 1;
  SP_CUDA(s, cudaMemcpyAsync(fb.h_out.p, fb.out, nl * sizeof(FrontInst), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(fb.h_error.p, fb.error, sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  s->stats.d2h_bytes += nl * sizeof(FrontInst) + sizeof(int32_t);
  if (*fb.h_error.p) {
    s->err = "root set: the heuristic changes by more than the bucket range allows along a path";
    return *fb.h_error.p;
  }
  // template node and h of every SubRoot: read by the host only after later
  // synchronisations (solution paths, the learned balancer)
  SP_CUDA(s, fb.h_leaf_node.reserve(n_subs));
  SP_CUDA(s, cudaMemcpyAsync(fb.h_leaf_node.p, fb.leaf_node, n_subs * sizeof(int32_t), cudaMemcpyDeviceToHost,
                             s->st));
  s->stats.d2h_bytes += n_subs * sizeof(int32_t);
  if (s->cfg.lb_mode == SP_LB_LEARNED) {
    SP_CUDA(s, fb.h_leaf_h.reserve(n_subs));
    SP_CUDA(s, cudaMemcpyAsync(fb.h_leaf_h.p, fb.leaf_h, n_subs, cudaMemcpyDeviceToHost, s->st));
    s->stats.d2h_bytes += n_subs;
  }
  // per instance only the buckets up to the last one in use (all leaves
  // counted, no interior children or goals above it)
  parallel_for(nl, [&](size_t k) {
    Instance &I = inst[live[k]];
    const FrontInst &O = fb.h_out.p[k];
    int top = kFrontBuckets - 1;
    while (top > 0 && O.leaf_cum[top - 1] == I.n_leaves && !O.child[top] && O.goal[top] == 0xFFFFFFFFu) --top;
    I.h0 = O.h0;
    I.leaf_cum.assign(O.leaf_cum, O.leaf_cum + top + 1);
    I.goal_key.assign(O.goal, O.goal + top + 1);
    I.interior.clear();
    uint64_t cum = 0;
    for (int b = 0; b <= top; ++b) {
      if (!O.child[b]) continue;
      cum += O.child[b];
      I.interior.push_back({I.h0 + (int32_t)b, cum});
    }
    I.last_load.assign(I.n_leaves, 0);
  }, nl * kFrontBuckets);
  return SP_OK;
}

// children generated this round by interior nodes within the limit
uint64_t interior_nodes(const Instance &I, int L) {
  auto it = std::upper_bound(I.interior.begin(), I.interior.end(), L,
                             [](int32_t v, const std::pair<int32_t, uint64_t> &e) { return v < e.first; });
  return it == I.interior.begin() ? 0 : std::prev(it)->second;
}

size_t active_leaves(const Instance &I, int L) {
  if (L < I.h0) return 0;
  return (size_t)(L - I.h0) >= I.leaf_cum.size() ? I.n_leaves : I.leaf_cum[(size_t)(L - I.h0)];
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

// The round's work: whole roots started as they are (direct, SubRoot ids in
// publication order) and roots first expanded `flags` levels by the split
// pre-pass.
struct RoundPlan {
  std::vector<uint32_t> direct;
  std::vector<Task> split;
  // the static planner writes straight into the solver's pinned staging
  // buffers (h_direct, h_split) instead; the vectors above stay empty
  bool staged = false;
  size_t staged_direct = 0, staged_split = 0;
  size_t n_direct() const { return staged ? staged_direct : direct.size(); }
  size_t n_split() const { return staged ? staged_split : split.size(); }
  size_t level_bound = 0;  // nodes one split level can hold
  size_t emit_bound = 0;   // pieces the split pre-pass can emit
  int max_k = 0;
};

void fold_ctl(sp_solver *s, const PoolCtl &ctl, int ri, float ms) {
  sp_stats &x = s->stats;
  x.kernel_ms += ms;
  x.tasks_donated += ctl.donated;
  x.dev_lane_steps += ctl.counters[0];
  x.dev_lane_slots += ctl.counters[1];
  x.dev_idle_cycles += ctl.counters[2];
  x.dev_warp_cycles += ctl.counters[3];
  x.dev_donate_tries += ctl.counters[4];
  x.dev_donate_notfree += ctl.counters[5];
  x.dev_donate_nowait += ctl.counters[6];
  x.dev_tasks_done += ctl.counters[7];
  x.round_kernel_ms[ri] = ms;
  x.round_donated[ri] = ctl.donated;
}

// Launch one round: uploads, split pre-pass, pool set-up, search; then the
// control block, split counters, per-root counts and solutions come back.
int launch_round(sp_solver *s, const RoundPlan &plan, size_t n_subs, size_t n_inst, float *ms,
                 bool multi = false) {
  const uint32_t n_direct = (uint32_t)plan.n_direct();
  const size_t n_split = plan.n_split();
  int rc = ensure_pool(s, n_direct + plan.emit_bound);
  if (rc) return rc;
  rc = ensure(s, &s->d_direct, &s->direct_cap, std::max<size_t>(n_direct, 1));
  if (rc) return rc;
  if (!s->d_cnt) SP_CUDA(s, cudaMalloc(&s->d_cnt, 4 * sizeof(uint32_t)));
  SP_CUDA(s, s->h_cnt.reserve(4));
  if (n_direct) {
    if (!plan.staged) {
      SP_CUDA(s, s->h_direct.reserve(n_direct));
      memcpy(s->h_direct.p, plan.direct.data(), n_direct * sizeof(uint32_t));
    }
    SP_CUDA(s, cudaMemcpyAsync(s->d_direct, s->h_direct.p, n_direct * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               s->st));
    s->stats.h2d_bytes += n_direct * sizeof(uint32_t);
  }
  s->h_cnt.p[0] = (uint32_t)n_split;
  s->h_cnt.p[1] = s->h_cnt.p[2] = s->h_cnt.p[3] = 0;
  SP_CUDA(s, cudaMemcpyAsync(s->d_cnt, s->h_cnt.p, 4 * sizeof(uint32_t), cudaMemcpyHostToDevice, s->st));
  if (n_split) {
    const size_t lb = std::max(plan.level_bound, n_split);
    rc = ensure(s, &s->d_split_a, &s->split_cap_a, lb);
    if (rc) return rc;
    rc = ensure(s, &s->d_split_b, &s->split_cap_b, lb);
    if (rc) return rc;
    rc = ensure(s, &s->d_emit, &s->emit_cap, std::max<size_t>(plan.emit_bound, 1));
    if (rc) return rc;
    if (!plan.staged) {
      SP_CUDA(s, s->h_split.reserve(n_split));
      memcpy(s->h_split.p, plan.split.data(), n_split * sizeof(Task));
    }
    SP_CUDA(s, cudaMemcpyAsync(s->d_split_a, s->h_split.p, n_split * sizeof(Task),
                               cudaMemcpyHostToDevice, s->st));
    s->stats.h2d_bytes += n_split * sizeof(Task);
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
  SP_CUDA(s, launch_pool_init(s->d_tasks, s->d_emit, plan.max_k ? s->d_cnt + 2 : nullptr, s->d_direct, n_direct,
                              s->d_seq, s->cap, s->d_ctl, multi ? s->d_subs : nullptr, multi ? s->mb.iter : nullptr,
                              s->st));
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
  P.poll_ns = SP_POLL_NS;
  const int block = s->cfg.threads_per_block == 128 ? 128 : 256;
  const uint32_t lanes = (uint32_t)(s->last_lanes > 0 ? s->last_lanes : s->num_sms * 1024);
  P.reserve = s->cfg.donate_reserve < 0 ? 0u : s->cfg.donate_reserve > 0 ? (uint32_t)s->cfg.donate_reserve
                                                                          : lanes / 16u;
  P.spread = std::max(1u, lanes / 32u);
  int grid = 0;
  if (multi) {
    MultiBufs &m = s->mb;
    P.inst_iter = m.iter;
    P.inst_out = m.out;
    P.inst_final = m.fin;
    P.inst_status = m.status;
    P.inst_sub_base = m.base;
    P.inst_nsub = m.nsub;
    P.sub_maxf = s->fb.leaf_maxf;
    P.inter_off = m.ioff;
    P.inter_len = m.ilen;
    P.inter_f = m.ifv;
    P.inter_cum = m.icum;
    P.goal_maxf = m.goal;
    P.inst_pair = m.pair;
    P.pair_nodes = (s->cfg.handback_nodes > 0 && n_inst * SP_PAIR_LANES <= (size_t)lanes) ? SP_PAIR_NODES : 0;
    P.iter_nodes = m.iter_nodes;
    P.sub_loads = m.loads;
    P.inst_fin_ns = m.fin_ns;
    P.t_begin_ns = m.t0_ns;
    P.n_subs = (uint32_t)n_subs;
    P.static_split = (s->cfg.lb_mode == SP_LB_STATIC_STEAL || s->cfg.lb_mode == SP_LB_LEARNED) ? 1 : 0;
    P.handback_nodes = (unsigned long long)s->cfg.handback_nodes;
    P.sub_growth = m.use_growth ? m.growth : nullptr;
    SP_CUDA(s, launch_search_multi(s->w, s->heur == SP_HEUR_PDB, block, s->cfg.blocks_per_sm, s->num_sms, P,
                                   s->st, &grid));
  } else {
    SP_CUDA(s, launch_search_round(s->w, s->heur == SP_HEUR_PDB, block, s->cfg.blocks_per_sm, s->num_sms, P,
                                   s->st, &grid));
  }
  SP_CUDA(s, cudaEventRecord(s->ev1, s->st));
  SP_CUDA(s, s->h_ctl.reserve(1));
  SP_CUDA(s, s->h_sub_nodes.reserve(std::max<size_t>(n_subs, 1)));
  SP_CUDA(s, s->h_sols.reserve(std::max<size_t>(n_inst, 1)));
  SP_CUDA(s, cudaMemcpyAsync(s->h_ctl.p, s->d_ctl, sizeof(PoolCtl), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(s->h_cnt.p, s->d_cnt, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->st));
  if (n_subs && !multi)
    SP_CUDA(s, cudaMemcpyAsync(s->h_sub_nodes.p, s->d_sub_nodes, n_subs * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, s->st));
  const size_t n_sol = multi ? 2 * n_inst : n_inst;  // multi: one record per instance and iteration parity
  SP_CUDA(s, s->h_sols.reserve(std::max<size_t>(n_sol, 1)));
  if (n_inst)
    SP_CUDA(s, cudaMemcpyAsync(s->h_sols.p, s->d_sol, n_sol * sizeof(Solution), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  SP_CUDA(s, cudaEventElapsedTime(ms, s->ev0, s->ev1));
  s->stats.d2h_bytes += sizeof(PoolCtl) + 16 + n_subs * 8 + n_sol * sizeof(Solution);
  s->stats.kernel_launches += 2;
  s->last_lanes = grid * block;
  s->last_emitted = s->h_cnt.p[2];
  if (!s->h_ctl.p->error && s->h_cnt.p[3]) s->h_ctl.p->error = (int32_t)s->h_cnt.p[3];
  return SP_OK;
}

// Static load balancing for the round: a root's work is predicted from its
// previous round (load x the instance's growth per threshold step); a root
// predicted above the round's piece size T (the round's predicted total
// over SP_SPLIT_PIECES_PER_LANE pieces per resident lane) is split ceil(log2(pred/T))
// levels by the device pre-pass -- the reference splits a root into
// ceil(load/avg) pieces (src/24puzzle_block_parallel_with_pdb.cu:839-897) --
// and whole roots are published in decreasing predicted size.  With the
// learned balancer every root's prediction comes from the model: its
// measured load times its own predicted growth, or the model's size estimate
// for a root the previous round did not search.
int plan_round(sp_solver *s, std::vector<Instance> &inst, const std::vector<int32_t> &limits,
               RoundPlan &plan) {
  const bool learned = s->cfg.lb_mode == SP_LB_LEARNED;
  const bool stat = s->cfg.lb_mode == SP_LB_STATIC_STEAL || learned;
  // candidates: the active roots of every live instance, instance by instance
  const size_t ni = inst.size();
  std::vector<size_t> off(ni + 1, 0);
  for (size_t i = 0; i < ni; ++i)
    off[i + 1] = off[i] + (inst[i].done ? 0 : active_leaves(inst[i], limits[i]));
  const size_t nc = off[ni];
  // candidate chunks for the worker pool; chunk c starts in instance c_inst[c]
  const size_t nchunk = std::max<size_t>(1, std::min<size_t>(128, nc / 2048));
  auto chunk_lo = [&](size_t c) { return nc * c / nchunk; };
  std::vector<size_t> c_inst(nchunk, 0);
  for (size_t c = 0; c < nchunk; ++c)
    c_inst[c] = (size_t)(std::upper_bound(off.begin(), off.end(), chunk_lo(c)) - off.begin()) - 1;
  // calls fn(j, i, q) for the candidates j of chunk c: root q of instance i
  auto for_chunk = [&](size_t c, auto fn) {
    size_t i = c_inst[c];
    for (size_t j = chunk_lo(c); j < chunk_lo(c + 1); ++j) {
      while (j >= off[i + 1]) ++i;
      fn(j, i, j - off[i]);
    }
  };
  if (!stat) {
    plan.direct.resize(nc);
    parallel_for(nchunk, [&](size_t c) {
      for_chunk(c, [&](size_t j, size_t i, size_t q) { plan.direct[j] = inst[i].sub_base + (uint32_t)q; });
    }, nc);
    return SP_OK;
  }
  // predicted load of each candidate: the previous round's load x the
  // instance's growth per threshold step (whose round total is the
  // instance's last total x growth), or, with the learned balancer, below
  std::vector<double> growth(ni, 0.0);
  double total = 0;
  for (size_t i = 0; i < ni; ++i) {
    const Instance &I = inst[i];
    if (off[i + 1] == off[i]) continue;
    double gr = 6.0;
    if (I.prev_total > 0 && I.last_total > 0)
      gr = std::min(30.0, std::max(2.0, (double)I.last_total / (double)I.prev_total));
    growth[i] = gr;
    total += (double)I.last_total * gr;
  }
  std::vector<double> lpred;  // learned balancer: per candidate
  if (learned && nc) {
    // The model predicts every active root: y(s) = log2(1 + nodes) of its
    // subtree at slack s = (limit - g - h) / 2 (clamped to the slacks it was
    // trained on).  A root measured in the previous round is predicted as
    // that load times its own growth 2^(y(s) - y(s - 1)) (in place of the
    // instance's common growth); a root without a measured load as 2^y(s) - 1.
    std::vector<uint32_t> q_sub;
    std::vector<int32_t> q_slack;
    std::vector<int32_t> lo_at(nc, -1);  // index of y(s - 1), -1 if not needed
    q_sub.reserve(2 * nc);
    q_slack.reserve(2 * nc);
    for (size_t i = 0; i < ni; ++i) {
      const Instance &I = inst[i];
      for (size_t q = 0; q < off[i + 1] - off[i]; ++q) {
        const int leaf_h = s->fb.h_leaf_h.p[I.sub_base + q];
        const int sl = std::min(kLbmMaxSlack, std::max(0, (limits[i] - (int)I.tmpl->D - leaf_h) / 2));
        q_sub.push_back(I.sub_base + (uint32_t)q);
        q_slack.push_back(sl);
        if (I.last_load[q]) {
          lo_at[off[i] + q] = (int32_t)q_sub.size();
          q_sub.push_back(I.sub_base + (uint32_t)q);
          q_slack.push_back(std::max(0, sl - 1));
        }
      }
    }
    std::vector<float> y(q_sub.size());
    int rc = s->lbm->predict_subs(s->d_subs, q_sub.data(), q_slack.data(), (int)q_sub.size(), y.data(), s->st,
                                  s->err);
    if (rc) return rc;
    s->stats.kernel_launches += 2 * (int)((q_sub.size() + 65535) / 65536);
    lpred.resize(nc);
    total = 0;
    size_t at = 0;
    for (size_t i = 0; i < ni; ++i) {
      const Instance &I = inst[i];
      for (size_t q = 0; q < off[i + 1] - off[i]; ++q) {
        const size_t j = off[i] + q;
        const double yh = std::min(60.0, std::max(0.0, (double)y[at]));
        double p;
        if (lo_at[j] >= 0) {
          const double step = std::min(kLbmMaxStep, std::max(0.0, yh - (double)y[(size_t)lo_at[j]]));
          p = (double)I.last_load[q] * std::exp2(step);
          at += 2;
        } else {
          p = std::exp2(yh) - 1.0;
          at += 1;
        }
        lpred[j] = p;
        total += p;
      }
    }
  }
  const double lanes = s->last_lanes > 0 ? (double)s->last_lanes : (double)s->num_sms * 1024.0;
  const double T = total / (lanes * (double)SP_SPLIT_PIECES_PER_LANE);
  static const size_t pow3[12] = {1, 3, 9, 27, 81, 243, 729, 2187, 6561, 19683, 59049, 177147};
  auto bound = [&](int kk) { return kk ? 4 * pow3[kk - 1] : (size_t)0; };
  const int kcap = std::min(10, std::max(1, s->cfg.static_split_cap));
  // pass 1, per chunk: the exponent of pred relative to T (ceil(log2(pred/T))
  // for pred > T) gives the split depth and the bucket of the longest-first
  // order (bucket 63 - e: larger predictions first); histograms of the
  // buckets (whole and split roots apart) and of the split depths
  std::vector<int8_t> k(nc, 0);
  std::vector<uint8_t> bucket(nc, 127);
  std::vector<uint32_t> hd(nchunk * 128, 0), hs(nchunk * 128, 0);
  std::vector<size_t> kh(nchunk * 11, 0);
  parallel_for(nchunk, [&](size_t c) {
    uint32_t *cd = &hd[c * 128], *cs = &hs[c * 128];
    size_t *ck = &kh[c * 11];
    for_chunk(c, [&](size_t j, size_t i, size_t q) {
      const double pred = learned ? lpred[j] : (double)inst[i].last_load[q] * growth[i];
      int e = -64;
      if (pred > 0 && T > 0) {
        std::frexp(pred / T, &e);  // pred/T in [2^(e-1), 2^e)
        e = std::max(-63, std::min(63, e));
      }
      const uint8_t b = (uint8_t)(63 - e);
      bucket[j] = b;
      int kk = 0;
      if (T > 0 && pred > T) {
        const int room = limits[i] - (int)inst[i].tmpl->D;  // levels left below the root
        kk = std::max(0, std::min(e, std::min(kcap, room - 1)));
      }
      k[j] = (int8_t)kk;
      ++ck[kk];
      ++(kk > 0 ? cs : cd)[b];
    });
  }, nc);
  // piece budget: the deepest splits are cut first, i.e. every depth is
  // capped at the largest cap whose pieces fit
  size_t cnt_k[11] = {0};
  for (size_t c = 0; c < nchunk; ++c)
    for (int kk = 0; kk <= 10; ++kk) cnt_k[kk] += kh[c * 11 + kk];
  const size_t budget = (size_t)1 << 22;
  int kmax = 10;
  for (; kmax > 0; --kmax) {
    size_t need = 0;
    for (int kk = 1; kk <= 10; ++kk) need += cnt_k[kk] * bound(std::min(kk, kmax));
    if (need <= budget) break;
  }
  if (kmax == 0)  // no split fits: every root goes whole
    for (size_t x = 0; x < hd.size(); ++x) hd[x] += hs[x], hs[x] = 0;
  // stable counting sort by bucket, split roots and whole roots apart:
  // every chunk scatters into its own ranges (pass 2)
  size_t nd = 0, nsp = 0;
  for (int b = 0; b < 128; ++b)
    for (size_t c = 0; c < nchunk; ++c) {
      const uint32_t a = hd[c * 128 + b], z = hs[c * 128 + b];
      hd[c * 128 + b] = (uint32_t)nd;
      hs[c * 128 + b] = (uint32_t)nsp;
      nd += a;
      nsp += z;
    }
  SP_CUDA(s, s->h_direct.reserve(std::max<size_t>(nd, 1)));
  SP_CUDA(s, s->h_split.reserve(std::max<size_t>(nsp, 1)));
  uint32_t *out_direct = s->h_direct.p;
  Task *out_split = s->h_split.p;
  plan.staged = true;
  plan.staged_direct = nd;
  plan.staged_split = nsp;
  parallel_for(nchunk, [&](size_t c) {
    uint32_t *cd = &hd[c * 128], *cs = &hs[c * 128];
    for_chunk(c, [&](size_t j, size_t i, size_t q) {
      const int kk = std::min((int)k[j], kmax);
      const uint32_t sub = inst[i].sub_base + (uint32_t)q;
      if (kk > 0) {
        Task t{};
        t.sub = sub;
        t.mask = 0xF;
        t.flags = (uint8_t)kk;
        out_split[cs[bucket[j]]++] = t;
      } else {
        out_direct[cd[bucket[j]]++] = sub;
      }
    });
  }, nc);
  for (int kk = 1; kk <= 10; ++kk) {
    const size_t cnt = cnt_k[kk];
    if (!cnt || kmax == 0) continue;
    const int ke = std::min(kk, kmax);
    plan.max_k = std::max(plan.max_k, ke);
    plan.emit_bound += cnt * bound(ke);
  }
  size_t level[12] = {0};
  for (int kk = 1; kk <= 10 && kmax > 0; ++kk)
    for (int l = 1; l <= std::min(kk, kmax); ++l) level[l] += cnt_k[kk] * 4 * pow3[l - 1];
  for (int l = 1; l < 12; ++l) plan.level_bound = std::max(plan.level_bound, level[l]);
  return SP_OK;
}

// Result path of a solved instance: the root-set tree prefix to its goal (a
// tree node) or to the device solution's root, then the device's moves.
// `leaf_node` maps a SubRoot to its template node.
void set_path(int w, Instance &I, const uint8_t *tiles, int host_goal, const Solution *sol,
              const int32_t *leaf_node) {
  std::vector<uint8_t> mv;
  int node = host_goal;
  uint32_t extra = 0;
  const uint32_t *pw = nullptr;
  if (node < 0) {
    node = leaf_node[sol->sub];
    extra = sol->len;
    pw = sol->path;
  }
  const FrontTemplate &T = *I.tmpl;
  for (int j = 0; j < T.depth[(size_t)node]; ++j) mv.push_back((uint8_t)((T.path[(size_t)node] >> (2 * j)) & 3u));
  for (uint32_t j = 0; j < extra; ++j) mv.push_back((uint8_t)((pw[j >> 4] >> (2 * (j & 15))) & 3u));
  sp_result *R = I.out;
  R->len = (int32_t)mv.size();
  if (mv.size() > SP_MAX_MOVES) {
    R->status = SP_ERR_PATH;
  } else {
    R->n_moves = R->len;
    memcpy(R->moves, mv.data(), mv.size());
    R->status = replay_ok(w, tiles, R->moves, R->n_moves) ? SP_OK : SP_ERR_PATH;
  }
}

// The shallowest root-set goal node (first in tree order) whose path stays
// within L, or -1.
int tree_goal(const Instance &I, int L) {
  uint32_t best = 0xFFFFFFFFu;
  for (size_t b = 0; b < I.goal_key.size() && I.h0 + (int)b <= L; ++b) best = std::min(best, I.goal_key[b]);
  return best == 0xFFFFFFFFu ? -1 : (int)(best & 0xFFFFFFu);
}

// Smallest maxf of a root-set goal node (INT32_MAX: none).
int32_t goal_maxf(const Instance &I) {
  for (size_t b = 0; b < I.goal_key.size(); ++b)
    if (I.goal_key[b] != 0xFFFFFFFFu) return I.h0 + (int)b;
  return 0x7FFFFFFF;
}

// Multi-iteration mode: every instance's threshold loop runs on the device in
// one launch (search.cu, `advance`); the host only prepares the tables and
// assembles the results.  Iterations in which no root-set leaf is active are
// finished here first.
int solve_multi(sp_solver *s, const uint8_t *tiles, std::vector<Instance> &inst, size_t n_subs,
                std::chrono::steady_clock::time_point t_start) {
  const size_t ni = inst.size();
  const int w = s->w, n = s->n;
  // limits: two per instance, by iteration parity (the device loop may run an
  // instance's next iteration beside the current one)
  std::vector<int32_t> h_iter(ni, 0), h_limit(2 * ni, 0), h_final(ni, -1), h_goal(ni, 0x7FFFFFFF);
  std::vector<uint32_t> h_out(ni, 0), h_base(ni, 0), h_nsub(ni, 0), h_ioff(ni, 0), h_ilen(ni, 0);
  std::vector<int32_t> h_if;
  std::vector<unsigned long long> h_icum;
  std::vector<uint32_t> direct;
  for (size_t i = 0; i < ni; ++i) {
    Instance &I = inst[i];
    h_base[i] = I.sub_base;
    if (I.done) continue;
    h_goal[i] = goal_maxf(I);
    h_ioff[i] = (uint32_t)h_if.size();
    h_ilen[i] = (uint32_t)I.interior.size();
    for (auto &e : I.interior) {
      h_if.push_back(e.first);
      h_icum.push_back(e.second);
    }
    h_nsub[i] = I.n_leaves;
    // iterations without any active leaf: the root-set tree holds them whole
    int L = I.h0;
    for (;;) {
      const size_t na = active_leaves(I, L);
      if (na) {
        for (size_t q = 0; q < na; ++q) direct.push_back(I.sub_base + (uint32_t)q);
        h_out[i] = (uint32_t)na;
        h_iter[i] = I.iter;
        h_limit[2 * i + (I.iter & 1)] = L;
        break;
      }
      sp_result *R = I.out;
      R->f_limit[I.iter] = L;
      R->nodes[I.iter] = interior_nodes(I, L);
      R->nodes_total += R->nodes[I.iter];
      s->stats.nodes += R->nodes[I.iter];
      s->stats.round_nodes[std::min(I.iter, SP_MAX_ROUNDS - 1)] += R->nodes[I.iter];
      R->n_iter = I.iter + 1;
      const int hg = tree_goal(I, L);
      if (hg >= 0) {
        set_path(w, I, tiles + i * (size_t)n, hg, nullptr, s->fb.h_leaf_node.p);
        I.done = true;
        break;
      }
      if (++I.iter >= SP_MAX_ITERS) {
        R->status = SP_ERR_LIMIT;
        I.done = true;
        break;
      }
      L += 2;
    }
    if (I.done) h_nsub[i] = 0;
  }
  if (h_if.empty()) {
    h_if.push_back(0);
    h_icum.push_back(0);
  }
  MultiBufs &m = s->mb;
  int rc = 0;
  if ((rc = ensure(s, &m.iter, &m.cap_iter, ni)) || (rc = ensure(s, &m.out, &m.cap_out, ni)) ||
      (rc = ensure(s, &m.fin, &m.cap_fin, ni)) || (rc = ensure(s, &m.status, &m.cap_status, ni)) ||
      (rc = ensure(s, &m.base, &m.cap_base, ni)) || (rc = ensure(s, &m.nsub, &m.cap_nsub, ni)) ||
      (rc = ensure(s, &m.ioff, &m.cap_ioff, ni)) || (rc = ensure(s, &m.ilen, &m.cap_ilen, ni)) ||
      (rc = ensure(s, &m.goal, &m.cap_goal, ni)) ||
      (rc = ensure(s, &m.ifv, &m.cap_ifv, h_if.size())) || (rc = ensure(s, &m.icum, &m.cap_icum, h_icum.size())) ||
      (rc = ensure(s, &m.iter_nodes, &m.cap_iter_nodes, ni * kMaxIters)) ||
      (rc = ensure(s, &m.loads, &m.cap_loads, 2 * std::max<size_t>(n_subs, 1))) ||
      (rc = ensure(s, &m.fin_ns, &m.cap_fin_ns, ni)) || (rc = ensure(s, &m.t0_ns, &m.cap_t0_ns, 1)) ||
      (rc = ensure(s, &m.pair, &m.cap_pair, ni)))
    return rc;
  // uploads through one pinned staging buffer (asynchronous copies)
  auto bytes16 = [](const auto &v) { return (v.size() * sizeof(v[0]) + 15) & ~(size_t)15; };
  const size_t stage_bytes = bytes16(h_iter) + bytes16(h_limit) + bytes16(h_out) + bytes16(h_final) +
                             bytes16(h_base) + bytes16(h_nsub) + bytes16(h_ioff) + bytes16(h_ilen) +
                             bytes16(h_goal) + bytes16(h_if) + bytes16(h_icum) + n_subs * kGrowthSlacks + 16;
  SP_CUDA(s, s->h_stage_up.reserve(stage_bytes));
  size_t stage_off = 0;
  auto up = [&](auto *dst, const auto &v) {
    const size_t b = v.size() * sizeof(v[0]);
    uint8_t *src = s->h_stage_up.p + stage_off;
    memcpy(src, v.data(), b);
    stage_off += (b + 15) & ~(size_t)15;
    return cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, s->st);
  };
  SP_CUDA(s, up(m.iter, h_iter));
  SP_CUDA(s, up(s->d_limit, h_limit));
  SP_CUDA(s, up(m.out, h_out));
  SP_CUDA(s, up(m.fin, h_final));
  SP_CUDA(s, cudaMemsetAsync(m.status, 0, ni * sizeof(int32_t), s->st));
  SP_CUDA(s, up(m.base, h_base));
  SP_CUDA(s, up(m.nsub, h_nsub));
  SP_CUDA(s, up(m.ioff, h_ioff));
  SP_CUDA(s, up(m.ilen, h_ilen));
  SP_CUDA(s, up(m.goal, h_goal));
  SP_CUDA(s, up(m.ifv, h_if));
  SP_CUDA(s, up(m.icum, h_icum));
  SP_CUDA(s, cudaMemsetAsync(m.iter_nodes, 0, ni * kMaxIters * sizeof(unsigned long long), s->st));
  SP_CUDA(s, cudaMemsetAsync(m.loads, 0, 2 * std::max<size_t>(n_subs, 1) * sizeof(unsigned long long), s->st));
  SP_CUDA(s, cudaMemsetAsync(s->d_sol, 0, 2 * ni * sizeof(Solution), s->st));
  SP_CUDA(s, cudaMemsetAsync(m.pair, 0, ni * sizeof(uint32_t), s->st));
  SP_CUDA(s, cudaMemsetAsync(m.fin_ns, 0, ni * sizeof(unsigned long long), s->st));
  SP_CUDA(s, cudaMemsetAsync(m.t0_ns, 0xFF, sizeof(unsigned long long), s->st));
  // learned balancer: every root's predicted growth per threshold step at
  // each slack, 2^(y(j+1) - y(j)) from the model's log2 sizes y, coded as
  // 16 * log2 in a byte; the device multiplies each root's measured load by
  // it to order and split the next iteration
  m.use_growth = false;
  if (s->cfg.lb_mode == SP_LB_LEARNED && n_subs) {
    if (!s->lbm || !s->lbm->ready()) {
      s->err = "SP_LB_LEARNED without a model (sp_lbm_init / sp_lbm_import)";
      return SP_ERR_ARG;
    }
    const int G = kGrowthSlacks;
    std::vector<uint32_t> gi(n_subs * G);
    std::vector<int32_t> gs(n_subs * G);
    for (size_t q = 0; q < n_subs; ++q)
      for (int j = 0; j < G; ++j) {
        gi[q * G + j] = (uint32_t)q;
        gs[q * G + j] = std::min(j, kLbmMaxSlack);
      }
    std::vector<float> y(gi.size());
    rc = s->lbm->predict_subs(s->d_subs, gi.data(), gs.data(), (int)gi.size(), y.data(), s->st, s->err);
    if (rc) return rc;
    s->stats.kernel_launches += 2 * (int)((gi.size() + 65535) / 65536);
    std::vector<uint8_t> code(n_subs * G);
    for (size_t q = 0; q < n_subs; ++q)
      for (int j = 0; j < G; ++j) {
        const int a = std::min(j, G - 2);
        const double step = (double)y[q * G + a + 1] - (double)y[q * G + a];
        code[q * G + j] = (uint8_t)std::lround(16.0 * std::min(kLbmMaxStep, std::max(0.0, step)));
      }
    if ((rc = ensure(s, &m.growth, &m.cap_growth, code.size()))) return rc;
    SP_CUDA(s, up(m.growth, code));
    s->stats.h2d_bytes += code.size();
    m.use_growth = true;
  }
  s->stats.h2d_bytes += ni * 40 + h_if.size() * 12;
  const double pre_s = ms_since(t_start) / 1000.0;  // host part before the launch
  for (auto &I : inst)
    if (I.done) I.out->seconds = pre_s;
  float ms = 0;
  if (!direct.empty()) {
    RoundPlan plan;
    plan.direct = std::move(direct);
    // later iterations publish up to every root at once, and split pieces
    // while the ring is below half full
    plan.emit_bound = n_subs + ((size_t)1 << 20);
    rc = launch_round(s, plan, n_subs, ni, &ms, true);
    if (rc) return rc;
    const PoolCtl &ctl = *s->h_ctl.p;
    fold_ctl(s, ctl, 0, ms);
    s->stats.tasks_initial += plan.direct.size();
    s->stats.round_tasks[0] = (int32_t)plan.direct.size();
    if (ctl.error) {
      char buf[160];
      snprintf(buf, sizeof buf, "device error %d (info %u) in the multi-iteration search", ctl.error,
               ctl.err_info[0]);
      s->err = buf;
      for (auto &I : inst)
        if (!I.done) {
          I.out->status = ctl.error;
          I.done = true;
        }
      return ctl.error;
    }
  }
  // results through one pinned staging buffer
  SP_CUDA(s, s->h_stage_dn.reserve(ni * (2 * sizeof(unsigned long long) + 2 * sizeof(int32_t) +
                                         kMaxIters * sizeof(unsigned long long)) + 64));
  unsigned long long *fin_ns = reinterpret_cast<unsigned long long *>(s->h_stage_dn.p);
  unsigned long long *t0 = fin_ns + ni;
  unsigned long long *itn = t0 + 1;
  int32_t *fin = reinterpret_cast<int32_t *>(itn + ni * kMaxIters);
  int32_t *st = fin + ni;
  SP_CUDA(s, cudaMemcpyAsync(fin_ns, m.fin_ns, ni * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(t0, m.t0_ns, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(fin, m.fin, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(st, m.status, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaMemcpyAsync(itn, m.iter_nodes, ni * kMaxIters * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  s->stats.d2h_bytes += ni * (8 + kMaxIters * 8);
  const Solution *sols = s->h_sols.p;
  int rounds = 0;
  const unsigned long long *loads = nullptr;
  for (size_t i = 0; i < ni; ++i) {
    Instance &I = inst[i];
    if (I.done) {
      rounds = std::max(rounds, I.out->n_iter);
      continue;
    }
    sp_result *R = I.out;
    const int r_end = fin[i] < 0 ? I.iter : fin[i];
    for (int r = I.iter; r <= r_end && r < SP_MAX_ITERS; ++r) {
      R->f_limit[r] = I.h0 + 2 * r;
      R->nodes[r] = itn[i * kMaxIters + (size_t)r];
      R->nodes_total += R->nodes[r];
      s->stats.nodes += R->nodes[r];
      s->stats.round_nodes[std::min(r, SP_MAX_ROUNDS - 1)] += R->nodes[r];
    }
    R->n_iter = r_end + 1;
    rounds = std::max(rounds, R->n_iter);
    if (fin_ns[i] && fin_ns[i] >= t0[0]) R->seconds = pre_s + 1e-9 * (double)(fin_ns[i] - t0[0]);
    if (fin[i] < 0) {
      R->status = SP_ERR_TIMEOUT;
    } else if (st[i] == kStatusHandback) {
      // continue in the round loop from iteration fin + 1 with the loads the
      // device measured in iteration fin
      R->seconds = 0.0;
      if (!loads) {
        const size_t nl = 2 * std::max<size_t>(n_subs, 1);
        SP_CUDA(s, s->h_loads.reserve(nl));
        SP_CUDA(s, cudaMemcpyAsync(s->h_loads.p, m.loads, nl * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                   s->st));
        SP_CUDA(s, cudaStreamSynchronize(s->st));
        s->stats.d2h_bytes += nl * sizeof(unsigned long long);
        loads = s->h_loads.p;
      }
      const int f = fin[i];
      const unsigned long long *lf = loads + (size_t)(f & 1) * n_subs + I.sub_base;
      uint64_t tot = 0;
      for (size_t q = 0; q < I.n_leaves; ++q) {
        I.last_load[q] = lf[q];
        tot += lf[q];
      }
      I.last_total = tot;
      I.prev_total = 0;
      if (f - 1 >= I.iter) {
        const uint64_t all = itn[i * kMaxIters + (size_t)(f - 1)], in = interior_nodes(I, I.h0 + 2 * (f - 1));
        I.prev_total = all > in ? all - in : 0;
      }
      I.iter = f + 1;
      continue;
    } else if (st[i]) {
      R->status = st[i];
    } else {
      const int L = I.h0 + 2 * fin[i];
      const int hg = tree_goal(I, L);
      set_path(w, I, tiles + i * (size_t)n, hg, hg < 0 ? &sols[2 * i + (fin[i] & 1)] : nullptr, s->fb.h_leaf_node.p);
    }
    I.done = true;
  }
  s->stats.rounds = rounds;
  const double wall = ms_since(t_start);
  for (auto &I : inst)
    if (I.done && I.out->seconds == 0.0) I.out->seconds = wall / 1000.0;
  s->stats.wall_ms = wall;
  return SP_OK;
}

int solve_impl(sp_solver *s, const uint8_t *tiles, int nin, sp_result *res) {
  auto t_start = std::chrono::steady_clock::now();
  memset(&s->stats, 0, sizeof(s->stats));
  if (s->heur == SP_HEUR_PDB && !s->pdb_ready) {
    s->err = "PDB heuristic selected but sp_pdb_build/sp_pdb_import not done";
    return SP_ERR_NO_PDB;
  }
  if (s->cfg.lb_mode == SP_LB_LEARNED && !(s->lbm && s->lbm->ready())) {
    s->err = "learned load balancing selected but no model (sp_lbm_init/sp_lbm_import)";
    return SP_ERR_ARG;
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
  }
  // root set: uniform-depth tree expansion to >= frontier_target leaves per
  // instance, on the device
  auto t_front = std::chrono::steady_clock::now();
  // a batch's root set is capped near 8 roots per resident lane: more roots
  // than that add work and no balance (donation splits what is left)
  size_t live = 0;
  for (auto &I : inst) live += !I.done;
  const double lanes = s->last_lanes > 0 ? (double)s->last_lanes : (double)s->num_sms * 768.0;
  int target = std::max(1, s->cfg.frontier_target);
  if (live) target = std::min(target, std::max(32, (int)(8.0 * lanes / (double)live)));
  size_t n_subs = 0;
  int rc = build_root_sets(s, tiles, inst, target, &n_subs);
  if (rc) return rc;
  if (inst.size() > s->inst_cap || !s->d_limit) {
    if (s->d_limit) cudaFree(s->d_limit);
    if (s->d_sol) cudaFree(s->d_sol);
    s->d_limit = nullptr;
    s->d_sol = nullptr;
    const size_t c = std::max<size_t>(inst.size(), 64);
    // two entries per instance: the device loop keeps one per iteration parity
    SP_CUDA(s, cudaMalloc(&s->d_limit, 2 * c * sizeof(int32_t)));
    SP_CUDA(s, cudaMalloc(&s->d_sol, 2 * c * sizeof(Solution)));
    s->inst_cap = c;
  }
  SP_CUDA(s, s->h_limits.reserve(inst.size()));
  s->stats.frontier_ms += ms_since(t_front);
  // persistent mode: the device loop; instances it hands back (large
  // iterations ahead) continue in the round loop below
  int round0 = 0;
  if (s->cfg.persistent) {
    rc = solve_multi(s, tiles, inst, n_subs, t_start);
    if (rc) return rc;
    bool left = false;
    for (auto &I : inst) left |= !I.done;
    if (!left) return SP_OK;
    round0 = 1;  // round statistics after the persistent launch's slot
  }

  std::vector<int32_t> limits(inst.size(), 0);
  for (int round = 0; round < SP_MAX_ITERS; ++round) {
    int active = 0;
    for (auto &I : inst) active += !I.done;
    if (!active) break;
    const auto t_round = std::chrono::steady_clock::now();
    const int ri = std::min(round + round0, SP_MAX_ROUNDS - 1);
    s->stats.round_instances[ri] = active;
    for (size_t i = 0; i < inst.size(); ++i) {
      limits[i] = inst[i].done ? -1 : inst[i].h0 + 2 * inst[i].iter;
      s->h_limits.p[i] = limits[i];
    }
    RoundPlan plan;
    rc = plan_round(s, inst, limits, plan);
    if (rc) return rc;
    SP_CUDA(s, cudaMemcpyAsync(s->d_limit, s->h_limits.p, inst.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               s->st));
    SP_CUDA(s, cudaMemsetAsync(s->d_sol, 0, inst.size() * sizeof(Solution), s->st));
    SP_CUDA(s, cudaMemsetAsync(s->d_sub_nodes, 0, std::max<size_t>(n_subs, 1) * sizeof(unsigned long long), s->st));
    s->stats.h2d_bytes += inst.size() * sizeof(int32_t);
    float ms = 0;
    const unsigned long long *sn = nullptr;
    const Solution *sols = nullptr;
    if (plan.n_direct() || plan.n_split()) {
      rc = launch_round(s, plan, n_subs, inst.size(), &ms);
      if (rc) return rc;
      const PoolCtl &ctl = *s->h_ctl.p;
      fold_ctl(s, ctl, ri, ms);
      s->stats.tasks_initial += plan.n_direct() + s->last_emitted;
      s->stats.round_tasks[ri] = (int32_t)(plan.n_direct() + s->last_emitted);
      if (ctl.error) {
        char buf[160];
        snprintf(buf, sizeof buf, "device error %d (info %u) in round %d", ctl.error, ctl.err_info[0], round);
        s->err = buf;
        for (auto &I : inst)
          if (!I.done) {
            I.out->status = ctl.error;
            I.done = true;
          }
        return ctl.error;
      }
      sn = s->h_sub_nodes.p;
      sols = s->h_sols.p;
    }
    ++s->stats.rounds;
    // fold results: per-root loads (parallel over instances), then the rest
    std::vector<uint64_t> dev_nodes(inst.size(), 0);
    size_t fold_work = 0;
    for (size_t i = 0; i < inst.size(); ++i)
      if (!inst[i].done) fold_work += active_leaves(inst[i], limits[i]);
    parallel_for(inst.size(), [&](size_t i) {
      Instance &I = inst[i];
      if (I.done) return;
      const size_t na = active_leaves(I, limits[i]);
      uint64_t dev = 0;
      for (size_t q = 0; q < na; ++q) {
        const uint64_t v = sn ? sn[I.sub_base + q] : 0;
        dev += v;
        I.last_load[q] = v;
      }
      dev_nodes[i] = dev;
    }, fold_work);
    for (size_t i = 0; i < inst.size(); ++i) {
      Instance &I = inst[i];
      if (I.done) continue;
      const int L = limits[i];
      const uint64_t dev = dev_nodes[i];
      const uint64_t nodes = interior_nodes(I, L) + dev;
      I.prev_total = I.last_total;
      I.last_total = dev;
      sp_result *R = I.out;
      R->f_limit[I.iter] = L;
      R->nodes[I.iter] = nodes;
      R->nodes_total += nodes;
      R->n_iter = I.iter + 1;
      s->stats.nodes += nodes;
      s->stats.round_nodes[ri] += nodes;
      const int host_goal = tree_goal(I, L);
      const bool dev_goal = sols && sols[i].flag != 0;
      if (host_goal >= 0 || dev_goal) {
        // path: root-set tree prefix, then the device's moves below its root
        set_path(w, I, tiles + i * (size_t)n, host_goal, host_goal < 0 ? &sols[i] : nullptr, s->fb.h_leaf_node.p);
        I.done = true;
        continue;
      }
      ++I.iter;
      if (I.iter >= SP_MAX_ITERS) {
        R->status = SP_ERR_LIMIT;
        I.done = true;
      }
    }
    const double now_s = ms_since(t_start) / 1000.0;
    for (auto &I : inst)
      if (I.done && I.out->seconds == 0.0) I.out->seconds = now_s;
    s->stats.round_host_ms[ri] = (float)(ms_since(t_round) - s->stats.round_kernel_ms[ri]);
  }
  const double wall = ms_since(t_start);
  int iters = 0;
  for (auto &I : inst) {
    if (I.out->seconds == 0.0) I.out->seconds = wall / 1000.0;
    if (!I.done && I.out->status == SP_OK) I.out->status = SP_ERR_LIMIT;
    iters = std::max(iters, I.out->n_iter);
  }
  if (round0) s->stats.rounds = iters;  // threshold iterations, as in persistent mode
  s->stats.wall_ms = wall;
  return SP_OK;
}

bool config_ok(const sp_config *c) {
  return (c->threads_per_block == 128 || c->threads_per_block == 256) && c->frontier_target >= 1 &&
         c->frontier_target <= (1 << 20) && c->blocks_per_sm >= 0 && c->blocks_per_sm <= 16 &&
         c->lb_mode >= SP_LB_STEAL && c->lb_mode <= SP_LB_LEARNED && c->donate_min_slack >= 0 &&
         c->steps_per_poll >= 1 && c->steps_per_poll <= 4096 && c->timeout_ms >= 100 &&
         c->timeout_ms <= 600000 && c->static_split_cap >= 1 && c->donate_reserve >= -1 &&
         (c->persistent == 0 || c->persistent == 1) && c->handback_nodes >= 0;
}

}  // namespace

extern "C" {

void sp_config_default(sp_config *c) {
  if (!c) return;
  c->frontier_target = 3072;    // measured: 1-1.3 % faster than 2048 on the 15-puzzle batches
  c->threads_per_block = 256;
  c->blocks_per_sm = 0;
  c->lb_mode = SP_LB_STATIC_STEAL;
  c->donate_min_slack = 6;
  c->steps_per_poll = 32;
  c->timeout_ms = 20000;
  c->static_split_cap = 10;
  c->donate_reserve = 0;
  c->persistent = 1;            // device loop for the small iterations,
  c->handback_nodes = 600000;   // round loop from ~6e5 predicted nodes per instance iteration
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
  cudaFree(s->d_direct);
  cudaFree(s->d_sub_nodes);
  cudaFree(s->d_limit);
  cudaFree(s->d_sol);
  cudaFree(s->d_boards);
  cudaFree(s->d_h);
  cudaFree(s->d_cnt);
  cudaFree(s->d_split_a);
  cudaFree(s->d_split_b);
  cudaFree(s->d_emit);
  s->mb.release();
  s->fb.release();
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

int sp_root_set_template(int width, int blank, int target, uint64_t *paths, uint32_t cap, uint32_t *n_nodes,
                         uint32_t *depth, uint32_t *n_leaves) {
  if ((width != 4 && width != 5) || blank < 0 || blank >= width * width || target < 1 || target > (1 << 20) ||
      (cap && !paths) || !n_nodes || !depth || !n_leaves)
    return SP_ERR_ARG;
  FrontTemplate T;
  if (!build_template(width, blank, target, T)) return SP_ERR_CAPACITY;
  const uint32_t n = (uint32_t)T.path.size();
  *n_nodes = n;
  *depth = T.D;
  *n_leaves = T.lev[T.D + 1] - T.lev[T.D];
  for (uint32_t x = 0; x < std::min(cap, n); ++x) paths[x] = T.path[x];
  return SP_OK;
}

int sp_heuristic(sp_solver *s, const uint8_t *tiles, int n, int32_t *h) {
  if (!s || (n > 0 && (!tiles || !h)) || n < 0) return SP_ERR_ARG;
  if (s->heur == SP_HEUR_PDB && !s->pdb_ready) return SP_ERR_NO_PDB;
  if (n == 0) return SP_OK;
  for (int i = 0; i < n; ++i) {
    const int st = check_instance(s->w, tiles + (size_t)i * s->n);
    if (st == SP_ERR_NOT_PERMUTATION) return st;
  }
  int rc = ensure(s, &s->d_boards, &s->boards_cap, (size_t)n * s->n);
  if (rc) return rc;
  rc = ensure(s, &s->d_h, &s->h_cap, (size_t)n);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(s->d_boards, tiles, (size_t)n * s->n, cudaMemcpyHostToDevice, s->st);
  if (e == cudaSuccess)
    e = launch_heuristic(s->w, s->heur == SP_HEUR_PDB, s->d_boards, n, s->d_h, s->d_ht, s->d_pdb, s->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, s->d_h, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
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
  const int rc = solve_impl(s, h.data(), n, results);
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
  RoundPlan plan;
  plan.direct.resize((size_t)n);
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
    plan.direct[(size_t)i] = (uint32_t)i;
  }
  // roots that are goals (the reference's dfs_kernel sets dev_flag for them,
  // src/24puzzle_block_parallel_with_pdb.cu:580-583)
  std::vector<int32_t> h((size_t)n);
  int rc = sp_heuristic(s, roots, n, h.data());
  if (rc) return rc;
  for (int i = 0; i < n; ++i)
    if (h[(size_t)i] == 0 && (*found < 0 || depth[i] < *found)) *found = depth[i];
  rc = ensure(s, &s->d_subs, &s->subs_cap, (size_t)n);
  if (rc) return rc;
  rc = ensure(s, &s->d_sub_nodes, &s->sub_nodes_cap, (size_t)n);
  if (rc) return rc;
  if (!s->d_limit || s->inst_cap < 1) {
    SP_CUDA(s, cudaMalloc(&s->d_limit, 64 * sizeof(int32_t)));
    SP_CUDA(s, cudaMalloc(&s->d_sol, 64 * sizeof(Solution)));
    s->inst_cap = 64;
  }
  SP_CUDA(s, cudaMemcpyAsync(s->d_subs, subs.data(), subs.size() * sizeof(SubRoot), cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemcpyAsync(s->d_limit, &limit, sizeof(int32_t), cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemsetAsync(s->d_sol, 0, sizeof(Solution), s->st));
  SP_CUDA(s, cudaMemsetAsync(s->d_sub_nodes, 0, (size_t)n * sizeof(unsigned long long), s->st));
  float ms = 0;
  rc = launch_round(s, plan, (size_t)n, 1, &ms);
  if (rc) return rc;
  const PoolCtl &ctl = *s->h_ctl.p;
  memcpy(nodes, s->h_sub_nodes.p, (size_t)n * sizeof(uint64_t));
  fold_ctl(s, ctl, 0, ms);
  s->stats.rounds = 1;
  s->stats.tasks_initial = (uint64_t)n;
  s->stats.round_tasks[0] = n;
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
  const Solution &sol = s->h_sols.p[0];
  if (sol.flag && sol.best) {
    const int d = (int)(0xFFFFFFFFu - sol.best);
    if (*found < 0 || d < *found) *found = d;
  }
  for (int i = 0; i < n; ++i) s->stats.nodes += nodes[i];
  return SP_OK;
}

int sp_selftest_stall(sp_solver *s, int timeout_ms, int32_t *device_status) {
  if (!s || !device_status || timeout_ms < 100 || timeout_ms > 60000) return SP_ERR_ARG;
  *device_status = SP_OK;
  int rc = ensure_pool(s, 1);
  if (rc) return rc;
  if ((rc = ensure(s, &s->d_subs, &s->subs_cap, 1)) || (rc = ensure(s, &s->d_sub_nodes, &s->sub_nodes_cap, 1)))
    return rc;
  if (!s->d_limit || s->inst_cap < 1) {
    SP_CUDA(s, cudaMalloc(&s->d_limit, 64 * sizeof(int32_t)));
    SP_CUDA(s, cudaMalloc(&s->d_sol, 64 * sizeof(Solution)));
    s->inst_cap = 64;
  }
  // an empty pool, then one task counted as queued at index 0 that no
  // producer ever publishes: every lane that claims it waits for it
  SP_CUDA(s, launch_pool_init(s->d_tasks, nullptr, nullptr, nullptr, 0, s->d_seq, s->cap, s->d_ctl, nullptr, nullptr,
                              s->st));
  SP_CUDA(s, s->h_cnt.reserve(4));
  s->h_cnt.p[0] = 1;
  SP_CUDA(s, cudaMemcpyAsync(&s->d_ctl->tail, s->h_cnt.p, sizeof(uint32_t), cudaMemcpyHostToDevice, s->st));
  SP_CUDA(s, cudaMemcpyAsync(&s->d_ctl->outstanding, s->h_cnt.p, sizeof(uint32_t), cudaMemcpyHostToDevice, s->st));
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
  P.donate = 1;
  P.timeout_ns = (unsigned long long)timeout_ms * 1000000ull;
  P.poll_ns = SP_POLL_NS;
  P.reserve = 0;
  P.spread = 1;
  int grid = 0;
  const int block = s->cfg.threads_per_block == 128 ? 128 : 256;
  SP_CUDA(s, launch_search_round(s->w, s->heur == SP_HEUR_PDB, block, s->cfg.blocks_per_sm, s->num_sms, P, s->st,
                                 &grid));
  SP_CUDA(s, s->h_ctl.reserve(1));
  SP_CUDA(s, cudaMemcpyAsync(s->h_ctl.p, s->d_ctl, sizeof(PoolCtl), cudaMemcpyDeviceToHost, s->st));
  SP_CUDA(s, cudaStreamSynchronize(s->st));
  *device_status = s->h_ctl.p->error;
  return SP_OK;
}

uint64_t sp_lbm_num_params(int width) {
  return (width == 4 || width == 5) ? (uint64_t)lbm::num_params(width) : 0;
}

static int lbm_model(sp_solver *s, bool need_ready) {
  if (!s) return SP_ERR_ARG;
  if (!s->lbm) s->lbm.reset(new lbm::Model(s->w));
  if (need_ready && !s->lbm->ready()) {
    s->err = "no model: call sp_lbm_init or sp_lbm_import first";
    return SP_ERR_ARG;
  }
  return SP_OK;
}

int sp_lbm_init(sp_solver *s, uint64_t seed) {
  int rc = lbm_model(s, false);
  return rc ? rc : s->lbm->init(seed, s->st, s->err);
}

int sp_lbm_import(sp_solver *s, const float *src, uint64_t n) {
  if (!src) return SP_ERR_ARG;
  int rc = lbm_model(s, false);
  return rc ? rc : s->lbm->import_params(src, (size_t)n, s->st, s->err);
}

int sp_lbm_export(sp_solver *s, float *dst, uint64_t n) {
  if (!dst) return SP_ERR_ARG;
  int rc = lbm_model(s, true);
  return rc ? rc : s->lbm->export_params(dst, (size_t)n, s->st, s->err);
}

static int lbm_check_rows(sp_solver *s, const uint8_t *tiles, const int32_t *slack, int n) {
  if (!tiles || !slack || n < 0) return SP_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    if (slack[i] < 0 || slack[i] > 255) {
      s->err = "slack must lie in 0..255";
      return SP_ERR_ARG;
    }
    uint32_t seen = 0;
    for (int c = 0; c < s->n; ++c) {
      const uint8_t t = tiles[(size_t)i * s->n + c];
      if (t >= s->n || ((seen >> t) & 1u)) {
        s->err = "tiles are not a permutation";
        return SP_ERR_NOT_PERMUTATION;
      }
      seen |= 1u << t;
    }
  }
  return SP_OK;
}

int sp_lbm_predict(sp_solver *s, const uint8_t *tiles, const int32_t *slack, int n, float *out) {
  int rc = lbm_model(s, true);
  if (!rc) rc = lbm_check_rows(s, tiles, slack, n);
  if (rc) return rc;
  if (!out) return SP_ERR_ARG;
  return n ? s->lbm->predict(tiles, slack, n, out, s->st, s->err) : SP_OK;
}

int sp_lbm_train_step(sp_solver *s, const uint8_t *tiles, const int32_t *slack, const float *target, int n,
                      float lr, float *loss) {
  int rc = lbm_model(s, true);
  if (!rc) rc = lbm_check_rows(s, tiles, slack, n);
  if (rc) return rc;
  if (!target || !(lr > 0.f)) return SP_ERR_ARG;
  return s->lbm->train_step(tiles, slack, target, n, lr, true, loss, nullptr, s->st, s->err);
}

int sp_lbm_gradients(sp_solver *s, const uint8_t *tiles, const int32_t *slack, const float *target, int n,
                     float *grads, float *loss) {
  int rc = lbm_model(s, true);
  if (!rc) rc = lbm_check_rows(s, tiles, slack, n);
  if (rc) return rc;
  if (!target || !grads) return SP_ERR_ARG;
  return s->lbm->train_step(tiles, slack, target, n, 0.f, false, loss, grads, s->st, s->err);
}

int sp_gemm_bf16_nt(const uint16_t *a, const uint16_t *b, float *c, int m, int n, int k) {
  if (!a || !b || !c) return SP_ERR_ARG;
  std::string err;
  return lbm::Model::gemm_nt(a, b, c, m, n, k, nullptr, err);
}

int sp_selftest_gemm_stall(int32_t starve_chunk, int32_t timeout_ms, int32_t *device_status) {
  if (!device_status) return SP_ERR_ARG;
  std::string err;
  int st = 0;
  const int rc = lbm::Model::gemm_stall_selftest(starve_chunk, timeout_ms, &st, nullptr, err);
  *device_status = st;
  return rc;
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
