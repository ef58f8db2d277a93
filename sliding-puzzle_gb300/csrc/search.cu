// Threshold-round search kernel of libslide.
//
// One launch searches one IDA* threshold for every unsolved instance of a
// batch.  It replaces the reference's per-round dfs_kernel
// (src/24puzzle_block_parallel_with_pdb.cu:520-648: one 32-thread block per
// root, 8 nodes x 4 moves per round, three __syncthreads per round, a
// 326-entry shared Node stack) with:
//
//  * one lane = one depth-first search over a task (a root-set node, possibly
//    narrowed to some of its first moves); no block barriers in the loop;
//  * the lane's path kept as 2-bit moves in shared memory (a [word][lane]
//    layout, so lanes never conflict on banks) and undone move by move;
//  * 15-puzzle boards packed 4 bits per cell in one 64-bit register, 24-puzzle
//    boards as bytes in shared memory;
//  * Manhattan distance updated from a per-(move, cell, tile) delta table in
//    shared memory (src/15puzzle_block_parallel.cu:271-272 updates it with two
//    constant-memory lookups);
//  * PDB indices kept per pattern as mixed-radix integers and updated by one
//    add per move, so a generated child costs one regular and one reflected
//    table lookup instead of the reference's eight
//    (src/24puzzle_block_parallel_with_pdb.cu:426-429); the idea of updating
//    only the moved tile's pattern is Horie's (src_horie/idas_pdb.cu:221-254);
//    undoing a move restores the two overwritten pattern values from a
//    per-level save in shared memory instead of looking them up again;
//  * generating a child and undoing a move share one code path (both slide
//    one tile into the blank), which keeps a warp's lanes converged while
//    they are at different points of their walks;
//  * load balance by a device task pool: lanes claim slots warp-aggregated
//    (ballot + one atomicAdd per warp); claims may run ahead of the pool's
//    tail, and while any lane waits, busy lanes donate the untried moves of
//    their shallowest open level as a new task (the reference's closest
//    counterpart is Horie's intra-warp sharing, src_horie/idas_dynamic.cu
//    :200-247; the reference's own balance is the host re-split of
//    :839-897, done by the host round loop here).
//
// The multi-iteration variant (MULTI) runs every instance's whole threshold
// loop in one launch: the warp whose lane finishes an instance's last task of
// an iteration publishes that instance's next iteration (warp_advance), so
// instances never wait for each other and the host is not involved between
// iterations.  Its heavy roots go out as split tasks that expand one level
// per claim (breadth-first across lanes); an instance whose next iteration
// is predicted to be large is handed back to the host round loop.
//
// Every wait is bounded: a warp whose lanes all wait and see no change of the
// pool for timeout_ns sets SP_ERR_TIMEOUT and every warp returns.  Nothing
// traps.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/slide.h"
#include "sp_defs.h"
#include "sp_device.cuh"
#include "sp_kernels.h"

namespace sp {

namespace {

// Pool words are read with GPU-scope relaxed loads (coherent across SMs, never
// served from a stale L1 line); readiness of a slot with an acquire load, so
// the record written before its release store is visible.
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int32_t ld_volatile(const int32_t *p) {
  int32_t v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Pattern-index field helpers.  Width 4: three 20-bit indices in one u64 per
// partition.  Width 5: four 28-bit indices, two per u64.
template <int W>
struct Idx;

template <>
struct Idx<4> {
  uint64_t a;
  __device__ __forceinline__ void clear() { a = 0; }
  __device__ __forceinline__ uint32_t get(int p) const { return (uint32_t)(a >> (20 * p)) & 0xFFFFFu; }
  __device__ __forceinline__ void add(int p, int32_t d) { a += (uint64_t)((int64_t)d << (20 * p)); }
};

template <>
struct Idx<5> {
  uint64_t a, b;
  __device__ __forceinline__ void clear() { a = b = 0; }
  __device__ __forceinline__ uint32_t get(int p) const {
    uint64_t w = (p >> 1) ? b : a;
    return (uint32_t)(w >> (28 * (p & 1))) & 0xFFFFFFFu;
  }
  __device__ __forceinline__ void add(int p, int32_t d) {
    uint64_t v = (uint64_t)((int64_t)d << (28 * (p & 1)));
    if (p >> 1) b += v; else a += v;
  }
};

__device__ __forceinline__ uint32_t byte_sum(uint32_t v) { return __dp4a(v, 0x01010101u, 0u); }

// The step's move arithmetic without compares: the four blank
// displacements as signed bytes of one immediate, and for the 24-puzzle the
// 4-bit legal-move mask of every cell packed into two 64-bit immediates
// (measured: -3 % step time on the 15-puzzle for the first, +5 % nodes/s on
// the 24-puzzle for both; the packed masks cost the 15-puzzle kernel a
// spill, so it keeps legal_moves).
constexpr uint64_t legal_pack(int w, int first, int count) {
  uint64_t v = 0;
  for (int c = 0; c < count; ++c) {
    const int cell = first + c, r = cell / w, cc = cell % w;
    const uint64_t m = (r > 0 ? 1u : 0u) | (cc < w - 1 ? 2u : 0u) | (cc > 0 ? 4u : 0u) | (r < w - 1 ? 8u : 0u);
    v |= m << (4 * c);
  }
  return v;
}
template <int W>
__device__ __forceinline__ uint32_t step_legal(int blank) {
  if (W == 4) return legal_moves(W, blank);
  const uint64_t w = blank < 16 ? legal_pack(5, 0, 16) : legal_pack(5, 16, 9);
  return (uint32_t)(w >> (4 * (blank & 15))) & 15u;
}
template <int W>
__device__ __forceinline__ int step_delta(int d) {
  constexpr uint32_t pack = W == 4 ? 0x04FF01FCu : 0x05FF01FBu;  // -W, +1, -1, +W
  return (int)(pack << (24 - 8 * d)) >> 24;
}
__device__ __forceinline__ uint32_t set_byte(uint32_t v, int p, uint32_t x) {
  return (v & ~(0xFFu << (8 * p))) | (x << (8 * p));
}

}  // namespace

// Multi-iteration mode: split-piece load in units of the instance's average
// root load (1, 2 and 4 measure alike).
#ifndef SP_MULTI_PIECE
#define SP_MULTI_PIECE 1.0
#endif

// Iteration r of instance i, published beside the one before it (warp
// advance below): its limit and solution record (those of r - 2, whose goal
// flag is clear), loads zeroed, its na roots (in maxf order, unsplit) at
// pool indices t0 ... t0 + na - 1, already reserved.  Kept out of line so
// that the search loop's registers do not pay for it.
__device__ __noinline__ void publish_second(const RoundParams &P, uint32_t i, int r, int L, uint32_t base,
                                            uint32_t ns, uint32_t t0, uint32_t na) {
  const int lane = threadIdx.x & 31;
  PoolCtl *ctl = P.ctl;
  if (lane == 0) {
    const_cast<int32_t *>(P.inst_limit)[2 * i + (r & 1)] = L;
    P.inst_pair[i] = 1u;
  }
  unsigned long long *lz = P.sub_loads + (size_t)(r & 1) * P.n_subs + base;
  for (uint32_t q = lane; q < ns; q += 32) lz[q] = 0;
  __threadfence();
  __syncwarp();
  const uint32_t mask = P.cap - 1u;
  for (uint32_t q = lane; q < na; q += 32) {
    const uint32_t t = t0 + q;
    bool free_slot = false;
    for (int spin = 0; spin < (1 << 14) && !free_slot; ++spin) {
      free_slot = ld_acquire(&P.seq[t & mask]) == t;
      if (!free_slot) __nanosleep(64);
    }
    if (!free_slot) {
      if (atomicCAS(&ctl->error, 0, SP_ERR_CAPACITY) == 0) ctl->err_info[0] = t;
      continue;
    }
    Task *D = &P.tasks[t & mask];
    D->sub = base + q;
    D->plen = 0;
    D->mask = 0xF;
    D->flags = (uint8_t)((r & 1) << 6);
    st_release(&P.seq[t & mask], t + 1u);
  }
  __syncwarp();
}

// Multi-iteration mode: the warp of the lane that finished an instance's last
// task of an iteration completes that iteration (adds the root-set interior
// count, checks for a goal) and publishes the next iteration's roots -- the
// threshold loop of src/24puzzle_block_parallel_with_pdb.cu:772-921 run on the
// device, per instance, with no barrier across instances.  Called by all 32
// lanes of a warp with the same instance i; `hist` is the warp's 32 words of
// shared memory.  Kept out of line: it is cold, and inlined its registers
// would crowd the search loop.  When the instance's next iteration is
// predicted small (below P.pair_nodes) it is published together with this
// one, and the call that completes such a pair settles both in order.
__device__ __noinline__ void warp_advance(const RoundParams &P, uint32_t i, uint32_t *hist) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  PoolCtl *ctl = P.ctl;
  auto interior = [&](int L) -> unsigned long long {
    const uint32_t off = P.inter_off[i];
    int lo = 0, hi = (int)P.inter_len[i];  // first entry with f > L
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (P.inter_f[off + mid] <= L) lo = mid + 1;
      else hi = mid;
    }
    return lo ? P.inter_cum[off + lo - 1] : 0ull;
  };
  // per instance, two limits and two solution records, by iteration parity
  int r = ld_volatile(&P.inst_iter[i]);
  int L = ld_volatile(&P.inst_limit[2 * i + (r & 1)]);
  if (lane == 0) atomicAdd(&P.iter_nodes[(size_t)i * kMaxIters + r], interior(L));
  if (ld_volatile(&P.inst_pair[i])) {
    // iterations r and r + 1 ran together and have both finished: r's goal
    // decides first (r + 1's counts are then never read)
    int stop = 0;
    if (lane == 0) stop = (ld_volatile(&P.sol[2 * i + (r & 1)].flag) != 0u || P.goal_maxf[i] <= L) ? 1 : 0;
    stop = __shfl_sync(FULL, stop, 0);
    if (stop || r + 1 >= kMaxIters) {
      if (lane == 0) {
        P.inst_final[i] = r;
        P.inst_fin_ns[i] = globaltimer();
        if (!stop) P.inst_status[i] = SP_ERR_LIMIT;
      }
      return;
    }
    ++r;
    L += 2;
    if (lane == 0) {
      P.inst_iter[i] = r;
      P.inst_pair[i] = 0u;
      atomicAdd(&P.iter_nodes[(size_t)i * kMaxIters + r], interior(L));
    }
  }
  for (;;) {
    // every task of iteration r has finished: the goal flag is final
    int stop = 0;
    if (lane == 0) stop = (ld_volatile(&P.sol[2 * i + (r & 1)].flag) != 0u || P.goal_maxf[i] <= L) ? 1 : 0;
    stop = __shfl_sync(FULL, stop, 0);
    if (stop || r + 1 >= kMaxIters) {
      if (lane == 0) {
        P.inst_final[i] = r;
        P.inst_fin_ns[i] = globaltimer();
        if (!stop) P.inst_status[i] = SP_ERR_LIMIT;
      }
      return;
    }
    ++r;
    L += 2;
    const uint32_t base = P.inst_sub_base[i], ns = P.inst_nsub[i];
    uint32_t lo = 0, hi = ns;  // active roots: prefix with maxf <= L
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (P.sub_maxf[base + mid] <= L) lo = mid + 1;
      else hi = mid;
    }
    const uint32_t na = lo;
    if (lane == 0) {
      P.inst_iter[i] = r;
      const_cast<int32_t *>(P.inst_limit)[2 * i + (r & 1)] = L;
      if (!na) atomicAdd(&P.iter_nodes[(size_t)i * kMaxIters + r], interior(L));
    }
    if (!na) continue;
    // loads of iteration r - 1 (summed by atomics in L2: read past L1)
    const unsigned long long *ld = P.sub_loads + (size_t)((r - 1) & 1) * P.n_subs + base;
    unsigned long long *nx = P.sub_loads + (size_t)(r & 1) * P.n_subs + base;
    unsigned long long tot = 0;
    for (uint32_t q = lane; q < na; q += 32) tot += __ldcg(ld + q);
    for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
    // the next iteration's size: this one's times the instance's growth
    double grow = 6.0;
    if (r >= 2) {
      const unsigned long long prev = __ldcg(&P.iter_nodes[(size_t)i * kMaxIters + (r - 2)]);
      if (prev) grow = fmin(30.0, fmax(2.0, (double)tot / (double)prev));
    }
    if (P.handback_nodes && (double)tot * grow >= (double)P.handback_nodes) {
      // a large iteration is next: the host round loop finishes this
      // instance (its loads of iteration r - 1 stay in `ld`)
      if (lane == 0) {
        P.inst_final[i] = r - 1;
        P.inst_fin_ns[i] = globaltimer();
        P.inst_status[i] = kStatusHandback;
      }
      return;
    }
    // next-iteration load of root q: its load times its predicted growth
    // (learned balancer; otherwise the load itself, the instance's growth
    // being common to all its roots)
    auto pred_load = [&](uint32_t q) -> double {
      double lq = (double)__ldcg(ld + q);
      if (P.sub_growth && lq > 0.0) {
        const int j = min(kGrowthSlacks - 1, max(0, (L - 2 - P.sub_maxf[base + q]) >> 1));
        lq *= exp2((double)P.sub_growth[(size_t)(base + q) * kGrowthSlacks + j] * (1.0 / 16.0));
      }
      return lq;
    };
    double ptot = (double)tot;
    if (P.sub_growth) {
      ptot = 0.0;
      for (uint32_t q = lane; q < na; q += 32) ptot += pred_load(q);
      for (int o = 16; o; o >>= 1) ptot += __shfl_xor_sync(FULL, ptot, o);
    }
    const double avg = ptot / (double)na;
    for (uint32_t q = lane; q < ns; q += 32) nx[q] = 0;
    // longest first: bucket = binary exponent of load / average (0 = no load)
    auto bucket = [&](double lq) -> int {
      if (!(lq > 0.0) || !(avg > 0.0)) return 0;
      int e = 0;
      frexp(lq / avg, &e);
      return min(31, max(1, e + 15));
    };
    hist[lane] = 0;
    __syncwarp();
    for (uint32_t q = lane; q < na; q += 32) atomicAdd(&hist[bucket(pred_load(q))], 1u);
    __syncwarp();
    const uint32_t c = hist[lane];
    uint32_t suf = c;  // roots in buckets >= lane
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_down_sync(FULL, suf, o);
      if (lane + o < 32) suf += v;
    }
    hist[lane] = suf - c;  // first position of bucket `lane`
    // iteration r + 1 goes out with r when it is predicted small: the two
    // run together and the instance advances once both have finished, so a
    // chain of small iterations is not paced by one iteration at a time
    uint32_t na2 = 0;
    if (P.pair_nodes && r + 2 < kMaxIters && (double)tot * grow * grow < (double)P.pair_nodes) {
      uint32_t lo2 = na, hi2 = ns;  // active roots of r + 1: prefix with maxf <= L + 2
      while (lo2 < hi2) {
        const uint32_t mid = (lo2 + hi2) >> 1;
        if (P.sub_maxf[base + mid] <= L + 2) lo2 = mid + 1;
        else hi2 = mid;
      }
      na2 = lo2;
    }
    // the whole iteration (pair) is outstanding before its first task is visible
    uint32_t t0 = 0;
    if (lane == 0) {
      atomicAdd(&P.inst_out[i], na + na2);
      atomicAdd(&ctl->outstanding, na + na2);
      t0 = atomicAdd(&ctl->tail, na + na2);
      __threadfence();
    }
    t0 = __shfl_sync(FULL, t0, 0);
    __syncwarp();
    const uint32_t mask = P.cap - 1u;
    for (uint32_t q = lane; q < na; q += 32) {
      const double lq = pred_load(q);
      const uint32_t t = t0 + atomicAdd(&hist[bucket(lq)], 1u);
      int kk = 0;
      const double piece = avg * SP_MULTI_PIECE;
      if (P.static_split && piece > 0 && lq > 2.0 * piece) {
        // static split from the loads just measured: a root with x pieces'
        // load goes out as a split task of about log(x)/log(2.4) levels (the
        // reference cuts it into ceil(load/avg) pieces,
        // src/24puzzle_block_parallel_with_pdb.cu:839-897)
        kk = (int)ceil(log(lq / piece) / log(2.4));
        kk = max(0, min(kk, min(10, L - (int)P.subs[base + q].g - 1)));
      }
      bool free_slot = false;
      for (int spin = 0; spin < (1 << 14) && !free_slot; ++spin) {
        free_slot = ld_acquire(&P.seq[t & mask]) == t;
        if (!free_slot) __nanosleep(64);
      }
      if (!free_slot) {
        if (atomicCAS(&ctl->error, 0, SP_ERR_CAPACITY) == 0) ctl->err_info[0] = t;
        continue;
      }
      Task *D = &P.tasks[t & mask];
      D->sub = base + q;
      D->plen = 0;
      D->mask = 0xF;
      D->flags = (uint8_t)(kk | ((r & 1) << 6));  // bit 6: the iteration's parity
      st_release(&P.seq[t & mask], t + 1u);
    }
    __syncwarp();
    if (na2) publish_second(P, i, r + 1, L + 2, base, ns, t0 + na, na2);
    return;
  }
}

// Resident threads per SM the search kernels are compiled for (the register
// budget: 768 threads leave 80 registers a thread; 24 warps per SM hide the
// pattern-table latency markedly better than 16).
// Most lanes of a warp that donate in one pass of its loop.
#ifndef SP_MAX_DONORS
#define SP_MAX_DONORS 8
#endif

// Longest sleep of a warp with no lane searching between pool polls (ns).
#ifndef SP_MAX_BACKOFF_NS
#define SP_MAX_BACKOFF_NS 16384
#endif

#ifndef SP_SEARCH_THREADS_PER_SM
#define SP_SEARCH_THREADS_PER_SM 768
#endif

template <int W, bool PDB, int BLOCK, int WORDS, bool MULTI>
__global__ void __launch_bounds__(BLOCK, SP_SEARCH_THREADS_PER_SM / BLOCK) search_round_kernel(RoundParams P) {
  constexpr int N = W * W;
  constexpr int BSTRIDE = 28;  // bytes per lane board (7 words: conflict-free same-cell access)
  constexpr int MAXLEV = WORDS * 16;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ uint32_t s_code[PDB ? 2 * N * N : 1];
  __shared__ uint8_t s_pat[PDB ? 2 * N : 1];
  __shared__ int8_t s_mdd[PDB ? 1 : 4 * N * N];
  __shared__ uint32_t s_stack[WORDS][BLOCK];
  __shared__ uint32_t s_prefix[kPathWords][BLOCK];  // the lane's task prefix (its pool slot is freed)
  // PDB: the two pattern values (regular, reflected) a descent overwrote, per
  // level, so that backtracking restores them without table lookups; levels
  // from HSAVE on look them up again
  constexpr int HSAVE = PDB ? (W == 4 ? 64 : 32) : 1;
  __shared__ uint16_t s_hsave[HSAVE][BLOCK];
  __shared__ __align__(16) uint8_t s_board[W == 5 ? BLOCK * BSTRIDE : 4];
  // multi-iteration mode: per-warp bucket counts of the longest-first publication
  __shared__ uint32_t s_hist[MULTI ? BLOCK / 32 : 1][32];
  __shared__ uint32_t s_cold[3][BLOCK];  // per-lane data of rare events (below)
  // block-wide cache of the pool state: at most one global poll per block per poll_ns
  __shared__ uint32_t s_pool[5];  // head, tail, error, outstanding, heartbeat
  __shared__ unsigned long long s_pool_t;
  if (threadIdx.x == 0) {
    s_pool[0] = s_pool[1] = s_pool[2] = s_pool[4] = 0;
    s_pool[3] = 1;
    s_pool_t = 0;
    if (MULTI) atomicMin(P.t_begin_ns, globaltimer());
  }

  const HeurTables *ht = P.ht;
  if (PDB) {
    for (int i = threadIdx.x; i < N * N; i += BLOCK) {
      s_code[i] = ht->code[0][i];
      s_code[N * N + i] = ht->code[1][i];
    }
    for (int i = threadIdx.x; i < N; i += BLOCK) {
      s_pat[i] = ht->pat[0][i];
      s_pat[N + i] = ht->pat[1][i];
    }
  } else {
    for (int i = threadIdx.x; i < 4 * N * N; i += BLOCK) s_mdd[i] = ht->mdd[i];
  }
  __syncthreads();

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  uint8_t *myboard = s_board + (W == 5 ? tid * BSTRIDE : 0);
  PoolCtl *ctl = P.ctl;

  // ---- lane state -------------------------------------------------------
  int state = 0;  // 0 idle, 1 holds a claimed slot, 2 searching
  uint32_t slot = 0;
  uint64_t b64 = 0;  // width-4 board
  int blank = 0, g = 0, h = 0, k = 0, it = 0, pre = -1, limit = 0;
  int rblank = 0, rpre = -1, groot = 0, plen = 0;
  uint32_t mask0 = 0, top = 0, sub = 0;
  uint64_t cut = 0;
  uint32_t lo = 0;  // donation walk cache: level | blank << 8 | (incoming move + 1) << 16
  unsigned long long cnt = 0;
  Idx<W> ir, iff;
  uint32_t hvr = 0, hvf = 0;
  ir.clear();
  iff.clear();
  unsigned long long c_tries = 0, c_notfree = 0, c_nowait = 0, c_done = 0, c_found = 0;  // donation counters
  // the task's instance; multi-iteration mode: bit 31 = the parity of the
  // task's iteration (kept in the same register: the search loop has none to spare)
  uint32_t cur_inst = 0;
  int splitk = 0;         // split task: hand every node at this relative depth to the pool
  bool emit_pending = false;
  // Rare per-lane events, flags in a register and their data in shared memory:
  //  * kAdvance: the lane finished an instance's iteration; the warp advances
  //    that instance (s_cold[0]) at the top of its next loop;
  //  * kDebt: a reserved pool index (s_cold[1]) whose ring slot did not free
  //    in time is owed: the lane kept the work and publishes a null task (no
  //    moves, SubRoot s_cold[2]) there later, so no index stays unpublished.
  constexpr uint32_t kAdvance = 1u, kDebt = 2u;
  uint32_t events = 0;

  auto tile_at = [&](int c) -> int {
    if (W == 4) return (int)((b64 >> (4 * c)) & 15u);
    return myboard[c];
  };
  // slide tile t from cell `from` into the blank at cell `to`
  auto slide = [&](int t, int from, int to) {
    if (W == 4) {
      b64 ^= ((uint64_t)t << (4 * from)) ^ ((uint64_t)t << (4 * to));
    } else {
      myboard[to] = (uint8_t)t;
      myboard[from] = 0;
    }
  };
  auto lookup = [&](int p, uint32_t idx) -> uint32_t {
    size_t off = (W == 4) ? ((size_t)p << 20) : (p ? ((size_t)1 << 28) : 0);
    return __ldg(P.pdb + off + idx);
  };
  auto stack_dir = [&](int i) -> int {
    uint32_t w = ((i >> 4) < (k >> 4)) ? s_stack[i >> 4][tid] : top;
    return (int)((w >> (2 * (i & 15))) & 3u);
  };
  auto task_dir = [&](int i) -> int {
    return (int)((s_prefix[i >> 4][tid] >> (2 * (i & 15))) & 3u);
  };
  // moves 0..len-1 of the lane's path below its SubRoot: task prefix then stack
  auto path_word = [&](int wi, int len) -> uint32_t {
    uint32_t out = 0;
    for (int b = 0; b < 16; ++b) {
      int j = wi * 16 + b;
      if (j >= len) break;
      int d = j < plen ? task_dir(j) : stack_dir(j - plen);
      out |= (uint32_t)d << (2 * b);
    }
    return out;
  };
  auto full_h = [&]() -> int {
    if (PDB) {
      ir.clear();
      iff.clear();
      for (int c = 0; c < N; ++c) {
        int t = tile_at(c);
        if (!t) continue;
        ir.add(s_pat[t], (int32_t)s_code[t * N + c]);
        iff.add(s_pat[N + t], (int32_t)s_code[N * N + t * N + c]);
      }
      hvr = hvf = 0;
      constexpr int NP = (W == 5) ? 4 : 3;
      for (int p = 0; p < NP; ++p) {
        hvr = set_byte(hvr, p, lookup(W == 5 ? (p != 0) : p, ir.get(p)));
        hvf = set_byte(hvf, p, lookup(W == 5 ? (p != 0) : p, iff.get(p)));
      }
      return (int)max(byte_sum(hvr), byte_sum(hvf));
    } else {
      int s = 0;
      for (int c = 0; c < N; ++c) {
        int t = tile_at(c);
        if (!t) continue;
        int dr = c / W - t / W, dc = c % W - t % W;
        s += abs(dr) + abs(dc);
      }
      return s;
    }
  };
  auto set_error = [&](int code, uint32_t info) {
    if (atomicCAS(&ctl->error, 0, code) == 0) ctl->err_info[0] = info;
  };
  // Wait a bounded time for the ring slot of reserved pool index t (normally
  // free at once: its previous occupant, index t - cap, was claimed long
  // before).
  auto slot_free = [&](uint32_t t, int spins) -> bool {
    for (int spin = 0; spin < spins; ++spin) {
      if (ld_acquire(&P.seq[t & (P.cap - 1u)]) == t) return true;
      __nanosleep(64);
    }
    return false;
  };
  auto finish_task = [&]() {
    ++c_done;
    state = 0;
    if (MULTI) {
      if (cnt) {
        // the instance stays in its current iteration while the task is
        // outstanding; the task's own is that one or, in a pair, the next
        const uint32_t ci = cur_inst & 0x7FFFFFFFu, tp = cur_inst >> 31;
        const int cur_iter = ld_volatile(&P.inst_iter[ci]);
        const int task_iter = cur_iter + (((uint32_t)cur_iter & 1u) != tp ? 1 : 0);
        atomicAdd(&P.iter_nodes[(size_t)ci * kMaxIters + task_iter], cnt);
        atomicAdd(&P.sub_loads[(size_t)tp * P.n_subs + sub], cnt);
      }
      __threadfence();
      // the last task of the iteration: the warp advances the instance at the
      // top of its next loop, and only then does this task leave
      // `outstanding`, so that never reads 0 while work is still to come
      if (atomicSub(&P.inst_out[cur_inst & 0x7FFFFFFFu], 1u) == 1u) {
        events |= kAdvance;
        s_cold[0][tid] = cur_inst & 0x7FFFFFFFu;
        return;
      }
    } else if (cnt) {
      atomicAdd(&P.sub_nodes[sub], cnt);
    }
    __threadfence();
    atomicSub(&ctl->outstanding, 1u);
  };
  // Copy the claimed record out of its ring slot, then free the slot for the
  // producer of index slot + cap.
  auto take_task = [&]() {
    const uint32_t s = slot & (P.cap - 1u);
    const Task *T = &P.tasks[s];
    sub = __ldcg(&T->sub);
    const uint32_t hdr = __ldcg((const uint32_t *)T + 1);
    plen = (int)(hdr & 0xFFFFu);
    mask0 = (hdr >> 16) & 0xFu;
    splitk = MULTI ? (int)((hdr >> 24) & 0x3Fu) : (int)(hdr >> 24);
    cur_inst = MULTI ? (hdr << 1) & 0x80000000u : 0u;  // the parity bit until start_task adds the instance
    for (int wi = 0; wi < kPathWords; ++wi) s_prefix[wi][tid] = __ldcg(&T->path[wi]);
    st_release(&P.seq[s], slot + P.cap);  // the copy above completes before the slot is reused
  };
  auto start_task = [&]() -> bool {
    const SubRoot *R = &P.subs[sub];
    const uint8_t *rb = R->board;
    if (W == 4) {
      uint4 v = *(const uint4 *)rb;
      const uint8_t *bb = (const uint8_t *)&v;
      b64 = 0;
      for (int c = 0; c < 16; ++c) b64 |= (uint64_t)(bb[c] & 15u) << (4 * c);
    } else {
      for (int c = 0; c < N; ++c) myboard[c] = rb[c];
    }
    uint4 tailv = *(const uint4 *)(rb + 16);
    const uint8_t *tb = (const uint8_t *)&tailv;
    blank = tb[25 - 16];
    g = tb[26 - 16];
    pre = tb[27 - 16] == kNoPre ? -1 : (int)tb[27 - 16];
    uint32_t inst = *(const uint32_t *)(tb + 12);
    if (MULTI) {
      limit = ld_volatile(&P.inst_limit[2 * inst + (cur_inst >> 31)]);
      cur_inst |= inst;
    } else {
      cur_inst = inst;
      limit = P.inst_limit[inst];
    }
    for (int i = 0; i < plen; ++i) {
      int d = task_dir(i);
      if (!((legal_moves(W, blank) >> d) & 1u)) {  // corrupt record: never index off the board
        set_error(SP_ERR_ARG, 0x100u + (uint32_t)i);
        return false;
      }
      int src = blank + move_delta(W, d);
      slide(tile_at(src), src, blank);
      blank = src;
      pre = d;
      ++g;
    }
    h = full_h();
    rblank = blank;
    rpre = pre;
    groot = g;
    lo = ((uint32_t)rblank << 8) | ((uint32_t)(rpre + 1) << 16);
    k = 0;
    it = 0;
    top = 0;
    cut = 0;
    cnt = 0;
    return g + h <= limit;
  };
  auto record_goal = [&]() {
    const uint32_t si = P.subs[sub].inst;
    Solution *S = &P.sol[MULTI ? 2 * si + (cur_inst >> 31) : si];
    atomicMax(&S->best, 0xFFFFFFFFu - (uint32_t)g);  // shortest goal depth over all lanes
    if (atomicCAS(&S->flag, 0u, 1u) == 0u) {
      int len = plen + k;
      S->sub = sub;
      S->len = (uint32_t)len;
      for (int wi = 0; wi < kPathWords; ++wi) S->path[wi] = path_word(wi, len);
      __threadfence();
    }
  };

  // One edge of the depth-first search: generate the next child of the
  // current node, or undo the move into the current node.  Both slide one
  // tile into the blank's cell and update the pattern index the same way, so
  // they share one code path (lanes of a warp at different points of their
  // walks stay converged); only the child's table lookups, the f-test and
  // the stack bookkeeping differ.  Returns true when the task is exhausted.
  auto step = [&]() -> bool {
    // minus the reverse of the move into this node: its bit from a nibble
    // table indexed by pre + 1 (pre = -1 at a task root without one)
    uint32_t cand = step_legal<W>(blank) & (0xFu << it) & ~((0x12480u >> (4 * (pre + 1))) & 15u);
    if (k == 0) cand &= mask0;
    const bool gen = cand != 0;
    if (!gen && k == 0) return true;
    int dm;  // the blank's move this step
    if (gen) {
      dm = __ffs(cand) - 1;
    } else {
      --k;
      if ((k & 15) == 15) top = s_stack[k >> 4][tid];
      dm = 3 - (int)((top >> (2 * (k & 15))) & 3u);  // the reverse of the move into level k + 1
    }
    const int from = blank + step_delta<W>(dm);
    const int t = tile_at(from);  // slides from `from` into the blank's cell
    int nh;
    uint32_t nhvr = hvr, nhvf = hvf;
    Idx<W> nir = ir, nif = iff;
    int pr = 0, pf = 0;
    if (PDB) {
      pr = s_pat[t];
      pf = s_pat[N + t];
      nir.add(pr, (int32_t)(s_code[t * N + blank] - s_code[t * N + from]));
      nif.add(pf, (int32_t)(s_code[N * N + t * N + blank] - s_code[N * N + t * N + from]));
      if (gen || k >= HSAVE) {
        nhvr = set_byte(hvr, pr, lookup(W == 5 ? (pr != 0) : pr, nir.get(pr)));
        nhvf = set_byte(hvf, pf, lookup(W == 5 ? (pf != 0) : pf, nif.get(pf)));
      } else {
        const uint32_t sv = s_hsave[k][tid];  // the values this level had before the descent
        nhvr = set_byte(hvr, pr, sv & 0xFFu);
        nhvf = set_byte(hvf, pf, sv >> 8);
      }
      nh = (int)max(byte_sum(nhvr), byte_sum(nhvf));
    } else {
      nh = h + s_mdd[(dm * N + from) * N + t];
    }
    if (gen) {
      ++cnt;
      if (g + 1 + nh > limit) {  // generated, not entered
        it = dm + 1;
        return false;
      }
      if (k + 1 >= MAXLEV || plen + k + 1 > kMaxPath) {
        set_error(SP_ERR_STACK_OVERFLOW, (uint32_t)(plen + k));
        return true;
      }
      if (PDB && k < HSAVE)
        s_hsave[k][tid] = (uint16_t)(((hvr >> (8 * pr)) & 0xFFu) | (((hvf >> (8 * pf)) & 0xFFu) << 8));
    }
    slide(t, from, blank);
    blank = from;
    h = nh;
    if (PDB) {
      ir = nir;
      iff = nif;
      hvr = nhvr;
      hvf = nhvf;
    }
    if (gen) {
      ++g;
      const int sh = 2 * (k & 15);
      top = (top & ~(3u << sh)) | ((uint32_t)dm << sh);
      if ((k & 15) == 15) s_stack[k >> 4][tid] = top;
      ++k;
      if (cut && k < 64) cut &= ~(1ull << k);  // cut is almost always 0
      pre = dm;
      it = 0;
      if (nh == 0) record_goal();
      if (splitk && k == 1) {
        // split task with `splitk` levels left: this child (already counted
        // as generated) becomes a task of its own with one level fewer
        // (published outside the step loop), so a heavy root is split
        // breadth-first by many lanes; the lane then steps back
        emit_pending = true;
        it = 4;
      }
    } else {
      --g;
      it = (3 - dm) + 1;  // the next sibling of the undone move
      if (cut && k < 64 && ((cut >> k) & 1ull)) it = 4;
      if (k == 0) pre = rpre;
      else if (k & 15) pre = (int)((top >> (2 * ((k - 1) & 15))) & 3u);
      else pre = (int)((s_stack[(k - 1) >> 4][tid] >> 30) & 3u);
    }
    return false;
  };

  // Give the untried moves of the shallowest open level (slack >= min_slack)
  // to a waiting lane.  Returns the level donated, or -1.
  auto find_donation = [&](uint32_t &mask_out) -> int {
    // resume at the first level not yet seen exhausted (`lo`): a level only
    // loses untried moves during a task, so the walk never needs to look
    // below it again; above the current depth the cache restarts at k
    int j = (int)(lo & 0xFFu), bl = (int)((lo >> 8) & 0xFFu), pr = (int)((lo >> 16) & 7u) - 1;
    if (k < j) {
      j = k;
      bl = blank;
      pr = pre;
    }
    const int lim = min(k, 63);
    int found = -1;
    for (; j <= lim; ++j) {
      if (limit - (groot + j) < P.min_slack) break;
      const int dj = j == k ? 0 : stack_dir(j);
      uint32_t un = legal_moves(W, bl) & (j == k ? (0xFu << it) : ((0xFu << (dj + 1)) & 0xFu));
      if (pr >= 0) un &= ~(1u << (3 - pr));
      if (j == 0) un &= mask0;
      if (!((cut >> j) & 1ull) && un) {
        mask_out = un;
        found = j;
        break;
      }
      if (j == k) break;
      bl += move_delta(W, dj);
      pr = dj;
    }
    lo = (uint32_t)min(j, 255) | ((uint32_t)bl << 8) | ((uint32_t)(pr + 1) << 16);
    return found;
  };

  unsigned long long last_change = 0;
  uint32_t last_out = 0xFFFFFFFFu, last_tail = 0xFFFFFFFFu, last_hb = 0xFFFFFFFFu, beat = 0;
  unsigned backoff = 256;  // idle-warp sleep, ns, doubled up to SP_MAX_BACKOFF_NS
  unsigned long long c_steps = 0, c_slots = 0, c_idle = 0;
  const long long t_begin = clock64();

  for (;;) {
    const long long t_iter = clock64();
    // pending work of the previous loop: instance advances, then owed indices
    if (MULTI) {
      unsigned pend = __ballot_sync(FULL, events & kAdvance);
      while (pend) {
        const int src = __ffs(pend) - 1;
        pend &= pend - 1u;
        warp_advance(P, s_cold[0][(tid & ~31) + src], s_hist[tid >> 5]);
        if (lane == src) {
          events &= ~kAdvance;
          __threadfence();
          atomicSub(&ctl->outstanding, 1u);
        }
      }
    }
    if ((events & kDebt) && ld_acquire(&P.seq[s_cold[1][tid] & (P.cap - 1u)]) == s_cold[1][tid]) {
      const uint32_t debt = s_cold[1][tid];
      Task *D = &P.tasks[debt & (P.cap - 1u)];
      D->sub = s_cold[2][tid];
      D->plen = 0;
      D->mask = 0;  // no first move: the claimant finishes it at once
      D->flags = 0;
      st_release(&P.seq[debt & (P.cap - 1u)], debt + 1u);
      events &= ~kDebt;
    }
    // 0. pool state from the block's cached copy (one global poll per block
    //    per poll_ns; a stale copy only delays, never corrupts, decisions:
    //    outstanding == 0 is final, tail and head only grow)
    uint32_t hd = 0, tl = 0, out = 0, hb = 0;
    int32_t err = 0;
    if (lane == 0) {
      volatile uint32_t *vp = (volatile uint32_t *)s_pool;
      const unsigned long long now = globaltimer();
      if (now - *(volatile unsigned long long *)&s_pool_t > P.poll_ns) {
        s_pool_t = now;
        vp[0] = ld_volatile(&ctl->head);
        vp[1] = ld_volatile(&ctl->tail);
        vp[2] = (uint32_t)ld_volatile(&ctl->error);
        vp[3] = ld_volatile(&ctl->outstanding);
        vp[4] = ld_volatile(&ctl->heartbeat);
      }
      hd = vp[0];
      tl = vp[1];
      err = (int32_t)vp[2];
      out = vp[3];
      hb = vp[4];
    }
    hd = __shfl_sync(FULL, hd, 0);
    tl = __shfl_sync(FULL, tl, 0);
    err = __shfl_sync(FULL, err, 0);
    out = __shfl_sync(FULL, out, 0);
    if (err) break;
    // 1. idle lanes claim pool indices, one atomic per warp
    const unsigned need = __ballot_sync(FULL, state == 0);
    if (need) {
      const int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&ctl->head, (uint32_t)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (state == 0) {
        slot = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
        state = 1;
      }
    }
    // 2. a claimed index becomes a task once its producer published it; only
    //    indices already reserved (below the cached tail) are polled
    if (state == 1 && slot < tl && ld_acquire(&P.seq[slot & (P.cap - 1u)]) == slot + 1u) {
      take_task();
      if (start_task()) state = 2;
      else finish_task();
    }
    // 3. nobody in the warp is searching: finished, failed or waiting
    const unsigned act = __ballot_sync(FULL, state == 2);
    if (!act) {
      if (out == 0) break;
      if (lane == 0) {
        const unsigned long long now = globaltimer();
        if (out != last_out || tl != last_tail || hb != last_hb || last_change == 0) {
          last_out = out;
          last_tail = tl;
          last_hb = hb;
          last_change = now;
        } else if (now - last_change > P.timeout_ns) {
          set_error(SP_ERR_TIMEOUT, out);
        }
      }
      __nanosleep(backoff);
      backoff = min(backoff * 2u, (unsigned)SP_MAX_BACKOFF_NS);
      c_idle += (unsigned long long)(clock64() - t_iter);
      continue;
    }
    backoff = 256;
    last_change = 0;  // a new idle spell starts its own no-progress clock
    if (lane == 0 && ((++beat & 127u) == 0u)) atomicAdd(&ctl->heartbeat, 1u);
    // 4. search
    c_slots += 32ull * (unsigned long long)P.steps;
    if (state == 2) {
      bool fin = false;
      for (int s = 0; s < P.steps; ++s) {
        ++c_steps;
        if (step()) {
          fin = true;
          break;
        }
        if (emit_pending) break;
      }
      if (emit_pending) {
        emit_pending = false;
        // the split is advisory: with a debt outstanding or the ring half
        // full, the lane searches the subtree itself
        bool emitted = false;
        if (!(events & kDebt) && (int32_t)(tl - hd) <= (int32_t)(P.cap >> 1)) {
          atomicAdd(&ctl->outstanding, 1u);
          if (MULTI) atomicAdd(&P.inst_out[cur_inst & 0x7FFFFFFFu], 1u);  // the lane's own task keeps it >= 1
          const uint32_t t = atomicAdd(&ctl->tail, 1u);
          if (slot_free(t, 4096)) {
            const int len = plen + k;
            Task *D = &P.tasks[t & (P.cap - 1u)];
            D->sub = sub;
            D->plen = (uint16_t)len;
            D->mask = 0xF;
            D->flags = (uint8_t)((splitk - 1) | (MULTI ? (cur_inst >> 31) << 6 : 0u));
            for (int wi = 0; wi < kPathWords; ++wi) D->path[wi] = path_word(wi, len);
            st_release(&P.seq[t & (P.cap - 1u)], t + 1u);
            emitted = true;
          } else {
            ++c_notfree;
            events |= kDebt;
            s_cold[1][tid] = t;
            s_cold[2][tid] = sub;
          }
        }
        if (!emitted) it = 0;
      }
      if (fin) finish_task();
    }
    // 5. donate while fewer than `reserve` tasks are queued (tail - head)
    if (P.donate && hd + P.reserve > tl) {
      uint32_t dmask = 0;
      int lev = (state == 2) ? find_donation(dmask) : -1;
      if (lev >= 0 && plen + lev > kMaxPath) lev = -1;  // prefix would not fit a record
      // donors: lanes whose open level is within one of the warp's shallowest,
      // at most `allowed` of them (more when the shortfall is large)
      const unsigned key = lev >= 0 ? (unsigned)lev : 0xFFFFFFFFu;
      const unsigned best = __reduce_min_sync(FULL, key);
      const uint32_t shortfall = hd + P.reserve - tl;
      const unsigned allowed = min((unsigned)SP_MAX_DONORS, 1u + shortfall / P.spread);
      const unsigned cand = __ballot_sync(FULL, lev >= 0 && (unsigned)lev <= best + 1u);
      const unsigned rank = __popc(cand & ((1u << lane) - 1u));
      const bool donor = ((cand >> lane) & 1u) && rank < allowed && !(events & kDebt);
      const unsigned donors = __ballot_sync(FULL, donor);
      if (lane == 0) {
        ++c_nowait;  // hungry polls
        if (donors) ++c_found;
      }
      uint32_t tbase = 0;
      const int lead = donors ? __ffs(donors) - 1 : 0;
      if (donors && lane == lead) {
        tbase = atomicAdd(&ctl->tail, (uint32_t)__popc(donors));
        atomicAdd(&ctl->outstanding, (uint32_t)__popc(donors));
      }
      tbase = __shfl_sync(FULL, tbase, lead);
      if (donor) {
        // the reserved index's ring slot is free once the slot's previous
        // occupant (index t - cap, claimed long before) was copied out, which
        // in practice it already is -- wait a bounded time, else keep the
        // branch and owe the index a null task
        const uint32_t mask = P.cap - 1u;
        ++c_tries;
        if (MULTI) atomicAdd(&P.inst_out[cur_inst & 0x7FFFFFFFu], 1u);  // the donor's own task keeps it >= 1
        const uint32_t t = tbase + (uint32_t)__popc(donors & ((1u << lane) - 1u));
        const bool ok = slot_free(t, 4096);
        if (!ok) {
          ++c_notfree;
          events |= kDebt;
          s_cold[1][tid] = t;
          s_cold[2][tid] = sub;
        }
        if (ok) {
          Task *D = &P.tasks[t & mask];
          const int nlen = plen + lev;
          D->sub = sub;
          D->plen = (uint16_t)nlen;
          D->mask = (uint8_t)dmask;
          D->flags = (uint8_t)(MULTI ? (cur_inst >> 31) << 6 : 0u);
          for (int wi = 0; wi < kPathWords; ++wi) D->path[wi] = path_word(wi, nlen);
          st_release(&P.seq[t & mask], t + 1u);
          atomicAdd(&ctl->donated, 1ull);
          if (lev == k) it = 4;
          else cut |= 1ull << lev;
        }
      }
    }
  }
  // efficiency counters (warp-aggregated)
  unsigned long long steps_w = c_steps, tries_w = c_tries, notfree_w = c_notfree, nowait_w = c_nowait,
                     done_w = c_done;
  for (int o = 16; o; o >>= 1) {
    steps_w += __shfl_xor_sync(FULL, steps_w, o);
    tries_w += __shfl_xor_sync(FULL, tries_w, o);
    notfree_w += __shfl_xor_sync(FULL, notfree_w, o);
    nowait_w += __shfl_xor_sync(FULL, nowait_w, o);
    done_w += __shfl_xor_sync(FULL, done_w, o);
  }
  if (lane == 0) {
    atomicAdd(&ctl->counters[0], steps_w);
    atomicAdd(&ctl->counters[1], c_slots);
    atomicAdd(&ctl->counters[2], c_idle);
    atomicAdd(&ctl->counters[3], (unsigned long long)(clock64() - t_begin));
    atomicAdd(&ctl->counters[4], tries_w);
    atomicAdd(&ctl->counters[5], notfree_w);
    atomicAdd(&ctl->counters[6], nowait_w);
    atomicAdd(&ctl->counters[7], done_w);
    atomicAdd(&ctl->counters[8], c_found);
  }
}

// Reset the ring (seq[s] = s: slot s free for index s), fill indices [0, n)
// with the round's root tasks and publish them (seq = index + 1).  The pieces
// of split roots (count on the device) come first, then the host's direct
// tasks, which the host orders by decreasing predicted size.
__global__ void pool_init_kernel(Task *tasks, const Task *emit, const uint32_t *n_emit, const uint32_t *direct,
                                 uint32_t n_direct, uint32_t *seq, uint32_t cap, PoolCtl *ctl, const SubRoot *subs,
                                 const int32_t *inst_iter) {
  const uint32_t ne = n_emit ? *n_emit : 0u;
  const uint32_t n = min(ne + n_direct, cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    if (i < n) {
      if (i < ne) {
        tasks[i] = emit[i];
      } else {  // a whole root: no prefix, every first move
        Task t{};
        t.sub = direct[i - ne];
        t.mask = 0xF;
        if (inst_iter) t.flags = (uint8_t)((inst_iter[subs[t.sub].inst] & 1) << 6);
        tasks[i] = t;
      }
      seq[i] = i + 1u;
    } else {
      seq[i] = i;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->head = 0;
    ctl->tail = n;
    ctl->outstanding = n;
    ctl->error = (ne + n_direct > cap) ? SP_ERR_CAPACITY : 0;
    ctl->donated = 0;
    ctl->heartbeat = 0;
    for (int c = 0; c < 16; ++c) ctl->counters[c] = 0;
  }
}

// One breadth-first level of the split pre-pass: each input node (a root, or
// a piece of one, at f <= limit) is expanded; every legal non-reverse child
// is counted as generated, exactly as the depth-first search would count it,
// and children within the limit go on to the next level or, at the last
// level, become pool tasks.  flags = levels still to expand.
template <int W, bool PDB>
__global__ void split_level_kernel(SplitArgs A) {
  constexpr int N = W * W;
  const uint32_t n_in = *A.n_in;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += gridDim.x * blockDim.x) {
    const Task T = A.in[i];
    const SubRoot R = A.subs[T.sub];
    uint8_t b[N];
    for (int c = 0; c < N; ++c) b[c] = R.board[c];
    int blank = R.blank, g = R.g, pre = R.pre == kNoPre ? -1 : (int)R.pre;
    bool ok = true;
    for (int q = 0; q < T.plen; ++q) {
      const int d = (int)((T.path[q >> 4] >> (2 * (q & 15))) & 3u);
      if (!((legal_moves(W, blank) >> d) & 1u)) { ok = false; break; }
      const int src = blank + move_delta(W, d);
      b[blank] = b[src];
      b[src] = 0;
      blank = src;
      pre = d;
      ++g;
    }
    if (!ok) {
      atomicCAS(A.error, 0, SP_ERR_ARG);
      continue;
    }
    const int L = A.inst_limit[R.inst];
    uint32_t mv = legal_moves(W, blank) & T.mask;
    if (pre >= 0) mv &= ~(1u << (3 - pre));
    unsigned long long cnt = 0;
    for (int d = 0; d < 4; ++d) {
      if (!((mv >> d) & 1u)) continue;
      ++cnt;
      const int src = blank + move_delta(W, d);
      b[blank] = b[src];
      b[src] = 0;
      const int hc = board_h<W, PDB>(b, A.ht, A.pdb);
      b[src] = b[blank];
      b[blank] = 0;
      if (g + 1 + hc > L) continue;
      Task C = T;
      const int q = T.plen;
      if (q >= kMaxPath) {
        atomicCAS(A.error, 0, SP_ERR_STACK_OVERFLOW);
        continue;
      }
      C.path[q >> 4] = (C.path[q >> 4] & ~(3u << (2 * (q & 15)))) | ((uint32_t)d << (2 * (q & 15)));
      C.plen = (uint16_t)(q + 1);
      C.mask = 0xF;
      C.flags = (uint8_t)(T.flags - 1);
      if (hc == 0) {  // a goal at the child: record it like the search does
        Solution *S = &A.sol[R.inst];
        atomicMax(&S->best, 0xFFFFFFFFu - (uint32_t)(g + 1));
        if (atomicCAS(&S->flag, 0u, 1u) == 0u) {
          S->sub = T.sub;
          S->len = (uint32_t)(q + 1);
          for (int wi = 0; wi < kPathWords; ++wi) S->path[wi] = C.path[wi];
          __threadfence();
        }
      }
      if (C.flags > 0) {
        const uint32_t at = atomicAdd(A.n_next, 1u);
        if (at < A.cap_next) A.next[at] = C;
        else atomicCAS(A.error, 0, SP_ERR_CAPACITY);
      } else {
        const uint32_t at = atomicAdd(A.n_out, 1u);
        if (at < A.cap_out) A.out[at] = C;
        else atomicCAS(A.error, 0, SP_ERR_CAPACITY);
      }
    }
    if (cnt) atomicAdd(&A.sub_nodes[T.sub], cnt);
  }
}

cudaError_t launch_split_level(int w, bool pdb, int num_sms, const SplitArgs &A, cudaStream_t st) {
  const int grid = num_sms * 8, block = 128;
  if (w == 4) {
    if (pdb) split_level_kernel<4, true><<<grid, block, 0, st>>>(A);
    else split_level_kernel<4, false><<<grid, block, 0, st>>>(A);
  } else {
    if (pdb) split_level_kernel<5, true><<<grid, block, 0, st>>>(A);
    else split_level_kernel<5, false><<<grid, block, 0, st>>>(A);
  }
  note_launch();
  return cudaGetLastError();
}

// Host launchers (template kernels stay in this translation unit).
template <bool MULTI>
static cudaError_t launch_impl(int w, bool pdb, int block, int blocks_per_sm, int num_sms, const RoundParams &P,
                               cudaStream_t st, int *grid_out) {
  void (*kern)(RoundParams) = nullptr;
#define SP_PICK(W, PD, B, WD) \
  if (w == W && pdb == PD && block == B) kern = search_round_kernel<W, PD, B, WD, MULTI>;
  SP_PICK(4, false, 256, 6)
  SP_PICK(4, true, 256, 6)
  SP_PICK(5, false, 256, 10)
  SP_PICK(5, true, 256, 10)
  SP_PICK(4, false, 128, 6)
  SP_PICK(4, true, 128, 6)
  SP_PICK(5, false, 128, 10)
  SP_PICK(5, true, 128, 10)
#undef SP_PICK
  if (!kern) return cudaErrorInvalidValue;
  int per_sm = blocks_per_sm;
  if (per_sm <= 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
  }
  const int grid = num_sms * per_sm;
  if (grid_out) *grid_out = grid;
  kern<<<grid, block, 0, st>>>(P);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_search_round(int w, bool pdb, int block, int blocks_per_sm, int num_sms,
                                const RoundParams &P, cudaStream_t st, int *grid_out) {
  return launch_impl<false>(w, pdb, block, blocks_per_sm, num_sms, P, st, grid_out);
}

cudaError_t launch_search_multi(int w, bool pdb, int block, int blocks_per_sm, int num_sms,
                                const RoundParams &P, cudaStream_t st, int *grid_out) {
  return launch_impl<true>(w, pdb, block, blocks_per_sm, num_sms, P, st, grid_out);
}

cudaError_t launch_pool_init(Task *tasks, const Task *emit, const uint32_t *n_emit, const uint32_t *direct,
                             uint32_t n_direct, uint32_t *seq, uint32_t cap, PoolCtl *ctl, const SubRoot *subs,
                             const int32_t *inst_iter, cudaStream_t st) {
  const uint32_t blocks = std::min<uint32_t>((cap + 255) / 256, 152u * 32u);
  pool_init_kernel<<<blocks, 256, 0, st>>>(tasks, emit, n_emit, direct, n_direct, seq, cap, ctl, subs, inst_iter);
  note_launch();
  return cudaGetLastError();
}

}  // namespace sp
