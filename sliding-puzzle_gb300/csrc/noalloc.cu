// sp_dfs_round_md_noalloc: one Manhattan-heuristic threshold round over a
// caller's root set that allocates no memory.
//
// Some callers cannot call cudaMalloc: embedders whose process owns the
// device allocator (a framework's caching pool that must see every device
// allocation, or a memory budget fixed at start-up), and tight real-time
// loops that must not enter the driver's allocator, whose latency is
// unbounded.  They pass device buffers for the inputs and outputs;
// everything else the round needs lives in one file-scope device array of
// fixed size, g_noalloc_scratch below.  Every GPU that loads the library
// holds that array (kNoAllocScratchBytes, about 7 MB) until the process
// exits.
//
// Limits and sharing: at most kNoAllocMaxRoots roots per call and a task
// pool of kNoAllocPoolCap slots; larger inputs are rejected with
// SP_ERR_CAPACITY before anything is launched.  All calls share the one
// array, which keeps what the last call left there: each call
// re-initialises what must start clean (heuristic tables, pool control
// block, ring sequence numbers, solution slot, output counters), and two
// calls whose work overlaps on the GPU (different streams, or different host
// threads) race on it -- serialise them.
//
// Set-up: every call takes the array's device address on the current device
// with cudaGetSymbolAddress (the host-side name g_noalloc_scratch is not a
// device address) and writes the heuristic tables with a kernel, so nothing
// is cached that a device reset could make stale; the SM count is cached
// once per device.  The call is synchronous: it reads the device status back
// and returns after the stream has drained.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/slide.h"
#include "sp_defs.h"
#include "sp_kernels.h"

namespace sp {
namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr uint32_t kNoAllocPoolCap = 1u << 17;  // ring slots (power of two)
constexpr int kNoAllocMaxRoots = 16384;
constexpr int kMaxDevices = 64;

// layout of the scratch array
constexpr size_t kOffTasks = 0;
constexpr size_t kOffSeq = align_up(kOffTasks + sizeof(Task) * kNoAllocPoolCap);
constexpr size_t kOffCtl = align_up(kOffSeq + sizeof(uint32_t) * kNoAllocPoolCap);
constexpr size_t kOffSubs = align_up(kOffCtl + sizeof(PoolCtl));
constexpr size_t kOffSol = align_up(kOffSubs + sizeof(SubRoot) * kNoAllocMaxRoots);
constexpr size_t kOffLimit = align_up(kOffSol + sizeof(Solution));
constexpr size_t kOffHt4 = align_up(kOffLimit + sizeof(int32_t) * 4);
constexpr size_t kOffHt5 = align_up(kOffHt4 + sizeof(HeurTables));
constexpr size_t kNoAllocScratchBytes = align_up(kOffHt5 + sizeof(HeurTables));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

int g_num_sms[kMaxDevices];  // 0 until read for that device
std::mutex g_setup_mu;

// The Manhattan delta table of width W (HeurTables::mdd: the change of h when
// the tile at `cell` slides into the blank after the blank's move d), one
// entry per thread; the rest of the record is unused by this path.
template <int W>
__global__ void noalloc_tables_kernel(unsigned char *base) {
  constexpr int N = W * W;
  HeurTables *ht = (HeurTables *)(base + (W == 4 ? kOffHt4 : kOffHt5));
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * N * N) return;
  const int t = i % N, c = (i / N) % N, d = i / (N * N);
  const int b = c - move_delta(W, d);
  int v = 0;
  if (t && b >= 0 && b < N)
    v = (abs(b / W - t / W) + abs(b % W - t % W)) - (abs(c / W - t / W) + abs(c % W - t % W));
  ht->mdd[i] = (int8_t)v;
}

// Root records from the caller's device arrays; Manhattan distance of each
// root; a root that is the goal sets *found (the reference's dfs_kernel flags
// such roots, src/24puzzle_block_parallel_with_pdb.cu:580-583).  Invalid
// tiles, depth or move codes set the control block's error.
template <int W>
__global__ void noalloc_prepare_kernel(const uint8_t *roots, const int32_t *depth, const int32_t *pre, int n,
                                       int limit, unsigned char *base, int32_t *found,
                                       unsigned long long *nodes) {
  constexpr int N = W * W;
  SubRoot *subs = (SubRoot *)(base + kOffSubs);
  PoolCtl *ctl = (PoolCtl *)(base + kOffCtl);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    *(int32_t *)(base + kOffLimit) = limit;
    ((Solution *)(base + kOffSol))->flag = 0;
    ((Solution *)(base + kOffSol))->best = 0;
  }
  if (i >= n) return;
  nodes[i] = 0;
  SubRoot r{};
  uint32_t seen = 0;
  int md = 0;
  for (int c = 0; c < N; ++c) {
    const uint8_t t = roots[(size_t)i * N + c];
    if (t >= N || ((seen >> t) & 1u)) {
      atomicCAS(&ctl->error, 0, SP_ERR_NOT_PERMUTATION);
      return;
    }
    seen |= 1u << t;
    r.board[c] = t;
    if (!t) r.blank = (uint8_t)c;
    else md += abs(c / W - t / W) + abs(c % W - t % W);
  }
  const int g = depth[i], p = pre[i];
  if (g < 0 || g > 255 || p < -1 || p > 3) {
    atomicCAS(&ctl->error, 0, SP_ERR_ARG);
    return;
  }
  r.g = (uint8_t)g;
  r.pre = p < 0 ? kNoPre : (uint8_t)p;
  r.inst = 0;
  subs[i] = r;
  if (md == 0) atomicMin(found, g);
}

// Ring reset and one whole-root task per root (index i = root i); no tasks
// when the preparation found an invalid root.
__global__ void noalloc_pool_kernel(unsigned char *base, int n) {
  Task *tasks = (Task *)(base + kOffTasks);
  uint32_t *seq = (uint32_t *)(base + kOffSeq);
  PoolCtl *ctl = (PoolCtl *)(base + kOffCtl);
  if (*(volatile int32_t *)&ctl->error) n = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kNoAllocPoolCap; i += gridDim.x * blockDim.x) {
    if (i < (uint32_t)n) {
      Task t{};
      t.sub = i;
      t.mask = 0xF;
      tasks[i] = t;
      seq[i] = i + 1u;
    } else {
      seq[i] = i;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->head = 0;
    ctl->tail = (uint32_t)n;
    ctl->outstanding = (uint32_t)n;
    ctl->donated = 0;
    ctl->heartbeat = 0;
    for (int c = 0; c < 16; ++c) ctl->counters[c] = 0;
  }
}

// *found: shortest goal depth among the roots and the search's solution, -1
// if none (INT32_MAX stands for "none" until here).
__global__ void noalloc_finish_kernel(unsigned char *base, int32_t *found) {
  const Solution *sol = (const Solution *)(base + kOffSol);
  int32_t f = *found;
  if (sol->flag && sol->best) f = min(f, (int32_t)(0xFFFFFFFFu - sol->best));
  *found = f == 0x7FFFFFFF ? -1 : f;
}

__global__ void noalloc_found_init_kernel(int32_t *found, unsigned char *base) {
  *found = 0x7FFFFFFF;
  ((PoolCtl *)(base + kOffCtl))->error = 0;
}

// The scratch array's device address on the current device `dev` and that
// device's SM count.  The address is taken on every call (it is cheap) so
// that a new primary context after a device reset is picked up.
int setup_device(int dev, unsigned char **base, int *num_sms) {
  void *ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return SP_ERR_CUDA;
  *base = (unsigned char *)ptr;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_num_sms[dev] &&
      (cudaDeviceGetAttribute(&g_num_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
       g_num_sms[dev] < 1)) {
    g_num_sms[dev] = 0;
    return SP_ERR_CUDA;
  }
  *num_sms = g_num_sms[dev];
  return SP_OK;
}

}  // namespace
}  // namespace sp

using namespace sp;

extern "C" int sp_dfs_round_md_noalloc(int width, const uint8_t *d_roots, const int32_t *d_depth,
                                       const int32_t *d_pre, int n, int limit, uint64_t *d_nodes,
                                       int32_t *d_found, void *stream) {
  if ((width != 4 && width != 5) || n < 0 || (n > 0 && (!d_roots || !d_depth || !d_pre || !d_nodes)) || !d_found)
    return SP_ERR_ARG;
  if (n > kNoAllocMaxRoots) return SP_ERR_CAPACITY;
  // an error the caller left pending is the caller's: report it without
  // clearing it, and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return SP_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SP_ERR_CUDA;
  unsigned char *base = nullptr;
  int num_sms = 0;
  const int rc = setup_device(dev, &base, &num_sms);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // each launch is checked at once; after a failed one the outputs are undefined
  auto launched = [](int k) {
    note_launch(k);
    return cudaGetLastError() == cudaSuccess;
  };
  const int nt = 4 * width * width * width * width;
  if (width == 4) noalloc_tables_kernel<4><<<(nt + 255) / 256, 256, 0, st>>>(base);
  else noalloc_tables_kernel<5><<<(nt + 255) / 256, 256, 0, st>>>(base);
  if (!launched(1)) return SP_ERR_CUDA;
  noalloc_found_init_kernel<<<1, 1, 0, st>>>(d_found, base);
  if (!launched(1)) return SP_ERR_CUDA;
  if (n > 0) {
    const int blocks = (n + 127) / 128;
    if (width == 4)
      noalloc_prepare_kernel<4><<<blocks, 128, 0, st>>>(d_roots, d_depth, d_pre, n, limit, base, d_found,
                                                        (unsigned long long *)d_nodes);
    else
      noalloc_prepare_kernel<5><<<blocks, 128, 0, st>>>(d_roots, d_depth, d_pre, n, limit, base, d_found,
                                                        (unsigned long long *)d_nodes);
    if (!launched(1)) return SP_ERR_CUDA;
    noalloc_pool_kernel<<<(kNoAllocPoolCap + 255) / 256, 256, 0, st>>>(base, n);
    if (!launched(1)) return SP_ERR_CUDA;
    RoundParams P{};
    P.subs = (const SubRoot *)(base + kOffSubs);
    P.tasks = (Task *)(base + kOffTasks);
    P.seq = (uint32_t *)(base + kOffSeq);
    P.cap = kNoAllocPoolCap;
    P.ctl = (PoolCtl *)(base + kOffCtl);
    P.inst_limit = (const int32_t *)(base + kOffLimit);
    P.sub_nodes = (unsigned long long *)d_nodes;
    P.sol = (Solution *)(base + kOffSol);
    P.ht = (const HeurTables *)(base + (width == 4 ? kOffHt4 : kOffHt5));
    P.pdb = nullptr;
    P.min_slack = 6;
    P.steps = 32;
    P.donate = 1;
    P.timeout_ns = 20000000000ull;
    P.poll_ns = 2000;
    const uint32_t lanes = (uint32_t)num_sms * 1024u;
    P.reserve = lanes / 16u;
    P.spread = lanes / 32u;
    int grid = 0;
    if (launch_search_round(width, false, 256, 0, num_sms, P, st, &grid) != cudaSuccess) return SP_ERR_CUDA;
  }
  noalloc_finish_kernel<<<1, 1, 0, st>>>(base, d_found);
  if (!launched(1)) return SP_ERR_CUDA;
  int32_t err = 0;
  if (cudaMemcpyAsync(&err, base + kOffCtl + offsetof(PoolCtl, error), sizeof(err), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SP_ERR_CUDA;
  return err;
}
