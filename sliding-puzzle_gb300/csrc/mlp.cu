// Learned load balancer on the GPU: layer-1 gather-sum, tcgen05 GEMMs with
// fused epilogues, Adam.  See lbm.h for the model.
//
// GEMM shape: C[M x 256] = A[M x K] . B[256 x K]^T with A and B bf16, K-major
// (K contiguous), fp32 accumulation in tensor memory.  One CTA of 4 warps
// computes one 128-row tile over a K range:
//   * thread 0 streams 64-wide K chunks of A (128 x 64) and B (256 x 64) into
//     shared memory with TMA (128-byte swizzle), two stages, completion on an
//     mbarrier, and issues four tcgen05.mma (M=128, N=256, K=16) per chunk;
//     tcgen05.commit frees a stage once its MMAs have read it;
//   * warp 0 allocates 256 TMEM columns (the 128 x 256 fp32 accumulator);
//   * after the last commit all four warps read their 32 accumulator rows
//     with tcgen05.ld (32x32b) and run the epilogue.
// The training step is four such GEMMs:
//   forward   Z2 = H1 . W2^T          epilogue: ReLU, layer 3, loss, dL/dy,
//                                     dH2 = dy w3 (Z2 > 0), d/dw3, d/db2
//   backward  dZ1 = dH2 . W2          epilogue: dH1 = dZ1 (H1 > 0), d/db1
//   dW2 = dH2^T . H1                  (split K over the batch, fp32 atomics)
//   dW1 = X^T . dH1                   (X = the one-hot input, ditto)
// Every mbarrier wait is bounded (2 s of %globaltimer); on expiry the CTA
// records an error, drains its copies in flight (bounded), frees its tensor
// memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/slide.h"
#include "lbm.h"
#include "sp_defs.h"
#include "sp_kernels.h"

namespace sp {
namespace lbm {

namespace {

constexpr int H = kHidden;
constexpr int BM = 128;                      // accumulator rows per CTA (TMEM lanes)
constexpr int BK = 64;                       // K per stage: one 128-byte swizzle row of bf16
constexpr int STAGES = 2;
constexpr int A_STAGE = BM * BK * 2;         // 16 KB
constexpr int B_STAGE = H * BK * 2;          // 32 KB
constexpr int SMEM_TILES = STAGES * (A_STAGE + B_STAGE);
constexpr int SMEM_BYTES = SMEM_TILES + 1024 /* alignment slack */ + 128 /* barriers, TMEM address */;
// kind::f16 instruction descriptor: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1),
// B bf16 (10-12 = 1), both K-major (15, 16 = 0), N >> 3 at 17-22, M >> 4 at 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(H >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

enum { EPI_F32 = 0, EPI_F32_ATOMIC = 1, EPI_FWD = 2, EPI_BWD1 = 3, EPI_INFER = 4 };

struct EpiArgs {
  float *C;          // EPI_F32 / EPI_F32_ATOMIC: C[row * 256 + col]
  int m_valid;       // rows >= m_valid are padding
  int ldt;           // leading dimension of the transposed bf16 outputs (the batch)
  float inv_b;       // 1 / batch rows, for the mean loss
  const float *b2, *w3, *b3;
  const float *target;
  float *y;
  __nv_bfloat16 *dH2, *dH2T;      // forward-train outputs
  const __nv_bfloat16 *H1;        // backward: ReLU mask of layer 1
  __nv_bfloat16 *dH1T;            // backward output
  float *gw3, *gb2, *gb3, *gb1, *loss;
  int *err;
  unsigned long long wait_ns;  // limit of every mbarrier wait (0: 2 s)
  int starve_kc1;              // self-test only: K chunk starve_kc1 - 1 gets no copies (0: none)
};

// ---- PTX wrappers ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false after limit_ns without the phase completing.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
  unsigned long long t0 = 0;
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u) {
      const unsigned long long now = gtimer();
      if (!t0) t0 = now;
      else if (now - t0 > limit_ns) return false;
    }
  }
}
__device__ __forceinline__ void tma_load_2d(const CUtensorMap *map, uint32_t dst, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t holder, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(holder), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
// 32 consecutive fp32 accumulator columns of this thread's row.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the
// 128-byte swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart (SBO),
// descriptor version 1, layout type 2 (128-byte swizzle).  The tile base is
// 1024-byte aligned; a K step of 16 elements inside the row adds 32 bytes.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;                       // version
  d |= (uint64_t)2 << 61;                       // 128-byte swizzle
  return d;
}

// In lane l: the sum over the warp's 32 lanes of v[l] (v is consumed).
__device__ __forceinline__ float warp_colsum(float (&v)[32], int lane) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float send = up ? v[i] : v[i + o];
      const float keep = up ? v[i + o] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// 32 bf16 values as four 16-byte stores.
__device__ __forceinline__ void store_bf16x32(__nv_bfloat16 *dst, const float (&v)[32]) {
  uint32_t p[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    p[i] = *reinterpret_cast<const uint32_t *>(&h);
  }
  uint4 *d = reinterpret_cast<uint4 *>(dst);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = make_uint4(p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]);
}

template <int EPI>
__global__ void __launch_bounds__(128, 1)
    umma_gemm_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int kc_per_cta,
                     int kc_total, EpiArgs E) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * A_STAGE;
  uint64_t *bars = (uint64_t *)(smem + SMEM_TILES);  // full[2], done[2], accum
  uint32_t *tmem_holder = (uint32_t *)(bars + 6);
  int *s_fail = (int *)(bars + 7);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const int kc0 = blockIdx.y * kc_per_cta;
  const int nk = min(kc_per_cta, kc_total - kc0);
  const uint32_t full0 = smem_u32(bars), done0 = smem_u32(bars + 2), accum = smem_u32(bars + 4);

  if (threadIdx.x == 0) {
    for (int i = 0; i < 5; ++i) mbar_init(smem_u32(bars + i), 1);
    *s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(smem_u32(tmem_holder), 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  const unsigned long long limit = E.wait_ns ? E.wait_ns : 2000000000ull;
  if (threadIdx.x == 0) {
    int issued = 0, consumed = 0;
    bool ok = nk > 0;
    // chunk kc's copies; the self-test's starved chunk gets none, so the
    // wait for it runs out (its stage's barrier never completes a phase)
    auto issue = [&](int kc) {
      const int s = kc % STAGES;
      if (kc0 + kc + 1 != E.starve_kc1) {
        mbar_expect_tx(full0 + 8 * s, A_STAGE + B_STAGE);
        tma_load_2d(&ta, smem_u32(sA + s * A_STAGE), full0 + 8 * s, (kc0 + kc) * BK, m0);
        tma_load_2d(&tb, smem_u32(sB + s * B_STAGE), full0 + 8 * s, (kc0 + kc) * BK, 0);
      }
      ++issued;
    };
    for (int kc = 0; kc < min(nk, STAGES); ++kc) issue(kc);
    for (int kc = 0; kc < nk && ok; ++kc) {
      const int s = kc % STAGES;
      const uint32_t ph = (uint32_t)(kc / STAGES) & 1u;
      if (!mbar_wait(full0 + 8 * s, ph, limit)) {
        ok = false;
        break;
      }
      ++consumed;
      tc_fence_after();
      const uint64_t ad = smem_desc(smem_u32(sA + s * A_STAGE));
      const uint64_t bd = smem_desc(smem_u32(sB + s * B_STAGE));
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)
        umma_bf16(tmem, ad + (uint64_t)(kk * 2), bd + (uint64_t)(kk * 2), kIdesc, (kc | kk) ? 1u : 0u);
      umma_commit(done0 + 8 * s);
      if (kc + STAGES < nk) {
        if (!mbar_wait(done0 + 8 * s, ph, limit)) {
          ok = false;
          break;
        }
        issue(kc + STAGES);
      }
    }
    if (!ok) {
      // drain: copies in flight land before the CTA leaves (bounded)
      for (int kc = consumed; kc < issued; ++kc)
        if (kc0 + kc + 1 != E.starve_kc1) mbar_wait(full0 + 8 * (kc % STAGES), (uint32_t)(kc / STAGES) & 1u, limit);
      *s_fail = 1;
      if (E.err) atomicExch(E.err, 1);
    }
    umma_commit(accum);  // arrives once every MMA issued above has completed
  }
  __syncthreads();
  const bool have = mbar_wait(accum, 0, limit) && !*(volatile int *)s_fail;
  if (!have && E.err) atomicExch(E.err, 1);
  tc_fence_after();

  if (have) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
    const bool valid = row < E.m_valid;
    if (EPI == EPI_F32 || EPI == EPI_F32_ATOMIC) {
      for (int c0 = 0; c0 < H; c0 += 32) {
        float v[32];
        tmem_ld32(tbase + c0, v);
        if (valid) {
          float *dst = E.C + (size_t)row * H + c0;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (EPI == EPI_F32) dst[j] = v[j];
            else atomicAdd(dst + j, v[j]);
          }
        }
      }
    } else if (EPI == EPI_FWD || EPI == EPI_INFER) {
      float yv = 0.f;
      for (int c0 = 0; c0 < H; c0 += 32) {
        float v[32];
        tmem_ld32(tbase + c0, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float z = v[j] + E.b2[c0 + j];
          if (z > 0.f) yv += z * E.w3[c0 + j];
        }
      }
      yv += E.b3[0];
      if (valid) E.y[row] = yv;
      if (EPI == EPI_FWD) {
        float dy = 0.f, l = 0.f;
        if (valid) {
          const float d = yv - E.target[row];
          l = d * d;
          dy = 2.f * d * E.inv_b;
        }
        l = warp_sum(l);
        const float sdy = warp_sum(dy);
        if (lane == 0) {
          atomicAdd(E.loss, l * E.inv_b);
          atomicAdd(E.gb3, sdy);
        }
        for (int c0 = 0; c0 < H; c0 += 32) {
          float v[32], gw[32], gb[32];
          tmem_ld32(tbase + c0, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float z = v[j] + E.b2[c0 + j];
            const float d = z > 0.f ? dy * E.w3[c0 + j] : 0.f;
            gw[j] = z > 0.f ? dy * z : 0.f;
            gb[j] = d;
            v[j] = d;
          }
          store_bf16x32(E.dH2 + (size_t)row * H + c0, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) E.dH2T[(size_t)(c0 + j) * E.ldt + row] = __float2bfloat16_rn(v[j]);
          const float s1 = warp_colsum(gw, lane);
          const float s2 = warp_colsum(gb, lane);
          atomicAdd(&E.gw3[c0 + lane], s1);
          atomicAdd(&E.gb2[c0 + lane], s2);
        }
      }
    } else if (EPI == EPI_BWD1) {
      for (int c0 = 0; c0 < H; c0 += 32) {
        float v[32];
        tmem_ld32(tbase + c0, v);
        const uint4 *hp = reinterpret_cast<const uint4 *>(E.H1 + (size_t)row * H + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint4 u = hp[q];
          const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const __nv_bfloat162 h2 = *reinterpret_cast<const __nv_bfloat162 *>(&w[e]);
            const int j = q * 8 + e * 2;
            if (!(__low2float(h2) > 0.f)) v[j] = 0.f;
            if (!(__high2float(h2) > 0.f)) v[j + 1] = 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) E.dH1T[(size_t)(c0 + j) * E.ldt + row] = __float2bfloat16_rn(v[j]);
        const float s = warp_colsum(v, lane);
        atomicAdd(&E.gb1[c0 + lane], s);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

// ---- layer 1: gather-sum of one-hot rows ----------------------------------
struct EmbedArgs {
  const uint8_t *boards;   // row r's tiles at boards + (idx ? idx[r] : r) * bstride
  const uint32_t *idx;
  int bstride;
  const int32_t *slack;
  int n;                   // real rows; rows n..grid*32-1 are padding (the goal, slack 0)
  const __nv_bfloat16 *W1; // [D][256]
  const float *b1;
  __nv_bfloat16 *H1;       // [rows][256]
  __nv_bfloat16 *H1T;      // [256][ldt] or null
  __nv_bfloat16 *XT;       // [Dpad][ldt] one-hot transposed (zeroed by the caller) or null
  int ldt;
};

template <int W>
__global__ void __launch_bounds__(256) embed_kernel(EmbedArgs A) {
  constexpr int N = W * W;
  constexpr int D = (N - 1) * N + 1;
  constexpr uint16_t kNone = 0xFFFFu;
  __shared__ uint16_t s_feat[32][N];
  __shared__ float s_slack[32];
  __shared__ __nv_bfloat16 s_ht[H][33];
  const int tid = threadIdx.x;
  const int row0 = blockIdx.x * 32;
  for (int e = tid; e < 32 * N; e += 256) s_feat[e / N][e % N] = kNone;
  __syncthreads();
  for (int e = tid; e < 32 * N; e += 256) {
    const int r = e / N, c = e % N, row = row0 + r;
    int t = c;
    if (row < A.n) {
      const size_t src = A.idx ? (size_t)A.idx[row] : (size_t)row;
      t = A.boards[src * (size_t)A.bstride + c];
    }
    if (t > 0 && t < N) s_feat[r][t - 1] = (uint16_t)((t - 1) * N + c);
  }
  if (tid < 32) s_slack[tid] = (row0 + tid < A.n) ? (float)A.slack[row0 + tid] : 0.f;
  __syncthreads();
  if (A.XT) {
    for (int e = tid; e < 32 * N; e += 256) {
      const int r = e / N, t = e % N, row = row0 + r;
      if (row >= A.n) continue;
      if (t < N - 1) {
        const uint16_t f = s_feat[r][t];
        if (f != kNone) A.XT[(size_t)f * A.ldt + row] = __float2bfloat16_rn(1.f);
      } else {
        A.XT[(size_t)(D - 1) * A.ldt + row] = __float2bfloat16_rn(s_slack[r]);
      }
    }
  }
  const int j = tid;
  const float bj = A.b1[j];
  const float sw = __bfloat162float(A.W1[(size_t)(D - 1) * H + j]);
  for (int r = 0; r < 32; ++r) {
    float acc = bj + s_slack[r] * sw;
    for (int t = 0; t < N - 1; ++t) {
      const uint16_t f = s_feat[r][t];
      if (f != kNone) acc += __bfloat162float(A.W1[(size_t)f * H + j]);
    }
    const __nv_bfloat16 hb = __float2bfloat16_rn(fmaxf(acc, 0.f));
    A.H1[(size_t)(row0 + r) * H + j] = hb;
    s_ht[j][r] = hb;
  }
  if (A.H1T) {
    __syncthreads();
    for (int e = tid; e < H * 32; e += 256) {
      const int jj = e >> 5, r = e & 31;
      A.H1T[(size_t)jj * A.ldt + row0 + r] = s_ht[jj][r];
    }
  }
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, size_t n, float lr, float c1, float c2) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
  }
}

// bf16 copies of the weights: W1 [D][256], W2 [out][in] and W2^T [in][out]
__global__ void refresh_kernel(const float *W1, size_t n1, const float *W2, __nv_bfloat16 *W1b, __nv_bfloat16 *W2b,
                               __nv_bfloat16 *W2Tb) {
  const size_t tot = n1 + (size_t)H * H;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      W1b[i] = __float2bfloat16_rn(W1[i]);
    } else {
      const size_t k = i - n1;
      const size_t o = k / H, in = k % H;
      const __nv_bfloat16 b = __float2bfloat16_rn(W2[k]);
      W2b[k] = b;
      W2Tb[in * H + o] = b;
    }
  }
}

// ---- host side -------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encode(std::string &err) {
  if (g_encode) return SP_OK;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      !fn || q != cudaDriverEntryPointSuccess) {
    err = "cuTensorMapEncodeTiled is not available from the driver";
    return SP_ERR_CUDA;
  }
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return SP_OK;
}

// 2-D bf16 tensor [rows][k] (k contiguous), boxes of box_rows x 64, 128-byte swizzle.
int make_map(CUtensorMap *m, const void *ptr, uint64_t rows, uint64_t k, uint32_t box_rows, std::string &err) {
  int rc = get_encode(err);
  if (rc) return rc;
  if (((uintptr_t)ptr & 15u) || (k % 64) || rows < box_rows) {
    err = "GEMM operand not aligned to the tile shape";
    return SP_ERR_ARG;
  }
  cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(k * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return SP_ERR_CUDA;
  }
  return SP_OK;
}

template <int EPI>
cudaError_t launch_gemm(const CUtensorMap &ta, const CUtensorMap &tb, int m_tiles, int kc_total, int splits,
                        const EpiArgs &E, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(umma_gemm_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  splits = std::max(1, std::min(splits, kc_total));
  const int per = (kc_total + splits - 1) / splits;
  splits = (kc_total + per - 1) / per;  // every CTA gets at least one chunk
  umma_gemm_kernel<EPI><<<dim3(m_tiles, splits), 128, SMEM_BYTES, st>>>(ta, tb, per, kc_total, E);
  note_launch(1);
  return cudaGetLastError();
}

uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

struct Buffers {
  int w = 0, D = 0, Dpad = 0;
  size_t np = 0, oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, ow3 = 0, ob3 = 0;
  float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
  __nv_bfloat16 *W1b = nullptr, *W2b = nullptr, *W2Tb = nullptr;
  int cap = 0;  // batch rows
  uint8_t *boards = nullptr;
  uint32_t *idx = nullptr;
  int32_t *slack = nullptr;
  float *target = nullptr, *y = nullptr, *scal = nullptr;  // scal: loss
  int *err = nullptr;
  __nv_bfloat16 *H1 = nullptr, *H1T = nullptr, *dH2 = nullptr, *dH2T = nullptr, *dH1T = nullptr, *XT = nullptr;
  void release() {
    void *ps[] = {P, G, M, V, W1b, W2b, W2Tb, boards, idx, slack, target, y, scal, err, H1, H1T, dH2, dH2T, dH1T, XT};
    for (void *p : ps)
      if (p) cudaFree(p);
  }
};

#define LBM_CUDA(x)                                                       \
  do {                                                                    \
    cudaError_t e_ = (x);                                                 \
    if (e_ != cudaSuccess) {                                              \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);              \
      return SP_ERR_CUDA;                                                 \
    }                                                                     \
  } while (0)

Model::Model(int width) : w_(width), b_(new Buffers) {
  Buffers &B = *b_;
  B.w = width;
  B.D = feature_dim(width);
  B.Dpad = feature_dim_padded(width);
  B.np = num_params(width);
  B.oW1 = 0;
  B.ob1 = (size_t)B.D * H;
  B.oW2 = B.ob1 + H;
  B.ob2 = B.oW2 + (size_t)H * H;
  B.ow3 = B.ob2 + H;
  B.ob3 = B.ow3 + H;
}

Model::~Model() {
  b_->release();
  delete b_;
}

int Model::init(uint64_t seed, cudaStream_t st, std::string &err) {
  Buffers &B = *b_;
  std::vector<float> p(B.np, 0.f);
  uint64_t s = seed;
  auto normal = [&]() {
    // Box-Muller on two 53-bit uniforms
    const double u1 = ((splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  };
  const int N = w_ * w_;
  const double s1 = std::sqrt(2.0 / N), s2 = std::sqrt(2.0 / H), s3 = std::sqrt(1.0 / H);
  for (size_t i = 0; i < (size_t)B.D * H; ++i) p[B.oW1 + i] = (float)(normal() * s1);
  for (size_t i = 0; i < (size_t)H * H; ++i) p[B.oW2 + i] = (float)(normal() * s2);
  for (size_t i = 0; i < (size_t)H; ++i) p[B.ow3 + i] = (float)(normal() * s3);
  p[B.ob3] = 8.f;
  return import_params(p.data(), p.size(), st, err);
}

int Model::import_params(const float *src, size_t n, cudaStream_t st, std::string &err) {
  Buffers &B = *b_;
  if (n != B.np) {
    err = "parameter count mismatch";
    return SP_ERR_ARG;
  }
  if (!B.P) {
    LBM_CUDA(cudaMalloc(&B.P, B.np * sizeof(float)));
    LBM_CUDA(cudaMalloc(&B.G, B.np * sizeof(float)));
    LBM_CUDA(cudaMalloc(&B.M, B.np * sizeof(float)));
    LBM_CUDA(cudaMalloc(&B.V, B.np * sizeof(float)));
    LBM_CUDA(cudaMalloc(&B.W1b, (size_t)B.D * H * 2));
    LBM_CUDA(cudaMalloc(&B.W2b, (size_t)H * H * 2));
    LBM_CUDA(cudaMalloc(&B.W2Tb, (size_t)H * H * 2));
    LBM_CUDA(cudaMalloc(&B.scal, 4 * sizeof(float)));
    LBM_CUDA(cudaMalloc(&B.err, sizeof(int)));
  }
  LBM_CUDA(cudaMemcpyAsync(B.P, src, B.np * sizeof(float), cudaMemcpyHostToDevice, st));
  LBM_CUDA(cudaMemsetAsync(B.M, 0, B.np * sizeof(float), st));
  LBM_CUDA(cudaMemsetAsync(B.V, 0, B.np * sizeof(float), st));
  LBM_CUDA(cudaMemsetAsync(B.err, 0, sizeof(int), st));
  refresh_kernel<<<256, 256, 0, st>>>(B.P + B.oW1, (size_t)B.D * H, B.P + B.oW2, B.W1b, B.W2b, B.W2Tb);
  note_launch(1);
  ++launches_;
  LBM_CUDA(cudaGetLastError());
  LBM_CUDA(cudaStreamSynchronize(st));
  adam_t_ = 0;
  ready_ = true;
  return SP_OK;
}

int Model::export_params(float *dst, size_t n, cudaStream_t st, std::string &err) {
  Buffers &B = *b_;
  if (!ready_) {
    err = "model not initialised";
    return SP_ERR_ARG;
  }
  if (n != B.np) {
    err = "parameter count mismatch";
    return SP_ERR_ARG;
  }
  LBM_CUDA(cudaMemcpyAsync(dst, B.P, B.np * sizeof(float), cudaMemcpyDeviceToHost, st));
  LBM_CUDA(cudaStreamSynchronize(st));
  return SP_OK;
}

int Model::ensure_batch(int n, std::string &err) {
  Buffers &B = *b_;
  const int need = (n + BM - 1) / BM * BM;
  if (need <= B.cap) return SP_OK;
  int cap = std::max(need, 1024);
  void *ps[] = {B.boards, B.idx, B.slack, B.target, B.y, B.H1, B.H1T, B.dH2, B.dH2T, B.dH1T, B.XT};
  for (void *p : ps)
    if (p) cudaFree(p);
  B.cap = 0;
  const int N = w_ * w_;
  LBM_CUDA(cudaMalloc(&B.boards, (size_t)cap * N));
  LBM_CUDA(cudaMalloc(&B.idx, (size_t)cap * 4));
  LBM_CUDA(cudaMalloc(&B.slack, (size_t)cap * 4));
  LBM_CUDA(cudaMalloc(&B.target, (size_t)cap * 4));
  LBM_CUDA(cudaMalloc(&B.y, (size_t)cap * 4));
  LBM_CUDA(cudaMalloc(&B.H1, (size_t)cap * H * 2));
  LBM_CUDA(cudaMalloc(&B.H1T, (size_t)cap * H * 2));
  LBM_CUDA(cudaMalloc(&B.dH2, (size_t)cap * H * 2));
  LBM_CUDA(cudaMalloc(&B.dH2T, (size_t)cap * H * 2));
  LBM_CUDA(cudaMalloc(&B.dH1T, (size_t)cap * H * 2));
  LBM_CUDA(cudaMalloc(&B.XT, (size_t)cap * B.Dpad * 2));
  B.cap = cap;
  return SP_OK;
}

static int launch_embed(int w, const EmbedArgs &A, int rows, cudaStream_t st) {
  if (w == 4) embed_kernel<4><<<rows / 32, 256, 0, st>>>(A);
  else embed_kernel<5><<<rows / 32, 256, 0, st>>>(A);
  note_launch(1);
  return cudaGetLastError() == cudaSuccess ? SP_OK : SP_ERR_CUDA;
}

int Model::forward_infer(int n, float *out, cudaStream_t st, std::string &err) {
  Buffers &B = *b_;
  const int rows = (n + BM - 1) / BM * BM;
  CUtensorMap ta, tb;
  int rc = make_map(&ta, B.H1, rows, H, BM, err);
  if (!rc) rc = make_map(&tb, B.W2b, H, H, H, err);
  if (rc) return rc;
  EpiArgs E{};
  E.m_valid = n;
  E.b2 = B.P + B.ob2;
  E.w3 = B.P + B.ow3;
  E.b3 = B.P + B.ob3;
  E.y = B.y;
  E.err = B.err;
  LBM_CUDA(launch_gemm<EPI_INFER>(ta, tb, rows / BM, H / BK, 1, E, st));
  launches_ += 1;
  int herr = 0;
  LBM_CUDA(cudaMemcpyAsync(out, B.y, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  LBM_CUDA(cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  LBM_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    err = "tensor-core GEMM wait timed out";
    return SP_ERR_TIMEOUT;
  }
  return SP_OK;
}

int Model::predict(const uint8_t *tiles, const int32_t *slack, int n, float *out, cudaStream_t st,
                   std::string &err) {
  if (!ready_) {
    err = "model not initialised";
    return SP_ERR_ARG;
  }
  Buffers &B = *b_;
  const int N = w_ * w_;
  const int chunk = 1 << 16;
  for (int off = 0; off < n; off += chunk) {
    const int m = std::min(chunk, n - off);
    int rc = ensure_batch(m, err);
    if (rc) return rc;
    LBM_CUDA(cudaMemcpyAsync(B.boards, tiles + (size_t)off * N, (size_t)m * N, cudaMemcpyHostToDevice, st));
    LBM_CUDA(cudaMemcpyAsync(B.slack, slack + off, (size_t)m * 4, cudaMemcpyHostToDevice, st));
    EmbedArgs A{};
    A.boards = B.boards;
    A.bstride = N;
    A.slack = B.slack;
    A.n = m;
    A.W1 = B.W1b;
    A.b1 = B.P + B.ob1;
    A.H1 = B.H1;
    const int rows = (m + BM - 1) / BM * BM;
    A.ldt = rows;
    if (launch_embed(w_, A, rows, st)) {
      err = "layer-1 kernel launch failed";
      return SP_ERR_CUDA;
    }
    launches_ += 1;
    rc = forward_infer(m, out + off, st, err);
    if (rc) return rc;
  }
  return SP_OK;
}

int Model::predict_subs(const SubRoot *d_subs, const uint32_t *idx, const int32_t *slack, int n, float *out,
                        cudaStream_t st, std::string &err) {
  if (!ready_) {
    err = "model not initialised";
    return SP_ERR_ARG;
  }
  Buffers &B = *b_;
  const int chunk = 1 << 16;
  for (int off = 0; off < n; off += chunk) {
    const int m = std::min(chunk, n - off);
    int rc = ensure_batch(m, err);
    if (rc) return rc;
    LBM_CUDA(cudaMemcpyAsync(B.idx, idx + off, (size_t)m * 4, cudaMemcpyHostToDevice, st));
    LBM_CUDA(cudaMemcpyAsync(B.slack, slack + off, (size_t)m * 4, cudaMemcpyHostToDevice, st));
    EmbedArgs A{};
    A.boards = reinterpret_cast<const uint8_t *>(d_subs);  // SubRoot.board is its first member
    A.idx = B.idx;
    A.bstride = (int)sizeof(SubRoot);
    A.slack = B.slack;
    A.n = m;
    A.W1 = B.W1b;
    A.b1 = B.P + B.ob1;
    A.H1 = B.H1;
    const int rows = (m + BM - 1) / BM * BM;
    A.ldt = rows;
    if (launch_embed(w_, A, rows, st)) {
      err = "layer-1 kernel launch failed";
      return SP_ERR_CUDA;
    }
    launches_ += 1;
    rc = forward_infer(m, out + off, st, err);
    if (rc) return rc;
  }
  return SP_OK;
}

int Model::train_step(const uint8_t *tiles, const int32_t *slack, const float *target, int n, float lr,
                      bool update, float *loss, float *grads, cudaStream_t st, std::string &err) {
  if (!ready_) {
    err = "model not initialised";
    return SP_ERR_ARG;
  }
  if (n <= 0 || n % BM) {
    err = "training batch must be a positive multiple of 128 rows";
    return SP_ERR_ARG;
  }
  Buffers &B = *b_;
  int rc = ensure_batch(n, err);
  if (rc) return rc;
  const int N = w_ * w_;
  LBM_CUDA(cudaMemcpyAsync(B.boards, tiles, (size_t)n * N, cudaMemcpyHostToDevice, st));
  LBM_CUDA(cudaMemcpyAsync(B.slack, slack, (size_t)n * 4, cudaMemcpyHostToDevice, st));
  LBM_CUDA(cudaMemcpyAsync(B.target, target, (size_t)n * 4, cudaMemcpyHostToDevice, st));
  LBM_CUDA(cudaMemsetAsync(B.G, 0, B.np * sizeof(float), st));
  LBM_CUDA(cudaMemsetAsync(B.scal, 0, 4 * sizeof(float), st));
  LBM_CUDA(cudaMemsetAsync(B.err, 0, sizeof(int), st));
  LBM_CUDA(cudaMemsetAsync(B.XT, 0, (size_t)B.Dpad * n * 2, st));
  EmbedArgs A{};
  A.boards = B.boards;
  A.bstride = N;
  A.slack = B.slack;
  A.n = n;
  A.W1 = B.W1b;
  A.b1 = B.P + B.ob1;
  A.H1 = B.H1;
  A.H1T = B.H1T;
  A.XT = B.XT;
  A.ldt = n;
  if (launch_embed(w_, A, n, st)) {
    err = "layer-1 kernel launch failed";
    return SP_ERR_CUDA;
  }
  CUtensorMap m_a, m_b;
  EpiArgs E{};
  E.ldt = n;
  E.inv_b = 1.f / (float)n;
  E.b2 = B.P + B.ob2;
  E.w3 = B.P + B.ow3;
  E.b3 = B.P + B.ob3;
  E.target = B.target;
  E.y = B.y;
  E.dH2 = B.dH2;
  E.dH2T = B.dH2T;
  E.H1 = B.H1;
  E.dH1T = B.dH1T;
  E.gw3 = B.G + B.ow3;
  E.gb2 = B.G + B.ob2;
  E.gb3 = B.G + B.ob3;
  E.gb1 = B.G + B.ob1;
  E.loss = B.scal;
  E.err = B.err;
  // forward + loss + layer-3 backward
  E.m_valid = n;
  if ((rc = make_map(&m_a, B.H1, n, H, BM, err)) || (rc = make_map(&m_b, B.W2b, H, H, H, err))) return rc;
  LBM_CUDA(launch_gemm<EPI_FWD>(m_a, m_b, n / BM, H / BK, 1, E, st));
  // dZ1 = dH2 . W2
  if ((rc = make_map(&m_a, B.dH2, n, H, BM, err)) || (rc = make_map(&m_b, B.W2Tb, H, H, H, err))) return rc;
  LBM_CUDA(launch_gemm<EPI_BWD1>(m_a, m_b, n / BM, H / BK, 1, E, st));
  // dW2 = dH2^T . H1 (K = batch, split over about 150 CTAs)
  const int kc = n / BK;
  E.C = B.G + B.oW2;
  E.m_valid = H;
  if ((rc = make_map(&m_a, B.dH2T, H, n, BM, err)) || (rc = make_map(&m_b, B.H1T, H, n, H, err))) return rc;
  LBM_CUDA(launch_gemm<EPI_F32_ATOMIC>(m_a, m_b, H / BM, kc, 75, E, st));
  // dW1 = X^T . dH1
  E.C = B.G + B.oW1;
  E.m_valid = B.D;
  if ((rc = make_map(&m_a, B.XT, B.Dpad, n, BM, err)) || (rc = make_map(&m_b, B.dH1T, H, n, H, err))) return rc;
  LBM_CUDA(launch_gemm<EPI_F32_ATOMIC>(m_a, m_b, B.Dpad / BM, kc, std::max(1, 150 / (B.Dpad / BM)), E, st));
  launches_ += 5;
  if (update) {
    ++adam_t_;
    const float c1 = 1.f - std::pow(0.9f, (float)adam_t_), c2 = 1.f - std::pow(0.999f, (float)adam_t_);
    adam_kernel<<<512, 256, 0, st>>>(B.P, B.G, B.M, B.V, B.np, lr, c1, c2);
    refresh_kernel<<<256, 256, 0, st>>>(B.P + B.oW1, (size_t)B.D * H, B.P + B.oW2, B.W1b, B.W2b, B.W2Tb);
    note_launch(2);
    launches_ += 2;
    LBM_CUDA(cudaGetLastError());
  }
  float hl = 0;
  int herr = 0;
  LBM_CUDA(cudaMemcpyAsync(&hl, B.scal, sizeof(float), cudaMemcpyDeviceToHost, st));
  LBM_CUDA(cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (grads) LBM_CUDA(cudaMemcpyAsync(grads, B.G, B.np * sizeof(float), cudaMemcpyDeviceToHost, st));
  LBM_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    err = "tensor-core GEMM wait timed out";
    return SP_ERR_TIMEOUT;
  }
  if (loss) *loss = hl;
  return SP_OK;
}

int Model::gemm_stall_selftest(int starve_chunk, int timeout_ms, int *device_status, cudaStream_t st,
                               std::string &err) {
  constexpr int M = BM, K = 4 * BK;
  if (starve_chunk < 0 || starve_chunk >= K / BK || timeout_ms < 10 || timeout_ms > 2000 || !device_status) {
    err = "selftest needs starve_chunk in [0, 4) and timeout_ms in [10, 2000]";
    return SP_ERR_ARG;
  }
  *device_status = SP_OK;
  void *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int *derr = nullptr;
  int rc = SP_OK;
  do {
    if (cudaMalloc(&dA, (size_t)M * K * 2) || cudaMalloc(&dB, (size_t)H * K * 2) ||
        cudaMalloc(&dC, (size_t)M * H * 4) || cudaMalloc((void **)&derr, sizeof(int))) {
      err = "cudaMalloc failed";
      rc = SP_ERR_CUDA;
      break;
    }
    if (cudaMemsetAsync(dA, 0, (size_t)M * K * 2, st) || cudaMemsetAsync(dB, 0, (size_t)H * K * 2, st) ||
        cudaMemsetAsync(derr, 0, sizeof(int), st)) {
      err = "memset failed";
      rc = SP_ERR_CUDA;
      break;
    }
    CUtensorMap ta, tb;
    if ((rc = make_map(&ta, dA, M, K, BM, err)) || (rc = make_map(&tb, dB, H, K, H, err))) break;
    EpiArgs E{};
    E.C = (float *)dC;
    E.m_valid = M;
    E.err = derr;
    E.wait_ns = (unsigned long long)timeout_ms * 1000000ull;
    E.starve_kc1 = starve_chunk + 1;
    if (launch_gemm<EPI_F32>(ta, tb, 1, K / BK, 1, E, st) != cudaSuccess) {
      err = "GEMM launch failed";
      rc = SP_ERR_CUDA;
      break;
    }
    int herr = 0;
    if (cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
      err = std::string("GEMM self-test failed: ") + cudaGetErrorString(cudaGetLastError());
      rc = SP_ERR_CUDA;
      break;
    }
    *device_status = herr ? SP_ERR_TIMEOUT : SP_OK;
  } while (0);
  if (dA) cudaFree(dA);
  if (dB) cudaFree(dB);
  if (dC) cudaFree(dC);
  if (derr) cudaFree(derr);
  return rc;
}

int Model::gemm_nt(const uint16_t *A, const uint16_t *Bm, float *C, int M, int N, int K, cudaStream_t st,
                   std::string &err) {
  if (M <= 0 || M % BM || N != H || K <= 0 || K % BK) {
    err = "gemm_nt needs M a multiple of 128, N = 256, K a multiple of 64";
    return SP_ERR_ARG;
  }
  void *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int *derr = nullptr;
  auto cleanup = [&]() {
    if (dA) cudaFree(dA);
    if (dB) cudaFree(dB);
    if (dC) cudaFree(dC);
    if (derr) cudaFree(derr);
  };
  int rc = SP_OK;
  std::string e2;
  do {
    if (cudaMalloc(&dA, (size_t)M * K * 2) || cudaMalloc(&dB, (size_t)N * K * 2) ||
        cudaMalloc(&dC, (size_t)M * N * 4) || cudaMalloc((void **)&derr, sizeof(int))) {
      err = "cudaMalloc failed";
      rc = SP_ERR_CUDA;
      break;
    }
    if (cudaMemcpyAsync(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice, st) ||
        cudaMemcpyAsync(dB, Bm, (size_t)N * K * 2, cudaMemcpyHostToDevice, st) ||
        cudaMemsetAsync(derr, 0, sizeof(int), st)) {
      err = "copy failed";
      rc = SP_ERR_CUDA;
      break;
    }
    CUtensorMap ta, tb;
    if ((rc = make_map(&ta, dA, M, K, BM, err)) || (rc = make_map(&tb, dB, N, K, H, err))) break;
    EpiArgs E{};
    E.C = (float *)dC;
    E.m_valid = M;
    E.err = derr;
    if (launch_gemm<EPI_F32>(ta, tb, M / BM, K / BK, 1, E, st) != cudaSuccess) {
      err = "GEMM launch failed";
      rc = SP_ERR_CUDA;
      break;
    }
    int herr = 0;
    if (cudaMemcpyAsync(C, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost, st) ||
        cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
      err = std::string("GEMM failed: ") + cudaGetErrorString(cudaGetLastError());
      rc = SP_ERR_CUDA;
      break;
    }
    if (herr) {
      err = "tensor-core GEMM wait timed out";
      rc = SP_ERR_TIMEOUT;
    }
  } while (0);
  cleanup();
  return rc;
}

}  // namespace lbm
}  // namespace sp
