// Learned load balancer: an MLP that predicts log2(1 + generated nodes) of a
// root's subtree at a threshold from the root's tile placement and its slack
// (threshold - f) / 2.  No reference counterpart: the reference balances
// only from the previous round's measured loads
// (src/24puzzle_block_parallel_with_pdb.cu:839-897).
//
// Architecture: one-hot tile placement ((N-1) x N features) + slack
// -> 256 ReLU -> 256 ReLU -> 1, BF16 weights and activations, FP32
// accumulation.  Layer 1 on a one-hot input is a gather-sum of N-1 weight rows
// (no GEMM); layers 2-3, the loss and the backward pass run as tcgen05 GEMMs
// with fused epilogues (mlp.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

namespace sp {

struct SubRoot;

namespace lbm {

constexpr int kHidden = 256;

inline int feature_dim(int w) { return (w * w - 1) * w * w + 1; }
inline int feature_dim_padded(int w) { return (feature_dim(w) + 127) / 128 * 128; }
// W1 [D][256], b1 [256], W2 [256 out][256 in], b2 [256], w3 [256], b3 [1]
inline size_t num_params(int w) {
  const size_t D = (size_t)feature_dim(w), H = kHidden;
  return D * H + H + H * H + H + H + 1;
}

struct Buffers;

class Model {
 public:
  explicit Model(int width);
  ~Model();
  Model(const Model &) = delete;
  Model &operator=(const Model &) = delete;

  // He-normal weights from a seeded xoshiro256** stream, zero biases,
  // b3 = 8 (about 256 nodes).
  int init(uint64_t seed, cudaStream_t st, std::string &err);
  int import_params(const float *src, size_t n, cudaStream_t st, std::string &err);
  int export_params(float *dst, size_t n, cudaStream_t st, std::string &err);
  bool ready() const { return ready_; }

  // Host arrays: tiles n x N, slack n; out n predictions.
  int predict(const uint8_t *tiles, const int32_t *slack, int n, float *out, cudaStream_t st,
              std::string &err);
  // Device SubRoots selected by host index lists (idx n, slack n).
  int predict_subs(const SubRoot *d_subs, const uint32_t *idx, const int32_t *slack, int n, float *out,
                   cudaStream_t st, std::string &err);
  // One mean-squared-error step on a batch (n a multiple of 128).  update:
  // apply Adam(lr); grads (optional, num_params floats) receives the
  // gradient; loss the batch's mean squared error.
  int train_step(const uint8_t *tiles, const int32_t *slack, const float *target, int n, float lr, bool update,
                 float *loss, float *grads, cudaStream_t st, std::string &err);

  // C[M x 256] = A[M x K] . B[256 x K]^T, bf16 in, fp32 out (host arrays):
  // the tcgen05 GEMM on its own, for tests.
  static int gemm_nt(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, cudaStream_t st,
                     std::string &err);
  // Self-test of the GEMM's bounded waits: a 128 x 256 x 256 GEMM whose K
  // chunk `starve_chunk` (0..3) never gets its copies, so the wait for it
  // runs out after timeout_ms; *device_status = SP_ERR_TIMEOUT when the
  // kernel gave up, drained its copies, freed its tensor memory and returned.
  static int gemm_stall_selftest(int starve_chunk, int timeout_ms, int *device_status, cudaStream_t st,
                                 std::string &err);

  uint64_t launches() const { return launches_; }

 private:
  int ensure_batch(int n, std::string &err);
  int forward_infer(int n, float *out, cudaStream_t st, std::string &err);

  int w_;
  bool ready_ = false;
  int adam_t_ = 0;
  uint64_t launches_ = 0;
  Buffers *b_;
};

}  // namespace lbm
}  // namespace sp
