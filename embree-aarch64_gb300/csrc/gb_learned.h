// gb_learned.h -- the learned hit proposer (gb_learned.cu).
//
// A proposer maps a ray to four BVH subtrees ("treelets") that it expects the
// ray to hit.  The traversal searches them before the whole tree (seeded
// stacks, gb_trace.cu), so a good guess ends an occlusion ray at once or
// lowers a closest-hit ray's tfar early, and the results stay those of the
// plain traversal.
//
// Network: a multiresolution hash-grid encoding (Mueller et al. 2022,
// "Instant neural graphics primitives") of the ray origin (8 levels) and
// direction (8 levels), 2 BF16 features per level and 2^18 entries per level,
// followed by a 32-64-64-64-4096 MLP with ReLU hidden layers.  The 4096
// outputs are the treelets' logits (softmax cross-entropy in training, top-4 in
// inference).  Products run on the BF16 tensor cores with FP32 accumulation.
//
// Parameters live in one FP32 array (the Adam master copy) with a BF16 mirror
// the kernels read:
//   [table: 16 levels x 2^18 entries x 2 features]
//   [W1 64x32][b1 64][W2 64x64][b2 64][W3 64x64][b3 64][W4 4096x64][b4 4096]
// Weights are stored [out][in] (row o holds the weights of output o).
#pragma once
#include <cstdint>
#include <vector>

#include "gb_common.h"

namespace gb {

constexpr int kLevels = 16;          // hash-grid levels: 8 origin + 8 direction
constexpr int kOriginLevels = 8;
constexpr int kLog2Table = 18;
constexpr uint32_t kTableSize = 1u << kLog2Table;
constexpr int kFeat = 2;
constexpr int kIn = kLevels * kFeat;  // 32
constexpr int kHidden = 64;
constexpr int kTreelets = 4096;
constexpr int kTopK = 4;

constexpr size_t kOffTable = 0;
constexpr size_t kOffW1 = (size_t)kLevels * kTableSize * kFeat;
constexpr size_t kOffB1 = kOffW1 + (size_t)kHidden * kIn;
constexpr size_t kOffW2 = kOffB1 + kHidden;
constexpr size_t kOffB2 = kOffW2 + (size_t)kHidden * kHidden;
constexpr size_t kOffW3 = kOffB2 + kHidden;
constexpr size_t kOffB3 = kOffW3 + (size_t)kHidden * kHidden;
constexpr size_t kOffW4 = kOffB3 + kHidden;
constexpr size_t kOffB4 = kOffW4 + (size_t)kTreelets * kHidden;
constexpr size_t kNumParams = kOffB4 + kTreelets;

// Grid resolution of level l: origin levels 16 * 2^l, direction levels 4 * 2^(l-8).
inline uint32_t level_resolution(int l) { return l < kOriginLevels ? (16u << l) : (4u << (l - kOriginLevels)); }

// Maps ray origins into [0,1]^3: q = (o - lo) * scale, clamped.
struct GridSpec {
  float lo[3];
  float scale[3];
};

struct TrainStats {
  double loss = 0;      // mean cross-entropy of the last epoch
  double top1 = 0;      // fraction of the last epoch's rays whose label ranked first
  double top4 = 0;      // ... within the top four
  uint32_t steps = 0;   // Adam steps taken so far
  uint32_t samples = 0; // labelled rays in the last training call
};

class Proposer {
 public:
  // node_of_treelet: BVH node index of each treelet root (<= kTreelets entries);
  // prim_treelet: treelet of each primitive, indexed geom_prefix[geomID] + primID;
  // geom_prefix: per geometry ID, the first primitive index (kInvalidID: none).
  cudaError_t init(const std::vector<uint32_t>& node_of_treelet, const std::vector<uint32_t>& prim_treelet,
                   const std::vector<uint32_t>& geom_prefix, const GridSpec& grid, uint32_t seed, cudaStream_t st);
  void release();
  ~Proposer() { release(); }

  // Trains on logged closest-hit records (RTCRayHit, device-accessible memory):
  // rays with a hit are labelled with their hit primitive's treelet.
  cudaError_t train(const char* records, uint64_t stride, uint32_t M, uint32_t epochs, uint32_t batch, float lr,
                    cudaStream_t st);
  // Top-4 proposals for M rays (RTCRay prefix of each record): node indices for
  // a seeded traversal (seeds, optional) and treelet indices (treelets, 4 per ray, optional).
  // d_count (optional, device): the number of rays is min(*d_count, M), read by the kernel.
  // err (optional, device): receives kErrIterationLimit if the tensor-core kernel timed out.
  cudaError_t predict(const char* rays, uint64_t stride, uint32_t M, uint4* seeds, uint32_t* treelets,
                      cudaStream_t st, const uint32_t* d_count = nullptr, uint32_t* err = nullptr);
  // Loss and gradients of one batch (rays + labels in device memory); grads
  // receives kNumParams floats (device).
  cudaError_t gradients(const char* rays, uint64_t stride, const int32_t* labels, uint32_t B, float* grads,
                        float* loss, cudaStream_t st);

  cudaError_t get_params(float* host, cudaStream_t st) const;
  cudaError_t set_params(const float* host, cudaStream_t st);

  uint32_t num_treelets = 0;
  uint32_t num_prims = 0;
  bool use_mma_sync = false;  // inference on mma.sync instead of tcgen05 (device key gpu.proposer=mma)
  GridSpec grid{};
  TrainStats stats;

 private:
  cudaError_t ensure_batch(uint32_t B);
  cudaError_t step_forward_backward(const char* rays, uint64_t stride, const uint32_t* idx, const int32_t* labels,
                                    uint32_t B, cudaStream_t st);

  float* P_ = nullptr;         // FP32 parameters (Adam master)
  uint16_t* Pb_ = nullptr;     // BF16 mirror
  float* G_ = nullptr;         // gradients
  float* m_ = nullptr;         // Adam moments
  float* v_ = nullptr;
  uint32_t* node_of_treelet_ = nullptr;
  uint32_t* prim_treelet_ = nullptr;
  uint32_t* geom_prefix_ = nullptr;
  uint32_t num_geom_ids_ = 0;
  float* acc_ = nullptr;       // device accumulators: loss sum, top1 count, top4 count, labelled count
  uint16_t* W4p_ = nullptr;    // output weights in the tensor cores' shared-memory layout
  uint16_t* H_ = nullptr;      // inference: last hidden layer of every tile (same layout)
  size_t hcap_ = 0;
  uint32_t* err_ = nullptr;    // error word of inference calls without one
  cudaError_t refresh_w4(cudaStream_t st);

  // batch scratch
  uint32_t cap_ = 0;
  uint16_t *X0_ = nullptr, *H1_ = nullptr, *H2_ = nullptr, *H3_ = nullptr, *dZ4_ = nullptr, *dZ_ = nullptr;
  float *Z_ = nullptr, *Z4_ = nullptr, *dH_ = nullptr, *dX0_ = nullptr;
};

// Chooses up to max_treelets (<= kTreelets) subtree roots over the BVH's
// triangles: starting from the root, the subtree with the most triangles is
// replaced by its internal children while the count allows and while the
// triangles it holds directly (which then belong to no treelet) are at most 1/8
// of it.  Outputs the roots and, per triangle record, the treelet that holds it
// (or kInvalidID).
cudaError_t choose_treelets(const DeviceBVH& bvh, cudaStream_t st, std::vector<uint32_t>* roots,
                            std::vector<uint32_t>* record_treelet, std::vector<uint32_t>* record_prim,
                            std::vector<uint32_t>* record_geom, uint32_t max_treelets = kTreelets);

}  // namespace gb
