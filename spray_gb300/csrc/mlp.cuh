// Learned domain-order proposal: a 54-64-64-64-8 MLP (BF16 weights, FP32
// accumulation) that reads a ray and the boxes of its first eight candidate
// domains and scores which candidate holds the closest hit.  The forward and
// backward GEMMs run on the 5th-generation tensor cores (tcgen05.mma with the
// accumulators in tensor memory); feature building, bias, ReLU, softmax and
// Adam run on the CUDA cores.  SpRay has no learned component: this is the
// proposal the scheduler consults to order work, never to decide a hit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace spray {
namespace mlp {

constexpr int kCand = 8;        // candidate domains scored per ray
constexpr int kIn = 6 + 6 * kCand;  // 54 input features
constexpr int kK = 64;          // padded input width
constexpr int kHid = 64;
constexpr int kOutPad = 16;     // 8 logits padded to the smallest N of an M=128 MMA
constexpr int kTile = 128;      // rows per MMA tile (one per thread of a 128-thread CTA)

// One fp32 parameter vector: W1 b1 W2 b2 W3 b3 W4 b4, weights row-major
// [out][in].  Padding (W1 columns 54..63, W4 rows 8..15) stays zero.
constexpr int kW1 = 0, kB1 = kW1 + kHid * kK;
constexpr int kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid, kB3 = kW3 + kHid * kHid;
constexpr int kW4 = kB3 + kHid, kB4 = kW4 + kOutPad * kHid;
constexpr int kParams = kB4 + kOutPad;  // 13520
constexpr int kPartial = kParams + 2;   // per-CTA gradient, loss sum, labelled rows

// A training pair: the ray, its candidate domains in (t, id) order and the
// position of the candidate that holds the closest hit (-1: none).
struct Sample {
  float org[3];
  float dir[3];
  uint16_t cand[kCand];
  int32_t ncand;
  int32_t label;
};
static_assert(sizeof(Sample) == 48, "sample layout");

// Feature normalisation: positions map to (p - centre) * scale.
struct Norm {
  float centre[3];
  float scale;
};

// Candidates read from the scheduler's per-ray lists (radiance rays).
struct ArenaSource {
  const uint32_t* count;     // alive rays
  const uint32_t* list;      // alive index -> sample
  const float4* org;
  const float4* dir;
  const uint2* arena;        // (domain | position << 16, entry t)
  const uint32_t* list_off;
  const uint32_t* list_cnt;
};

struct Net {
  const float* params;       // kParams floats
  const float* boxes;        // 6 floats per domain: min xyz, max xyz
  Norm norm;
  int* error;                // set to nonzero when a bounded wait gave up
};

// Inference over the live rays of a wavefront: pred[i] = predicted position
// (0..7) of the candidate holding the hit of alive ray i (0 when it has fewer
// than two candidates).
void launchPredictArena(cudaStream_t s, const Net& net, const ArenaSource& src, uint8_t* pred,
                        int nblocks);
// Inference over samples (test hook): logits [n][8] (invalid candidates get
// -inf) and the argmax.
void launchPredictSamples(cudaStream_t s, const Net& net, const Sample* samples, int64_t n,
                          float* logits, int32_t* pred, int nblocks);
// Top-1 accuracy on held-out samples: counts[3] (zeroed by the caller) +=
// labelled samples with at least two candidates, those whose argmax is the
// label, and those whose label is the nearest candidate (the accuracy of
// always predicting position 0, i.e. the front-to-back order).
void launchEvaluate(cudaStream_t s, const Net& net, const Sample* samples, int64_t n, unsigned long long* counts,
                    int nblocks);
// Gradient of the mean cross-entropy over the labelled rows of a batch:
// every CTA writes a partial [kPartial] (gradient, loss sum, labelled rows).
// `inv_count` scales the loss gradient (1 / labelled rows of the whole batch).
void launchGrad(cudaStream_t s, const Net& net, const Sample* batch, int64_t n, float inv_count,
                float* partial, int nblocks);
// Sums `nparts` partials in order into grad[kParams + 2] and, when lr > 0,
// applies one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at step `step`.
void launchReduceAdam(cudaStream_t s, const float* partial, int nparts, float* grad, float* params,
                      float* m, float* v, float lr, int step);
// Training-pair emission after the hits of a depth are resolved: every alive
// ray with at least two candidates and a hit appends (ray, candidates, label).
// Pairs are appended in alive order (stable compaction), so the buffer's
// content does not depend on thread timing; `label`, `flag` (one per alive
// ray), `sel`, `nsel` and `block_tmp` (nblocks words) are scratch.
void launchCollect(cudaStream_t s, const ArenaSource& src, const uint64_t* ray_key,
                   const DomainDev* domains, Sample* out, unsigned long long* filled,
                   uint64_t capacity, int8_t* label, uint8_t* flag, uint32_t* sel, uint32_t* nsel,
                   uint32_t* block_tmp, int nblocks);
// Predicted hits per domain: counts[d] += 1 for the predicted candidate d of
// every alive ray with at least one candidate (counts zeroed by the caller).
void launchPredCount(cudaStream_t s, const ArenaSource& src, const uint8_t* pred, uint32_t* counts,
                     int nblocks);
// CTAs of the gradient kernel (one per SM: it holds all 512 tensor-memory columns).
int gradBlocks(int num_sms);

}  // namespace mlp
}  // namespace spray
