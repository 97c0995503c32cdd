// Domain-parallel (in-situ) execution across ranks.
//
// SpRay's in-situ tracer (insitu::MultiThreadTracer,
// src/insitu/insitu_multithread_tracer.inl:313-442) pins every domain to one
// MPI rank (InsituPartition::partition, src/render/data_partition.h:60-137),
// traces rays only in the domains its rank owns, and after each bounce
// composites the per-sample closest-hit distances with an MPI MIN all-reduce
// and the occlusion bits with a BOR all-reduce (VBuf::compositeTbuf and
// compositeObuf, src/insitu/insitu_vbuf.h:109-129).
//
// Here each rank's tracer keeps the whole ray state of a wavefront (camera
// rays, shading, compaction and retirement are replicated: they are cheap
// next to traversal and need no geometry), holds only its own domains'
// geometry and BVHs, and traverses only its own domains' queue entries.
// Three reductions per depth join the ranks, all through caller-supplied
// callbacks (NCCL, MPI or gloo):
//   1. MIN over the packed 64-bit hit keys (t bits << 32 | global triangle):
//      the t-buffer composite; afterwards every rank knows every ray's
//      closest hit, and the ordering of the keys makes the winner the same
//      on every rank;
//   2. MAX over the bytes of the resolved hit attributes (normal, colour):
//      only the rank whose domain holds the winning hit writes them, the
//      others leave zeros, so the maximum of each byte is the owner's byte;
//   3. MAX over the shadow rays' occlusion flags (0/1): the BOR composite.
// The image every rank accumulates is therefore the single-rank image, bit
// for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spray_gpu.h"
#include "kernels.cuh"
#include "spray_math.cuh"
#include "tracer_internal.h"

namespace spray {

namespace {

// Morton::compute (src/render/morton.h:33-52): each coordinate in [0, 1]
// scaled to 10 bits, the bits of x, y, z interleaved (x highest).
uint32_t spreadBits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

uint32_t morton3(float x, float y, float z) {
  auto q = [](float c) { return (uint32_t)std::min(std::max(c * 1024.0f, 0.0f), 1023.0f); };
  return spreadBits(q(x)) * 4 + spreadBits(q(y)) * 2 + spreadBits(q(z));
}

__global__ void kFillKeys(uint64_t* keys, const uint32_t* count, uint64_t value) {
  const uint32_t n = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) keys[i] = value;
}

}  // namespace

// InsituPartition::partition: domain centres in the scene box mapped to
// [0, 1]^3 (glm's translate * scale), Morton codes, domains sorted by code,
// then consecutive shares of ndomains / num_ranks domains per rank, wrapping
// to rank 0 for the remainder.  The reference sorts with std::sort, which
// leaves equal codes in no particular order; this sort is stable (equal codes
// keep domain order).
std::vector<int> insituPartition(const float* bounds, int nd, int num_ranks) {
  if (nd <= 0 || num_ranks <= 0) throw std::invalid_argument("partition needs domains and ranks");
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int d = 0; d < nd; ++d)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], bounds[6 * d + c]);
      hi[c] = std::max(hi[c], bounds[6 * d + 3 + c]);
    }
  float sf[3], off[3];
  for (int c = 0; c < 3; ++c) {
    const float diag = hi[c] - lo[c];
    sf[c] = 1.0f / diag;
    off[c] = 0.0f - lo[c] * sf[c];
  }
  std::vector<std::pair<uint32_t, int>> codes(nd);
  for (int d = 0; d < nd; ++d) {
    float u[3];
    for (int c = 0; c < 3; ++c) {
      const float centre = (bounds[6 * d + c] + bounds[6 * d + 3 + c]) * 0.5f;
      u[c] = centre * sf[c] + off[c];
    }
    codes[d] = {morton3(u[0], u[1], u[2]), d};
  }
  std::stable_sort(codes.begin(), codes.end(),
                   [](const std::pair<uint32_t, int>& a, const std::pair<uint32_t, int>& b) {
                     return a.first < b.first;
                   });
  const int shares = std::max(nd / num_ranks, 1);
  std::vector<int> owner(nd, 0);
  int rank = 0, s = 0;
  for (int k = 0; k < nd; ++k) {
    owner[codes[k].second] = rank;
    if (++s == shares) {
      s = 0;
      if (++rank == num_ranks) rank = 0;
    }
  }
  return owner;
}

void Tracer::setInsitu(int num_ranks, int rank, const spray_gpu_reduce_ops* ops) {
  if (has_scene) throw StateError("set the domain partition before the scene");
  if (num_ranks < 1 || rank < 0 || rank >= num_ranks)
    throw std::invalid_argument("rank must be in [0, num_ranks)");
  if (num_ranks > 1 && (!ops || !ops->min_u64 || !ops->max_u8))
    throw std::invalid_argument("domain-parallel tracing needs the min_u64 and max_u8 reductions");
  if (num_ranks > 1 && (cfg.schedule_policy > 1 || cfg.debug_capture))
    throw std::invalid_argument("domain-parallel tracing runs the in-core speculative order "
                                "(schedule_policy 0 or 1) without debug capture");
  insitu_ranks = num_ranks;
  insitu_rank = rank;
  reduce = ops ? *ops : spray_gpu_reduce_ops{};
}

// Pinned host staging of the reductions (host_buffers mode), grown as needed.
char* Tracer::reduceStage(size_t bytes) {
  if (bytes > h_reduce_cap) {
    if (h_reduce) CK(cudaFreeHost(h_reduce));
    h_reduce = nullptr;
    h_reduce_cap = 0;
    CK(cudaMallocHost(&h_reduce, bytes));
    h_reduce_cap = bytes;
  }
  return h_reduce;
}

void Tracer::reduceCall(bool keys, void* dev, int64_t n, size_t elem) {
  const size_t bytes = (size_t)n * elem;
  reduce_bytes += (int64_t)bytes;
  if (n <= 0) return;
  int rc;
  if (reduce.host_buffers) {
    char* h = reduceStage(bytes);
    CK(cudaMemcpyAsync(h, dev, bytes, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    rc = keys ? reduce.min_u64(reduce.user, reinterpret_cast<uint64_t*>(h), n, nullptr)
              : reduce.max_u8(reduce.user, reinterpret_cast<uint8_t*>(h), n, nullptr);
    if (rc != 0) throw std::runtime_error("a domain-parallel reduction failed (" + std::to_string(rc) + ")");
    CK(cudaMemcpyAsync(dev, h, bytes, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
  } else {
    rc = keys ? reduce.min_u64(reduce.user, reinterpret_cast<uint64_t*>(dev), n, stream)
              : reduce.max_u8(reduce.user, reinterpret_cast<uint8_t*>(dev), n, stream);
    if (rc != 0) throw std::runtime_error("a domain-parallel reduction failed (" + std::to_string(rc) + ")");
  }
}

// One launch over the queue entries of this rank's domains (keys = domains,
// every owned domain one segment).  Entries of other ranks' domains are not
// traced; their records read as misses for the resolve pass.
void Tracer::traceOwned(bool shadow, int S) {
  std::vector<uint32_t> ks(D + 1);
  CK(cudaMemcpyAsync(ks.data(), d_key_start, (D + 1) * 4, cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  std::vector<uint32_t> seg(2 * (size_t)D + 2, 0u);
  int nseg = 0;
  uint32_t run = 0;
  for (int d = 0; d < D; ++d) {
    if (owner[d] != insitu_rank || ks[d + 1] == ks[d]) continue;
    seg[nseg] = ks[d];
    seg[D + 1 + nseg] = run;
    run += ks[d + 1] - ks[d];
    ++nseg;
  }
  seg[D + 1 + nseg] = run;
  if (!shadow) {
    kFillKeys<<<num_sms * 4, 256, 0, stream>>>(d_rec_key, d_num_entries, kNoHit);
    launches += 1;
  }
  if (nseg == 0) return;
  CK(cudaMemcpyAsync(d_segs, seg.data(), seg.size() * 4, cudaMemcpyHostToDevice, stream));
  CK(cudaMemsetAsync(d_work, 0, 4, stream));
  TraceArgs ta = traceArgs(0, S);
  ta.seg_begin = d_segs;
  ta.seg_prefix = d_segs + D + 1;
  ta.nseg = nseg;
  cudaEvent_t e0 = poolEvent(), e1 = poolEvent();
  CK(cudaEventRecord(e0, stream));
  if (shadow) launchTraceOccluded(stream, ta, traceBlocks());
  else launchTraceClosest(stream, ta, traceBlocks());
  CK(cudaEventRecord(e1, stream));
  (shadow ? occl_events : trace_events).push_back({e0, e1});
  launches += 1;
  // the segment table is pageable host memory copied above; it must stay
  // alive until the copy has read it
  CK(cudaStreamSynchronize(stream));
}

}  // namespace spray
