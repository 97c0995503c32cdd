// Per-domain BVH build on the GPU: binned SAH over the FP32 triangles,
// collapsed into the 4-wide BvhNode4 layout the traversal kernels read.
//
// SpRay rebuilds an Embree BVH (bvh4.triangle4v) whenever it loads a domain
// (TriMeshBuffer::load -> rtcCommit, src/render/trimesh_buffer.cc:104,222-224).
// Here every domain of a batch is built at once, one CTA per domain:
//   kPrep      per triangle: exact float box, centroid 0.5 (lo + hi), index
//   kBuild     binary binned-SAH splits.  Tasks above kSmallTask triangles
//              are split by the whole CTA: 16 bins per axis (count, triangle
//              box, centroid box) in warp-private shared-memory bins, the SAH
//              sweep, then a stable partition (block scan) from one index
//              buffer into the other; the children's boxes and centroid
//              boxes come from the bins.
//   kBuildSmall the tasks of at most kSmallTask triangles, one warp each,
//              warps of every SM pulling from one counter: depth first,
//              continuing with the smaller child so a warp's stack stays
//              within log2(kSmallTask) + 1 entries.
//   kCollapse  4-wide nodes: each node takes its binary node's children and
//              opens the inner child with the largest box until it holds
//              four (the host builder's rule), one warp per domain
//   kTris      leaf-ordered triangles (3 float4, v0.w = the face index)
// Boxes are exact min/max of the float vertices, so the traversal's
// conservative box test never misses a triangle, and the hit (t, triangle)
// key makes the traced image independent of the tree's shape.  Every stack
// and list is bounded; running out of room sets an error flag that the host
// turns into an error (no kernel waits on anything).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh.h"
#include "tracer_internal.h"

namespace spray {
namespace gbvh {

namespace {

constexpr int kBins = 16;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kSmallTask = 256;        // tasks of at most this many triangles go to a warp
constexpr int kWarpStack = 12;         // >= log2(kSmallTask) + 2
constexpr int kBigStack = 64;          // CTA task stack (depth first, smaller child first)
constexpr int kMaxBatchDomains = 4096; // domains built together (kBuildSmall's shared prefix)
constexpr float kTraversalCost = 1.0f;  // relative to one triangle test, as the host builder

enum : int { kErrStack = 1, kErrSmallList = 2, kErrNodes = 4, kErrQueue = 8, kErrLeaf = 16, kErrPartition = 32 };

struct Dom {
  const float* v;        // vertices (3 floats each), device
  const uint32_t* f;     // faces (3 indices each), device
  uint32_t nf;
  uint64_t tri_base;     // offset of the domain's triangles in the batch arrays
  uint64_t node_base;    // offset of its binary nodes (capacity 2 nf)
  uint64_t small_base;   // offset of its small-task list (capacity nf / 64 + 64)
  uint64_t q_base;       // offset of its collapse queue (capacity 2 nf)
  uint64_t out_base;     // offset of its 4-wide nodes (capacity nf)
};

struct BNode {  // binary node
  float lo[3];
  int32_t left;   // -1: leaf
  float hi[3];
  int32_t right;
  uint32_t first, count;
};

struct Task {
  uint32_t node, first, count, parity;  // parity: which index buffer holds the range
  float clo[3], chi[3];                 // centroid bounds
};

struct Batch {
  const Dom* doms;
  float4* tlo;           // triangle box lo (w unused)
  float4* thi;
  float4* cen;           // centroid
  uint32_t* idx[2];      // double-buffered permutation, domain-relative triangle numbers
  uint32_t* order;       // final leaf order
  BNode* nodes;
  Task* small;
  uint32_t* nnodes;      // binary nodes per domain
  uint32_t* nsmall;      // small tasks per domain
  BvhNode4* out;         // 4-wide nodes
  uint32_t* nout;        // 4-wide nodes per domain
  int32_t* depth;        // 4-wide depth per domain (root = 1)
  int2* queue;           // collapse queue: (binary node, 4-wide node)
  int* error;
};

__device__ __forceinline__ int ordf(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float unordf(int b) { return __int_as_float(b >= 0 ? b : b ^ 0x7fffffff); }

__device__ __forceinline__ float halfArea(const float lo[3], const float hi[3]) {
  const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  if (dx < 0.f || dy < 0.f || dz < 0.f) return 0.f;
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int binOf(float c, float lo, float scale) {
  int b = (int)((c - lo) * scale);
  return min(max(b, 0), kBins - 1);
}

// Bin statistics of one axis: count, triangle box (lo, hi), centroid box.
// Min/max as order-preserving ints so shared-memory atomics apply.
struct Bins {
  int cnt[3][kBins];
  int blo[3][kBins][3], bhi[3][kBins][3];
  int clo[3][kBins][3], chi[3][kBins][3];
};

__device__ void clearBins(Bins* b, int lane, int width) {
  int* p = reinterpret_cast<int*>(b);
  constexpr int n = sizeof(Bins) / 4;
  for (int i = lane; i < n; i += width) {
    // counts 0, minima +max, maxima -max (as ordered ints)
    const int off = i;
    int v = 0;
    if (off >= 3 * kBins) {
      const int k = (off - 3 * kBins) / (3 * kBins * 3);  // 0 blo, 1 bhi, 2 clo, 3 chi
      v = (k == 0 || k == 2) ? 0x7fffffff : (int)0x80000000;
    }
    p[i] = v;
  }
}

__device__ __forceinline__ void addToBins(Bins* b, const float4 lo, const float4 hi, const float4 c,
                                          const float clo[3], const float scale[3]) {
  const float cc[3] = {c.x, c.y, c.z};
  const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!(scale[a] > 0.f)) continue;
    const int k = binOf(cc[a], clo[a], scale[a]);
    atomicAdd(&b->cnt[a][k], 1);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      atomicMin(&b->blo[a][k][q], ordf(l3[q]));
      atomicMax(&b->bhi[a][k][q], ordf(h3[q]));
      atomicMin(&b->clo[a][k][q], ordf(cc[q]));
      atomicMax(&b->chi[a][k][q], ordf(cc[q]));
    }
  }
}

// The SAH sweep over merged bins of one axis: best split b (left = bins < b)
// and its cost; cost = +inf when the axis cannot split.
__device__ void sweepAxis(const Bins* m, int a, float* best_cost, int* best_split) {
  *best_cost = INFINITY;
  *best_split = -1;
  float la[kBins];
  int lc[kBins];
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  int n = 0;
  for (int b = 0; b < kBins - 1; ++b) {
    if (m->cnt[a][b]) {
      for (int q = 0; q < 3; ++q) {
        lo[q] = fminf(lo[q], unordf(m->blo[a][b][q]));
        hi[q] = fmaxf(hi[q], unordf(m->bhi[a][b][q]));
      }
    }
    n += m->cnt[a][b];
    la[b] = n ? halfArea(lo, hi) : 0.f;
    lc[b] = n;
  }
  for (int q = 0; q < 3; ++q) {
    lo[q] = FLT_MAX;
    hi[q] = -FLT_MAX;
  }
  n = 0;
  for (int b = kBins - 1; b > 0; --b) {
    if (m->cnt[a][b]) {
      for (int q = 0; q < 3; ++q) {
        lo[q] = fminf(lo[q], unordf(m->blo[a][b][q]));
        hi[q] = fmaxf(hi[q], unordf(m->bhi[a][b][q]));
      }
    }
    n += m->cnt[a][b];
    if (lc[b - 1] == 0 || n == 0) continue;
    const float cost = la[b - 1] * (float)lc[b - 1] + halfArea(lo, hi) * (float)n;
    if (cost < *best_cost) {
      *best_cost = cost;
      *best_split = b;
    }
  }
}

// Union of bins [b0, b1) of axis a: triangle box and centroid box.
__device__ void binUnion(const Bins* m, int a, int b0, int b1, float blo[3], float bhi[3], float clo[3],
                         float chi[3]) {
  for (int q = 0; q < 3; ++q) {
    blo[q] = clo[q] = FLT_MAX;
    bhi[q] = chi[q] = -FLT_MAX;
  }
  for (int b = b0; b < b1; ++b) {
    if (!m->cnt[a][b]) continue;
    for (int q = 0; q < 3; ++q) {
      blo[q] = fminf(blo[q], unordf(m->blo[a][b][q]));
      bhi[q] = fmaxf(bhi[q], unordf(m->bhi[a][b][q]));
      clo[q] = fminf(clo[q], unordf(m->clo[a][b][q]));
      chi[q] = fmaxf(chi[q], unordf(m->chi[a][b][q]));
    }
  }
}

__global__ void kPrep(Batch B, int ndoms) {
  const Dom d = B.doms[blockIdx.y];
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < d.nf; t += gridDim.x * blockDim.x) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int c = 0; c < 3; ++c) {
      const float* p = d.v + 3 * (size_t)d.f[3 * (size_t)t + c];
      for (int q = 0; q < 3; ++q) {
        lo[q] = fminf(lo[q], p[q]);
        hi[q] = fmaxf(hi[q], p[q]);
      }
    }
    const uint64_t g = d.tri_base + t;
    B.tlo[g] = make_float4(lo[0], lo[1], lo[2], 0.f);
    B.thi[g] = make_float4(hi[0], hi[1], hi[2], 0.f);
    B.cen[g] = make_float4(0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2]), 0.f);
    B.idx[0][g] = t;
  }
  (void)ndoms;
}

struct Shared {
  Bins bins[kWarps];     // warp-private bins of the CTA-wide split (and per-warp small builds)
  Task stack[kBigStack];
  Task wstack[kWarps][kWarpStack];
  int scan[kWarps];
  int nstack;
  int nnodes;
  int nsmall;
  Task cur;
  int axis, split, stop;
  int running_left, running_right;
  float res[16];
};

// Writes node `id` and its range into the final order when it is a leaf.
__device__ void writeNode(const Batch& B, const Dom& d, uint32_t id, const float lo[3], const float hi[3],
                          int left, int right, uint32_t first, uint32_t count) {
  BNode n;
  for (int q = 0; q < 3; ++q) {
    n.lo[q] = lo[q];
    n.hi[q] = hi[q];
  }
  n.left = left;
  n.right = right;
  n.first = first;
  n.count = count;
  B.nodes[d.node_base + id] = n;
}

// Copies a leaf's range from its buffer into the final order (one group).
__device__ void copyLeaf(const Batch& B, const Dom& d, const Task& t, int lane, int width) {
  for (uint32_t i = lane; i < t.count; i += width)
    B.order[d.tri_base + t.first + i] = B.idx[t.parity][d.tri_base + t.first + i];
}

// Stable partition of a task's range into the other buffer, CTA-wide.
// Returns (in shared) the number of left elements.
__device__ void partitionCta(const Batch& B, const Dom& d, Shared& S, const Task& t, int axis, int split,
                             bool by_half) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t* src = B.idx[t.parity] + d.tri_base;
  uint32_t* dst = B.idx[t.parity ^ 1] + d.tri_base;
  const float scale = by_half ? 0.f : kBins / (t.chi[axis] - t.clo[axis]);
  // left count: from the bins (or half)
  uint32_t nleft;
  if (by_half) {
    nleft = t.count / 2;
  } else {
    nleft = 0;
    for (int b = 0; b < split; ++b) nleft += (uint32_t)S.bins[0].cnt[axis][b];
  }
  if (tid == 0) {
    S.running_left = 0;
    S.running_right = 0;
  }
  __syncthreads();
  for (uint32_t base = 0; base < t.count; base += kThreads) {
    const uint32_t i = base + tid;
    bool isl = false;
    uint32_t tri = 0;
    if (i < t.count) {
      tri = src[t.first + i];
      if (by_half) {
        isl = i < nleft;
      } else {
        const float4 c = B.cen[d.tri_base + tri];
        const float cc = axis == 0 ? c.x : axis == 1 ? c.y : c.z;
        isl = binOf(cc, t.clo[axis], scale) < split;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, isl);
    if (lane == 0) S.scan[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kWarps; ++w) {
      if (w < warp) before += S.scan[w];
      total += S.scan[w];
    }
    const int lrank = before + __popc(m & ((1u << lane) - 1u));
    if (i < t.count) {
      // positions stay inside the task's range even if the counts disagreed
      const uint32_t pos = isl ? (uint32_t)(S.running_left + lrank)
                               : nleft + (uint32_t)(S.running_right + (int)(i - base) - lrank);
      if (pos < t.count) dst[t.first + pos] = tri;
    }
    __syncthreads();
    if (tid == 0) {
      S.running_left += total;
      S.running_right += (int)min((uint32_t)kThreads, t.count - base) - total;
    }
    __syncthreads();
  }
  if (tid == 0 && (uint32_t)S.running_left != nleft) atomicOr(B.error, kErrPartition);
}

// Box and centroid box of the range [first, first + count) of buffer
// `parity`, reduced by one group (CTA when width == kThreads, else a warp).
__device__ void rangeBounds(const Batch& B, const Dom& d, uint32_t parity, uint32_t first, uint32_t count,
                            int lane, int width, Bins* scratch, float blo[3], float bhi[3], float clo[3],
                            float chi[3], bool cta) {
  // reuse bin 0 of axis 0 of the scratch bins as the accumulator
  if (lane < 3) {
    scratch->blo[0][0][lane] = 0x7fffffff;
    scratch->bhi[0][0][lane] = (int)0x80000000;
    scratch->clo[0][0][lane] = 0x7fffffff;
    scratch->chi[0][0][lane] = (int)0x80000000;
  }
  if (cta) __syncthreads();
  else __syncwarp();
  float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  float cl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ch[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint32_t i = lane; i < count; i += width) {
    const uint64_t g = d.tri_base + B.idx[parity][d.tri_base + first + i];
    const float4 a = B.tlo[g], b = B.thi[g], c = B.cen[g];
    l[0] = fminf(l[0], a.x), l[1] = fminf(l[1], a.y), l[2] = fminf(l[2], a.z);
    h[0] = fmaxf(h[0], b.x), h[1] = fmaxf(h[1], b.y), h[2] = fmaxf(h[2], b.z);
    cl[0] = fminf(cl[0], c.x), cl[1] = fminf(cl[1], c.y), cl[2] = fminf(cl[2], c.z);
    ch[0] = fmaxf(ch[0], c.x), ch[1] = fmaxf(ch[1], c.y), ch[2] = fmaxf(ch[2], c.z);
  }
  for (int q = 0; q < 3; ++q) {
    atomicMin(&scratch->blo[0][0][q], ordf(l[q]));
    atomicMax(&scratch->bhi[0][0][q], ordf(h[q]));
    atomicMin(&scratch->clo[0][0][q], ordf(cl[q]));
    atomicMax(&scratch->chi[0][0][q], ordf(ch[q]));
  }
  if (cta) __syncthreads();
  else __syncwarp();
  for (int q = 0; q < 3; ++q) {
    blo[q] = unordf(scratch->blo[0][0][q]);
    bhi[q] = unordf(scratch->bhi[0][0][q]);
    clo[q] = unordf(scratch->clo[0][0][q]);
    chi[q] = unordf(scratch->chi[0][0][q]);
  }
  if (cta) __syncthreads();
  else __syncwarp();
}

// Builds the subtree of a small task with one warp, depth first; binary node
// ids come from the domain's counter in global memory.
__device__ void buildSmall(const Batch& B, const Dom& d, Shared& S, Task root, int warp, int lane,
                           uint32_t* node_counter) {
  Bins* bins = &S.bins[warp];
  Task* st = S.wstack[warp];
  int sp = 0;
  Task t = root;
  while (true) {
    // t's node is already written (box); decide leaf or split
    bool leaf = t.count <= 2;
    int axis = -1, split = -1;
    float best = INFINITY;
    float nlo[3], nhi[3];
    if (!leaf) {
      clearBins(bins, lane, 32);
      __syncwarp();
      float scale[3];
      for (int a = 0; a < 3; ++a) {
        const float ext = t.chi[a] - t.clo[a];
        scale[a] = ext > 0.f ? kBins / ext : 0.f;
      }
      for (uint32_t i = lane; i < t.count; i += 32) {
        const uint64_t g = d.tri_base + B.idx[t.parity][d.tri_base + t.first + i];
        addToBins(bins, B.tlo[g], B.thi[g], B.cen[g], t.clo, scale);
      }
      __syncwarp();
      // every lane sweeps the three axes (cheap) and agrees on the result
      for (int a = 0; a < 3; ++a) {
        if (!(scale[a] > 0.f)) continue;
        float c;
        int s;
        sweepAxis(bins, a, &c, &s);
        if (s >= 0 && c < best) {
          best = c;
          axis = a;
          split = s;
        }
      }
      const BNode& self = B.nodes[d.node_base + t.node];
      for (int q = 0; q < 3; ++q) {
        nlo[q] = self.lo[q];
        nhi[q] = self.hi[q];
      }
      const float area = halfArea(nlo, nhi);
      const float leaf_cost = area * (float)t.count;
      const float split_cost = kTraversalCost * area + best;
      if (axis < 0) leaf = t.count <= (uint32_t)kMaxLeafTris;
      else leaf = t.count <= (uint32_t)kMaxLeafTris && leaf_cost <= split_cost;
    }
    if (leaf) {
      if (t.count > (uint32_t)kMaxLeafTris) {
        if (lane == 0) atomicOr(B.error, kErrLeaf);
        return;
      }
      copyLeaf(B, d, t, lane, 32);
    } else {
      // stable warp partition into the other buffer
      const uint32_t* src = B.idx[t.parity] + d.tri_base;
      uint32_t* dst = B.idx[t.parity ^ 1] + d.tri_base;
      const bool by_half = axis < 0;
      uint32_t nleft = 0;
      if (by_half) nleft = t.count / 2;
      else
        for (int b = 0; b < split; ++b) nleft += (uint32_t)bins->cnt[axis][b];
      const float scale = by_half ? 0.f : kBins / (t.chi[axis] - t.clo[axis]);
      uint32_t rl = 0, rr = 0;
      for (uint32_t base = 0; base < t.count; base += 32) {
        const uint32_t i = base + lane;
        bool isl = false;
        uint32_t tri = 0;
        if (i < t.count) {
          tri = src[t.first + i];
          if (by_half) {
            isl = i < nleft;
          } else {
            const float4 c = B.cen[d.tri_base + tri];
            isl = binOf(axis == 0 ? c.x : axis == 1 ? c.y : c.z, t.clo[axis], scale) < split;
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, isl);
        const uint32_t lr = __popc(m & ((1u << lane) - 1u));
        if (i < t.count) {
          const uint32_t pos = isl ? rl + lr : nleft + rr + (lane - lr);
          if (pos < t.count) dst[t.first + pos] = tri;
        }
        rl += __popc(m);
        rr += min(32u, t.count - base) - __popc(m);
      }
      __syncwarp();
      if (rl != nleft) {
        if (lane == 0) atomicOr(B.error, kErrPartition);
        return;
      }
      // children's boxes: from the bins, or reduced over the halves
      float blo[2][3], bhi[2][3], clo[2][3], chi[2][3];
      if (!by_half) {
        binUnion(bins, axis, 0, split, blo[0], bhi[0], clo[0], chi[0]);
        binUnion(bins, axis, split, kBins, blo[1], bhi[1], clo[1], chi[1]);
      } else {
        rangeBounds(B, d, t.parity ^ 1, t.first, nleft, lane, 32, bins, blo[0], bhi[0], clo[0], chi[0], false);
        rangeBounds(B, d, t.parity ^ 1, t.first + nleft, t.count - nleft, lane, 32, bins, blo[1], bhi[1],
                    clo[1], chi[1], false);
      }
      int ids = 0;
      if (lane == 0) ids = (int)atomicAdd(node_counter, 2u);
      ids = __shfl_sync(0xffffffffu, ids, 0);
      if ((uint32_t)ids + 2 > 2 * d.nf) {
        if (lane == 0) atomicOr(B.error, kErrNodes);
        return;
      }
      Task kid[2];
      for (int k = 0; k < 2; ++k) {
        kid[k].node = (uint32_t)(ids + k);
        kid[k].first = k == 0 ? t.first : t.first + nleft;
        kid[k].count = k == 0 ? nleft : t.count - nleft;
        kid[k].parity = t.parity ^ 1;
        for (int q = 0; q < 3; ++q) {
          kid[k].clo[q] = clo[k][q];
          kid[k].chi[q] = chi[k][q];
        }
        if (lane == 0)
          writeNode(B, d, kid[k].node, blo[k], bhi[k], -1, -1, kid[k].first, kid[k].count);
      }
      if (lane == 0) {
        BNode* self = &B.nodes[d.node_base + t.node];
        self->left = ids;
        self->right = ids + 1;
      }
      __syncwarp();
      // continue with the smaller child, push the larger
      const int small = kid[0].count <= kid[1].count ? 0 : 1;
      if (sp >= kWarpStack) {
        if (lane == 0) atomicOr(B.error, kErrStack);
        return;
      }
      if (lane == 0) st[sp] = kid[1 - small];
      ++sp;
      __syncwarp();
      t = kid[small];
      continue;
    }
    if (sp == 0) return;
    --sp;
    __syncwarp();
    t = st[sp];
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kThreads) kBuild(Batch B) {
  extern __shared__ __align__(16) unsigned char smem[];
  Shared& S = *reinterpret_cast<Shared*>(smem);
  const Dom d = B.doms[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // root
  float blo[3], bhi[3], clo[3], chi[3];
  rangeBounds(B, d, 0, 0, d.nf, tid, kThreads, &S.bins[0], blo, bhi, clo, chi, true);
  if (tid == 0) {
    writeNode(B, d, 0, blo, bhi, -1, -1, 0, d.nf);
    S.nnodes = 1;
    S.nsmall = 0;
    S.nstack = 0;
    Task r;
    r.node = 0;
    r.first = 0;
    r.count = d.nf;
    r.parity = 0;
    for (int q = 0; q < 3; ++q) {
      r.clo[q] = clo[q];
      r.chi[q] = chi[q];
    }
    if (d.nf > (uint32_t)kSmallTask) S.stack[S.nstack++] = r;
    else B.small[d.small_base + S.nsmall++] = r;
  }
  __syncthreads();
  // CTA-wide splits of the large tasks
  while (true) {
    if (tid == 0) {
      if (S.nstack > 0) S.cur = S.stack[--S.nstack];
      else S.cur.count = 0;
    }
    __syncthreads();
    const Task t = S.cur;
    if (t.count == 0) break;
    for (int w = 0; w < kWarps; ++w) clearBins(&S.bins[w], tid, kThreads);
    __syncthreads();
    float scale[3];
    for (int a = 0; a < 3; ++a) {
      const float ext = t.chi[a] - t.clo[a];
      scale[a] = ext > 0.f ? kBins / ext : 0.f;
    }
    for (uint32_t i = tid; i < t.count; i += kThreads) {
      const uint64_t g = d.tri_base + B.idx[t.parity][d.tri_base + t.first + i];
      addToBins(&S.bins[warp], B.tlo[g], B.thi[g], B.cen[g], t.clo, scale);
    }
    __syncthreads();
    // merge the warps' bins into bins[0]
    {
      constexpr int n = sizeof(Bins) / 4;
      int* m0 = reinterpret_cast<int*>(&S.bins[0]);
      for (int i = tid; i < n; i += kThreads) {
        int v = m0[i];
        const bool is_cnt = i < 3 * kBins;
        const int k = is_cnt ? -1 : (i - 3 * kBins) / (3 * kBins * 3);
        for (int w = 1; w < kWarps; ++w) {
          const int x = reinterpret_cast<const int*>(&S.bins[w])[i];
          if (is_cnt) v += x;
          else if (k == 0 || k == 2) v = min(v, x);
          else v = max(v, x);
        }
        m0[i] = v;
      }
    }
    __syncthreads();
    if (tid < 3) {
      float c = INFINITY;
      int s = -1;
      if (scale[tid] > 0.f) sweepAxis(&S.bins[0], tid, &c, &s);
      S.res[tid] = c;
      S.res[3 + tid] = __int_as_float(s);
    }
    __syncthreads();
    if (tid == 0) {
      int axis = -1, split = -1;
      float best = INFINITY;
      for (int a = 0; a < 3; ++a) {
        const int s = __float_as_int(S.res[3 + a]);
        if (s >= 0 && S.res[a] < best) {
          best = S.res[a];
          axis = a;
          split = s;
        }
      }
      S.axis = axis;
      S.split = split;
    }
    __syncthreads();
    const int axis = S.axis, split = S.split;
    partitionCta(B, d, S, t, axis, split, axis < 0);
    uint32_t nleft = 0;
    if (axis < 0) nleft = t.count / 2;
    else
      for (int b = 0; b < split; ++b) nleft += (uint32_t)S.bins[0].cnt[axis][b];
    float kb[2][3], kh[2][3], kc[2][3], kx[2][3];
    if (axis >= 0) {
      binUnion(&S.bins[0], axis, 0, split, kb[0], kh[0], kc[0], kx[0]);
      binUnion(&S.bins[0], axis, split, kBins, kb[1], kh[1], kc[1], kx[1]);
    }
    __syncthreads();
    if (axis < 0) {
      rangeBounds(B, d, t.parity ^ 1, t.first, nleft, tid, kThreads, &S.bins[1], kb[0], kh[0], kc[0], kx[0], true);
      rangeBounds(B, d, t.parity ^ 1, t.first + nleft, t.count - nleft, tid, kThreads, &S.bins[1], kb[1], kh[1],
                  kc[1], kx[1], true);
    }
    if (tid == 0) {
      const int ids = S.nnodes;
      S.nnodes += 2;
      if ((uint32_t)ids + 2 > 2 * d.nf) {
        atomicOr(B.error, kErrNodes);
      } else {
        BNode* self = &B.nodes[d.node_base + t.node];
        self->left = ids;
        self->right = ids + 1;
        Task kid[2];
        for (int k = 0; k < 2; ++k) {
          kid[k].node = (uint32_t)(ids + k);
          kid[k].first = k == 0 ? t.first : t.first + nleft;
          kid[k].count = k == 0 ? nleft : t.count - nleft;
          kid[k].parity = t.parity ^ 1;
          for (int q = 0; q < 3; ++q) {
            kid[k].clo[q] = kc[k][q];
            kid[k].chi[q] = kx[k][q];
          }
          writeNode(B, d, kid[k].node, kb[k], kh[k], -1, -1, kid[k].first, kid[k].count);
        }
        // depth first, smaller child on top of the stack
        const int small = kid[0].count <= kid[1].count ? 0 : 1;
        for (int k : {1 - small, small}) {
          if (kid[k].count > (uint32_t)kSmallTask) {
            if (S.nstack < kBigStack) S.stack[S.nstack++] = kid[k];
            else atomicOr(B.error, kErrStack);
          } else {
            const uint32_t cap = d.nf / 64 + 64;
            if ((uint32_t)S.nsmall < cap) B.small[d.small_base + S.nsmall++] = kid[k];
            else atomicOr(B.error, kErrSmallList);
          }
        }
      }
    }
    // stop on an error flag (any block's): one thread reads it, all follow
    if (tid == 0) S.stop = *((volatile int*)B.error);
    __syncthreads();
    if (S.stop) break;
  }
  __syncthreads();
  // the small tasks go to kBuildSmall, whose warps spread over every SM
  if (tid == 0) {
    B.nnodes[blockIdx.x] = (uint32_t)S.nnodes;
    B.nsmall[blockIdx.x] = (uint32_t)S.nsmall;
  }
  (void)lane;
  (void)warp;
}

// The small tasks of every domain of the batch, one warp per task, warps of
// all CTAs pulling from one counter (`next`): a domain's subtrees are built
// in parallel on every SM instead of by its one CTA.
__global__ void __launch_bounds__(kThreads) kBuildSmall(Batch B, int nb, uint32_t* next) {
  extern __shared__ __align__(16) unsigned char smem[];
  Shared& S = *reinterpret_cast<Shared*>(smem);
  uint32_t* prefix = reinterpret_cast<uint32_t*>(smem + sizeof(Shared));  // [nb + 1]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    uint32_t run = 0;
    for (int d = 0; d < nb; ++d) {
      prefix[d] = run;
      run += B.nsmall[d];
    }
    prefix[nb] = run;
  }
  __syncthreads();
  const uint32_t total = prefix[nb];
  while (true) {
    uint32_t k = 0;
    int stop = 0;
    if (lane == 0) {
      k = atomicAdd(next, 1u);
      stop = *((volatile int*)B.error);
    }
    k = __shfl_sync(0xffffffffu, k, 0);
    stop = __shfl_sync(0xffffffffu, stop, 0);
    if (k >= total || stop) break;
    // the domain of task k: last d with prefix[d] <= k
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (prefix[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    const Dom d = B.doms[lo];
    const Task t = B.small[d.small_base + (k - prefix[lo])];
    buildSmall(B, d, S, t, warp, lane, &B.nnodes[lo]);
  }
}

// 4-wide collapse, one warp per domain: a queue of (binary node, 4-wide
// node) pairs; each item gathers up to four children by opening the inner
// child with the largest box, allocates 4-wide nodes for the inner ones and
// queues them.
__global__ void kCollapse(Batch B) {
  const Dom d = B.doms[blockIdx.x];
  const int lane = threadIdx.x;
  __shared__ int qhead, qtail, nout, maxdepth, stop;
  int2* q = B.queue + d.q_base;
  const BNode* bn = B.nodes + d.node_base;
  BvhNode4* out = B.out + d.out_base;
  const uint32_t qcap = 2 * d.nf + 4, ocap = d.nf + 4;
  if (lane == 0) {
    q[0] = make_int2(0, 0);
    out[0].pad[0] = 1;  // the root's depth
    qhead = 0;
    qtail = 1;
    nout = 1;
    maxdepth = 1;
  }
  __syncwarp();
  // items carry the 4-wide node id in .y; depth is tracked in a parallel
  // pass: a node's depth = its parent's + 1, recorded in out[].pad[0]
  while (true) {
    const int head = qhead, tail = qtail;
    __syncwarp();
    if (head >= tail) break;
    const int take = min(32, tail - head);
    if (lane < take) {
      const int2 it = q[head + lane];
      const BNode& root = bn[it.x];
      int kids[4];
      int nk = 0;
      if (root.left < 0) {
        kids[nk++] = it.x;  // a single leaf root: one child, the leaf itself
      } else {
        kids[nk++] = root.left;
        kids[nk++] = root.right;
        while (nk < 4) {
          int best = -1;
          float best_area = -1.f;
          for (int i = 0; i < nk; ++i) {
            const BNode& k = bn[kids[i]];
            if (k.left >= 0) {
              const float a = halfArea(k.lo, k.hi);
              if (a > best_area) {
                best_area = a;
                best = i;
              }
            }
          }
          if (best < 0) break;
          const int opened = kids[best];
          kids[best] = bn[opened].left;
          kids[nk++] = bn[opened].right;
        }
      }
      const int my_depth = out[it.y].pad[0];  // set by the parent (root: 1)
      BvhNode4 node;
      for (int c = 0; c < 4; ++c) {
        node.lox[c] = node.loy[c] = node.loz[c] = INFINITY;
        node.hix[c] = node.hiy[c] = node.hiz[c] = -INFINITY;
        node.child[c] = kEmptyChild;
        node.pad[c] = 0;
      }
      node.pad[0] = my_depth;
      int ninner = 0;
      for (int c = 0; c < nk; ++c) ninner += bn[kids[c]].left >= 0 ? 1 : 0;
      const int base = ninner ? atomicAdd(&nout, ninner) : 0;
      const int qb = ninner ? atomicAdd(&qtail, ninner) : 0;
      int used = 0;
      bool ok = (uint32_t)(base + ninner) <= ocap && (uint32_t)(qb + ninner) <= qcap;
      for (int c = 0; c < nk && ok; ++c) {
        const BNode& k = bn[kids[c]];
        node.lox[c] = k.lo[0];
        node.loy[c] = k.lo[1];
        node.loz[c] = k.lo[2];
        node.hix[c] = k.hi[0];
        node.hiy[c] = k.hi[1];
        node.hiz[c] = k.hi[2];
        if (k.left < 0) {
          if (k.count > (uint32_t)kMaxLeafTris || k.first >= (1u << 27) || k.count == 0) {
            ok = false;
            break;
          }
          node.child[c] = ~(int32_t)((k.first << 3) | (k.count - 1));
        } else {
          const int id = base + used;
          node.child[c] = id;
          out[id].pad[0] = my_depth + 1;  // read when the child's item is processed
          q[qb + used] = make_int2(kids[c], id);
          ++used;
        }
      }
      if (!ok) {
        atomicOr(B.error, kErrQueue);
      } else {
        atomicMax(&maxdepth, my_depth);
        // keep the depth in pad[0] until the child items have read theirs;
        // cleared by kFinish
        out[it.y] = node;
      }
    }
    __syncwarp();
    if (lane == 0) {
      qhead = head + take;
      stop = *((volatile int*)B.error);
    }
    __syncwarp();
    if (stop) break;
  }
  __syncwarp();
  if (lane == 0) {
    B.nout[blockIdx.x] = (uint32_t)nout;
    B.depth[blockIdx.x] = maxdepth;
  }
}

// Clears the depth bookkeeping kept in pad[0] of every 4-wide node.
__global__ void kFinish(Batch B) {
  const Dom d = B.doms[blockIdx.y];
  const uint32_t n = B.nout[blockIdx.y];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    B.out[d.out_base + i].pad[0] = 0;
}

// Leaf-ordered triangles: 3 float4 per triangle, v0.w = the face index bits.
__global__ void kTris(Batch B, float4* tris) {
  const Dom d = B.doms[blockIdx.y];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < d.nf; k += gridDim.x * blockDim.x) {
    const uint32_t prim = B.order[d.tri_base + k];
    const uint32_t* fi = d.f + 3 * (size_t)prim;
    for (int c = 0; c < 3; ++c) {
      const float* p = d.v + 3 * (size_t)fi[c];
      tris[3 * (d.tri_base + k) + c] = make_float4(p[0], p[1], p[2], c == 0 ? __uint_as_float(prim) : 0.f);
    }
  }
}

}  // namespace

size_t sharedBytes() { return sizeof(Shared); }

}  // namespace gbvh

// Builds the BVHs of `n` domains (vertices and faces in host memory) on the
// current device and returns them in the packs (nodes, leaf-ordered
// triangles, depth).  Domains go in batches of at most `batch_tris`
// triangles to bound the device memory the build holds.
void buildBvhsOnDevice(const spray_gpu_domain* src, const std::vector<int>& which, std::vector<DomainPack>& packs,
                       cudaStream_t stream, uint64_t batch_tris) {
  using namespace gbvh;
  size_t k = 0;
  const size_t smem = sharedBytes();
  CK(cudaFuncSetAttribute(kBuild, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, sms = 1;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int small_blocks = 4 * sms;
  CK(cudaFuncSetAttribute(kBuildSmall, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)(smem + (kMaxBatchDomains + 1) * 4)));
  while (k < which.size()) {
    // the batch: consecutive domains up to batch_tris triangles (at least one)
    size_t j = k;
    uint64_t tris = 0, verts = 0;
    // (at most kMaxBatchDomains domains: kBuildSmall keeps their prefix in shared memory)
    while (j < which.size() && (j - k) < (size_t)kMaxBatchDomains &&
           (j == k || tris + (uint64_t)src[which[j]].num_faces <= batch_tris)) {
      tris += (uint64_t)src[which[j]].num_faces;
      verts += (uint64_t)src[which[j]].num_vertices;
      ++j;
    }
    const int nb = (int)(j - k);
    std::vector<Dom> hd(nb);
    uint64_t small = 0;
    for (int i = 0; i < nb; ++i) small += (uint64_t)src[which[k + i]].num_faces / 64 + 64;
    // device buffers of the batch
    float* dv = nullptr;
    uint32_t* df = nullptr;
    CK(cudaMalloc(&dv, std::max<uint64_t>(verts, 1) * 12));
    CK(cudaMalloc(&df, std::max<uint64_t>(tris, 1) * 12));
    Batch B{};
    Dom* ddoms = nullptr;
    float4* dtris = nullptr;
    CK(cudaMalloc(&ddoms, nb * sizeof(Dom)));
    CK(cudaMalloc(&B.tlo, tris * sizeof(float4)));
    CK(cudaMalloc(&B.thi, tris * sizeof(float4)));
    CK(cudaMalloc(&B.cen, tris * sizeof(float4)));
    CK(cudaMalloc(&B.idx[0], tris * 4));
    CK(cudaMalloc(&B.idx[1], tris * 4));
    CK(cudaMalloc(&B.order, tris * 4));
    CK(cudaMalloc(&B.nodes, (2 * tris + 4 * nb) * sizeof(BNode)));
    CK(cudaMalloc(&B.small, small * sizeof(Task)));
    CK(cudaMalloc(&B.nnodes, nb * 4));
    CK(cudaMalloc(&B.nsmall, nb * 4));
    CK(cudaMalloc(&B.out, (tris + 4 * nb) * sizeof(BvhNode4)));
    CK(cudaMalloc(&B.nout, nb * 4));
    CK(cudaMalloc(&B.depth, nb * 4));
    CK(cudaMalloc(&B.queue, (2 * tris + 4 * nb) * sizeof(int2)));
    CK(cudaMalloc(&B.error, 4));
    uint32_t* small_next = nullptr;
    CK(cudaMalloc(&small_next, 4));
    CK(cudaMalloc(&dtris, 3 * tris * sizeof(float4)));
    CK(cudaMemsetAsync(B.error, 0, 4, stream));
    uint64_t vo = 0, fo = 0, so = 0, oo = 0;
    for (int i = 0; i < nb; ++i) {
      const spray_gpu_domain& s = src[which[k + i]];
      CK(cudaMemcpyAsync(dv + 3 * vo, s.vertices, (size_t)s.num_vertices * 12, cudaMemcpyHostToDevice, stream));
      CK(cudaMemcpyAsync(df + 3 * fo, s.faces, (size_t)s.num_faces * 12, cudaMemcpyHostToDevice, stream));
      hd[i].v = dv + 3 * vo;
      hd[i].f = df + 3 * fo;
      hd[i].nf = (uint32_t)s.num_faces;
      hd[i].tri_base = fo;
      hd[i].node_base = 2 * fo + 4 * (uint64_t)i;
      hd[i].small_base = so;
      hd[i].q_base = 2 * fo + 4 * (uint64_t)i;
      hd[i].out_base = oo;
      vo += (uint64_t)s.num_vertices;
      fo += (uint64_t)s.num_faces;
      so += (uint64_t)s.num_faces / 64 + 64;
      oo += (uint64_t)s.num_faces + 4;
    }
    CK(cudaMemcpyAsync(ddoms, hd.data(), nb * sizeof(Dom), cudaMemcpyHostToDevice, stream));
    B.doms = ddoms;
    const int gx = 64;
    kPrep<<<dim3(gx, nb), 256, 0, stream>>>(B, nb);
    kBuild<<<nb, kThreads, smem, stream>>>(B);
    CK(cudaMemsetAsync(small_next, 0, 4, stream));
    kBuildSmall<<<small_blocks, kThreads, smem + (nb + 1) * 4, stream>>>(B, nb, small_next);
    kCollapse<<<nb, 32, 0, stream>>>(B);
    kFinish<<<dim3(gx, nb), 256, 0, stream>>>(B);
    kTris<<<dim3(gx, nb), 256, 0, stream>>>(B, dtris);
    CK(cudaGetLastError());
    int err = 0;
    std::vector<uint32_t> nout(nb);
    std::vector<int32_t> depth(nb);
    CK(cudaMemcpyAsync(&err, B.error, 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(nout.data(), B.nout, nb * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(depth.data(), B.depth, nb * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (err == 0) {
      for (int i = 0; i < nb; ++i) {
        DomainPack& p = packs[which[k + i]];
        p.nodes.resize(nout[i]);
        p.tris.resize(3 * (size_t)hd[i].nf);
        CK(cudaMemcpyAsync(p.nodes.data(), B.out + hd[i].out_base, nout[i] * sizeof(BvhNode4),
                           cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(p.tris.data(), dtris + 3 * hd[i].tri_base, 3 * (size_t)hd[i].nf * sizeof(float4),
                           cudaMemcpyDeviceToHost, stream));
        p.bvh_depth = depth[i];
      }
      CK(cudaStreamSynchronize(stream));
    }
    for (void* ptr : {(void*)dv, (void*)df, (void*)ddoms, (void*)B.tlo, (void*)B.thi, (void*)B.cen,
                      (void*)B.idx[0], (void*)B.idx[1], (void*)B.order, (void*)B.nodes, (void*)B.small,
                      (void*)B.nnodes, (void*)B.nsmall, (void*)B.out, (void*)B.nout, (void*)B.depth,
                      (void*)B.queue, (void*)B.error, (void*)dtris, (void*)small_next})
      cudaFree(ptr);
    if (err) throw std::runtime_error("device BVH build ran out of room (error flags " + std::to_string(err) + ")");
    k = j;
  }
}

}  // namespace spray
