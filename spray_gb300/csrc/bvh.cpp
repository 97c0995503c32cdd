// Binned-SAH BVH build, collapsed to 4-wide nodes.  See bvh.h.
#include "bvh.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace spray {
namespace {

struct Box {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; ++k) {
      lo[k] = FLT_MAX;
      hi[k] = -FLT_MAX;
    }
  }
  void grow(const Box& b) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], b.lo[k]);
      hi[k] = std::max(hi[k], b.hi[k]);
    }
  }
  void grow(const float p[3]) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], p[k]);
      hi[k] = std::max(hi[k], p[k]);
    }
  }
  float halfArea() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.f;
    return dx * dy + dy * dz + dz * dx;
  }
};

struct BinNode {  // binary build node
  Box box;
  int left = -1, right = -1;  // children (inner)
  uint32_t first = 0, count = 0;  // leaf range into the index array
  bool leaf() const { return left < 0; }
};

#ifndef SPRAY_SAH_TRAVERSAL_COST
#define SPRAY_SAH_TRAVERSAL_COST 1.0f
#endif
constexpr int kBins = 16;
constexpr float kTraversalCost = SPRAY_SAH_TRAVERSAL_COST;  // relative to one triangle test
constexpr float kTriCost = 1.0f;

struct Builder {
  const float* v;
  const uint32_t* f;
  std::vector<Box> tbox;
  std::vector<float> cent;  // 3 per triangle
  std::vector<uint32_t> idx;
  std::vector<BinNode> nodes;

  void triBox(uint32_t t, Box* b) {
    b->reset();
    for (int c = 0; c < 3; ++c) b->grow(&v[3 * (size_t)f[3 * (size_t)t + c]]);
  }

  int build(uint32_t first, uint32_t count) {
    int id = (int)nodes.size();
    nodes.emplace_back();
    Box box, cbox;
    box.reset();
    cbox.reset();
    for (uint32_t i = first; i < first + count; ++i) {
      box.grow(tbox[idx[i]]);
      cbox.grow(&cent[3 * (size_t)idx[i]]);
    }
    nodes[id].box = box;
    nodes[id].first = first;
    nodes[id].count = count;
    if (count <= 2) return id;
    // binned SAH over centroid bounds
    float best_cost = FLT_MAX;
    int best_axis = -1, best_split = -1;
    for (int a = 0; a < 3; ++a) {
      float ext = cbox.hi[a] - cbox.lo[a];
      if (!(ext > 0.f)) continue;
      Box bb[kBins];
      uint32_t bc[kBins] = {0};
      for (int b = 0; b < kBins; ++b) bb[b].reset();
      float scale = kBins / ext;
      for (uint32_t i = first; i < first + count; ++i) {
        int b = (int)((cent[3 * (size_t)idx[i] + a] - cbox.lo[a]) * scale);
        b = std::min(std::max(b, 0), kBins - 1);
        bb[b].grow(tbox[idx[i]]);
        ++bc[b];
      }
      float la[kBins];
      uint32_t lc[kBins];
      Box acc;
      acc.reset();
      uint32_t n = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        acc.grow(bb[b]);
        n += bc[b];
        la[b] = acc.halfArea();
        lc[b] = n;
      }
      acc.reset();
      n = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        n += bc[b];
        if (lc[b - 1] == 0 || n == 0) continue;
        float cost = la[b - 1] * lc[b - 1] + acc.halfArea() * n;
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = a;
          best_split = b;
        }
      }
    }
    float leaf_cost = box.halfArea() * count * kTriCost;
    float split_cost = kTraversalCost * box.halfArea() + kTriCost * best_cost;
    uint32_t mid;
    if (best_axis < 0) {
      if (count <= (uint32_t)kMaxLeafTris) return id;
      // all centroids coincide: split the range in half
      mid = first + count / 2;
    } else {
      if (count <= (uint32_t)kMaxLeafTris && leaf_cost <= split_cost) return id;
      float ext = cbox.hi[best_axis] - cbox.lo[best_axis];
      float scale = kBins / ext;
      auto it = std::partition(idx.begin() + first, idx.begin() + first + count, [&](uint32_t t) {
        int b = (int)((cent[3 * (size_t)t + best_axis] - cbox.lo[best_axis]) * scale);
        b = std::min(std::max(b, 0), kBins - 1);
        return b < best_split;
      });
      mid = (uint32_t)(it - idx.begin());
      if (mid == first || mid == first + count) mid = first + count / 2;
    }
    int l = build(first, mid - first);
    int r = build(mid, first + count - mid);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }
};

struct Collapser {
  const Builder& b;
  BvhBuildResult* out;
  int maxdepth = 0;

  // Emits a 4-wide node for binary node `bn`; returns its index.
  int emit(int bn, int depth) {
    maxdepth = std::max(maxdepth, depth);
    int id = (int)out->nodes.size();
    out->nodes.emplace_back();
    // gather up to 4 children by opening the largest inner child
    int kids[4];
    int nk = 0;
    kids[nk++] = b.nodes[bn].left;
    kids[nk++] = b.nodes[bn].right;
    while (nk < 4) {
      int best = -1;
      float best_area = -1.f;
      for (int i = 0; i < nk; ++i) {
        const BinNode& k = b.nodes[kids[i]];
        if (!k.leaf() && k.box.halfArea() > best_area) {
          best_area = k.box.halfArea();
          best = i;
        }
      }
      if (best < 0) break;
      int opened = kids[best];
      kids[best] = b.nodes[opened].left;
      kids[nk++] = b.nodes[opened].right;
    }
    BvhNode4 node;
    for (int c = 0; c < 4; ++c) {
      node.lox[c] = node.loy[c] = node.loz[c] = INFINITY;
      node.hix[c] = node.hiy[c] = node.hiz[c] = -INFINITY;
      node.child[c] = kEmptyChild;
      node.pad[c] = 0;
    }
    int child_ref[4];
    for (int c = 0; c < nk; ++c) {
      const BinNode& k = b.nodes[kids[c]];
      if (k.leaf()) {
        if (k.count > (uint32_t)kMaxLeafTris || k.first >= (1u << 27))
          throw std::runtime_error("bvh: leaf does not fit the node encoding");
        child_ref[c] = ~(int32_t)((k.first << 3) | (k.count - 1));
      } else {
        child_ref[c] = -1;  // filled after recursion
      }
    }
    for (int c = 0; c < nk; ++c) {
      const BinNode& k = b.nodes[kids[c]];
      node.lox[c] = k.box.lo[0];
      node.loy[c] = k.box.lo[1];
      node.loz[c] = k.box.lo[2];
      node.hix[c] = k.box.hi[0];
      node.hiy[c] = k.box.hi[1];
      node.hiz[c] = k.box.hi[2];
    }
    out->nodes[id] = node;
    for (int c = 0; c < nk; ++c) {
      if (!b.nodes[kids[c]].leaf()) child_ref[c] = emit(kids[c], depth + 1);
      out->nodes[id].child[c] = child_ref[c];
    }
    return id;
  }
};

}  // namespace

void buildBvh4(const float* vertices, const uint32_t* faces, uint32_t num_faces,
               BvhBuildResult* out) {
  out->nodes.clear();
  out->tri_order.clear();
  if (num_faces == 0) throw std::runtime_error("bvh: empty mesh");
  Builder b;
  b.v = vertices;
  b.f = faces;
  b.tbox.resize(num_faces);
  b.cent.resize(3 * (size_t)num_faces);
  b.idx.resize(num_faces);
  for (uint32_t t = 0; t < num_faces; ++t) {
    b.triBox(t, &b.tbox[t]);
    for (int k = 0; k < 3; ++k) b.cent[3 * (size_t)t + k] = 0.5f * (b.tbox[t].lo[k] + b.tbox[t].hi[k]);
    b.idx[t] = t;
  }
  b.nodes.reserve(2 * (size_t)num_faces / 2 + 8);
  int root = b.build(0, num_faces);
  out->tri_order = b.idx;
  Collapser c{b, out};
  if (b.nodes[root].leaf()) {
    // a single leaf: wrap it into one node with one child
    BvhNode4 node;
    for (int k = 0; k < 4; ++k) {
      node.lox[k] = node.loy[k] = node.loz[k] = INFINITY;
      node.hix[k] = node.hiy[k] = node.hiz[k] = -INFINITY;
      node.child[k] = kEmptyChild;
      node.pad[k] = 0;
    }
    const BinNode& k = b.nodes[root];
    node.lox[0] = k.box.lo[0];
    node.loy[0] = k.box.lo[1];
    node.loz[0] = k.box.lo[2];
    node.hix[0] = k.box.hi[0];
    node.hiy[0] = k.box.hi[1];
    node.hiz[0] = k.box.hi[2];
    if (k.count > (uint32_t)kMaxLeafTris) throw std::runtime_error("bvh: root leaf too large");
    node.child[0] = ~(int32_t)((k.first << 3) | (k.count - 1));
    out->nodes.push_back(node);
    out->depth = 1;
    return;
  }
  c.emit(root, 1);
  out->depth = c.maxdepth;
}

}  // namespace spray

namespace spray {
namespace {

struct DomBuild {
  const float* boxes;
  std::vector<int> ids;
  std::vector<DomNode>* out;

  void bounds(int first, int count, float lo[3], float hi[3]) const {
    for (int k = 0; k < 3; ++k) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
    for (int i = first; i < first + count; ++i)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], boxes[6 * ids[i] + k]);
        hi[k] = std::max(hi[k], boxes[6 * ids[i] + 3 + k]);
      }
    // enlarge outward by a relative 1e-6 (plus a tiny absolute term)
    for (int k = 0; k < 3; ++k) {
      lo[k] = (float)((double)lo[k] - (std::fabs((double)lo[k]) + 1e-30) * 1e-6);
      hi[k] = (float)((double)hi[k] + (std::fabs((double)hi[k]) + 1e-30) * 1e-6);
    }
  }

  // Returns the child reference for ids[first, first + count).
  int32_t build(int first, int count) {
    if (count == 1) return ~(int32_t)ids[first];
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = first; i < first + count; ++i)
      for (int k = 0; k < 3; ++k) {
        float c = 0.5f * (boxes[6 * ids[i] + k] + boxes[6 * ids[i] + 3 + k]);
        clo[k] = std::min(clo[k], c);
        chi[k] = std::max(chi[k], c);
      }
    int axis = 0;
    for (int k = 1; k < 3; ++k)
      if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
    int mid = first + count / 2;
    std::nth_element(ids.begin() + first, ids.begin() + mid, ids.begin() + first + count, [&](int a, int b) {
      float ca = boxes[6 * a + axis] + boxes[6 * a + 3 + axis];
      float cb = boxes[6 * b + axis] + boxes[6 * b + 3 + axis];
      return ca < cb || (ca == cb && a < b);
    });
    int id = (int)out->size();
    out->emplace_back();
    DomNode node;
    std::memset(&node, 0, sizeof(node));
    bounds(first, mid - first, node.lo0, node.hi0);
    bounds(mid, first + count - mid, node.lo1, node.hi1);
    node.c0 = build(first, mid - first);
    node.c1 = build(mid, first + count - mid);
    (*out)[id] = node;
    return id;
  }
};

}  // namespace

void buildDomainBvh(const float* boxes, int n, std::vector<DomNode>* out) {
  out->clear();
  if (n < 2) throw std::runtime_error("domain hierarchy needs at least two domains");
  DomBuild b{boxes, std::vector<int>(n), out};
  for (int i = 0; i < n; ++i) b.ids[i] = i;
  b.build(0, n);
}

namespace {

struct DomCollapse {
  const std::vector<DomNode>& bin;
  std::vector<BvhNode4>* out;

  static void setSlot(BvhNode4& nd, int k, const float lo[3], const float hi[3], int32_t child) {
    nd.lox[k] = lo[0];
    nd.loy[k] = lo[1];
    nd.loz[k] = lo[2];
    nd.hix[k] = hi[0];
    nd.hiy[k] = hi[1];
    nd.hiz[k] = hi[2];
    nd.child[k] = child;
  }

  // 4-wide node for binary inner node b; returns its index.
  int emit(int b) {
    const int id = (int)out->size();
    out->emplace_back();
    BvhNode4 nd;
    std::memset(&nd, 0, sizeof(nd));
    for (int k = 0; k < 4; ++k) {
      const float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
      setSlot(nd, k, lo, hi, kEmptyChild);
    }
    int pending[4] = {-1, -1, -1, -1};  // binary inner node behind each slot
    int k = 0;
    for (int s = 0; s < 2; ++s) {
      const DomNode& n = bin[b];
      const int32_t c = s ? n.c1 : n.c0;
      if (c < 0) {
        setSlot(nd, k++, s ? n.lo1 : n.lo0, s ? n.hi1 : n.hi0, c);
        continue;
      }
      const DomNode& m = bin[c];
      for (int t = 0; t < 2; ++t) {
        const int32_t g = t ? m.c1 : m.c0;
        setSlot(nd, k, t ? m.lo1 : m.lo0, t ? m.hi1 : m.hi0, g);
        if (g >= 0) pending[k] = g;
        ++k;
      }
    }
    (*out)[id] = nd;
    for (int q = 0; q < 4; ++q)
      if (pending[q] >= 0) {
        const int child = emit(pending[q]);
        (*out)[id].child[q] = child;
      }
    return id;
  }
};

}  // namespace

void buildDomainBvh4(const float* boxes, int n, std::vector<BvhNode4>* out) {
  std::vector<DomNode> bin;
  buildDomainBvh(boxes, n, &bin);
  out->clear();
  DomCollapse c{bin, out};
  c.emit(0);
}

}  // namespace spray
