// Per-domain bounding volume hierarchy: binned-SAH binary build collapsed into
// 4-wide nodes.  Replaces the Embree triangle BVH SpRay rebuilds on every
// domain load (src/render/trimesh_buffer.cc:104,224); here it is built once per
// domain and kept with the domain's geometry.
#pragma once

#include <cstdint>
#include <vector>

namespace spray {

// One 128-byte node: child boxes in SoA form, then the child references.
//   child >= 0 : index of an inner node (domain-relative)
//   child <  0 : leaf, ~child = (first_triangle << 3) | (count - 1)
//   child == kEmptyChild : unused slot, with an empty box (lo = +inf, hi = -inf)
struct alignas(16) BvhNode4 {
  float lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
  int32_t child[4];
  int32_t pad[4];
};
static_assert(sizeof(BvhNode4) == 128, "node must be one 128-byte line");

constexpr int kMaxLeafTris = 8;
constexpr int32_t kEmptyChild = (int32_t)0x80000000;

// Binary hierarchy over the domain boxes (median splits); the scheduler
// descends its 4-wide collapse (buildDomainBvh4) to find the domains a ray may
// overlap before it runs SpRay's exact slab test on them.
// Node boxes are enlarged outward so a conservative node test never rejects a
// domain the exact test accepts.  c0/c1 >= 0: inner node; < 0: leaf ~domain.
struct alignas(16) DomNode {
  float lo0[3];
  int32_t c0;
  float hi0[3];
  float pad0;
  float lo1[3];
  int32_t c1;
  float hi1[3];
  float pad1;
};
static_assert(sizeof(DomNode) == 64, "domain node must be 64 bytes");

// boxes: 6 floats per domain (min xyz, max xyz); n >= 2.
void buildDomainBvh(const float* boxes, int n, std::vector<DomNode>* out);

// The same hierarchy collapsed to 4-wide nodes in the BvhNode4 layout (root
// at 0): each node holds the children of its binary node's children (a leaf
// child keeps its own slot), boxes unchanged (enlarged outward), child < 0 a
// leaf ~domain, unused slots empty (lo = +inf, hi = -inf, kEmptyChild).
void buildDomainBvh4(const float* boxes, int n, std::vector<BvhNode4>* out);

struct BvhBuildResult {
  std::vector<BvhNode4> nodes;     // nodes[0] is the root
  std::vector<uint32_t> tri_order;  // leaf order -> original face index
  int depth = 0;                    // deepest node level (root = 1)
};

// Builds the BVH of a triangle mesh.  Boxes are exact min/max of the float
// vertices, so traversal with a conservative box test never misses a triangle.
void buildBvh4(const float* vertices, const uint32_t* faces, uint32_t num_faces,
               BvhBuildResult* out);

}  // namespace spray
