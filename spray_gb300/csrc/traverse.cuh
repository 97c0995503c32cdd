// Per-thread BVH walks of one (ray, domain) pair, shared by the queue
// kernels (trace.cu) and the round loop of the non-speculative tracer
// (rounds.cu): the 4-wide node test, the closest-hit walk and the any-hit
// walk.  Scene::intersect / Scene::occluded (src/render/scene.inl:189-209)
// with tnear = 1e-3.
#pragma once

#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {
namespace {

// Box test slack: (1 + 2*gamma(3)) rounded up (Ize, "Robust BVH Ray
// Traversal", JCGT 2(2), 2013), so rounding never culls a box the ray touches.
constexpr float kBoxSlack = 1.0000004f;
constexpr int kStack = 64;

struct TravRay {
  V3 org, dir, inv;
  int sx, sy, sz;  // 1 when the direction component is negative
  RayShear sh;
};

__device__ __forceinline__ TravRay makeTravRay(V3 org, V3 dir) {
  TravRay r;
  r.org = org;
  r.dir = dir;
  r.inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  r.sx = r.inv.x < 0.0f;
  r.sy = r.inv.y < 0.0f;
  r.sz = r.inv.z < 0.0f;
  r.sh = makeShear(dir);
  return r;
}

// Intersects the four children of a node; returns a mask of hit children and
// their entry distances.  Near and far planes are picked by the direction's
// sign, so an empty slot (lo = +inf, hi = -inf) can never be entered.  Per
// child: t0 = max(max(tx0, ty0), max(tz0, tnear)), t1 = min(min(tx1, ty1),
// min(tz1, tfar)) * kBoxSlack with tx = (plane - org.x) * inv.x; children
// (0, 1) and (2, 3) share the packed subtractions and products.
__device__ __forceinline__ int testChildren(const BvhNode4* __restrict__ nodes, int node,
                                            const TravRay& r, float tnear, float tfar,
                                            float tn[4]) {
  // the node stores lo/hi per axis as float4 pairs; the ray's signs pick the
  // near and far plane of each pair by address
  const float4* p = reinterpret_cast<const float4*>(nodes + node);
  const float4 nx = __ldg(p + r.sx), fx = __ldg(p + (r.sx ^ 1));
  const float4 ny = __ldg(p + 2 + r.sy), fy = __ldg(p + (3 - r.sy));
  const float4 nz = __ldg(p + 4 + r.sz), fz = __ldg(p + (5 - r.sz));
  const unsigned long long ox = f2pack(r.org.x, r.org.x), oy = f2pack(r.org.y, r.org.y),
                           oz = f2pack(r.org.z, r.org.z);
  const unsigned long long ix = f2pack(r.inv.x, r.inv.x), iy = f2pack(r.inv.y, r.inv.y),
                           iz = f2pack(r.inv.z, r.inv.z);
  int mask = 0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float2 ax = f2subMul(h ? f2pack(nx.z, nx.w) : f2pack(nx.x, nx.y), ox, ix);
    const float2 ay = f2subMul(h ? f2pack(ny.z, ny.w) : f2pack(ny.x, ny.y), oy, iy);
    const float2 az = f2subMul(h ? f2pack(nz.z, nz.w) : f2pack(nz.x, nz.y), oz, iz);
    const float2 bx = f2subMul(h ? f2pack(fx.z, fx.w) : f2pack(fx.x, fx.y), ox, ix);
    const float2 by = f2subMul(h ? f2pack(fy.z, fy.w) : f2pack(fy.x, fy.y), oy, iy);
    const float2 bz = f2subMul(h ? f2pack(fz.z, fz.w) : f2pack(fz.x, fz.y), oz, iz);
    const float t00 = fmaxf(fmaxf(ax.x, ay.x), fmaxf(az.x, tnear));
    const float t01 = fmaxf(fmaxf(ax.y, ay.y), fmaxf(az.y, tnear));
    const float t10 = fminf(fminf(bx.x, by.x), fminf(bz.x, tfar)) * kBoxSlack;
    const float t11 = fminf(fminf(bx.y, by.y), fminf(bz.y, tfar)) * kBoxSlack;
    tn[2 * h] = t00;
    tn[2 * h + 1] = t01;
    if (t00 <= t10) mask |= 1 << (2 * h);
    if (t01 <= t11) mask |= 1 << (2 * h + 1);
  }
  return mask;
}

// The same test in scalar arithmetic (fewer live registers), for the
// occlusion walk.
__device__ __forceinline__ int testChildrenScalar(const BvhNode4* __restrict__ nodes, int node,
                                                  const TravRay& r, float tnear, float tfar,
                                                  float tn[4]) {
  const float4* p = reinterpret_cast<const float4*>(nodes + node);
  const float4 nx = __ldg(p + r.sx), fx = __ldg(p + (r.sx ^ 1));
  const float4 ny = __ldg(p + 2 + r.sy), fy = __ldg(p + (3 - r.sy));
  const float4 nz = __ldg(p + 4 + r.sz), fz = __ldg(p + (5 - r.sz));
  const float nxa[4] = {nx.x, nx.y, nx.z, nx.w}, fxa[4] = {fx.x, fx.y, fx.z, fx.w};
  const float nya[4] = {ny.x, ny.y, ny.z, ny.w}, fya[4] = {fy.x, fy.y, fy.z, fy.w};
  const float nza[4] = {nz.x, nz.y, nz.z, nz.w}, fza[4] = {fz.x, fz.y, fz.z, fz.w};
  int mask = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float t0 = fmaxf(fmaxf((nxa[c] - r.org.x) * r.inv.x, (nya[c] - r.org.y) * r.inv.y),
                     fmaxf((nza[c] - r.org.z) * r.inv.z, tnear));
    float t1 = fminf(fminf((fxa[c] - r.org.x) * r.inv.x, (fya[c] - r.org.y) * r.inv.y),
                     fminf((fza[c] - r.org.z) * r.inv.z, tfar)) *
               kBoxSlack;
    tn[c] = t0;
    if (t0 <= t1) mask |= 1 << c;
  }
  return mask;
}

__device__ __forceinline__ int4 loadChildren(const BvhNode4* __restrict__ nodes, int node) {
  const int4* p = reinterpret_cast<const int4*>(nodes + node);
  return __ldg(p + 6);
}

__device__ __forceinline__ int childAt(int4 c, int k) {
  return k == 0 ? c.x : (k == 1 ? c.y : (k == 2 ? c.z : c.w));
}

// Upper bound on node visits of one traversal; reaching it means a corrupt
// hierarchy, which is reported through Counters::error_flags.
constexpr int kMaxSteps = 1 << 20;

__device__ __forceinline__ void raise(Counters* ctr, unsigned long long bit) {
  atomicOr(&ctr->error_flags, bit);
}

// Marks the end of a traversal (never a child reference: empty slots are skipped).
constexpr int kDone = (int)kEmptyChild;
// Inner-node expansions a lane runs before its warp checks for idle lanes.
constexpr int kNodeBudget = 8;

// Traversal state of one (ray, domain) entry, kept across the rounds of the
// persistent loop so that a lane can be refilled as soon as its entry ends.
struct Walk {
  const BvhNode4* nodes;
  const float4* tris;
  int num_nodes, num_tris;
  int cur, sp, steps;
};

__device__ __forceinline__ Walk startWalk(const SceneDev& sc, const DomainDev& dom) {
  Walk w;
  const DomArrays g = domArrays(sc, dom);
  w.nodes = g.nodes;
  w.tris = g.tris;
  w.num_nodes = dom.num_nodes;
  w.num_tris = dom.num_tris;
  w.cur = 0;
  w.sp = 0;
  w.steps = 0;
  return w;
}

// Closest hit in one domain.  best_key enters as the key to beat and leaves as
// the best found; returns true when this domain improved it.
//
// While-while traversal: a thread expands inner nodes until the nearest
// pending entry is a leaf (the loop ends when every active thread holds a
// leaf or has finished), then the threads test their leaves together.  Inner
// nodes and leaves share one near-to-far stack, so a leaf is tested only after
// every nearer subtree, and entries beyond the best hit are dropped on pop.
// The hit does not depend on the order: the packed (t | triangle) key is a
// total order and a subtree is skipped only when its box starts beyond the
// best t found.
__device__ bool traverseClosest(const SceneDev& sc, const DomainDev& dom, const TravRay& r,
                                uint64_t& best_key, float& best_t, uint32_t& best_prim,
                                float& best_u, float& best_v, Counters* ctr,
                                uint32_t& nnodes, uint32_t& ntris) {
  const DomArrays g = domArrays(sc, dom);
  const BvhNode4* nodes = g.nodes;
  const float4* tris = g.tris;
  uint2 stack[kStack];
  int sp = 0;
  bool found = false;
  // node and triangle counts of this walk (32 bits: a walk is bounded by
  // kMaxSteps); the node count is also the step bound's counter
  uint32_t steps = 0, tested = 0;
  auto finish = [&]() {
    nnodes += steps;
    ntris += tested;
    return found;
  };
  auto pop = [&]() -> int {
    while (sp > 0) {
      const uint2 e = stack[--sp];
      if (__uint_as_float(e.y) <= best_t) return (int)e.x;
    }
    return kDone;
  };
  // triangles of one leaf; false on a corrupt leaf reference
  auto testLeaf = [&](int lf) -> bool {
    const uint32_t v = ~(uint32_t)lf;
    const uint32_t first = v >> 3, cnt = (v & 7u) + 1u;
    if (first + cnt > (uint32_t)dom.num_tris) {
      raise(ctr, kErrBadNode);
      return false;
    }
    tested += cnt;
    for (uint32_t q = 0; q < cnt; ++q) {
      const float4* tp = tris + 3 * (size_t)(first + q);
      const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
      float t, u, vv;
      if (intersectTriangle(r.sh, r.org, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(cc.x, cc.y, cc.z),
                            kRayEpsilon, __int_as_float(0x7f800000), &t, &u, &vv)) {
        const uint32_t prim = __float_as_uint(a.w);
        const uint64_t key = packHitKey(t, dom.gprim_base + prim);
        if (key < best_key) {
          best_key = key;
          best_t = t;
          best_prim = prim;
          best_u = u;
          best_v = vv;
          found = true;
        }
      }
    }
    return true;
  };
  int cur = 0;
  while (cur != kDone) {
    // inner nodes until the nearest pending entry is a leaf
    while (cur >= 0) {
      if (++steps > (uint32_t)kMaxSteps) {
        raise(ctr, kErrTraversalBound);
        return finish();
      }
      if ((unsigned)cur >= (unsigned)dom.num_nodes) {
        raise(ctr, kErrBadNode);
        return finish();
      }
      float tn[4];
      const int mask = testChildren(nodes, cur, r, kRayEpsilon, best_t, tn);
      const int4 ch = loadChildren(nodes, cur);
      // Children sorted near to far by a key of the entry t with its two low
      // bits replaced by the slot: t >= tnear > 0, so the bits order like the
      // value, and the key's t (rounded down by at most 3 ulp) stays a lower
      // bound of the entry.  A five-comparator network keeps it in registers.
      uint32_t k[4];
#pragma unroll
      for (int c = 0; c < 4; ++c)
        k[c] = ((mask & (1 << c)) && childAt(ch, c) != kEmptyChild)
                   ? (__float_as_uint(tn[c]) & ~3u) | (uint32_t)c
                   : 0xffffffffu;
      auto cswap = [](uint32_t& x, uint32_t& y) {
        const uint32_t lo = min(x, y), hi = max(x, y);
        x = lo;
        y = hi;
      };
      cswap(k[0], k[1]);
      cswap(k[2], k[3]);
      cswap(k[0], k[2]);
      cswap(k[1], k[3]);
      cswap(k[1], k[2]);
      // The nearest child continues the walk when it starts within the best
      // hit; the others go on the stack far to near.  Every other child starts
      // at least as far as the nearest, so when the nearest is beyond the best
      // hit all of them are (pop would drop them) and the walk pops instead.
      if (k[0] != 0xffffffffu && __uint_as_float(k[0] & ~3u) <= best_t) {
#pragma unroll
        for (int j = 3; j >= 1; --j) {
          if (k[j] == 0xffffffffu) continue;
          if (sp == kStack) {
            raise(ctr, kErrTraversalBound);
            return finish();
          }
          stack[sp++] = make_uint2((uint32_t)childAt(ch, (int)(k[j] & 3u)), k[j] & ~3u);
        }
        cur = childAt(ch, (int)(k[0] & 3u));
      } else {
        cur = pop();
      }
    }
    if (cur == kDone) break;
    if (!testLeaf(cur)) return finish();
    cur = pop();
  }
  return finish();
}

// Any hit in (tnear, tfar) in one domain, the whole walk at once: the last
// hit child continues, the others are pushed.  Returns true on a hit.
__device__ bool traverseAny(const SceneDev& sc, const DomainDev& dom, const TravRay& r, float tfar,
                            Counters* ctr, uint32_t& nnodes, uint32_t& ntris) {
  const DomArrays g = domArrays(sc, dom);
  int stack[kStack];
  int sp = 0, cur = 0;
  uint32_t steps = 0;
  while (cur != kDone) {
    while (cur >= 0) {
      if (++steps > (uint32_t)kMaxSteps || (unsigned)cur >= (unsigned)dom.num_nodes) {
        raise(ctr, steps > (uint32_t)kMaxSteps ? kErrTraversalBound : kErrBadNode);
        nnodes += steps;
        return false;
      }
      float tn[4];
      const int mask = testChildren(g.nodes, cur, r, kRayEpsilon, tfar, tn);
      const int4 ch = loadChildren(g.nodes, cur);
      int next = kDone;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (!(mask & (1 << c))) continue;
        const int ref = childAt(ch, c);
        if (ref == kEmptyChild) continue;
        if (next != kDone) {
          if (sp == kStack) {
            raise(ctr, kErrTraversalBound);
            nnodes += steps;
            return false;
          }
          stack[sp++] = next;
        }
        next = ref;
      }
      cur = next != kDone ? next : (sp > 0 ? stack[--sp] : kDone);
    }
    if (cur == kDone) break;
    const uint32_t v = ~(uint32_t)cur;
    const uint32_t first = v >> 3, cnt = (v & 7u) + 1u;
    if (first + cnt > (uint32_t)dom.num_tris) {
      raise(ctr, kErrBadNode);
      nnodes += steps;
      return false;
    }
    ntris += cnt;
    for (uint32_t q = 0; q < cnt; ++q) {
      const float4* tp = g.tris + 3 * (size_t)(first + q);
      const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
      float t, u, vv;
      if (intersectTriangle(r.sh, r.org, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(cc.x, cc.y, cc.z),
                            kRayEpsilon, tfar, &t, &u, &vv)) {
        nnodes += steps;
        return true;
      }
    }
    cur = sp > 0 ? stack[--sp] : kDone;
  }
  nnodes += steps;
  return false;
}

}  // namespace
}  // namespace spray
