// Descent of the 4-wide hierarchy over the domain boxes, shared by the
// scheduler (sched.cu) and the non-speculative round loop (rounds.cu).
#pragma once

#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {

// Calls consider(d) for every domain d of the 4-wide hierarchy over the domain
// boxes (8 float4 per node, BvhNode4 layout; NN nodes) whose node boxes the ray
// (org, inv = 1 / dir) enters within (1e-3, t1].  The node boxes are enlarged
// outward and the test widened by 2 ulp, so the descent is conservative: the
// caller's exact slab test at the leaf decides.  Children go near to far, so
// domains arrive roughly in entry order.
template <class F>
__device__ __forceinline__ void descendDomains(const float4* nodes, int NN, V3 org, V3 inv, float t1, F&& consider,
                                               Counters* ctr) {
  const int sx = inv.x < 0.0f, sy = inv.y < 0.0f, sz = inv.z < 0.0f;
  const float tfar = t1 * 1.0000004f;
  int stack[32];
  int sp = 0;
  int node = 0;
  for (int steps = 0; steps < NN + 4; ++steps) {
    const float4* nd = nodes + 8 * node;
    const float4 nx = nd[sx], fx = nd[sx ^ 1], ny = nd[2 + sy], fy = nd[3 - sy];
    const float4 nz = nd[4 + sz], fz = nd[5 - sz];
    const int4 ch = *reinterpret_cast<const int4*>(nd + 6);
    const float nxa[4] = {nx.x, nx.y, nx.z, nx.w}, fxa[4] = {fx.x, fx.y, fx.z, fx.w};
    const float nya[4] = {ny.x, ny.y, ny.z, ny.w}, fya[4] = {fy.x, fy.y, fy.z, fy.w};
    const float nza[4] = {nz.x, nz.y, nz.z, nz.w}, fza[4] = {fz.x, fz.y, fz.z, fz.w};
    const int cha[4] = {ch.x, ch.y, ch.z, ch.w};
    uint32_t k[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float t0 = fmaxf(fmaxf((nxa[c] - org.x) * inv.x, (nya[c] - org.y) * inv.y),
                             fmaxf((nza[c] - org.z) * inv.z, kRayEpsilon));
      const float tt = fminf(fminf((fxa[c] - org.x) * inv.x, (fya[c] - org.y) * inv.y),
                             fminf((fza[c] - org.z) * inv.z, tfar)) * 1.0000004f;
      // (entry t with the slot in its two low bits: t > 0 orders like its bits)
      k[c] = (t0 <= tt && cha[c] != kEmptyChild) ? ((__float_as_uint(t0) & ~3u) | (uint32_t)c) : 0xffffffffu;
    }
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
    int inner[4], ni = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (k[j] == 0xffffffffu) break;
      const int ref = cha[k[j] & 3u];
      if (ref < 0) consider(~ref);
      else inner[ni++] = ref;
    }
    // the nearest inner child next, the others on the stack far to near
    for (int j = ni - 1; j >= 1; --j) {
      if (sp < 32) stack[sp++] = inner[j];
      else atomicAdd(&ctr->list_overflows, 1ull);  // unreachable: depth <= 8, 3 per level
    }
    if (ni > 0) {
      node = inner[0];
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
}

}  // namespace spray
