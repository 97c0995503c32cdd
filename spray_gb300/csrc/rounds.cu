// The reference's non-speculative image tracer in rounds (schedule_policy 5).
//
// baseline::ImageTracer::trace (src/baseline/baseline_image_tracer.inl:28-131)
// queues every eye ray of the image in its first domain, then repeats rounds
// until every queue is empty: LoadAnyOnceImageSched
// (src/baseline/baseline_schedulers.cc:43-62) picks the one domain holding the
// most queued radiance and shadow rays, the domain is loaded, and its queued
// rays run there (InsituTracer::processRays, processShadow, processRay2,
// src/baseline/baseline_insitu_tracer.inl:545-766):
//   * a shadow ray not occluded here moves on to its next domain, or adds its
//     weight to the image when its domain list is exhausted;
//   * a radiance ray that finds a hit nearer than its best so far is shaded
//     here when no later domain starts before that hit, and otherwise moves
//     on; a hit not nearer sends the ray back to the domain of its best hit
//     for shading, as does the end of its list;
//   * shading tests each shadow ray in this domain first and queues it in the
//     next domain of its list; the bounce ray runs in this domain at once
//     (temp_q), then follows its own list.
// DomainIntersector::intersect (src/baseline/baseline_isector.h:44-98)
// recomputes a ray's domain list (every box hit with tnear = 1e-3, sorted by
// (t, id)) each time the ray moves.
//
// Here a round is one launch over the chosen domain's entries, one thread per
// queued ray, which follows the ray's chain of spawned bounce rays in the
// domain.  The rays the round queues elsewhere are partitioned by domain into
// an append-only arena: every domain keeps a host list of its segments, and
// the round's per-domain counts come back to the host, which keeps the queue
// lengths and picks the next domain exactly as the reference does (its
// std::sort over (id, count), counts descending).  A queue's count depends
// only on the rays' own states, not on the order in which a round ran them,
// so the sequence of rounds, the loads of the domain cache and every visit
// count equal the reference loop's; only the order in which contributions are
// added to a pixel differs.
#include <algorithm>
#include <cstring>
#include <utility>

#include "domain_walk.cuh"
#include "kernels.cuh"
#include "shade.cuh"
#include "spray_math.cuh"
#include "tracer_internal.h"
#include "traverse.cuh"

namespace spray {

namespace {

constexpr int kRoundNone = 0x7fffffff;  // INT_MAX: no domain, no list position
constexpr uint32_t kRoundShadow = 1u;   // meta.z flag bits above the 8-bit depth
constexpr uint32_t kRoundShade = 2u;    // DRAY_FLAG_SHADE: back in the domain of its hit for shading
// List positions a ray can reach: the list holds the kMaxList nearest domains.
constexpr int kRoundList = kMaxList + 1;
// Retries of a pixel's compare-and-swap before the error flag is raised.
constexpr int kCasLimit = 1 << 20;
constexpr uint32_t kNoRay = 0xffffffffu;  // no ray (pool exhausted, nothing spawned)

struct RoundArgs {
  SceneDev scene;
  const float* boxes;  // 6 floats per domain
  int D;
  const float4* dnodes;  // 4-wide hierarchy over the boxes (8 float4 per node), null: every box
  int dnode_count;
  RoundRays rays;
  uint32_t* pool_count;
  uint32_t pool_cap;
  // the round: domain, and its entries as segments of the arena
  int id;
  const uint32_t* arena;
  const uint32_t* seg;  // nseg start offsets, then nseg + 1 prefix sums
  int nseg;
  // rays queued elsewhere this round: (domain, ray)
  uint2* out;
  uint32_t* out_count;
  uint32_t out_cap;
  float4* image;
  ViewDev view;
  ShadeEnv env;
  Counters* ctr;
  unsigned long long* visits_shade;
  uint32_t* hist;  // the round's partition: D counts, total, overflow flag, queued count
};

// Words after the D counts of the round's histogram.
constexpr int kHistExtra = 3;

// The kernel that starts a round (kRoundEyes, kRoundRays) zeroes the
// histogram the partition after it fills (the host has read the last one).
__device__ __forceinline__ void zeroHist(uint32_t* hist, int D) {
  if (blockIdx.x == 0)
    for (int d = threadIdx.x; d < D + kHistExtra; d += blockDim.x) hist[d] = 0u;
}

// One thread's counts, added to the frame's counters when it ends: the nodes
// and triangles of its walks (closest hit, occlusion), its visits and the
// rays it spawned.
struct WalkCounts {
  uint32_t rnodes, rtris, snodes, stris;
  uint32_t vrad, vshadow, vshade, nshadow, nbounce;
};

__device__ __forceinline__ uint32_t depthOf(int4 m) { return (uint32_t)m.z & 0xffu; }
__device__ __forceinline__ uint32_t flagsOf(int4 m) { return (uint32_t)m.z >> 8; }

// DomainIntersector::intersect on one ray: the next list position (a new ray,
// domain_pos == kRoundNone, starts past `current` when that domain is the
// list's first), its domain (-1 when the list is exhausted) and the entry
// distance of the domain after it.
__device__ int advanceRay(const RoundArgs& a, V3 org, V3 dir, float tmax, int current, int& domain_pos,
                          float& next_tdom) {
  const V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  // the `need` nearest (t, id) pairs in order: positions p and p + 1, p at
  // most domain_pos + 1 (or 1 for a new ray)
  const int need = domain_pos == kRoundNone ? 3 : domain_pos + 3;
  if (need > kRoundList) {
    atomicAdd(&a.ctr->list_overflows, 1ull);
    domain_pos = kRoundNone;
    next_tdom = __int_as_float(0x7f800000);
    return -1;
  }
  float lt[kRoundList];
  int ld[kRoundList];
  int cnt = 0, n = 0;
  auto consider = [&](int d) {
    float t;
    if (!slabTest(&a.boxes[6 * d], &a.boxes[6 * d + 3], org, inv, kRayEpsilon, tmax, &t)) return;
    ++n;
    if (cnt == need && (lt[cnt - 1] < t || (lt[cnt - 1] == t && ld[cnt - 1] < d))) return;
    int j = cnt < need ? cnt++ : need - 1;
    while (j > 0 && (lt[j - 1] > t || (lt[j - 1] == t && ld[j - 1] > d))) {
      lt[j] = lt[j - 1];
      ld[j] = ld[j - 1];
      --j;
    }
    lt[j] = t;
    ld[j] = d;
  };
  if (a.dnode_count > 0) descendDomains(a.dnodes, a.dnode_count, org, inv, tmax, consider, a.ctr);
  else
    for (int d = 0; d < a.D; ++d) consider(d);
  int p;
  if (domain_pos == kRoundNone) p = (n > 0 && ld[0] == current) ? 1 : 0;
  else p = domain_pos + 1;
  if (p < n) {
    next_tdom = p + 1 < n ? lt[p + 1] : __int_as_float(0x7f800000);
    domain_pos = p;
    return ld[p];
  }
  domain_pos = kRoundNone;
  next_tdom = __int_as_float(0x7f800000);
  return -1;
}

__device__ __forceinline__ void queueRay(const RoundArgs& a, int d, uint32_t ray) {
  const uint32_t k = atomicAdd(a.out_count, 1u);
  if (k < a.out_cap) a.out[k] = make_uint2((uint32_t)d, ray);
  else atomicAdd(&a.ctr->arena_overflows, 1ull);
}

// px = (float)((double)px + v), atomically; after kCasLimit lost races the
// addition is dropped and the error flag raised.
__device__ __forceinline__ void addChannel(float* px, double v, Counters* ctr) {
  unsigned int* p = reinterpret_cast<unsigned int*>(px);
  unsigned int old = *p;
  for (int k = 0; k < kCasLimit; ++k) {
    const float nv = (float)((double)__uint_as_float(old) + v);
    const unsigned int seen = atomicCAS(p, old, __float_as_uint(nv));
    if (seen == old) return;
    old = seen;
  }
  atomicOr(&ctr->error_flags, kErrRetireContention);
}

// HdrImage::add with the retire scale, from CommitBufferB::retire
// (src/baseline/baseline_commit_buffer.h:49-63)
__device__ __forceinline__ void retire(const RoundArgs& a, int pixid, float4 w) {
  float* px = reinterpret_cast<float*>(a.image + a.view.pixel_base + pixid);
  const double s = a.view.scale;
  addChannel(px, s * (double)w.x, a.ctr);
  addChannel(px + 1, s * (double)w.y, a.ctr);
  addChannel(px + 2, s * (double)w.z, a.ctr);
}

__device__ uint32_t newRay(const RoundArgs& a) {
  const uint32_t r = atomicAdd(a.pool_count, 1u);
  if (r >= a.pool_cap) {
    atomicAdd(&a.ctr->arena_overflows, 1ull);
    return kNoRay;
  }
  return r;
}

// colour byte -> float, i * SPRAY_1_OVER_255 rounded once (util::unpack)
__device__ __forceinline__ V3 unpackRound(uint32_t c) {
  return v3((float)((double)((c >> 16) & 0xffu) * kOneOver255), (float)((double)((c >> 8) & 0xffu) * kOneOver255),
            (float)((double)(c & 0xffu) * kOneOver255));
}

// The shader of a hit in the round's domain: shadow rays tested here first,
// then queued in their next domain or retired; returns the bounce ray, if
// any, for the caller to run in this domain next.
__device__ uint32_t shadeHere(const RoundArgs& a, const DomainDev& dom, float4 o4, float4 d4, float4 w4,
                              int4 meta, int prim, float u, float v, WalkCounts& wc) {
  const float t = w4.w;
  const DomArrays g = domArrays(a.scene, dom);
  const uint32_t* f = g.faces + 3 * (size_t)prim;
  const uint32_t i0 = f[0], i1 = f[1], i2 = f[2];
  const uint32_t col = interpolateColor(g.colors[i0], g.colors[i1], g.colors[i2], u, v);
  const float* nb = g.normals;
  const V3 ns = interpolateNormal(v3(nb[3 * (size_t)i0], nb[3 * (size_t)i0 + 1], nb[3 * (size_t)i0 + 2]),
                                  v3(nb[3 * (size_t)i1], nb[3 * (size_t)i1 + 1], nb[3 * (size_t)i1 + 2]),
                                  v3(nb[3 * (size_t)i2], nb[3 * (size_t)i2 + 1], nb[3 * (size_t)i2 + 2]), u, v);
  const V3 org = v3(o4.x, o4.y, o4.z), dir = v3(d4.x, d4.y, d4.z);
  const V3 pos = v3(dir.x * t + org.x, dir.y * t + org.y, dir.z * t + org.z);
  const int pixid = meta.x, samid = meta.y;
  const uint32_t depth = depthOf(meta) + 1u;
  uint32_t bounce = kNoRay;
  shadeHit(
      a.env, a.view, dir, v3(w4.x, w4.y, w4.z), pos, ns, unpackRound(col), dom.bsdf, dom.bsdf_p, pixid, samid,
      (int)depth,
      [&](int, V3 wi, V3 w, float tmax, bool valid) {
        if (!valid) return;
        ++wc.nshadow;
        ++wc.vshadow;
        const TravRay tr = makeTravRay(pos, wi);
        if (traverseAny(a.scene, dom, tr, tmax, a.ctr, wc.snodes, wc.stris)) return;
        const uint32_t s = newRay(a);
        if (s == kNoRay) return;
        int dp = kRoundNone;
        float nt;
        const int nd = advanceRay(a, pos, wi, tmax, a.id, dp, nt);
        a.rays.org[s] = make_float4(pos.x, pos.y, pos.z, tmax);
        a.rays.dir[s] = make_float4(wi.x, wi.y, wi.z, nt);
        a.rays.wgt[s] = make_float4(w.x, w.y, w.z, __int_as_float(0x7f800000));
        a.rays.meta[s] = make_int4(pixid, samid, (int)(depth | (kRoundShadow << 8)), dp);
        a.rays.hit[s] = make_int4(kRoundNone, 0, 0, 0);
        if (nd >= 0) queueRay(a, nd, s);
        else retire(a, pixid, make_float4(w.x, w.y, w.z, 0.f));
      },
      [&](V3 wi, V3 w) {
        const uint32_t b = newRay(a);
        if (b == kNoRay) return;
        a.rays.org[b] = make_float4(pos.x, pos.y, pos.z, __int_as_float(0x7f800000));
        a.rays.dir[b] = make_float4(wi.x, wi.y, wi.z, __int_as_float(0x7f800000));
        a.rays.wgt[b] = make_float4(w.x, w.y, w.z, __int_as_float(0x7f800000));
        a.rays.meta[b] = make_int4(pixid, samid, (int)depth, kRoundNone);
        a.rays.hit[b] = make_int4(kRoundNone, 0, 0, 0);
        ++wc.nbounce;
        bounce = b;
      });
  return bounce;
}

// processRay2 on a radiance ray in the round's domain; returns a bounce ray
// spawned by its shading.
__device__ uint32_t runRadiance(const RoundArgs& a, const DomainDev& dom, uint32_t ray, WalkCounts& wc) {
  const float4 o4 = a.rays.org[ray], d4 = a.rays.dir[ray];
  float4 w4 = a.rays.wgt[ray];
  int4 meta = a.rays.meta[ray];
  int4 hit = a.rays.hit[ray];
  if (flagsOf(meta) & kRoundShade) {
    ++wc.vshade;
    return shadeHere(a, dom, o4, d4, w4, meta, hit.y, __int_as_float(hit.z), __int_as_float(hit.w), wc);
  }
  ++wc.vrad;
  const V3 org = v3(o4.x, o4.y, o4.z), dir = v3(d4.x, d4.y, d4.z);
  const TravRay tr = makeTravRay(org, dir);
  uint64_t key = kNoHit;
  float t = __int_as_float(0x7f800000), u = 0.f, v = 0.f;
  uint32_t prim = 0;
  const bool found = traverseClosest(a.scene, dom, tr, key, t, prim, u, v, a.ctr, wc.rnodes, wc.rtris);
  const float next_tdom = d4.w;
  auto moveOn = [&]() {
    int dp = meta.w;
    float nt;
    const int nd = advanceRay(a, org, dir, __int_as_float(0x7f800000), a.id, dp, nt);
    a.rays.dir[ray] = make_float4(d4.x, d4.y, d4.z, nt);
    meta.w = dp;
    a.rays.meta[ray] = meta;
    if (nd >= 0) queueRay(a, nd, ray);
  };
  auto sendBack = [&]() {
    meta.z |= (int)(kRoundShade << 8);
    a.rays.meta[ray] = meta;
    queueRay(a, hit.x, ray);
  };
  if (found) {
    if (t < w4.w) {
      w4.w = t;
      hit = make_int4(a.id, (int)prim, __float_as_int(u), __float_as_int(v));
      a.rays.wgt[ray] = w4;
      a.rays.hit[ray] = hit;
      if (isinf(next_tdom) || t < next_tdom)
        return shadeHere(a, dom, o4, d4, w4, meta, (int)prim, u, v, wc);
      moveOn();
    } else {
      sendBack();
    }
  } else if (isinf(next_tdom)) {
    if (hit.x != kRoundNone) sendBack();
  } else {
    moveOn();
  }
  return kNoRay;
}

// processShadow: not occluded here -> the next domain, or retired
__device__ void runShadow(const RoundArgs& a, const DomainDev& dom, uint32_t ray, WalkCounts& wc) {
  ++wc.vshadow;
  const float4 o4 = a.rays.org[ray], d4 = a.rays.dir[ray];
  const V3 org = v3(o4.x, o4.y, o4.z), dir = v3(d4.x, d4.y, d4.z);
  if (traverseAny(a.scene, dom, makeTravRay(org, dir), o4.w, a.ctr, wc.snodes, wc.stris)) return;
  int4 meta = a.rays.meta[ray];
  int dp = meta.w;
  float nt;
  const int nd = advanceRay(a, org, dir, o4.w, a.id, dp, nt);
  meta.w = dp;
  a.rays.meta[ray] = meta;
  a.rays.dir[ray] = make_float4(d4.x, d4.y, d4.z, nt);
  if (nd >= 0) queueRay(a, nd, ray);
  else retire(a, meta.x, a.rays.wgt[ray]);
}

// One round: every ray queued in domain a.id, each with the bounce rays its
// shading spawns in turn (InsituTracer::processRays' temp_q).
__global__ void __launch_bounds__(128) kRoundRays(RoundArgs a) {
  zeroHist(a.hist, a.D);
  const uint32_t n = a.seg[2 * a.nseg];
  const DomainDev dom = a.scene.domains[a.id];
  WalkCounts wc{};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    // segment holding item i: last prefix <= i
    int lo = 0, hi = a.nseg - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.seg[a.nseg + mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    uint32_t ray = a.arena[a.seg[lo] + (i - a.seg[a.nseg + lo])];
    if (flagsOf(a.rays.meta[ray]) & kRoundShadow) {
      runShadow(a, dom, ray, wc);
      continue;
    }
    // each spawned ray is one depth deeper: the chain ends within `bounces`
    for (int guard = 0; guard <= a.view.bounces && ray != kNoRay; ++guard) {
      ray = runRadiance(a, dom, ray, wc);
      if (ray == kNoRay) break;
      // a new ray: its list position only, then this domain first
      const float4 o4 = a.rays.org[ray], d4 = a.rays.dir[ray];
      int4 meta = a.rays.meta[ray];
      int dp = kRoundNone;
      float nt;
      advanceRay(a, v3(o4.x, o4.y, o4.z), v3(d4.x, d4.y, d4.z), __int_as_float(0x7f800000), kRoundNone, dp, nt);
      meta.w = dp;
      a.rays.meta[ray] = meta;
      a.rays.dir[ray] = make_float4(d4.x, d4.y, d4.z, nt);
    }
  }
  if (wc.rnodes) atomicAdd(&a.ctr->nodes_radiance, (unsigned long long)wc.rnodes);
  if (wc.rtris) atomicAdd(&a.ctr->tris_radiance, (unsigned long long)wc.rtris);
  if (wc.snodes) atomicAdd(&a.ctr->nodes_shadow, (unsigned long long)wc.snodes);
  if (wc.stris) atomicAdd(&a.ctr->tris_shadow, (unsigned long long)wc.stris);
  if (wc.vrad) atomicAdd(&a.ctr->visits_radiance, (unsigned long long)wc.vrad);
  if (wc.vshadow) atomicAdd(&a.ctr->visits_shadow, (unsigned long long)wc.vshadow);
  if (wc.vshade) atomicAdd(a.visits_shade, (unsigned long long)wc.vshade);
  if (wc.nshadow) atomicAdd(&a.ctr->rays_shadow, (unsigned long long)wc.nshadow);
  if (wc.nbounce) atomicAdd(&a.ctr->rays_bounce, (unsigned long long)wc.nbounce);
}

// genEyeRays + isectEyeDomains over the image as one tile (ImgSchedNop,
// src/baseline/baseline_tilers.h:35-47): sample s of pixel p has id
// spp * p + s, which seeds its jitter when spp > 1 (pixel corners at 1 spp).
__global__ void kRoundEyes(RoundArgs a, int64_t n) {
  zeroHist(a.hist, a.D);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ViewDev& vw = a.view;
  const CameraDev& cam = vw.cam;
  const int spp = vw.spp;
  const int pixid = (int)(i / spp), s = (int)(i % spp);
  const int x = pixid % vw.image_w, y = pixid / vw.image_w;
  const int samid = spp > 1 ? spp * pixid + s : pixid;
  float fx = (float)x, fy = (float)y;
  if (spp > 1) {
    uint32_t st = rngSeed(samid);
    fx = (float)x + rngNext(st);
    fy = (float)y + rngNext(st);
  }
  const V3 pos = v3(cam.pos[0], cam.pos[1], cam.pos[2]);
  const V3 d = cameraRay(cam, fx, fy);
  int dp = kRoundNone;
  float nt;
  const int first = advanceRay(a, pos, d, __int_as_float(0x7f800000), kRoundNone, dp, nt);
  a.rays.org[i] = make_float4(pos.x, pos.y, pos.z, __int_as_float(0x7f800000));
  a.rays.dir[i] = make_float4(d.x, d.y, d.z, nt);
  a.rays.wgt[i] = make_float4(1.f, 1.f, 1.f, __int_as_float(0x7f800000));
  a.rays.meta[i] = make_int4(pixid, samid, 0, dp);
  a.rays.hit[i] = make_int4(kRoundNone, 0, 0, 0);
  if (first >= 0) queueRay(a, first, (uint32_t)i);
}

// The round's queued rays into the arena, grouped by domain: counts, their
// offsets (after `base`), then the entries.
__global__ void kRoundCount(const uint2* out, const uint32_t* out_count, uint32_t out_cap, uint32_t* hist) {
  const uint32_t n = min(*out_count, out_cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&hist[out[i].x], 1u);
}

// Also records the overflow flag and the queued count, and clears the queue
// counter for the next round (the scatter reads the recorded count).
__global__ void __launch_bounds__(1024) kRoundOffsets(uint32_t* hist, int D, uint32_t base, uint32_t* cursor,
                                                      uint32_t* out_count, uint32_t out_cap, const Counters* ctr) {
  uint32_t* total = hist + D;
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = base;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int c0 = 0; c0 < D; c0 += blockDim.x) {
    const int d = c0 + threadIdx.x;
    const uint32_t v = d < D ? hist[d] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t before = (w > 0 ? warp_sums[w - 1] : 0u) + x - v;
    if (d < D) cursor[d] = carry + before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *total = carry - base;
    if (ctr->arena_overflows) hist[D + 1] = 1u;
    hist[D + 2] = min(*out_count, out_cap);
    *out_count = 0u;
  }
}

__global__ void kRoundScatter(const uint2* out, uint32_t* hist, int D, uint32_t* cursor, uint32_t* arena,
                              uint32_t arena_cap, Counters* ctr) {
  const uint32_t n = hist[D + 2];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint2 e = out[i];
    const uint32_t k = atomicAdd(&cursor[e.x], 1u);
    if (k < arena_cap) {
      arena[k] = e.y;
    } else {
      atomicAdd(&ctr->arena_overflows, 1ull);
      hist[D + 1] = 1u;
    }
  }
}

}  // namespace

// LoadAnyOnceSched::scheduleImage (src/baseline/baseline_schedulers.cc:43-62):
// the domain with the most queued rays; equal counts keep the order std::sort
// leaves them in when given the ids ascending.  Returns -1 when every count is 0.
int loadAnyOnceNext(const std::vector<int64_t>& counts) {
  // a unique largest count is the answer whatever the sort does with ties
  int64_t best = 0;
  int at = -1, ties = 0;
  for (size_t i = 0; i < counts.size(); ++i) {
    if (counts[i] > best) {
      best = counts[i];
      at = (int)i;
      ties = 1;
    } else if (counts[i] == best && best > 0) {
      ++ties;
    }
  }
  if (at < 0 || ties == 1) return at;
  std::vector<std::pair<int, int64_t>> rc(counts.size());
  for (size_t i = 0; i < counts.size(); ++i) rc[i] = {(int)i, counts[i]};
  std::sort(rc.begin(), rc.end(),
            [](const std::pair<int, int64_t>& x, const std::pair<int, int64_t>& y) { return x.second > y.second; });
  return rc.empty() || rc[0].second == 0 ? -1 : rc[0].first;
}

void Tracer::freeRounds() {
  devFree(rr.org);
  devFree(rr.dir);
  devFree(rr.wgt);
  devFree(rr.meta);
  devFree(rr.hit);
  devFree(d_rr_pool);
  devFree(d_rr_arena);
  devFree(d_rr_out);
  devFree(d_rr_hist);
  devFree(d_rr_cursor);
  devFree(d_rr_seg);
  if (h_rr) cudaFreeHost(h_rr);
  h_rr = nullptr;
  rr_pool_cap = rr_arena_cap = rr_seg_cap = 0;
}

void Tracer::ensureRounds(uint64_t pool, uint64_t arena, uint64_t segs) {
  if (pool > 0xfffffff0ull || arena > 0xfffffff0ull)
    throw OverflowError("the frame needs more than 2^32 rays or queue entries");
  if (pool > rr_pool_cap) {
    devFree(rr.org);
    devFree(rr.dir);
    devFree(rr.wgt);
    devFree(rr.meta);
    devFree(rr.hit);
    devFree(d_rr_out);
    devAlloc(&rr.org, pool);
    devAlloc(&rr.dir, pool);
    devAlloc(&rr.wgt, pool);
    devAlloc(&rr.meta, pool);
    devAlloc(&rr.hit, pool);
    devAlloc(&d_rr_out, pool);  // a ray is queued at most once per round
    rr_pool_cap = pool;
  }
  if (arena > rr_arena_cap) {
    devFree(d_rr_arena);
    devAlloc(&d_rr_arena, arena);
    rr_arena_cap = arena;
  }
  if (!d_rr_pool) devAlloc(&d_rr_pool, 2);
  if (!d_rr_hist) {
    devAlloc(&d_rr_hist, (size_t)D + kHistExtra);
    devAlloc(&d_rr_cursor, (size_t)D);
  }
  if (segs > rr_seg_cap) {
    devFree(d_rr_seg);
    if (h_rr) cudaFreeHost(h_rr);
    h_rr = nullptr;
    devAlloc(&d_rr_seg, 2 * segs + 1);
    // pinned: the segment table going out, the round's counts coming back
    CK(cudaMallocHost(&h_rr, (2 * segs + 1 + (size_t)D + kHistExtra) * sizeof(uint32_t)));
    rr_seg_cap = segs;
  }
}

void Tracer::traceRounds() {
  if (fviews.size() != 1) throw std::invalid_argument("schedule_policy 5 traces one view per frame");
  if (cfg.num_ranks != 1) throw std::invalid_argument("schedule_policy 5 traces the whole image on one rank");
  const ViewDev& vw = hviews[0];
  const int64_t eyes = (int64_t)vw.image_w * vw.image_h * vw.spp;
  const int S = std::max(slotsFor(vw.ao_mode, vw.ao_samples, vw.ao_light_shadow), 1);
  // rays: the eye rays and, per hit, its shadow rays and a bounce ray; queue
  // entries: a few visits per ray.  Overflows retrace with twice the room.
  uint64_t pool = (uint64_t)eyes * (uint64_t)(2 + S), arena = 4 * pool;
  std::vector<int> sched;
  for (int attempt = 0; attempt < 4; ++attempt, pool *= 2, arena *= 2) {
    ensureRounds(pool, arena, 64);
    CK(cudaMemsetAsync(d_ctr, 0, sizeof(Counters), stream));
    CK(cudaMemsetAsync(d_image, 0, (size_t)frame_pixels * sizeof(float4), stream));
    CK(cudaMemsetAsync(d_rr_pool, 0, 2 * sizeof(unsigned long long), stream));
    RoundArgs a{};
    a.scene = sceneDev();
    a.boxes = d_dboxes;
    a.D = D;
    a.dnodes = reinterpret_cast<const float4*>(d_dnodes);
    a.dnode_count = dnode_count;
    a.rays = rr;
    a.pool_count = reinterpret_cast<uint32_t*>(d_rr_pool);
    a.pool_cap = (uint32_t)rr_pool_cap;
    a.id = -1;
    a.arena = d_rr_arena;
    a.seg = d_rr_seg;
    a.out = d_rr_out;
    a.out_count = reinterpret_cast<uint32_t*>(d_rr_pool) + 1;
    a.out_cap = (uint32_t)rr_pool_cap;
    a.image = d_image;
    a.view = vw;
    a.env = ShadeEnv{d_lights, (int)lights.size(), {cfg.ks[0], cfg.ks[1], cfg.ks[2]}, cfg.shininess, d_ctr};
    a.ctr = d_ctr;
    a.visits_shade = d_rr_pool + 1;
    a.hist = d_rr_hist;
    // the pool counter and the round's queue counter share d_rr_pool[0];
    // visits_shade lives in d_rr_pool[1]
    CK(cudaMemcpyAsync(a.pool_count, &eyes, sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(a.out_count, 0, sizeof(uint32_t), stream));
    kRoundEyes<<<(unsigned)((eyes + 255) / 256), 256, 0, stream>>>(a, eyes);
    launches += 1;
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> segs(D);
    std::vector<int64_t> counts(D, 0);
    uint64_t arena_fill = 0;
    bool overflow = false;
    uint32_t* h_seg = h_rr;
    // the round's queued rays into the arena; counts back to the host
    auto partition = [&]() -> bool {
      const int blocks = num_sms * 4;
      kRoundCount<<<blocks, 256, 0, stream>>>(d_rr_out, a.out_count, a.out_cap, d_rr_hist);
      kRoundOffsets<<<1, 1024, 0, stream>>>(d_rr_hist, D, (uint32_t)arena_fill, d_rr_cursor, a.out_count,
                                            a.out_cap, d_ctr);
      kRoundScatter<<<blocks, 256, 0, stream>>>(d_rr_out, d_rr_hist, D, d_rr_cursor, d_rr_arena,
                                                (uint32_t)rr_arena_cap, d_ctr);
      launches += 3;
      uint32_t* h_hist = h_rr + 2 * rr_seg_cap + 1;
      CK(cudaMemcpyAsync(h_hist, d_rr_hist, ((size_t)D + kHistExtra) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                         stream));
      CK(cudaStreamSynchronize(stream));
      d2h_bytes += ((size_t)D + kHistExtra) * sizeof(uint32_t);
      if (h_hist[D + 1]) return false;
      uint64_t off = arena_fill;
      for (int d = 0; d < D; ++d) {
        if (!h_hist[d]) continue;
        segs[d].push_back({(uint32_t)off, h_hist[d]});
        counts[d] += h_hist[d];
        off += h_hist[d];
      }
      arena_fill += h_hist[D];
      return true;
    };
    if (!partition()) overflow = true;
    sched.clear();
    const size_t log0 = dbg[{SPRAY_DBG_LOADS, 0}].size();
    while (!overflow) {
      const int id = loadAnyOnceNext(counts);
      if (id < 0) break;
      sched.push_back(id);
      load_pass = (int)sched.size();
      if (ooc) {
        int slot, evicted;
        const bool hit = lru.load(id, &slot, &evicted);
        logLoad(id, hit ? 1 : 0, hit ? -1 : evicted);
        if (!hit) {
          if (evicted >= 0) hdoms[evicted].resident = 0;
          loadDomain(id, slot, stream);
          DomainDev* sd = reinterpret_cast<DomainDev*>(h_stage);
          std::memcpy(sd, hdoms.data(), D * sizeof(DomainDev));
          CK(cudaMemcpyAsync(d_domains, sd, D * sizeof(DomainDev), cudaMemcpyHostToDevice, stream));
          h2d_bytes += D * sizeof(DomainDev);
        }
      } else {
        logLoad(id, 1, -1);  // in core every domain is resident
      }
      // the domain's segments
      std::vector<std::pair<uint32_t, uint32_t>>& sg = segs[id];
      const int nseg = (int)sg.size();
      if ((uint64_t)nseg > rr_seg_cap) {
        CK(cudaStreamSynchronize(stream));  // h_rr is about to be replaced
        ensureRounds(rr_pool_cap, rr_arena_cap, std::max<uint64_t>(nseg, 2 * rr_seg_cap));
        h_seg = h_rr;
      }
      uint32_t run = 0;
      for (int k = 0; k < nseg; ++k) {
        h_seg[k] = sg[k].first;
        h_seg[nseg + k] = run;
        run += sg[k].second;
      }
      h_seg[2 * nseg] = run;
      CK(cudaMemcpyAsync(d_rr_seg, h_seg, (2 * (size_t)nseg + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice,
                         stream));
      h2d_bytes += (2 * (size_t)nseg + 1) * sizeof(uint32_t);
      sg.clear();
      counts[id] = 0;
      a.id = id;
      a.nseg = nseg;
      a.scene = sceneDev();
      const int blocks = (int)std::min<int64_t>((run + 127) / 128, (int64_t)num_sms * 16);
      cudaEvent_t t0 = poolEvent(), t1 = poolEvent();
      record(t0);
      kRoundRays<<<std::max(blocks, 1), 128, 0, stream>>>(a);
      record(t1);
      trace_events.push_back({t0, t1});
      launches += 1;
      if (!partition()) overflow = true;
    }
    if (!overflow) {
      rounds = (int64_t)sched.size();
      unsigned long long vs = 0;
      CK(cudaMemcpy(&vs, d_rr_pool + 1, sizeof(vs), cudaMemcpyDeviceToHost));
      visits_shade = (int64_t)vs;
      CK(cudaMemcpyAsync(&d_ctr->rays_primary, &eyes, sizeof(eyes), cudaMemcpyHostToDevice, stream));
      return;
    }
    // retrace: the load log, loads and copies of the failed attempt are dropped
    dbg[{SPRAY_DBG_LOADS, 0}].resize(log0);
    domain_loads = 0;
  }
  throw OverflowError("the round loop's ray pool or queue arena could not be grown enough");
}

}  // namespace spray
