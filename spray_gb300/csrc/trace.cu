// Closest-hit and occlusion traversal of per-domain queues, and closest-hit
// resolution across the domains a ray visited.
//
// Replaces Scene::intersect / Scene::occluded (src/render/scene.inl:189-209),
// which SpRay calls once per (ray, domain) queue entry with tnear = 1e-3 and
// tfar = infinity.  Here persistent warps pull 32 entries at a time from the
// domain-partitioned queue; each thread walks the entry's domain BVH (4-wide
// nodes, conservative box test) and tests triangles with the watertight test.
// A closest hit is folded into the ray's packed (t | triangle) key with a
// 64-bit atomicMin, so the winner does not depend on the order in which the
// domains were visited.
#include "kernels.cuh"
#include "spray_math.cuh"
#include "traverse.cuh"

#ifndef SPRAY_TRACE_MIN_BLOCKS
#define SPRAY_TRACE_MIN_BLOCKS 4
#endif

namespace spray {

namespace {

// Any hit in (tnear, tfar), the same rounds.  Returns true when the walk has
// ended; *hit tells whether it ended on a hit.
__device__ __forceinline__ bool anyRound(Walk& w, int* stack, const TravRay& r, float tfar, bool* hit,
                                         Counters* ctr, unsigned long long& nnodes,
                                         unsigned long long& ntris) {
  *hit = false;
  for (int k = 0; w.cur >= 0; ++k) {
    if (k == kNodeBudget) return false;
    if (++w.steps > kMaxSteps) {
      raise(ctr, kErrTraversalBound);
      return true;
    }
    if ((unsigned)w.cur >= (unsigned)w.num_nodes) {
      raise(ctr, kErrBadNode);
      return true;
    }
    float tn[4];
    ++nnodes;
    // scalar: the packed test's registers make the refilling walk spill
    const int mask = testChildrenScalar(w.nodes, w.cur, r, kRayEpsilon, tfar, tn);
    const int4 ch = loadChildren(w.nodes, w.cur);
    // the last child hit continues the walk; the earlier ones are pushed
    // (the order a push of all of them and a pop would give)
    int next = kDone;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (!(mask & (1 << c))) continue;
      const int ref = childAt(ch, c);
      if (ref == kEmptyChild) continue;
      if (next != kDone) {
        if (w.sp == kStack) {
          raise(ctr, kErrTraversalBound);
          return true;
        }
        stack[w.sp++] = next;
      }
      next = ref;
    }
    w.cur = next != kDone ? next : (w.sp > 0 ? stack[--w.sp] : kDone);
  }
  if (w.cur == kDone) return true;
  const uint32_t v = ~(uint32_t)w.cur;
  const uint32_t first = v >> 3, cnt = (v & 7u) + 1u;
  if (first + cnt > (uint32_t)w.num_tris) {
    raise(ctr, kErrBadNode);
    return true;
  }
  ntris += cnt;
  for (uint32_t q = 0; q < cnt; ++q) {
    const float4* tp = w.tris + 3 * (size_t)(first + q);
    const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
    float t, u, vv;
    if (intersectTriangle(r.sh, r.org, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(cc.x, cc.y, cc.z),
                          kRayEpsilon, tfar, &t, &u, &vv)) {
      *hit = true;
      return true;
    }
  }
  w.cur = w.sp > 0 ? stack[--w.sp] : kDone;
  return w.cur == kDone;
}

__device__ __forceinline__ int findKey(const uint32_t* ks, int nkeys, uint32_t e) {
  // last key with ks[key] <= e (segments may be empty)
  int lo = 0, hi = nkeys - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ks[mid] <= e) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Key offsets and, out of core, the segment table into shared memory.
__device__ __forceinline__ void loadTables(const TraceArgs& a, uint32_t* skeys, uint32_t* sbeg,
                                           uint32_t* spre) {
  for (int k = threadIdx.x; k <= a.nkeys; k += blockDim.x) skeys[k] = a.key_start[k];
  if (a.nseg > 0) {
    for (int k = threadIdx.x; k < a.nseg; k += blockDim.x) sbeg[k] = a.seg_begin[k];
    for (int k = threadIdx.x; k <= a.nseg; k += blockDim.x) spre[k] = a.seg_prefix[k];
  }
  __syncthreads();
}

// Work index -> entry index (identity without a segment table).
__device__ __forceinline__ uint32_t entryOf(const TraceArgs& a, const uint32_t* sbeg,
                                            const uint32_t* spre, uint32_t w) {
  if (a.nseg == 0) return w;
  int lo = 0, hi = a.nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (spre[mid] <= w) lo = mid;
    else hi = mid - 1;
  }
  return sbeg[lo] + (w - spre[lo]);
}

}  // namespace

__device__ __forceinline__ uint32_t lanesBelow() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Adds a warp's in-place counts (nodes, triangles, hits) to the counters.
__device__ __forceinline__ void warpAddInplace(Counters* ctr, uint32_t n, uint32_t t, uint32_t h, int lane) {
  unsigned long long sn = n, st = t, sh = h;
  for (int o = 16; o; o >>= 1) {
    sn += __shfl_down_sync(0xffffffffu, sn, o);
    st += __shfl_down_sync(0xffffffffu, st, o);
    sh += __shfl_down_sync(0xffffffffu, sh, o);
  }
  if (lane == 0) {
    if (sn) atomicAdd(&ctr->nodes_inplace, sn);
    if (st) atomicAdd(&ctr->tris_inplace, st);
    if (sh) atomicAdd(&ctr->hits_inplace, sh);
  }
}

// Closest hits: warps take 32 consecutive entries at a time, so the lanes of a
// warp walk coherent rays (consecutive samples of the same domain queue).
// kPack: culled entries are dropped before the warp's lanes are assigned
// (in core); out of core the per-batch launches keep the 32 consecutive
// entries a warp takes (packing across culled entries measured slower there:
// the batches are small and the packed rays less coherent).
template <bool kPack>
__global__ void __launch_bounds__(256, SPRAY_TRACE_MIN_BLOCKS) kTraceClosest(TraceArgs a) {
  extern __shared__ uint32_t skeys[];
  const int D = a.scene.num_domains;
  uint32_t* sbeg = skeys + a.nkeys + 1;
  uint32_t* spre = sbeg + a.nseg;
  loadTables(a, skeys, sbeg, spre);
  uint32_t E0 = 0, E = *a.num_entries;
  if (a.nseg > 0) {
    E = spre[a.nseg];
  } else if (a.bucket >= 0 && E > 0) {
    E0 = skeys[a.bucket * D];
    E = a.bucket + 1 < kDepthBuckets ? skeys[(a.bucket + 1) * D] : skeys[a.nkeys];
  }
  const int lane = threadIdx.x & 31;
  // per-thread counts in 32 bits (entries are 32-bit indices); node and
  // triangle counts go to the global counters before they could wrap
  uint32_t visits = 0, culled = 0, nnodes = 0, ntris = 0;
  // out of core: nodes, triangles and hits of the entries traced in place
  uint32_t ipn = 0, ipt = 0, iph = 0;
  // Live entries waiting for a lane, in queue order: a warp takes 32 entries
  // at a time, drops the ones the culling test rejects (kPack) and traces 32
  // live ones together, so that culled entries leave no lane idle.
  __shared__ uint32_t sbuf[8][64];
  uint32_t* buf = sbuf[threadIdx.x >> 5];
  const uint32_t below = lanesBelow();
  int nbuf = 0;
  bool exhausted = false;
  while (true) {
    while (nbuf < 32 && !exhausted) {
      uint32_t base = 0;
      if (lane == 0) base = E0 + atomicAdd(a.work, 32u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= E) {
        exhausted = true;
        break;
      }
      if (base + 32u >= E) exhausted = true;
      const uint32_t w = base + lane;
      bool live = false;
      uint32_t ce = 0;
      if (w < E) {
        ce = entryOf(a, sbeg, spre, w);
        live = true;
        if (kPack && a.cull) {
          const uint2 ent = a.entries[ce];
          const uint64_t cur = *((volatile uint64_t*)&a.ray_key[ent.x & kRayIdMask]);
          if (cur != kNoHit && __uint_as_float(ent.y) > hitKeyT(cur)) {
            a.rec_key[ce] = kNoHit;
            ++culled;
            live = false;
          }
        }
      }
      const uint32_t lm = __ballot_sync(0xffffffffu, live);
      if (live) buf[nbuf + __popc(lm & below)] = ce;
      nbuf += __popc(lm);
      __syncwarp();
    }
    if (nbuf == 0) break;
    const int take = min(nbuf, 32), rest = nbuf - take;
    const bool has = lane < take;
    const uint32_t mine = has ? buf[lane] : 0u;
    const uint32_t moved = lane < rest ? buf[take + lane] : 0u;
    __syncwarp();
    if (lane < rest) buf[lane] = moved;
    __syncwarp();
    nbuf = rest;
    if (!has) continue;
    const uint32_t e = mine;
    const uint2 ent = a.entries[e];
    const uint32_t ray = ent.x & kRayIdMask;
    const float tdom = __uint_as_float(ent.y);
    const int d = findKey(skeys, a.nkeys, e) % D;
    const DomainDev dom = a.scene.domains[d];
    uint64_t best_key = kNoHit;
    float best_t = __int_as_float(0x7f800000);
    if (a.cull) {
      uint64_t cur = *((volatile uint64_t*)&a.ray_key[ray]);
      if (cur != kNoHit) {
        best_key = cur;
        best_t = hitKeyT(cur);
        if (tdom > best_t) {
          a.rec_key[e] = kNoHit;
          ++culled;
          continue;
        }
      }
    }
    ++visits;
    const float4 o = a.rays.org[ray], dd = a.rays.dir[ray];
    TravRay r = makeTravRay(v3(o.x, o.y, o.z), v3(dd.x, dd.y, dd.z));
    uint32_t prim = 0;
    float u = 0.f, v = 0.f;
    const uint32_t n0 = nnodes, t0 = ntris;
    const bool hit = traverseClosest(a.scene, dom, r, best_key, best_t, prim, u, v, a.ctr, nnodes, ntris);
    if (!kPack && dom.resident == 2) {
      ipn += nnodes - n0;
      ipt += ntris - t0;
      iph += hit ? 1u : 0u;
    }
    if (hit && kPack) {
      // in core the winner's colour and normal are interpolated by kResolve:
      // the record keeps the barycentrics
      atomicMin((unsigned long long*)&a.ray_key[ray], (unsigned long long)best_key);
      a.rec_key[e] = best_key;
      a.rec_attr[e] = make_float4(u, v, 0.f, 0.f);
    } else if (hit) {
      // out of core the domain may leave the cache before resolve: interpolate now
      atomicMin((unsigned long long*)&a.ray_key[ray], (unsigned long long)best_key);
      const DomArrays g = domArrays(a.scene, dom);
      const uint32_t* f = g.faces + 3 * (size_t)prim;
      const uint32_t i0 = f[0], i1 = f[1], i2 = f[2];
      uint32_t col = interpolateColor(g.colors[i0], g.colors[i1], g.colors[i2], u, v);
      const float* nb = g.normals;
      V3 ns = interpolateNormal(v3(nb[3 * (size_t)i0], nb[3 * (size_t)i0 + 1], nb[3 * (size_t)i0 + 2]),
                                v3(nb[3 * (size_t)i1], nb[3 * (size_t)i1 + 1], nb[3 * (size_t)i1 + 2]),
                                v3(nb[3 * (size_t)i2], nb[3 * (size_t)i2 + 1], nb[3 * (size_t)i2 + 2]),
                                u, v);
      a.rec_key[e] = best_key;
      a.rec_attr[e] = make_float4(ns.x, ns.y, ns.z, __uint_as_float(col));
    } else {
      a.rec_key[e] = kNoHit;
    }
    if ((nnodes | ntris) & 0x80000000u) {
      atomicAdd(&a.ctr->nodes_radiance, (unsigned long long)nnodes);
      atomicAdd(&a.ctr->tris_radiance, (unsigned long long)ntris);
      nnodes = ntris = 0;
    }
    if (!kPack && ((ipn | ipt) & 0x80000000u)) {
      atomicAdd(&a.ctr->nodes_inplace, (unsigned long long)ipn);
      atomicAdd(&a.ctr->tris_inplace, (unsigned long long)ipt);
      ipn = ipt = 0;
    }
  }
  unsigned long long sv = visits, sc = culled, sn = nnodes, st = ntris;
  for (int o = 16; o; o >>= 1) {
    sv += __shfl_down_sync(0xffffffffu, sv, o);
    sc += __shfl_down_sync(0xffffffffu, sc, o);
    sn += __shfl_down_sync(0xffffffffu, sn, o);
    st += __shfl_down_sync(0xffffffffu, st, o);
  }
  if (lane == 0) {
    if (sv) atomicAdd(&a.ctr->visits_radiance, sv);
    if (sc) atomicAdd(&a.ctr->visits_culled, sc);
    if (sn) atomicAdd(&a.ctr->nodes_radiance, sn);
    if (st) atomicAdd(&a.ctr->tris_radiance, st);
  }
  if (!kPack) warpAddInplace(a.ctr, ipn, ipt, iph, lane);
}

void launchTraceClosest(cudaStream_t s, const TraceArgs& a, int nblocks) {
  size_t smem = (size_t)(a.nkeys + 2 + 2 * a.nseg) * 4;
  if (a.nseg == 0) kTraceClosest<true><<<nblocks, 256, smem, s>>>(a);
  else kTraceClosest<false><<<nblocks, 256, smem, s>>>(a);
}

// Domains whose first global face resolve keeps in shared memory for the
// winner's domain search (more domains search the device table).
constexpr int kResolveSmemDomains = 4096;

// The entry that holds a ray's final key publishes its colour and normal:
// recorded by the trace out of core (kInterp false), interpolated here from
// the recorded barycentrics in core (TriMeshBuffer::updateIntersection,
// src/render/trimesh_buffer.cc:328-360).
template <bool kInterp>
__global__ void kResolve(TraceArgs a, float4* hit_ns) {
  __shared__ uint32_t sprim[kInterp ? kResolveSmemDomains : 1];
  const int D = a.scene.num_domains;
  const bool stab = kInterp && D <= kResolveSmemDomains;
  if (stab)
    for (int k = threadIdx.x; k < D; k += blockDim.x) sprim[k] = a.scene.domains[k].gprim_base;
  if (kInterp) __syncthreads();
  const uint32_t E = *a.num_entries;
  // four entries per thread per step, their loads in flight together
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e0 < E; e0 += 4 * stride) {
    uint64_t k[4];
    uint32_t ray[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint64_t e = e0 + q * stride;
      k[q] = e < E ? a.rec_key[e] : kNoHit;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) ray[q] = k[q] != kNoHit ? a.entries[e0 + q * stride].x & kRayIdMask : 0u;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (k[q] == kNoHit || a.ray_key[ray[q]] != k[q]) continue;
      const float4 rec = a.rec_attr[e0 + q * stride];
      if (!kInterp) {
        hit_ns[ray[q]] = rec;
        continue;
      }
      // the winner's domain: the last whose first global face is <= the hit's
      const uint32_t gprim = (uint32_t)k[q];
      int lo = 0, hi = D - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((stab ? sprim[mid] : a.scene.domains[mid].gprim_base) <= gprim) lo = mid;
        else hi = mid - 1;
      }
      const DomainDev dom = a.scene.domains[lo];
      const DomArrays g = domArrays(a.scene, dom);
      const uint32_t* f = g.faces + 3 * (size_t)(gprim - dom.gprim_base);
      const uint32_t i0 = f[0], i1 = f[1], i2 = f[2];
      const float u = rec.x, v = rec.y;
      const uint32_t col = interpolateColor(g.colors[i0], g.colors[i1], g.colors[i2], u, v);
      const float* nb = g.normals;
      const V3 ns = interpolateNormal(v3(nb[3 * (size_t)i0], nb[3 * (size_t)i0 + 1], nb[3 * (size_t)i0 + 2]),
                                      v3(nb[3 * (size_t)i1], nb[3 * (size_t)i1 + 1], nb[3 * (size_t)i1 + 2]),
                                      v3(nb[3 * (size_t)i2], nb[3 * (size_t)i2 + 1], nb[3 * (size_t)i2 + 2]),
                                      u, v);
      hit_ns[ray[q]] = make_float4(ns.x, ns.y, ns.z, __uint_as_float(col));
    }
  }
}

void launchResolve(cudaStream_t s, const TraceArgs& a, float4* hit_ns, int nblocks, bool interpolate) {
  if (interpolate) kResolve<true><<<nblocks, 256, 0, s>>>(a, hit_ns);
  else kResolve<false><<<nblocks, 256, 0, s>>>(a, hit_ns);
}

// Occlusion with persistent, refilling warps: each round, the lanes whose
// entry has ended take the next entries (one warp-aggregated atomic), then
// every busy lane advances its walk by one while-while round.  Used for AO
// frames, whose short bounded rays end early and unevenly; path-traced frames
// use kTraceOccludedBatch (measured faster there).
// kOoc: out-of-core batch launch, which also counts the work of domains traced
// in place from host memory (the in-core launch leaves that out).
template <bool kOoc>
__global__ void __launch_bounds__(256, SPRAY_TRACE_MIN_BLOCKS) kTraceOccluded(TraceArgs a) {
  extern __shared__ uint32_t skeys[];
  const int D = a.scene.num_domains;
  uint32_t* sbeg = skeys + a.nkeys + 1;
  uint32_t* spre = sbeg + a.nseg;
  loadTables(a, skeys, sbeg, spre);
  const uint32_t E = a.nseg > 0 ? spre[a.nseg] : *a.num_entries;
  const int lane = threadIdx.x & 31;
  const uint32_t below = lanesBelow();
  unsigned long long visits = 0, nnodes = 0, ntris = 0, ipn = 0, ipt = 0;
  int stack[kStack];
  Walk w{};
  TravRay r{};
  float tfar = 0.0f;
  uint32_t ray = 0;
  bool has = false, exhausted = false, inplace = false;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, !has);
    if (idle && !exhausted) {
      const uint32_t need = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(a.work, need);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + need >= E) exhausted = true;
      const uint32_t wi = base + __popc(idle & below);
      if (!has && wi < E) {
        const uint32_t e = entryOf(a, sbeg, spre, wi);
        ray = a.entries[e].x & kRayIdMask;
        if (!*((volatile uint8_t*)&a.sh.occluded[ray])) {
          const int d = findKey(skeys, a.nkeys, e) % D;
          ++visits;
          const float4 hp = a.sh.hitpos[ray / a.slots];
          const float4 dd = a.sh.dir[ray];
          r = makeTravRay(v3(hp.x, hp.y, hp.z), v3(dd.x, dd.y, dd.z));
          tfar = dd.w;
          w = startWalk(a.scene, a.scene.domains[d]);
          inplace = kOoc && a.scene.domains[d].resident == 2;
          has = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, has)) {
      if (exhausted) break;
      continue;
    }
    bool hit = false;
    const unsigned long long n0 = kOoc ? nnodes : 0ull, t0 = kOoc ? ntris : 0ull;
    if (has && anyRound(w, stack, r, tfar, &hit, a.ctr, nnodes, ntris)) {
      has = false;
      if (hit) a.sh.occluded[ray] = 1;
    }
    if (kOoc && inplace) {
      ipn += nnodes - n0;
      ipt += ntris - t0;
    }
  }
  for (int o = 16; o; o >>= 1) {
    visits += __shfl_down_sync(0xffffffffu, visits, o);
    nnodes += __shfl_down_sync(0xffffffffu, nnodes, o);
    ntris += __shfl_down_sync(0xffffffffu, ntris, o);
    if (kOoc) {
      ipn += __shfl_down_sync(0xffffffffu, ipn, o);
      ipt += __shfl_down_sync(0xffffffffu, ipt, o);
    }
  }
  if (lane == 0) {
    if (visits) atomicAdd(&a.ctr->visits_shadow, visits);
    if (nnodes) atomicAdd(&a.ctr->nodes_shadow, nnodes);
    if (ntris) atomicAdd(&a.ctr->tris_shadow, ntris);
    if (kOoc && ipn) atomicAdd(&a.ctr->nodes_inplace, ipn);
    if (kOoc && ipt) atomicAdd(&a.ctr->tris_inplace, ipt);
  }
}

// Occlusion in batches: a warp takes 32 entries at a time, drops those whose
// shadow ray is already occluded, queues the rest in a per-warp FIFO (queue
// order kept) and walks 32 of them together, each lane to the end of its walk.
template <bool kOoc>
__global__ void __launch_bounds__(256, SPRAY_TRACE_MIN_BLOCKS) kTraceOccludedBatch(TraceArgs a) {
  extern __shared__ uint32_t skeys[];
  const int D = a.scene.num_domains;
  uint32_t* sbeg = skeys + a.nkeys + 1;
  uint32_t* spre = sbeg + a.nseg;
  loadTables(a, skeys, sbeg, spre);
  const uint32_t E = a.nseg > 0 ? spre[a.nseg] : *a.num_entries;
  const int lane = threadIdx.x & 31;
  const uint32_t below = lanesBelow();
  __shared__ uint32_t sbuf[8][64];
  uint32_t* buf = sbuf[threadIdx.x >> 5];
  uint32_t visits = 0, nnodes = 0, ntris = 0, ipn = 0, ipt = 0;
  int nbuf = 0;
  bool exhausted = false;
  while (true) {
    while (nbuf < 32 && !exhausted) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(a.work, 32u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= E) {
        exhausted = true;
        break;
      }
      if (base + 32u >= E) exhausted = true;
      const uint32_t wi = base + lane;
      bool live = false;
      uint32_t ce = 0;
      if (wi < E) {
        ce = entryOf(a, sbeg, spre, wi);
        live = !*((volatile uint8_t*)&a.sh.occluded[a.entries[ce].x & kRayIdMask]);
      }
      const uint32_t lm = __ballot_sync(0xffffffffu, live);
      if (live) buf[nbuf + __popc(lm & below)] = ce;
      nbuf += __popc(lm);
      __syncwarp();
    }
    if (nbuf == 0) break;
    const int take = min(nbuf, 32), rest = nbuf - take;
    const bool has = lane < take;
    const uint32_t mine = has ? buf[lane] : 0u;
    const uint32_t moved = lane < rest ? buf[take + lane] : 0u;
    __syncwarp();
    if (lane < rest) buf[lane] = moved;
    __syncwarp();
    nbuf = rest;
    if (!has) continue;
    const uint32_t e = mine;
    const uint32_t ray = a.entries[e].x & kRayIdMask;
    if (*((volatile uint8_t*)&a.sh.occluded[ray])) continue;
    const int d = findKey(skeys, a.nkeys, e) % D;
    ++visits;
    const float4 hp = a.sh.hitpos[ray / a.slots];
    const float4 dd = a.sh.dir[ray];
    const TravRay r = makeTravRay(v3(hp.x, hp.y, hp.z), v3(dd.x, dd.y, dd.z));
    const uint32_t n0 = nnodes, t0 = ntris;
    if (traverseAny(a.scene, a.scene.domains[d], r, dd.w, a.ctr, nnodes, ntris)) a.sh.occluded[ray] = 1;
    if (kOoc && a.scene.domains[d].resident == 2) {
      ipn += nnodes - n0;
      ipt += ntris - t0;
    }
    if ((nnodes | ntris) & 0x80000000u) {
      atomicAdd(&a.ctr->nodes_shadow, (unsigned long long)nnodes);
      atomicAdd(&a.ctr->tris_shadow, (unsigned long long)ntris);
      nnodes = ntris = 0;
    }
    if (kOoc && ((ipn | ipt) & 0x80000000u)) {
      atomicAdd(&a.ctr->nodes_inplace, (unsigned long long)ipn);
      atomicAdd(&a.ctr->tris_inplace, (unsigned long long)ipt);
      ipn = ipt = 0;
    }
  }
  unsigned long long sv = visits, sn = nnodes, st = ntris;
  for (int o = 16; o; o >>= 1) {
    sv += __shfl_down_sync(0xffffffffu, sv, o);
    sn += __shfl_down_sync(0xffffffffu, sn, o);
    st += __shfl_down_sync(0xffffffffu, st, o);
  }
  if (lane == 0) {
    if (sv) atomicAdd(&a.ctr->visits_shadow, sv);
    if (sn) atomicAdd(&a.ctr->nodes_shadow, sn);
    if (st) atomicAdd(&a.ctr->tris_shadow, st);
  }
  if (kOoc) warpAddInplace(a.ctr, ipn, ipt, 0u, lane);
}

void launchTraceOccluded(cudaStream_t s, const TraceArgs& a, int nblocks) {
  size_t smem = (size_t)(a.nkeys + 2 + 2 * a.nseg) * 4;
  const bool ooc = a.nseg > 0;
  if (a.refill) {
    if (ooc) kTraceOccluded<true><<<nblocks, 256, smem, s>>>(a);
    else kTraceOccluded<false><<<nblocks, 256, smem, s>>>(a);
  } else {
    if (ooc) kTraceOccludedBatch<true><<<nblocks, 256, smem, s>>>(a);
    else kTraceOccludedBatch<false><<<nblocks, 256, smem, s>>>(a);
  }
}

// One block per listed domain; the same cull test as kTraceClosest.  The
// entries are taken in rounds of 8 per thread; with a cap, the block stops
// after the round in which its counts settle the caller's questions (over the
// cap; with shadows, also one live shadow entry).  Culled radiance entries of
// the rounds counted get rec_key = kNoHit; a domain whose counting stopped
// early has live entries and is traced, which writes every entry's record.
__device__ __forceinline__ uint32_t blockSum(uint32_t v, uint32_t* ws) {
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  uint32_t t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
  return t;
}

__global__ void __launch_bounds__(256) kCountLive(LiveArgs a) {
  __shared__ uint32_t ws[8];
  const int d = a.domains[blockIdx.x];
  const uint32_t round = 8 * blockDim.x;
  uint32_t nr = 0, ns = 0;  // block totals of the rounds counted
  bool stop = false;
  for (int b = a.rbucket0; a.rentries && b < a.rbucket0 + a.rbuckets && !stop; ++b) {
    const uint32_t e0 = a.rkey_start[b * a.D + d], e1 = a.rkey_start[b * a.D + d + 1];
    for (uint32_t r0 = e0; r0 < e1 && !stop; r0 += round) {
      uint32_t c = 0;
      const uint32_t r1 = min(e1, r0 + round);
      for (uint32_t e = r0 + threadIdx.x; e < r1; e += blockDim.x) {
        const uint2 ent = a.rentries[e];
        bool live = true;
        if (a.cull) {
          const uint64_t cur = a.ray_key[ent.x & kRayIdMask];
          live = !(cur != kNoHit && __uint_as_float(ent.y) > hitKeyT(cur));
        }
        if (live) ++c;
        else a.rec_key[e] = kNoHit;
      }
      nr += blockSum(c, ws);
      stop = a.cap && nr > a.cap;
    }
  }
  if (a.sentries) {
    const uint32_t e0 = a.skey_start[d], e1 = a.skey_start[d + 1];
    stop = false;
    for (uint32_t r0 = e0; r0 < e1 && !stop; r0 += round) {
      uint32_t c = 0;
      const uint32_t r1 = min(e1, r0 + round);
      for (uint32_t e = r0 + threadIdx.x; e < r1; e += blockDim.x)
        if (!a.occluded[a.sentries[e].x & kRayIdMask]) ++c;
      ns += blockSum(c, ws);
      stop = a.cap && ns > 0 && nr + ns > a.cap;
    }
  }
  if (threadIdx.x == 0) {
    a.live[d] = nr;
    a.live[a.D + d] = ns;
  }
}

void launchCountLive(cudaStream_t s, const LiveArgs& a) {
  if (a.ndomains > 0) kCountLive<<<a.ndomains, 256, 0, s>>>(a);
}

}  // namespace spray
