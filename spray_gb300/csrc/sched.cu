// Primary-ray generation, the speculative scheduler (ray -> per-domain
// queues), stable stream compaction and the domain scores.
#include <algorithm>
#include <cfloat>
#include <stdexcept>

#include "domain_walk.cuh"
#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {

__device__ __forceinline__ uint32_t laneMaskLt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t warpExclusiveScan(uint32_t v, uint32_t* total) {
  const int lane = threadIdx.x & 31;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// ---------------------------------------------------------------- primary rays
// Eye rays of SpRay's Tracer::genSingleEyes / genMultiEyes
// (src/ooc/ooc_tracer.inl:84-172) with Camera::generateRay
// (src/render/camera.h:173-209): u = x / W, v = y / H, jitter drawn from a
// sampler seeded with the tile-local sample id when pixel_samples > 1.
//
// With eye culling (cull.live set), a sample whose pixel lies in a screen bin
// that no domain box's projection touches is a miss without a domain list (the
// exact slab test of every domain fails for it): its record is not written,
// live[i] = 0, and a compaction of `live` makes the alive list.  It still
// counts as a primary ray.
__global__ void kGenPrimary(const ViewDev* __restrict__ views, const TileDev* __restrict__ tiles, int ntiles,
                            int64_t nsamples, RayBuf rays, uint32_t* alive_list, uint32_t* alive_count,
                            EyeCull cull, Counters* ctr) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    if (!cull.live) *alive_count = (uint32_t)nsamples;
    atomicAdd(&ctr->rays_primary, (unsigned long long)nsamples);
  }
  if (i >= nsamples) return;
  // last tile with sample_base <= i
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].sample_base <= i) lo = mid;
    else hi = mid - 1;
  }
  const TileDev tl = tiles[lo];
  const ViewDev& vw = views[tl.view];
  const CameraDev& cam = vw.cam;
  const int spp = tl.spp;
  int32_t bufid = (int32_t)(i - tl.sample_base);
  int32_t lp = spp > 1 ? bufid / spp : bufid;
  int x = tl.x + lp % tl.w;
  int y = tl.y + lp / tl.w;
  if (cull.live) {
    const int bin = vw.bin_base + (y >> cull.bin_shift) * vw.bins_x + (x >> cull.bin_shift);
    const bool live = cull.bin_start[bin] != cull.bin_start[bin + 1];
    cull.live[i] = live;
    if (!live) return;
  }
  float fx = (float)x, fy = (float)y;
  if (spp > 1) {
    uint32_t st = rngSeed(bufid);
    fx = (float)x + rngNext(st);
    fy = (float)y + rngNext(st);
  }
  const V3 d = cameraRay(cam, fx, fy);
  rays.org[i] = make_float4(cam.pos[0], cam.pos[1], cam.pos[2], 0.f);
  rays.dir[i] = make_float4(d.x, d.y, d.z, 0.f);
  rays.pixid[i] = y * vw.image_w + x;
  rays.samid[i] = bufid;
  rays.view[i] = (uint16_t)tl.view;
  if (!cull.live) alive_list[i] = (uint32_t)i;
}

// The culled eye rays of a wave: its samples less the live ones the
// compaction kept (one thread; a counter per culled warp would serialise
// hundreds of thousands of atomics on one address).
__global__ void kCountCulled(const uint32_t* alive_count, int64_t nsamples, Counters* ctr) {
  ctr->eyes_culled += (unsigned long long)(nsamples - (int64_t)*alive_count);
}

void launchCountCulled(cudaStream_t s, const uint32_t* alive_count, int64_t nsamples, Counters* ctr) {
  kCountCulled<<<1, 1, 0, s>>>(alive_count, nsamples, ctr);
}

void launchGenPrimary(cudaStream_t s, const ViewDev* views, const TileDev* tiles, int ntiles, int64_t nsamples,
                      RayBuf rays, uint32_t* alive_list, uint32_t* alive_count, const EyeCull& cull,
                      Counters* ctr) {
  int threads = 256;
  int64_t blocks = (nsamples + threads - 1) / threads;
  if (blocks < 1) blocks = 1;
  kGenPrimary<<<(unsigned)blocks, threads, 0, s>>>(views, tiles, ntiles, nsamples, rays, alive_list, alive_count,
                                                   cull, ctr);
}

// ---------------------------------------------------------------- schedule
// Pass 1: per ray, the slab test against every domain AABB with t0 = 1e-3 and
// t1 = the ray's end (infinity for every ray of the reference), sorted by
// (t, id) (src/render/rays.h:71-79).  Shadow rays start with the domain that
// spawned them, then list the other domains with their index in the full
// sorted list as depth (ooc_isector.h:147-174).  Lists go to an arena, the
// per-(key, warp) histogram to global memory.
__device__ __forceinline__ bool fitsList(int cnt, int j) { return j < cnt; }

// kMinBlocks 6 caps the kernel at 40 registers (a few spills) so that six
// blocks fit an SM when shared memory allows; with larger domain tables
// shared memory holds fewer blocks and the variant for five (46 registers,
// no spills) runs instead.  kSharedTables: the domain boxes and the domain
// hierarchy are staged in shared memory (small tables); otherwise they are
// read through the read-only cache, which leaves the shared memory to the
// per-warp histograms (512 domains: 34 KB of tables per block would hold the
// kernel at two blocks per SM).
template <int kMinBlocks, bool kSharedTables>
__global__ void __launch_bounds__(kSchedThreads, kMinBlocks) kSchedLists(SchedArgs a,
                                                             const DomainDev* __restrict__ doms,
                                                             int D, int nkeys, int nwarps) {
  extern __shared__ uint32_t smem[];
  const int NN = a.dnode_count;
  const int table_words = kSharedTables ? 32 * NN + 6 * D : 0;
  float4* stage_node = reinterpret_cast<float4*>(smem);  // 8 float4 per hierarchy node (BvhNode4)
  float* stage_box = reinterpret_cast<float*>(smem + 32 * NN);
  const float4* snode = kSharedTables ? stage_node : reinterpret_cast<const float4*>(a.dnodes);
  const float* sbox = kSharedTables ? stage_box : a.dboxes;
  uint32_t* hist = smem + table_words;  // per warp: nkeys 16-bit counters, packed in pairs
  const int hwords = (nkeys + 1) >> 1;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (kSharedTables) {
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
      for (int c = 0; c < 3; ++c) {
        stage_box[6 * d + c] = doms[d].bmin[c];
        stage_box[6 * d + 3 + c] = doms[d].bmax[c];
      }
    }
    for (int k = threadIdx.x; k < 8 * NN; k += blockDim.x)
      stage_node[k] = reinterpret_cast<const float4*>(a.dnodes)[k];
  }
  uint32_t* h = hist + (size_t)wib * hwords;
  __syncthreads();
  const uint32_t n = *a.count;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  const int nch = chunksFor(n, a.nchunks, nwarps);
  const uint64_t csize = chunkSize(n, nch);
  // chunks round-robin over the warps; a chunk's counts fit 16 bits (csize < 2^16)
  for (int ch = gw; ch < nch; ch += nwarps) {
  const uint64_t r0 = min((uint64_t)n, (uint64_t)ch * csize);
  const uint64_t r1 = min((uint64_t)n, r0 + csize);
  if (!a.defer_hist) {
    for (int k = lane; k < hwords; k += 32) h[k] = 0;
    __syncwarp();
  }
  // the next group's ray ids load while this group is scheduled
  uint32_t nrid = r0 + lane < r1 ? a.list[r0 + lane] : 0u;
  for (uint64_t base = r0; base < r1; base += 32) {
    const uint64_t i = base + lane;
    const bool active = i < r1;
    const uint32_t rid_cur = nrid;
    nrid = base + 32 + lane < r1 ? a.list[base + 32 + lane] : 0u;
    float lt[kMaxList];
    uint32_t ld[kMaxList];
    int cnt = 0;
    int origin = -1;
    bool origin_in_list = false;
    float origin_t = 0.f;
    if (active) {
      const uint32_t rid = rid_cur;
      V3 org, dir;
      float t1 = INFINITY;
      if (!a.shadow) {
        float4 o = a.rays.org[rid], d4 = a.rays.dir[rid];
        org = v3(o.x, o.y, o.z);
        dir = v3(d4.x, d4.y, d4.z);
        a.ray_key[rid] = kNoHit;
      } else {
        float4 hp = a.sh.hitpos[rid / a.slots];
        float4 d4 = a.sh.dir[rid];
        org = v3(hp.x, hp.y, hp.z);
        origin = __float_as_int(hp.w);
        dir = v3(d4.x, d4.y, d4.z);
        t1 = d4.w;
        a.sh.occluded[rid] = 0;
      }
      V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
      // exact slab test of domain d, kept in (t, id) order
      auto consider = [&](int d) {
        float t;
        if (!slabTest(&sbox[6 * d], &sbox[6 * d + 3], org, inv, kRayEpsilon, t1, &t)) return;
        if (cnt == kMaxList) {
          atomicAdd(&a.ctr->list_overflows, 1ull);
          if (lt[kMaxList - 1] < t || (lt[kMaxList - 1] == t && (int)ld[kMaxList - 1] < d)) return;
          --cnt;
        }
        int j = cnt;
        while (j > 0 && (lt[j - 1] > t || (lt[j - 1] == t && (int)ld[j - 1] > d))) {
          lt[j] = lt[j - 1];
          ld[j] = ld[j - 1];
          --j;
        }
        lt[j] = t;
        ld[j] = (uint32_t)d;
        ++cnt;
      };
      if (a.bin_start) {
        // primary rays: the domains whose projected box covers this pixel's bin
        const int pid = a.rays.pixid[rid];
        const ViewDev& vw = a.views[a.rays.view[rid]];
        const int bx = (pid % vw.image_w) >> a.bin_shift, by = (pid / vw.image_w) >> a.bin_shift;
        const int bin = vw.bin_base + by * vw.bins_x + bx;
        const uint32_t c0 = a.bin_start[bin], c1 = a.bin_start[bin + 1];
        for (uint32_t c = c0; c < c1; ++c) consider((int)a.bin_ids[c]);
      } else if (NN == 0) {
        for (int d = 0; d < D; ++d) consider(d);
      } else {
        // conservative descent of the 4-wide domain hierarchy, exact slab
        // test at the leaves (descendDomains)
        descendDomains(snode, NN, org, inv, t1, consider, a.ctr);
      }
      if (a.shadow) {
        for (int j = 0; j < cnt; ++j)
          if ((int)ld[j] == origin) {
            origin_in_list = true;
            origin_t = lt[j];
          }
      }
    }
    // entries this lane emits
    uint32_t nemit = 0;
    if (active) nemit = a.shadow ? (uint32_t)(cnt + 1 - (origin_in_list ? 1 : 0)) : (uint32_t)cnt;
    uint32_t total;
    uint32_t pos = warpExclusiveScan(nemit, &total);
    unsigned long long wbase = 0;
    if (lane == 0 && total) wbase = atomicAdd(a.arena_top, (unsigned long long)total);
    wbase = __shfl_sync(0xffffffffu, wbase, 0);
    bool fits = wbase + total <= a.arena_cap;
    if (!fits && lane == 0 && total) atomicAdd(&a.ctr->arena_overflows, 1ull);
    if (active) {
      a.list_off[i] = (uint32_t)(wbase + pos);
      a.list_cnt[i] = fits ? nemit : 0u;
      if (fits) {
        uint2* out = a.arena + wbase + pos;
        int o = 0;
        if (a.shadow) {
          out[o++] = make_uint2((uint32_t)origin | (1u << 31), __float_as_uint(origin_t));
          uint32_t key = (uint32_t)origin;
          if (!a.defer_hist) atomicAdd(&h[key >> 1], 1u << ((key & 1u) << 4));
        }
        for (int j = 0; j < cnt; ++j) {
          uint32_t d = ld[j];
          if (a.shadow && (int)d == origin) continue;
          out[o++] = make_uint2(d | ((uint32_t)j << 16), __float_as_uint(lt[j]));
          uint32_t key = a.order_by_depth ? (uint32_t)(min(j, kDepthBuckets - 1) * D) + d : d;
          if (!a.defer_hist) atomicAdd(&h[key >> 1], 1u << ((key & 1u) << 4));
        }
      }
    }
    if (a.want_stats) {
      // DomainStats counts, one global atomic per distinct (domain, depth) of the warp
      for (int j = 0; j < kMaxList; ++j) {
        const bool has = active && fitsList(cnt, j) && j < a.list_size &&
                         !(a.shadow && (int)ld[j] == origin);
        if (!__any_sync(0xffffffffu, has)) break;
        const uint32_t key = has ? ld[j] * (uint32_t)a.list_size + (uint32_t)j : 0xffffffffu;
        const uint32_t m = __match_any_sync(0xffffffffu, key);
        if (has && (__ffs(m) - 1) == lane)
          atomicAdd((unsigned long long*)&a.dstats[key], (unsigned long long)__popc(m));
      }
    }
  }
  __syncwarp();
  if (!a.defer_hist) {
    for (int k = lane; k < nkeys; k += 32) a.hist[(size_t)ch * nkeys + k] = (h[k >> 1] >> ((k & 1) << 4)) & 0xffffu;
    __syncwarp();
  }
  }
}

// Pass 2: exclusive scan of the histogram in key-major order (every chunk of
// key 0, then every chunk of key 1, ...).  The table is stored chunk-major,
// hist[chunk * nkeys + key], so that passes 1 and 3 move a chunk's counters as
// one contiguous row.  The chunks are cut into G groups: (a) per group and key
// the column sum; (b) per key the exclusive scan of its G group sums, and in
// the block that finishes last the scan of the key totals; (c) per group and
// key the running offsets, written back in place.  scan_tmp holds the group
// sums [G][nkeys], the key bases [nkeys] and a ticket word.
constexpr int kScanMaxGroups = 1024;

__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[32];
  __shared__ uint32_t ws_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t wt;
  uint32_t x = warpExclusiveScan(v, &wt);
  if (lane == 31) ws[w] = wt;
  __syncthreads();
  if (w == 0) {
    uint32_t y = lane < nw ? ws[lane] : 0u, t2;
    uint32_t e = warpExclusiveScan(y, &t2);
    if (lane < nw) ws[lane] = e;
    if (lane == 0) ws_total = t2;
  }
  __syncthreads();
  uint32_t r = x + ws[w];
  *total = ws_total;
  __syncthreads();
  return r;
}

// (a) grid (groups, key tiles): one thread per (group, key)
__global__ void kHistColumns(const uint32_t* __restrict__ hist, const uint32_t* count, int nchunks, int nwarps,
                             int nkeys, uint32_t* __restrict__ colsum, uint32_t* ticket) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *ticket = 0u;
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= nkeys) return;
  const int nch = chunksFor(*count, nchunks, nwarps);
  const int per = (nch + (int)gridDim.x - 1) / (int)gridDim.x;
  const int c0 = min(nch, (int)blockIdx.x * per), c1 = min(nch, c0 + per);
  uint32_t s = 0;
#pragma unroll 8
  for (int c = c0; c < c1; ++c) s += hist[(size_t)c * nkeys + k];
  colsum[(size_t)blockIdx.x * nkeys + k] = s;
}

// (b) one block per 32 keys: lane = key, the 32 warps split the groups
__global__ void __launch_bounds__(1024) kHistKeyScan(uint32_t* colsum, int G, int nkeys, uint32_t* keybase,
                                                     uint32_t* ticket, uint32_t* key_start,
                                                     uint32_t* num_entries, unsigned long long entry_cap,
                                                     Counters* ctr) {
  __shared__ uint32_t wsum[32][33];
  __shared__ int is_last;
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const int gper = (G + 31) / 32;
  const int g0 = min(G, w * gper), g1 = min(G, g0 + gper);
  uint32_t s = 0;
  if (k < nkeys) {
#pragma unroll 8
    for (int g = g0; g < g1; ++g) s += colsum[(size_t)g * nkeys + k];
  }
  wsum[w][lane] = s;
  __syncthreads();
  if (w == 0) {
    uint32_t run = 0;
    for (int j = 0; j < 32; ++j) {
      const uint32_t v = wsum[j][lane];
      wsum[j][lane] = run;
      run += v;
    }
    if (k < nkeys) keybase[k] = run;  // the key's total until the last block scans them
  }
  __syncthreads();
  if (k < nkeys) {
    uint32_t run = wsum[w][lane];
    int g = g0;
    for (; g + 8 <= g1; g += 8) {
      uint32_t v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = colsum[(size_t)(g + j) * nkeys + k];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        colsum[(size_t)(g + j) * nkeys + k] = run;
        run += v[j];
      }
    }
    for (; g < g1; ++g) {
      const uint32_t v = colsum[(size_t)g * nkeys + k];
      colsum[(size_t)g * nkeys + k] = run;
      run += v;
    }
  }
  // the last block to finish scans the key totals
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nkeys; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < nkeys ? __ldcg(keybase + i) : 0u;
    uint32_t tot;
    const uint32_t e = blockExclusiveScan(v, &tot);
    if (i < nkeys) {
      keybase[i] = carry + e;
      key_start[i] = carry + e;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    uint32_t total = carry;
    key_start[nkeys] = total;
    if (total > entry_cap) {
      atomicAdd(&ctr->entry_overflows, 1ull);
      total = 0;
    }
    *num_entries = total;
  }
}

// (c) grid (groups, key tiles): the running offsets of each chunk
__global__ void kHistApply(uint32_t* __restrict__ hist, const uint32_t* count, int nchunks, int nwarps,
                           int nkeys, const uint32_t* __restrict__ colsum,
                           const uint32_t* __restrict__ keybase) {
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= nkeys) return;
  const int nch = chunksFor(*count, nchunks, nwarps);
  const int per = (nch + (int)gridDim.x - 1) / (int)gridDim.x;
  const int c0 = min(nch, (int)blockIdx.x * per), c1 = min(nch, c0 + per);
  uint32_t run = keybase[k] + colsum[(size_t)blockIdx.x * nkeys + k];
  // rows in batches of 8, every load issued before the batch's stores (the
  // compiler cannot prove that a row's store and the next row's load differ)
  int c = c0;
  for (; c + 8 <= c1; c += 8) {
    uint32_t v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = hist[(size_t)(c + j) * nkeys + k];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      hist[(size_t)(c + j) * nkeys + k] = run;
      run += v[j];
    }
  }
  for (; c < c1; ++c) {
    const uint32_t v = hist[(size_t)c * nkeys + k];
    hist[(size_t)c * nkeys + k] = run;
    run += v;
  }
}

// Groups of the scan for this table and workspace (0 when the workspace
// cannot hold even one group).
static int scanGroups(int nkeys, int nch, size_t scan_words) {
  if (scan_words < (size_t)2 * nkeys + 1) return 0;
  const size_t fit = (scan_words - nkeys - 1) / nkeys;
  const int g = (int)std::min<size_t>(std::min<size_t>(fit, kScanMaxGroups), (size_t)std::max(nch, 1));
  const int per = (std::max(nch, 1) + g - 1) / g;
  return (std::max(nch, 1) + per - 1) / per;
}

size_t scanTmpWords(int nkeys, int nchunks) {
  const size_t g = (size_t)std::min(std::max(nchunks, 1), kScanMaxGroups);
  return g * nkeys + nkeys + 1;
}

// Pass 3: stable scatter.  Each warp re-reads its rays in order, flattens
// their entries into shared memory and ranks them per key with match_any, so
// every domain's queue keeps ray order (the order a single-threaded
// Isector::isectAll pushes them, ooc_isector.h:133-144).  The flattened entries
// of 32 rays pass through a window of kScatterWindow entries per warp, in
// order, so that the staging buffer stays small and many warps fit per SM.
constexpr int kScatterWindow = 256;

__global__ void __launch_bounds__(128) kSchedScatter(SchedArgs a, int D, int nkeys, int nwarps) {
  extern __shared__ uint32_t smem[];
  const int wpb = blockDim.x >> 5;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* running = smem + (size_t)wib * nkeys;
  uint32_t* fkey = smem + (size_t)wpb * nkeys + (size_t)wib * kScatterWindow * 3;
  uint32_t* fw0 = fkey + kScatterWindow;
  uint32_t* fw1 = fw0 + kScatterWindow;
  const int gw = blockIdx.x * wpb + wib;
  if (gw >= nwarps) return;
  const uint32_t n = *a.count;
  if (*a.num_entries == 0) return;
  const int nch = chunksFor(n, a.nchunks, nwarps);
  const uint64_t csize = chunkSize(n, nch);
  const uint32_t lt = laneMaskLt();
  for (int ch = gw; ch < nch; ch += nwarps) {
  const uint64_t r0 = min((uint64_t)n, (uint64_t)ch * csize);
  const uint64_t r1 = min((uint64_t)n, r0 + csize);
  if (r0 >= r1) break;
  __syncwarp();
  for (int k = lane; k < nkeys; k += 32) running[k] = a.hist[(size_t)ch * nkeys + k];
  __syncwarp();
  // the next group's list sizes, offsets, ray ids and predictions load while
  // this group is flattened and ranked
  uint32_t ncnt = 0, noff = 0, nrid = 0, np = 0xffu;
  if (r0 + lane < r1) {
    ncnt = a.list_cnt[r0 + lane];
    noff = a.list_off[r0 + lane];
    nrid = a.list[r0 + lane];
    if (a.pred) np = a.pred[r0 + lane];
  }
  for (uint64_t base = r0; base < r1; base += 32) {
    const uint32_t cnt = ncnt, off = noff, rid = nrid, p = np;
    {
      const uint64_t j = base + 32 + lane;
      ncnt = 0;
      noff = 0;
      nrid = 0;
      np = 0xffu;
      if (j < r1) {
        ncnt = a.list_cnt[j];
        noff = a.list_off[j];
        nrid = a.list[j];
        if (a.pred) np = a.pred[j];
      }
    }
    uint32_t total;
    const uint32_t pos = warpExclusiveScan(cnt, &total);
    for (uint32_t w0 = 0; w0 < total; w0 += kScatterWindow) {
      const uint32_t w1 = min(total, w0 + (uint32_t)kScatterWindow);
      // this lane's entries that fall in [w0, w1)
      const uint32_t lo = max(pos, w0), hi = min(pos + cnt, w1);
      for (uint32_t f = lo; f < hi; ++f) {
        const uint2 e = a.arena[off + (f - pos)];
        const uint32_t d = e.x & 0xffffu;
        const uint32_t depth = (e.x >> 16) & 0x7fffu;
        const uint32_t origin = e.x >> 31;
        const uint32_t key = a.order_by_depth ? bucketOf(depth, p) * D + d : d;
        const uint32_t pos = min(depth, 31u);
        // the key (< 2^18) with the list position in the top byte
        fkey[f - w0] = key | (pos << 24);
        fw0[f - w0] = (a.pack_depth ? (rid & ((1u << kPackedIdBits) - 1u)) | (pos << kPackedIdBits)
                                    : (rid & kRayIdMask)) |
                      (origin << 31);
        fw1[f - w0] = e.y;
      }
      __syncwarp();
      for (uint32_t s = w0; s < w1; s += 32) {
        const uint32_t e = s + lane;
        const bool valid = e < w1;
        const uint32_t kp = valid ? fkey[e - w0] : 0xffffffffu;
        const uint32_t key = valid ? (kp & 0xffffffu) : 0xffffffffu;
        const uint32_t m = __match_any_sync(0xffffffffu, key);
        uint32_t rank = 0;
        if (valid) rank = running[key] + __popc(m & lt);
        __syncwarp();
        if (valid && (__ffs(m) - 1) == lane) running[key] += __popc(m);
        __syncwarp();
        if (valid && rank < a.entry_cap) {
          a.entries[rank] = make_uint2(fw0[e - w0], fw1[e - w0]);
          if (a.dbg_depth) a.dbg_depth[rank] = (uint8_t)(kp >> 24);
        }
      }
      __syncwarp();
    }
  }
  }
}

// Deferred histogram: the per-(key, warp) counts of kSchedLists, recounted
// from the per-ray lists with the same ray partition, after the learned
// proposal has set each ray's bucket boundary.
__global__ void __launch_bounds__(128) kSchedHist(SchedArgs a, int D, int nkeys, int nwarps) {
  extern __shared__ uint32_t smem[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* h = smem + (size_t)wib * nkeys;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  if (gw >= nwarps) return;
  const uint32_t n = *a.count;
  const int nch = chunksFor(n, a.nchunks, nwarps);
  const uint64_t csize = chunkSize(n, nch);
  for (int ch = gw; ch < nch; ch += nwarps) {
  for (int k = lane; k < nkeys; k += 32) h[k] = 0;
  __syncwarp();
  const uint64_t r0 = min((uint64_t)n, (uint64_t)ch * csize);
  const uint64_t r1 = min((uint64_t)n, r0 + csize);
  for (uint64_t i = r0 + lane; i < r1; i += 32) {
    const uint32_t cnt = a.list_cnt[i], off = a.list_off[i];
    const uint32_t p = a.pred ? a.pred[i] : 0xffu;
    for (uint32_t j = 0; j < cnt; ++j) {
      const uint2 e = a.arena[off + j];
      const uint32_t d = e.x & 0xffffu;
      const uint32_t depth = (e.x >> 16) & 0x7fffu;
      const uint32_t key = a.order_by_depth ? bucketOf(depth, p) * D + d : d;
      atomicAdd(&h[key], 1u);
    }
  }
  __syncwarp();
  for (int k = lane; k < nkeys; k += 32) a.hist[(size_t)ch * nkeys + k] = h[k];
  __syncwarp();
  }
}

// Domain tables up to this size are staged in shared memory by kSchedLists.
constexpr size_t kSharedTableBytes = 8192;

static bool tablesShared(int D, int dnode_count) {
  return (size_t)dnode_count * 128 + (size_t)6 * D * 4 <= kSharedTableBytes;
}

static size_t listsSmem(int D, int nkeys, int dnode_count, bool shared_tables) {
  return (shared_tables ? (size_t)dnode_count * 128 + (size_t)6 * D * 4 : 0) +
         (size_t)(kSchedThreads / 32) * ((nkeys + 1) / 2) * 4;
}

// Resident blocks per SM of a kSchedLists variant with this shared memory.
template <int kMinBlocks, bool kShared>
static int listsOccupancy(size_t smem) {
  cudaFuncSetAttribute(kSchedLists<kMinBlocks, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kSchedLists<kMinBlocks, kShared>, kSchedThreads,
                                                    smem) != cudaSuccess ||
      bps < 1)
    bps = 1;
  return bps;
}

// The register-capped variant when shared memory lets six blocks share an SM.
template <bool kShared>
static bool listsCapped(size_t smem) { return listsOccupancy<6, kShared>(smem) >= 6; }

template <bool kShared>
static int blocksFor(size_t smem) {
  return listsCapped<kShared>(smem) ? listsOccupancy<6, kShared>(smem) : listsOccupancy<5, kShared>(smem);
}

int schedBlocksPerSm(int D, int nkeys, int dnode_count) {
  const bool shared = tablesShared(D, dnode_count);
  const size_t smem = listsSmem(D, nkeys, dnode_count, shared);
  return shared ? blocksFor<true>(smem) : blocksFor<false>(smem);
}

template <bool kShared>
static void launchLists(cudaStream_t s, const SchedArgs& a, const DomainDev* domains, int D, int nwarps,
                        int nblocks) {
  const int nkeys = a.order_by_depth ? kDepthBuckets * D : D;
  // the variant is chosen for the allocation's key count (4 D), as in schedBlocksPerSm
  const bool capped = listsCapped<kShared>(listsSmem(D, kDepthBuckets * D, a.dnode_count, kShared));
  const size_t smem1 = listsSmem(D, nkeys, a.dnode_count, kShared);
  if (capped) {
    cudaFuncSetAttribute(kSchedLists<6, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    kSchedLists<6, kShared><<<nblocks, kSchedThreads, smem1, s>>>(a, domains, D, nkeys, nwarps);
  } else {
    cudaFuncSetAttribute(kSchedLists<5, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    kSchedLists<5, kShared><<<nblocks, kSchedThreads, smem1, s>>>(a, domains, D, nkeys, nwarps);
  }
}

void launchSchedLists(cudaStream_t s, const SchedArgs& a, const DomainDev* domains, int D, int nwarps,
                      int nblocks) {
  // without a box array (the allocation-free entry point) the tables are staged
  if (!a.dboxes || tablesShared(D, a.dnode_count)) launchLists<true>(s, a, domains, D, nwarps, nblocks);
  else launchLists<false>(s, a, domains, D, nwarps, nblocks);
}

void launchSchedule(cudaStream_t s, const SchedArgs& a, const DomainDev* domains, int D, int nwarps,
                    int nblocks, uint32_t* scan_tmp, size_t scan_words) {
  launchSchedLists(s, a, domains, D, nwarps, nblocks);
  launchSchedPartition(s, a, D, nwarps, scan_tmp, scan_words);
}

void launchSchedPartition(cudaStream_t s, const SchedArgs& a, int D, int nwarps, uint32_t* scan_tmp,
                          size_t scan_words) {
  const int nkeys = a.order_by_depth ? kDepthBuckets * D : D;
  if (a.defer_hist) {
    const size_t smemh = (size_t)4 * nkeys * 4;
    cudaFuncSetAttribute(kSchedHist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemh);
    kSchedHist<<<(nwarps + 3) / 4, 128, smemh, s>>>(a, D, nkeys, nwarps);
  }
  const int nch = a.nchunks;
  const int G = scanGroups(nkeys, nch, scan_words);
  if (G < 1) throw std::runtime_error("histogram scan workspace too small");
  uint32_t* colsum = scan_tmp;
  uint32_t* keybase = scan_tmp + (size_t)G * nkeys;
  uint32_t* ticket = keybase + nkeys;
  const int bt = std::min(256, (nkeys + 31) / 32 * 32);
  const dim3 grid(G, (nkeys + bt - 1) / bt);
  kHistColumns<<<grid, bt, 0, s>>>(a.hist, a.count, nch, nwarps, nkeys, colsum, ticket);
  kHistKeyScan<<<(nkeys + 31) / 32, 1024, 0, s>>>(colsum, G, nkeys, keybase, ticket, a.key_start,
                                                   a.num_entries, a.entry_cap, a.ctr);
  kHistApply<<<grid, bt, 0, s>>>(a.hist, a.count, nch, nwarps, nkeys, colsum, keybase);
  const int wpb = 4;
  size_t smem3 = (size_t)wpb * nkeys * 4 + (size_t)wpb * kScatterWindow * 3 * 4;
  cudaFuncSetAttribute(kSchedScatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3);
  kSchedScatter<<<(nwarps + wpb - 1) / wpb, wpb * 32, smem3, s>>>(a, D, nkeys, nwarps);
}

// ---------------------------------------------------------------- compaction
// Elements per block of the compaction passes: whole groups of n_mul (the
// shadow slots of one alive ray), so that a block's range is the range of
// alive rays a shader block with the same grid covered (kShade's block counts).
__host__ __device__ __forceinline__ uint64_t compactPer(uint64_t units, uint32_t n_mul, uint32_t blocks) {
  return (units + blocks - 1) / blocks * n_mul;
}

__global__ void kCompactCount(const uint8_t* __restrict__ flag, const uint32_t* n_dev,
                              uint32_t n_mul, uint64_t n_host, uint32_t* block_tmp,
                              const uint32_t* __restrict__ src) {
  __shared__ uint32_t ws[32];
  const uint64_t n = n_dev ? (uint64_t)(*n_dev) * n_mul : n_host;
  const uint64_t per = compactPer(n_dev ? *n_dev : n_host, n_dev ? n_mul : 1u, gridDim.x);
  const uint64_t b0 = min(n, per * blockIdx.x), b1 = min(n, b0 + per);
  uint32_t c = 0;
  for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) c += flag[src ? src[i] : i] != 0;
  for (int o = 16; o; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0u;
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) block_tmp[blockIdx.x] = v;
  }
}

__global__ void __launch_bounds__(1024) kCompactScan(uint32_t* block_tmp, int nblocks,
                                                     uint32_t* count) {
  __shared__ uint32_t part[1024];
  const int per = (nblocks + 1023) / 1024;
  const int b0 = min(nblocks, per * (int)threadIdx.x), b1 = min(nblocks, b0 + per);
  uint32_t sum = 0;
  for (int i = b0; i < b1; ++i) sum += block_tmp[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
  for (int i = b0; i < b1; ++i) {
    uint32_t v = block_tmp[i];
    block_tmp[i] = run;
    run += v;
  }
  if (threadIdx.x == 1023) *count = part[1023];
}

// block_tmp holds each block's first output position, or with `count` set,
// each block's kept count: the block then adds the counts before its own and
// the last block writes the total to *count (no separate scan launch).
__global__ void kCompactWrite(const uint8_t* __restrict__ flag, const uint32_t* n_dev,
                              uint32_t n_mul, uint64_t n_host, const uint32_t* block_tmp,
                              uint32_t* list, int32_t* index_of, const uint32_t* __restrict__ src,
                              uint32_t* count = nullptr) {
  __shared__ uint32_t ws[33];
  const uint64_t n = n_dev ? (uint64_t)(*n_dev) * n_mul : n_host;
  const uint64_t per = compactPer(n_dev ? *n_dev : n_host, n_dev ? n_mul : 1u, gridDim.x);
  const uint64_t b0 = min(n, per * blockIdx.x), b1 = min(n, b0 + per);
  uint32_t base;
  if (count) {
    uint32_t sum = 0;
    for (uint32_t k = threadIdx.x; k < blockIdx.x; k += blockDim.x) sum += block_tmp[k];
    for (int o = 16; o; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = sum;
    __syncthreads();
    base = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) base += ws[k];
    __syncthreads();
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *count = base + block_tmp[blockIdx.x];
  } else {
    base = block_tmp[blockIdx.x];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t lt = laneMaskLt();
  // four elements per thread per round (element s + k * blockDim + thread:
  // order row k, warp, lane), so that a round's loads overlap and its two
  // barriers cover 4 x blockDim elements
  __shared__ uint32_t wk[4][8];
  for (uint64_t s = b0; s < b1; s += 4 * (uint64_t)blockDim.x) {
    uint32_t id[4], bal[4];
    bool f[4], valid[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t i = s + (uint64_t)k * blockDim.x + threadIdx.x;
      valid[k] = i < b1;
      id[k] = valid[k] ? (src ? src[i] : (uint32_t)i) : 0u;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      f[k] = valid[k] && flag[id[k]] != 0;
      bal[k] = __ballot_sync(0xffffffffu, f[k]);
      if (lane == 0) wk[k][w] = __popc(bal[k]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (int k = 0; k < 4; ++k)
        for (int q = 0; q < nw; ++q) {
          const uint32_t v = wk[k][q];
          wk[k][q] = run;
          run += v;
        }
      ws[32] = run;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!valid[k]) continue;
      if (f[k]) {
        const uint32_t p = base + wk[k][w] + __popc(bal[k] & lt);
        list[p] = id[k];
        if (index_of) index_of[id[k]] = (int32_t)p;
      } else if (index_of) {
        index_of[id[k]] = -1;
      }
    }
    base += ws[32];
    __syncthreads();
  }
}

void launchCompact(cudaStream_t s, const uint8_t* flag, const uint32_t* n_dev, uint32_t n_mul,
                   uint64_t n_host, uint32_t* list, uint32_t* count, int32_t* index_of,
                   uint32_t* block_tmp, int nblocks) {
  kCompactCount<<<nblocks, 256, 0, s>>>(flag, n_dev, n_mul, n_host, block_tmp, nullptr);
  kCompactScan<<<1, 1024, 0, s>>>(block_tmp, nblocks, count);
  kCompactWrite<<<nblocks, 256, 0, s>>>(flag, n_dev, n_mul, n_host, block_tmp, list, index_of, nullptr);
}

void launchCompactCounted(cudaStream_t s, const uint8_t* flag, const uint32_t* n_dev, uint32_t n_mul,
                          uint32_t* list, uint32_t* count, int32_t* index_of, const uint32_t* src,
                          uint32_t* block_tmp, int nblocks) {
  kCompactWrite<<<nblocks, 256, 0, s>>>(flag, n_dev, n_mul, 0, block_tmp, list, index_of, src, count);
}

void launchCompactList(cudaStream_t s, const uint32_t* src, const uint32_t* n_dev, const uint8_t* flag,
                       uint32_t* list, uint32_t* count, int32_t* index_of, uint32_t* block_tmp, int nblocks) {
  kCompactCount<<<nblocks, 256, 0, s>>>(flag, n_dev, 1, 0, block_tmp, src);
  kCompactScan<<<1, 1024, 0, s>>>(block_tmp, nblocks, count);
  kCompactWrite<<<nblocks, 256, 0, s>>>(flag, n_dev, 1, 0, block_tmp, list, index_of, src);
}

// ---------------------------------------------------------------- scores
// DomainStats::schedule (src/ooc/ooc_domain_stats.cc:60-111):
// score[d] = sum_k count[d][k] * (L - k), processed in descending score.  The
// reference sorts with an unstable sort; ties are ordered by domain id here.
__global__ void kScores(const long long* __restrict__ dstats, int D, int L, long long* scores,
                        int32_t* order) {
  extern __shared__ long long sc[];
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    long long v = 0;
    for (int k = 0; k < L; ++k) v += dstats[(size_t)d * L + k] * (long long)(L - k);
    sc[d] = v;
    scores[d] = v;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    long long v = sc[d];
    int rank = 0;
    for (int e = 0; e < D; ++e) rank += (sc[e] > v) || (sc[e] == v && e < d);
    order[rank] = d;
  }
}

void launchScores(cudaStream_t s, const long long* dstats, int ndomains, int list_size,
                  long long* scores, int32_t* order) {
  kScores<<<1, 1024, (size_t)ndomains * sizeof(long long), s>>>(dstats, ndomains, list_size, scores,
                                                               order);
}

}  // namespace spray
