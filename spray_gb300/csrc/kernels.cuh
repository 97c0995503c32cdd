// Device data layout and kernel launchers of the wavefront tracer.
//
// One frame is traced as a sequence of wavefronts ("waves").  A wave holds
// whole blocking tiles (src/render/tile.cc:317-391), so every sample keeps the
// tile-local id SpRay seeds its random streams with.  Per bounce a wave runs:
//   schedule  : slab test of every live ray against every domain AABB, sorted
//               (t, id) domain list, stable partition of the (ray, domain)
//               entries into per-domain queues        (ooc_isector.h:116-174)
//   trace     : closest hit of each entry in its domain's BVH, folded into a
//               per-ray packed 64-bit (t | triangle) atomicMin
//   resolve   : the entry that owns the minimum publishes colour and normal
//   shade     : AO / path-tracing shader spawns shadow rays and the bounce ray
//                                                     (ooc_shader_ao.h, ooc_shader_pt.h)
//   schedule + occlusion of the shadow rays, then retire into the image
//                                                     (ooc_tcontext.inl:123-135)
// Counts live in device memory so a bounce needs no host round trip.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bvh.h"
#include "spray_math.cuh"

namespace spray {

constexpr int kMaxList = 32;       // longest per-ray domain list handled
constexpr int kMaxEmit = kMaxList + 1;  // entries per ray: list plus a shadow ray's own domain
constexpr int kRayIdBits = 31;     // entry word 0: ray id | origin << 31
constexpr uint32_t kRayIdMask = (1u << kRayIdBits) - 1u;
// The allocation-free scheduler's entries keep the list position in bits
// 26..30 (ray id | position << 26 | origin << 31, ray ids below 2^26).
constexpr int kPackedIdBits = 26;
// Shadow rays one wavefront may hold (alive samples x slots).
constexpr int64_t kMaxWaveShadowRays = (int64_t)1 << 28;
constexpr int kMaxSlots = 64;      // shadow rays per hit
constexpr int kSchedThreads = 256;
constexpr int kDepthBuckets = 4;   // key = min(depth, 3) * D + domain when ordering by depth
constexpr int kDomainBvhMin = 16;     // domain counts from which the scheduler descends a hierarchy

struct DomainDev {
  float bmin[3], bmax[3];  // world AABB used by the scheduler
  int32_t node_base;       // first BVH node of the domain (in its cache slot)
  int32_t tri_base;        // first leaf-order triangle record
  uint32_t gprim_base;     // global number of the domain's face 0
  int32_t vert_base;       // first vertex (colours, normals)
  int32_t face_base;       // first index triple (original face order)
  int32_t bsdf;
  float bsdf_p[3];
  int32_t resident;        // 1: geometry in a device slot (the *_base offsets); 2: traced in
                           // place from pinned host memory (the src_* pointers); 0: neither
  int32_t num_nodes;       // BVH nodes of the domain
  int32_t num_tris;        // triangles of the domain
  // out of core: the domain's arrays in mapped pinned host memory, read over
  // the host link when the domain is traced in place
  const BvhNode4* src_nodes;
  const float4* src_tris;
  const uint32_t* src_faces;
  const uint32_t* src_colors;
  const float* src_normals;
};

// Bits of Counters::error_flags.
constexpr unsigned long long kErrGlassBothLobes = 1ull;  // glass hit needing two rays
constexpr unsigned long long kErrBadNode = 2ull;         // node or leaf index out of range
constexpr unsigned long long kErrTraversalBound = 4ull;  // traversal exceeded its step bound
constexpr unsigned long long kErrRetireContention = 8ull;  // an image addition lost its race too often

struct SceneDev {
  const DomainDev* domains;
  int32_t num_domains;
  const BvhNode4* nodes;
  const float4* tris;       // 3 float4 per triangle, v0.w = domain-local face id
  const uint32_t* faces;    // 3 per face
  const uint32_t* colors;   // per vertex
  const float* normals;     // 3 per vertex
};

// A domain's geometry, wherever it is: its device slot, or pinned host memory.
struct DomArrays {
  const BvhNode4* nodes;
  const float4* tris;        // 3 per triangle, leaf order
  const uint32_t* faces;     // 3 per face, original order; indices into colors / normals
  const uint32_t* colors;
  const float* normals;      // 3 per vertex
};

__device__ __forceinline__ DomArrays domArrays(const SceneDev& sc, const DomainDev& d) {
  DomArrays a;
  if (d.resident == 2) {
    a.nodes = d.src_nodes;
    a.tris = d.src_tris;
    a.faces = d.src_faces;
    a.colors = d.src_colors;
    a.normals = d.src_normals;
  } else {
    a.nodes = sc.nodes + d.node_base;
    a.tris = sc.tris + 3 * (size_t)d.tri_base;
    a.faces = sc.faces + 3 * (size_t)d.face_base;
    a.colors = sc.colors + d.vert_base;
    a.normals = sc.normals + 3 * (size_t)d.vert_base;
  }
  return a;
}

struct Counters {
  unsigned long long rays_primary;
  unsigned long long rays_shadow;
  unsigned long long rays_bounce;
  unsigned long long visits_radiance;
  unsigned long long visits_shadow;
  unsigned long long visits_culled;
  unsigned long long list_overflows;
  unsigned long long arena_overflows;
  unsigned long long entry_overflows;
  unsigned long long error_flags;
  unsigned long long nodes_radiance;  // BVH nodes fetched by closest-hit traversal
  unsigned long long tris_radiance;   // triangles tested by closest-hit traversal
  unsigned long long nodes_shadow;
  unsigned long long tris_shadow;
  // out of core: work done in domains traced in place from pinned host memory
  // (resident == 2), whose node, triangle and shading reads cross the host link
  unsigned long long nodes_inplace;
  unsigned long long tris_inplace;
  unsigned long long hits_inplace;    // closest hits whose faces, colours and normals were read there
  unsigned long long eyes_culled;     // primary rays resolved as misses by the screen bins
};

// Radiance rays of a wave, indexed by sample.
struct RayBuf {
  float4* org;
  float4* dir;
  float4* wgt;
  int32_t* pixid;   // pixel inside the sample's view (y * width + x)
  int32_t* samid;
  uint16_t* view;   // view of the sample
};

// Shadow rays of a bounce, indexed by alive_index * slots + slot.
struct ShadowBuf {
  float4* dir;       // xyz, w = tmax
  float4* wgt;       // xyz, w = 1 when the ray exists
  float4* hitpos;    // per alive ray: hit point, w = origin domain (as float bits)
  uint8_t* occluded;
};

struct CameraDev {
  float pos[3];
  float ll[3];   // lower-left corner of the image plane
  float wv[3];   // full-width vector
  float hv[3];   // full-height vector
  float image_w, image_h;
};

// Camera::generateRay (src/render/camera.h:173-209): the unit direction
// through image point (fx, fy), u = fx / W, v = fy / H.
__device__ __forceinline__ V3 cameraRay(const CameraDev& cam, float fx, float fy) {
  const float u = fx / cam.image_w;
  const float v = fy / cam.image_h;
  const V3 ll = v3(cam.ll[0], cam.ll[1], cam.ll[2]);
  const V3 wv = v3(cam.wv[0], cam.wv[1], cam.wv[2]);
  const V3 hv = v3(cam.hv[0], cam.hv[1], cam.hv[2]);
  const V3 pos = v3(cam.pos[0], cam.pos[1], cam.pos[2]);
  return normalize(((ll + u * wv) + v * hv) - pos);
}

struct TileDev {
  int32_t x, y, w, h;
  int64_t sample_base;  // first sample of the tile inside the wave
  int64_t pix_base;     // first pixel of the tile among the wave's pixels
  int32_t view;         // view the tile belongs to
  int32_t spp;          // samples per pixel of that view
};

// One view of a frame: camera, image and shader settings.  A frame may trace
// several views in the same wavefronts (multi-view batches); every sample
// carries its view.
struct ViewDev {
  CameraDev cam;
  int32_t image_w, image_h, spp;
  int32_t ao_mode, ao_samples, bounces, rr_depth, ao_light_shadow;
  float ao_max_distance;
  int64_t pixel_base;   // first pixel of the view in the frame's image buffer
  double scale;         // retire weight scale, 1 / spp
  int32_t bin_base;     // the view's first screen bin in the frame's bin table
  int32_t bins_x;       // screen bins per image row
};

// Scheduling of one ray set into per-domain queues.
struct SchedArgs {
  int shadow;                 // 0 radiance, 1 shadow rays
  const uint32_t* count;      // number of rays (device)
  const uint32_t* list;       // ray ids (sample for radiance, shadow id for shadow)
  RayBuf rays;                // radiance rays
  ShadowBuf sh;               // shadow rays
  int slots;                  // shadow slots per alive ray
  int order_by_depth;         // key = min(depth,3)*D + domain, else domain
  int list_size;              // SPRAY_RAY_DOMAIN_LIST_SIZE, for the domain statistics
  uint64_t* ray_key;          // radiance: reset to kNoHit per scheduled ray
  const BvhNode4* dnodes;     // 4-wide hierarchy over the domain boxes (null: test every domain)
  int dnode_count;
  const float* dboxes;        // domain boxes, 6 floats each (null: staged from the domain table)
  // primary rays: candidate domains per screen bin (null: not primary rays);
  // a ray's bins are those of its view (ViewDev::bin_base, bins_x)
  const uint32_t* bin_start;  // [all views' bins + 1]
  const uint16_t* bin_ids;
  const ViewDev* views;
  int bin_shift;
  // outputs
  uint2* arena;               // per-ray sorted (domain | depth << 16, tdom) lists
  unsigned long long* arena_top;
  unsigned long long arena_cap;
  uint32_t* list_off;         // per scheduled ray
  uint32_t* list_cnt;
  uint32_t* hist;             // [nchunks][nkeys]
  int nchunks;                // ray chunks, each with its own histogram column
  long long* dstats;          // [D][list_size] ray counts per (domain, depth)
  int want_stats;             // fill dstats (out-of-core order, debug hooks)
  uint2* entries;             // partitioned entries
  unsigned long long entry_cap;
  uint32_t* key_start;        // [nkeys + 1]
  uint32_t* num_entries;      // total entries (device)
  Counters* ctr;
  // learned order: per scheduled ray the predicted list position of its hit;
  // with order_by_depth the entries at or before it form bucket 0 and the
  // later ones buckets 1, 2, 3+ (null: bucket = list position, capped at 3)
  const uint8_t* pred;
  int defer_hist;             // kSchedLists leaves the histogram to the partition step
  int pack_depth;             // entries in the packed format (kPackedIdBits)
  uint8_t* dbg_depth;         // debug capture: list position of every entry (or null)
};

// Two fp32 values in one 64-bit register for Blackwell's packed arithmetic
// (sub.rn.f32x2, mul.rn.f32x2): each half is rounded exactly like the scalar
// instruction, so the box test below gives the same bits as scalar code.
__device__ __forceinline__ unsigned long long f2pack(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 f2unpack(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
// (a - b) * c per half
__device__ __forceinline__ float2 f2subMul(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long d, e;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(e) : "l"(d), "l"(c));
  return f2unpack(e);
}

// Rays per chunk of the scheduler: a multiple of 32 covering n rays in at
// most nchunks chunks (chunk c holds rays [c * size, (c + 1) * size)).
__host__ __device__ __forceinline__ uint64_t chunkSize(uint64_t n, int nchunks) {
  return (((n + (uint64_t)nchunks - 1) / (uint64_t)nchunks) + 31u) & ~(uint64_t)31u;
}

// Chunks in use for n rays: about kChunkRays rays each, at least one per
// scheduling warp and at most the nchunks rows the histogram holds, so that
// the histogram (rows x keys) shrinks with the wave.  Read from the device's
// ray count by every kernel of one schedule, so a captured frame adapts too.
constexpr uint64_t kChunkRays = 1024;
__host__ __device__ __forceinline__ int chunksFor(uint64_t n, int nchunks, int nwarps) {
  uint64_t want = (n + kChunkRays - 1) / kChunkRays;
  if (want < (uint64_t)nwarps) want = (uint64_t)nwarps;
  if (want > (uint64_t)nchunks) want = (uint64_t)nchunks;
  return want < 1 ? 1 : (int)want;
}

// Depth bucket of the entry at list position j (p = predicted position, 0xff none).
__host__ __device__ __forceinline__ uint32_t bucketOf(uint32_t j, uint32_t p) {
  if (p == 0xffu) return j < 3u ? j : 3u;
  if (j <= p) return 0u;
  return j - p < 3u ? j - p : 3u;
}

struct TraceArgs {
  SceneDev scene;
  const uint2* entries;
  const uint32_t* num_entries;
  const uint32_t* key_start;
  int nkeys;
  unsigned int* work;         // work-stealing counter (zeroed before launch)
  int bucket;                 // depth bucket to trace (-1 = every entry)
  const uint32_t* seg_begin;  // out of core: first entry of each segment to trace
  const uint32_t* seg_prefix; // exclusive prefix of the segment lengths (nseg + 1)
  int nseg;                   // 0 = no segment table
  RayBuf rays;
  ShadowBuf sh;
  int slots;
  uint64_t* ray_key;
  uint64_t* rec_key;          // per entry
  float4* rec_attr;           // per entry: Ns xyz, colour bits in w
  int cull;
  int refill;                 // occlusion: refilling walk (AO rays) instead of batches
  Counters* ctr;
};

struct ShadeArgs {
  SceneDev scene;
  const uint32_t* count;      // alive rays
  const uint32_t* list;       // alive samples
  RayBuf rays;                // rays of this bounce
  RayBuf next;                // bounce rays for the next depth
  uint8_t* next_flag;         // per sample
  const uint64_t* ray_key;
  float4* hit_ns;             // per sample: resolved Ns xyz, colour bits in w
  ShadowBuf sh;
  uint8_t* shadow_flag;       // per shadow id
  int slots;
  int depth;                  // actual depth of the rays being shaded
  // shader configuration: per view (AO or PT, samples, bounces, ...) and shared
  const ViewDev* views;
  float ks[3], shininess;
  const float* lights;        // 13 floats per light: type, pos, radiance, e1, e2
  int num_lights;
  Counters* ctr;
  // Optional (null: not written): per block, the shadow rays and the bounce
  // rays it emitted.  Block b shades alive rays [b * per, (b + 1) * per) with
  // per = ceil(alive / blocks), the ranges of the compaction passes launched
  // with as many blocks, which then need no count pass.
  uint32_t* blk_shadow;
  uint32_t* blk_next;
};

// ---------------------------------------------------------------- launchers
// Views (cameras) and tiles are read from device memory, so a captured frame
// follows camera changes.
// Screen bins for eye culling: pixel (x, y) of a view lies in bin
// view.bin_base + (y >> bin_shift) * view.bins_x + (x >> bin_shift), which
// lists the domains bin_start[b] .. bin_start[b + 1]; live (one byte per
// sample) receives 1 for the samples whose bin lists a domain.
// live == nullptr: no culling, every sample alive.
struct EyeCull {
  const uint32_t* bin_start = nullptr;
  int bin_shift = 0;
  uint8_t* live = nullptr;
};
void launchGenPrimary(cudaStream_t s, const ViewDev* views, const TileDev* tiles, int ntiles,
                      int64_t nsamples, RayBuf rays, uint32_t* alive_list, uint32_t* alive_count,
                      const EyeCull& cull, Counters* ctr);
// Adds nsamples - *alive_count to Counters::eyes_culled (after the live flags' compaction).
void launchCountCulled(cudaStream_t s, const uint32_t* alive_count, int64_t nsamples, Counters* ctr);
// scan_tmp holds scan_words words, at least scanTmpWords(nkeys, nchunks) for
// the fastest scan (fewer give a scan over fewer chunk groups).  Launches 5
// kernels.
void launchSchedule(cudaStream_t s, const SchedArgs& a, const DomainDev* domains, int ndomains,
                    int nwarps, int nblocks, uint32_t* scan_tmp, size_t scan_words);
// Workspace words of the histogram scan for nkeys keys and nchunks chunks.
size_t scanTmpWords(int nkeys, int nchunks);
// The two halves of launchSchedule: the per-ray domain lists (1 kernel), then
// the partition into queues (histogram when deferred, scan, scatter: 4 or 5).
void launchSchedLists(cudaStream_t s, const SchedArgs& a, const DomainDev* domains, int ndomains,
                      int nwarps, int nblocks);
void launchSchedPartition(cudaStream_t s, const SchedArgs& a, int ndomains, int nwarps,
                          uint32_t* scan_tmp, size_t scan_words);
// Resident blocks per SM of the scheduling kernel for this shared-memory use.
int schedBlocksPerSm(int D, int nkeys, int dnode_count);
void launchTraceClosest(cudaStream_t s, const TraceArgs& a, int nblocks);
// The winners' colour and normal into hit_ns: interpolated from the records'
// barycentrics after an in-core closest-hit launch (interpolate), copied from
// the records after out-of-core and domain-parallel launches.
void launchResolve(cudaStream_t s, const TraceArgs& a, float4* hit_ns, int nblocks, bool interpolate);
void launchTraceOccluded(cudaStream_t s, const TraceArgs& a, int nblocks);
void launchShade(cudaStream_t s, const ShadeArgs& a, int nblocks);
// Stable compaction of flag[i] != 0 for i < n (n from *n_dev or n_host when
// n_dev is null) into list, count and, optionally, index_of[i] (-1 if unset).
// The element count is (*n_dev) * n_mul when n_dev is set, else n_host.
void launchCompact(cudaStream_t s, const uint8_t* flag, const uint32_t* n_dev, uint32_t n_mul,
                   uint64_t n_host, uint32_t* list, uint32_t* count, int32_t* index_of,
                   uint32_t* block_tmp, int nblocks);
// Adds the unoccluded shadow rays of every pixel of a wave (npix pixels over
// ntiles tiles) to the frame image, samples of a pixel in order.
// Stable compaction of a list: keeps src[i] (i < *n_dev) where flag[src[i]] is
// set, in order, into list and count; index_of[src[i]] = new position or -1.
// list must not alias src.
void launchCompactList(cudaStream_t s, const uint32_t* src, const uint32_t* n_dev, const uint8_t* flag,
                       uint32_t* list, uint32_t* count, int32_t* index_of, uint32_t* block_tmp, int nblocks);
// The write pass of launchCompact / launchCompactList when block_tmp already
// holds each block's kept count (kShade's block counts): each block adds the
// counts before its own, the last writes *count.  One launch.
void launchCompactCounted(cudaStream_t s, const uint8_t* flag, const uint32_t* n_dev, uint32_t n_mul,
                          uint32_t* list, uint32_t* count, int32_t* index_of, const uint32_t* src,
                          uint32_t* block_tmp, int nblocks);
// Adds the unoccluded shadow rays of the alive list's samples (*count of them,
// shadow slot k of entry j at j * slots + k) to their pixels.
void launchRetire(cudaStream_t s, float4* image, const ViewDev* views, const uint32_t* list, const uint32_t* count,
                  const RayBuf& rays, const ShadowBuf& sh, const uint8_t* flag, int slots, int nblocks);
// Uploads the constant tables of the shader (once per device).
void initShadeTables();
void launchScores(cudaStream_t s, const long long* dstats, int ndomains, int list_size,
                  long long* scores, int32_t* order);
// Out of core: entries of each listed domain that are still live.  A radiance
// entry is dead when its ray already holds a hit nearer than the entry's
// domain (its record is then written as a miss, as the trace kernel would);
// a shadow entry is dead when its ray is already occluded.  live[d] counts
// radiance entries and live[D + d] shadow entries.  Either queue may be null.
struct LiveArgs {
  const uint2* rentries;
  const uint32_t* rkey_start;  // key = bucket * D + domain
  int rbucket0, rbuckets;      // the radiance buckets counted: [rbucket0, rbucket0 + rbuckets)
  const uint64_t* ray_key;
  uint64_t* rec_key;
  const uint2* sentries;
  const uint32_t* skey_start;
  const uint8_t* occluded;
  const int32_t* domains;  // the domains to count
  int ndomains;
  int D;
  int cull;
  uint32_t* live;
  // 0: exact counts.  Else a domain's counting may stop once its radiance
  // count exceeds `cap` and, with shadows, once radiance + shadow exceed it and
  // one live shadow entry was seen: the counts then read cap + 1 or more (the
  // caller only compares them with cap and with 0).
  uint32_t cap;
};
void launchCountLive(cudaStream_t s, const LiveArgs& a);

}  // namespace spray
