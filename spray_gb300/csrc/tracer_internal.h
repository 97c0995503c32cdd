// Internal host-side tracer object behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <list>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/spray_gpu.h"
#include "kernels.cuh"
#include "mlp.cuh"

namespace spray {

struct StateError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OverflowError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct IoError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define CK(x)                                                                               \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess)                                                                  \
      throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_) + " at " + __FILE__ + \
                      ":" + std::to_string(__LINE__));                                      \
  } while (0)

int fail(int code, const std::string& msg);
// Domain -> rank of SpRay's in-situ partition (insitu.cu).
std::vector<int> insituPartition(const float* bounds, int nd, int num_ranks);

struct HostTile {
  int x, y, w, h;
  int view = 0;
};

struct Wave {
  int first_tile;
  int num_tiles;
  int64_t samples;
  int64_t pixels;
};

// One view of a frame (multi-view batches trace several in the same wavefronts).
struct FrameView {
  CameraDev cam;
  int w, h, spp;
  int ao_mode, ao_samples, bounces, rr_depth, ao_light_shadow;
  float ao_max_distance;
};

// A domain prepared for the device: BVH, leaf-ordered triangles and the
// per-vertex shading data.
struct DomainPack {
  float bounds[6] = {0, 0, 0, 0, 0, 0};  // world AABB: min xyz, max xyz
  int32_t bsdf = 0;
  float bsdf_p[3] = {0, 0, 0};
  int64_t nv = 0, nf = 0;
  std::vector<BvhNode4> nodes;
  std::vector<float4> tris;
  std::vector<uint32_t> faces;
  std::vector<uint32_t> colors;
  std::vector<float> normals;
  int bvh_depth = 0;
  // triangles this domain numbers in the scene-wide triangle count (the hit
  // keys' primitive ids); -1: nf.  A domain another rank owns keeps its count
  // but no geometry, so every rank numbers triangles the same way.
  int64_t prim_count = -1;
};

// Device slots of the out-of-core domain cache, least recently used first.
// Device arrays of n elements (at least one), freed and nulled by devFree.
template <class T>
inline void devAlloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  CK(cudaMalloc((void**)p, n * sizeof(T)));
}
template <class T>
inline void devFree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// Ray pool of the non-speculative round loop (rounds.cu), one entry per ray.
struct RoundRays {
  float4* org;  // xyz; w = occlusion range of a shadow ray (infinite for radiance)
  float4* dir;  // xyz; w = entry distance of the domain after the current one
  float4* wgt;  // rgb; w = t of the nearest hit so far
  int4* meta;   // pixel, sample, depth | flags << 8, list position
  int4* hit;    // domain of the nearest hit, its triangle (domain-local), u, v bits
};

// LoadAnyOnceSched::scheduleImage on per-domain queue counts (rounds.cu):
// the domain to run next, -1 when every count is zero.
int loadAnyOnceNext(const std::vector<int64_t>& counts);

struct LruSlots {
  int capacity = 0;
  std::list<std::pair<int, int>> blocks;  // (slot, domain)
  std::map<int, std::list<std::pair<int, int>>::iterator> where;
  void init(int cap);
  // Returns true on a hit; on a miss `slot` is the slot to fill and `evicted`
  // the domain that lived there (-1 if the slot was free).
  bool load(int domain, int* slot, int* evicted);
};

// Normals, BVH and leaf-ordered triangles of one domain (TriMeshBuffer::load
// and its Embree build, src/render/trimesh_buffer.cc:117-326).
// Host preparation of one domain: checks, vertex normals, faces, colours and,
// with `bvh`, the BVH and leaf-ordered triangles (otherwise left empty for
// buildBvhsOnDevice).
void buildPack(const spray_gpu_domain& src, int d, DomainPack& p, bool bvh = true);
// The BVHs (nodes, leaf-ordered triangles, depth) of the domains `which` of
// `src`, built on the current device (bvh_build.cu).
void buildBvhsOnDevice(const spray_gpu_domain* src, const std::vector<int>& which, std::vector<DomainPack>& packs,
                       cudaStream_t stream, uint64_t batch_tris);
// Prepared-domain blobs: one file per domain holding everything buildPack
// makes, so that a scene is prepared once and loaded without rebuilding.
std::string domainBlobPath(const std::string& dir, int d);
void writeDomainBlob(const std::string& path, const DomainPack& p);
void readDomainBlob(const std::string& path, DomainPack* p);
void prepareScene(const spray_gpu_domain* domains, int nd, const std::string& dir);

std::vector<HostTile> makeTiles(int W, int H, int spp, int num_ranks, int rank, int64_t max_samples);
void computeVertexNormals(const float* v, int64_t nv, const uint32_t* f, int64_t nf, float* n);
CameraDev makeCamera(const float p[3], const float l[3], const float up[3], float vfov, int W, int H);

class Tracer {
 public:
  explicit Tracer(const spray_gpu_config& c);
  ~Tracer();
  void setScene(const spray_gpu_domain* doms, int nd, const spray_gpu_light* ls, int nl);
  // the same from blobs written by writeDomainBlob (no normal or BVH build)
  void setScenePrepared(const std::string& dir, int nd, const spray_gpu_light* ls, int nl);
  void setCamera(const float p[3], const float l[3], const float up[3], float vfov);
  void trace(float* out, bool out_is_device, spray_gpu_stats* st);
  // several views in one frame: images back to back in `out`, view order
  void traceViews(const spray_gpu_view* views, int n, float* out, bool out_is_device, spray_gpu_stats* st);
  int64_t debugCount(int what, int bounce) const;
  const std::vector<char>* debugData(int what, int bounce) const;
  const std::vector<char>* domainBvh(int what, int domain);
  // domain-parallel (in-situ) execution, before setScene (insitu.cu)
  void setInsitu(int num_ranks, int rank, const spray_gpu_reduce_ops* ops);

 private:
  int slots() const;
  int slotsFor(int ao_mode, int ao_samples, int ao_light_shadow) const;
  int maxBounces() const;
  int traceBlocks() const;
  void traceFrame(float* out, bool out_is_device, spray_gpu_stats* st);
  void planWaves();
  void ensureBuffers(int64_t nsamples);
  void freeScene();
  void freeBuffers();
  void traceWave(const Wave& w, bool capture);
  void traceWaveBatched(const Wave& w);
  void beginWave(const Wave& w);
  ShadeArgs shadeArgs(int b, int S);
  void schedule(bool shadow, int order_by_depth, uint32_t* count, uint32_t* list, int S,
                bool primary = false, bool into_shadow_queues = false, bool predicted = false);
  // learned domain-order proposal (schedule_policy 3)
  bool learned() const { return cfg.schedule_policy == 3; }
  // the non-speculative round loop (schedule_policy 5)
  bool rounded() const { return cfg.schedule_policy == 5; }
  void setupProposal();
  void freeProposal();
  mlp::ArenaSource arenaSource() const;
  mlp::Net proposalNet() const;
  void collectPairs();
  void predictDomainCounts(bool run_predict);
  void trainProposal();
  void buildScreenBins();
  void binView(const FrameView& f, std::vector<uint16_t>* lists, int bins_x) const;
  TraceArgs traceArgs(int order_by_depth, int S);
  SceneDev sceneDev() const;
  cudaEvent_t poolEvent();
  void captureRays(int b);
  void captureQueues(int what, int b, int order_by_depth);
  void captureScores(int b);
  void captureHits(int b);
  void captureShadows(int b, int S);
  void installScene(std::vector<DomainPack>& packs, const spray_gpu_light* ls, int nl);
  void setupOutOfCore(std::vector<DomainPack>& packs, int capacity, size_t max_nodes, size_t max_tris,
                      size_t max_verts, size_t slot_bytes);
  void loadDomain(int d, int slot, cudaStream_t s);
  void traceOutOfCore(bool shadow, const std::vector<int>& order, int S);
  // domain-parallel (in-situ) execution (insitu.cu)
  bool situ() const { return insitu_ranks > 1; }
  void traceOwned(bool shadow, int S);
  void reduceCall(bool keys, void* dev, int64_t n, size_t elem);
  char* reduceStage(size_t bytes);
  int insitu_ranks = 1, insitu_rank = 0;
  spray_gpu_reduce_ops reduce{};
  std::vector<int> owner;      // domain -> rank of the partition
  char* h_reduce = nullptr;    // pinned staging of the reductions
  size_t h_reduce_cap = 0;
  int64_t reduce_bytes = 0;    // bytes passed to the reductions during the frame
  // One pass over the domains for the radiance queues (buckets [rb_first,
  // rb_first + rb_count) of rbuckets) and/or the shadow queues; by_live orders
  // the domains by live entries, most first, instead of resident-first.
  void oocPass(bool with_radiance, bool with_shadow, int S, int rbuckets, int rb_first = 0,
               int rb_count = -1, bool by_live = false);
  std::vector<int> residentFirst(const std::vector<int>& order) const;
  std::vector<int> scoreOrder();
  // non-speculative round loop (schedule_policy 5, rounds.cu)
  void traceRounds();
  void ensureRounds(uint64_t pool, uint64_t arena, uint64_t segs);
  void freeRounds();
  RoundRays rr{};
  unsigned long long* d_rr_pool = nullptr;  // [0]: ray count | round queue count << 32, [1]: shading-only visits
  uint32_t* d_rr_arena = nullptr;           // queue entries (ray ids), grouped by domain per round
  uint2* d_rr_out = nullptr;                // the round's queued rays: (domain, ray)
  uint32_t* d_rr_hist = nullptr;            // per-domain counts of the round, total last
  uint32_t* d_rr_cursor = nullptr;
  uint32_t* d_rr_seg = nullptr;             // segment table of the round's domain
  uint32_t* h_rr = nullptr;                 // pinned: segment table, then the round's counts
  uint64_t rr_pool_cap = 0, rr_arena_cap = 0, rr_seg_cap = 0;
  int64_t rounds = 0, visits_shade = 0;

  spray_gpu_config cfg;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t cstream = nullptr;  // out-of-core domain copies, ahead of the traces
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> sched_events, trace_events, occl_events, copy_events;

  // scene
  bool has_scene = false, has_camera = false;
  int D = 0;
  int max_bvh_depth = 0;
  size_t total_tris = 0;
  size_t scene_bytes = 0;
  std::vector<DomainDev> hdoms;
  std::vector<spray_gpu_light> lights;
  DomainDev* d_domains = nullptr;
  BvhNode4* d_nodes = nullptr;
  float4* d_tris = nullptr;
  uint32_t* d_faces = nullptr;
  uint32_t* d_colors = nullptr;
  float* d_normals = nullptr;
  float* d_lights = nullptr;
  CameraDev cam{};
  std::vector<FrameView> fviews;     // the views of the frame being traced
  std::vector<ViewDev> hviews;
  ViewDev* d_views = nullptr;
  size_t views_cap = 0;
  int64_t frame_pixels = 0, image_cap = 0, tiles_cap = 0;
  uint64_t plan_sig = 0;             // layout of the planned waves (a change recaptures the graph)
  std::vector<TileDev> wave_tiles;   // every wave's tiles, sample bases relative to the wave
  // in-core frame captured as a CUDA graph; recaptured when buffers change
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t buf_gen = 1, graph_gen = 0;
  int64_t graph_launches = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> graph_sched, graph_trace, graph_occl;
  void captureFrame();
  void record(cudaEvent_t e);
  bool capturing = false;
  void dropGraph();
  std::vector<size_t> domain_verts;

  // out-of-core cache
  bool ooc = false;
  int cache_capacity = 0;
  size_t slot_nodes = 0, slot_tris = 0, slot_verts = 0, cache_slot_bytes = 0;
  char* h_pinned = nullptr;       // prepared domains, pinned
  std::vector<size_t> host_off;   // per domain offset into h_pinned
  char* h_stage = nullptr;        // pinned staging of the domain and segment tables
  uint32_t* d_segs = nullptr;
  BvhNode4* d_dnodes = nullptr;  // 4-wide hierarchy over the domain boxes
  float* d_dboxes = nullptr;     // domain boxes for the scheduler, 6 floats each
  int dnode_count = 0;
  // screen bins of candidate domains for the primary rays
  static constexpr int kBinShift = 4;
  static constexpr int kBinSize = 1 << kBinShift;
  bool use_bins = true;
  std::vector<unsigned char> bins_key;  // camera and image the current bins were built for
  std::vector<int32_t> bin_view_base, bin_view_x;  // per view: first bin, bins per row
  uint32_t* d_bin_start = nullptr;
  uint16_t* d_bin_ids = nullptr;
  size_t bin_start_cap = 0, bin_ids_cap = 0;
  LruSlots lru;
  int64_t domain_loads = 0;

  // frame plan
  std::vector<HostTile> tiles;
  std::vector<Wave> waves;

  // wave buffers
  int64_t cap_samples = 0;
  uint64_t cap_entries = 0, needed_entries = 0;
  int sched_blocks = 0, sched_warps = 0, sched_chunks = 0, compact_blocks = 0;
  int cur = 0;
  RayBuf rays[2] = {};
  int32_t* d_pixid = nullptr;
  int32_t* d_samid = nullptr;
  uint16_t* d_view = nullptr;
  uint32_t* d_alive_list = nullptr;
  uint32_t* d_alive_list2 = nullptr;   // the other depth's alive list (ping-pong)
  uint32_t* d_alive_count2 = nullptr;
  uint32_t* d_alive_count = nullptr;
  uint8_t* d_next_flag = nullptr;
  uint64_t* d_ray_key = nullptr;
  float4* d_hit_ns = nullptr;
  ShadowBuf sh = {};
  uint8_t* d_shadow_flag = nullptr;
  uint32_t* d_shadow_list = nullptr;
  uint32_t* d_shadow_count = nullptr;
  uint2* d_arena = nullptr;
  unsigned long long* d_arena_top = nullptr;
  uint32_t* d_list_off = nullptr;
  uint32_t* d_list_cnt = nullptr;
  uint32_t* d_hist = nullptr;
  long long* d_dstats = nullptr;
  // learned proposal: parameters | Adam m | Adam v | gradient, per-CTA
  // partials, domain boxes, collected pairs, per-alive-ray prediction and
  // collection scratch, predicted hits per domain
  float* d_mlp = nullptr;
  float* d_mlp_partial = nullptr;
  float* d_boxes = nullptr;
  mlp::Sample* d_pairs = nullptr;
  unsigned long long* d_pairs_filled = nullptr;
  uint8_t* d_pred = nullptr;
  int8_t* d_lab = nullptr;
  uint8_t* d_lflag = nullptr;
  uint32_t* d_lsel = nullptr;
  uint32_t* d_lnsel = nullptr;
  uint32_t* d_predcount = nullptr;
  int* d_mlp_err = nullptr;
  unsigned long long* d_mlp_eval = nullptr;  // held-out evaluation counters
  mlp::Norm mlp_norm{};
  uint64_t pairs_cap = 0;
  bool proposal_trained = false;
  bool use_pred_order = false;  // this pass orders domains by predicted hits
  int frames_collected = 0;
  int adam_step = 0;
  double learn_ms = 0.0, learn_loss = 0.0, learn_top1 = 0.0, learn_top1_nearest = 0.0;
  int64_t learn_eval_pairs = 0;
  int64_t pairs_filled = 0;
  uint2* d_sentries = nullptr;     // batched out of core: shadow queues beside the radiance ones
  uint32_t* d_skey_start = nullptr;
  uint32_t* d_snum_entries = nullptr;
  uint32_t* d_live = nullptr;      // live entries per domain (radiance, shadow)
  int32_t* d_live_doms = nullptr;
  uint32_t* h_live = nullptr;      // pinned: domain list (D) + live counts (2 D)
  uint2* d_entries = nullptr;
  uint32_t* d_key_start = nullptr;
  uint32_t* d_num_entries = nullptr;
  uint64_t* d_rec_key = nullptr;
  float4* d_rec_attr = nullptr;
  unsigned int* d_work = nullptr;
  uint32_t* d_scan_tmp = nullptr;
  uint8_t* d_dbg_depth = nullptr;  // debug capture only
  uint32_t* d_block_tmp2 = nullptr;  // compaction counts from the shader
  size_t scan_words = 0;
  uint32_t* d_block_tmp = nullptr;
  float4* d_image = nullptr;
  long long* d_scores = nullptr;
  int32_t* d_order = nullptr;
  TileDev* d_tiles = nullptr;
  Counters* d_ctr = nullptr;

  // frame accounting
  int64_t launches = 0;
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
  int64_t inplace_domains = 0;  // (domain, batch) pairs traced in place this frame
  std::map<std::pair<int, int>, std::vector<char>> dbg;
  std::map<std::pair<int, int>, std::vector<char>> bvh_dump;  // (what, domain): domainBvh copies
  int load_pass = 0;  // passes over the domains in this frame (the request log's pass numbers)
  void logLoad(int d, int outcome, int evicted);
};

}  // namespace spray
