/*
 * spray_gpu.h -- C ABI of the GB300 (sm_103a) speculative domain-parallel
 * ray tracer.
 *
 * The reference has no plugin or FFI boundary: its tracer is a compile-time
 * template argument of the renderer, SprayRenderer<TracerT>
 * (src/render/spray_renderer.h:45-78), which calls
 *   tracer_.init(cfg, camera_, &scene_, &image_)   (src/render/spray_renderer.inl:58)
 *   tracer_.trace()                                 (src/render/spray_renderer.inl:364)
 * on an ooc::Tracer<ShaderAo|ShaderPt<Scene<InfiniteCache|LruCache>>>
 * (src/apps/spray_ooc.cc:56-104, src/ooc/ooc_tracer.h:52-103).
 * The entry points below are what a binding of that tracer concept needs:
 * create/configure (Config + Tracer::init), scene upload (Scene::init and the
 * domain cache), camera (Camera::init), trace one frame into an HdrImage
 * buffer (Tracer::trace), destroy.  Test hooks expose the intermediate queues
 * and hits of the first wavefront for comparison with a CPU oracle.
 *
 * Conventions: every function returns 0 on success or a SPRAY_GPU_E* code;
 * spray_gpu_last_error() returns a message for the calling thread's last
 * failure.  No C++ exception crosses this boundary.  A tracer is used by one
 * thread at a time; calls block until the GPU work they issue has finished
 * unless stated otherwise.  The library copies all caller data it keeps.
 */
#ifndef SPRAY_GPU_H_
#define SPRAY_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPRAY_GPU_OK 0
#define SPRAY_GPU_EINVAL 1    /* bad argument or configuration */
#define SPRAY_GPU_ECUDA 2     /* CUDA runtime error or no usable GPU */
#define SPRAY_GPU_EIO 3       /* scene or PLY file could not be read */
#define SPRAY_GPU_ESTATE 4    /* call out of order (e.g. trace before scene) */
#define SPRAY_GPU_EOVERFLOW 5 /* a ray overlapped more domains than the list holds */
#define SPRAY_GPU_ENOMEM 6    /* device or pinned host allocation failed */
#define SPRAY_GPU_ETIMEOUT 7  /* a bounded device-side wait gave up */

typedef struct spray_gpu_tracer spray_gpu_tracer;
typedef struct spray_scene spray_scene;

/* Run parameters.  Mirrors spray::Config (src/render/config.h:34-95) with the
 * defaults of Config::Config() (src/render/config.cc:33-73); fields after
 * `nthreads` are extensions that are off (0) in reference-exact mode. */
typedef struct spray_gpu_config {
  int32_t image_w;              /* --width (400) */
  int32_t image_h;              /* --height (400) */
  int32_t ao_mode;              /* --ao-mode: 1 = ShaderAo, 0 = ShaderPt (0) */
  int32_t ao_samples;           /* --ao-samples (8); area-light samples in PT */
  int32_t pixel_samples;        /* --pixel-samples (4) */
  int32_t bounces;              /* --bounces (1) */
  float ks[3];                  /* --blinn ks (unset in the reference without --blinn; 0 here) */
  float shininess;              /* --blinn shininess (0) */
  float fov;                    /* --fov, vertical, degrees (90) */
  int32_t cache_size;           /* --cache-size: <0 every domain resident, else LRU capacity in domains (-1) */
  int32_t max_samples_per_rank; /* --max-samples-per-rank (1048576) */
  int32_t list_size;            /* SPRAY_RAY_DOMAIN_LIST_SIZE (16) */
  int32_t history_size;         /* SPRAY_SPECU_HISTORY_SIZE (4) */
  int32_t nthreads;             /* --nthreads; not used by the GPU path (1) */
  int32_t num_ranks;            /* image-space ranks (mpi::worldSize) sharing the frame (1) */
  int32_t rank;                 /* this rank: renders vertical stripe `rank` (mpi::worldRank) (0) */
  /* ---- extensions ---- */
  int32_t ao_light_shadow;      /* AO: one extra shadow ray toward light 0 (0) */
  float ao_max_distance;        /* AO rays end at this distance; 0 = unbounded (0) */
  int32_t rr_depth;             /* Russian roulette on bounce rays from this depth; 0 = off (0) */
  int32_t cull;                 /* skip (ray, domain) pairs entered beyond the closest hit found so far (1) */
  int64_t cache_bytes;          /* device domain-cache cap in bytes; 0 = use cache_size (0) */
  int64_t wave_samples;         /* samples per wavefront; 0 = up to 64 M (always at most 2^28 / shadow slots) */
  int32_t debug_capture;        /* keep the first wavefront's stage buffers for the debug hooks (0) */
  int32_t device;               /* CUDA device ordinal (0) */
  int32_t schedule_policy;      /* out-of-core domain order: 0 DomainStats score order (the
                                   reference's), 1 resident domains first, 2 batched: the shadow
                                   rays of depth b and the radiance rays of depth b+1 share one
                                   pass over the domains, resident domains go first, and a domain
                                   whose entries were all culled before its turn is not loaded;
                                   3 learned: policy 2 out of core, plus the learned domain-order
                                   proposal (a small MLP trained online on the tracer's own
                                   (ray, winning domain) pairs) orders the work: in core, each
                                   ray's entries up to its predicted domain are traced first and
                                   the later ones front to back; out of core, domains holding
                                   more predicted hits go first; 4 non-speculative: the
                                   LoadAnyOnce baseline (src/baseline/baseline_schedulers.cc) --
                                   one pass per list position, a ray waits only in the queue of its
                                   next domain, domains with the most pending rays first;
                                   5 non-speculative rounds: the reference's baseline image tracer
                                   itself (src/baseline/baseline_image_tracer.inl:28-131), in core
                                   or out of core -- each round runs the one domain holding the
                                   most queued rays (LoadAnyOnceImageSched), a ray moves on to its
                                   next domain only when no hit lies in front of it, the rays a
                                   hit spawns run in that domain first; whole image on one rank,
                                   one view.  Images are unchanged (0) */
  int32_t ooc_batch;            /* out-of-core, policy 2: domains made resident per traced batch,
                                   at most half the cache capacity so that the next batch's copies
                                   overlap this batch's traces; 0 = half the capacity (0) */
  int64_t learn_samples;        /* policy 3: training pairs collected before training (16777216) */
  int32_t learn_batch;          /* policy 3: Adam batch size (65536) */
  int32_t learn_epochs;         /* policy 3: passes over the collected pairs (2) */
  float learn_lr;               /* policy 3: Adam learning rate (0.001) */
  int32_t learn_seed;           /* policy 3: weight initialisation seed (1) */
  int32_t learn_frames;         /* policy 3: train after this many frames even if fewer pairs
                                   were collected (4) */
  int32_t graphs;               /* in core: capture the frame's launches once into a CUDA graph and
                                   replay it while the buffers stay the same (1) */
  int32_t ooc_inplace;          /* out-of-core, policies 2 and 3: a domain that is not resident and
                                   has at most this many live entries in a batch is traced in place
                                   from pinned host memory (read over the host link) instead of
                                   being copied into the cache; 0 = always copy (16384) */
  /* ---- launch shapes (spray_gb300/autotune.py searches them) ---- */
  int32_t trace_blocks_per_sm;  /* CTAs of 256 threads per SM in a traversal launch; 0 = 4 */
  int32_t sched_chunks_per_warp;/* ray chunks (each with a histogram column) per scheduling warp;
                                   0 = 8 */
  int32_t bucket_launches;      /* in core with culling: closest-hit launches per depth, 1 = one
                                   launch over the depth buckets in order (fastest), 4 = one per
                                   bucket (visit counts repeat exactly); 0 = 1 (0) */
  int32_t learn_buckets;        /* policy 3: 1 = also trace each ray's candidates up to the
                                   predicted one first (in core and inside an out-of-core batch);
                                   0 = the prediction only orders the out-of-core domain loads,
                                   every ray keeps its front-to-back order (0) */
  int32_t bvh_device;           /* 1: set_scene builds the domains' BVHs on the GPU (binned SAH,
                                   4-wide nodes); 0: on the host cores (1) */
} spray_gpu_config;

/* One domain: a triangle mesh in world space (transform already applied, as
 * TriMeshBuffer::load does, src/render/trimesh_buffer.cc:117-169) and the
 * world AABB the scheduler tests rays against (Domain::world_aabb,
 * src/render/domain.h:30-40).  Vertex normals are computed by the library in
 * face order (TriMeshBuffer::computeNormals, trimesh_buffer.cc:267-326). */
typedef struct spray_gpu_domain {
  const float* vertices;    /* 3 * num_vertices floats */
  const uint32_t* faces;    /* 3 * num_faces vertex indices */
  const uint32_t* colors;   /* num_vertices packed 0x00RRGGBB, or NULL (black) */
  int64_t num_vertices;
  int64_t num_faces;
  float world_bounds[6];    /* min x y z, max x y z */
  int32_t bsdf_type;        /* 0 diffuse, 1 mirror, 2 glass, 3 transmission */
  float bsdf_params[3];     /* albedo / reflectance, or eta_exterior, eta_interior */
} spray_gpu_domain;

/* A light (src/render/light.h:41-89): point (position, radiance), diffuse
 * hemisphere (radiance), or -- extension -- an emissive quad (position =
 * corner, edge1, edge2, radiance). */
typedef struct spray_gpu_light {
  int32_t type;             /* 0 point, 1 diffuse hemisphere, 2 quad */
  float position[3];
  float radiance[3];
  float edge1[3];
  float edge2[3];
} spray_gpu_light;

/* One view of a multi-view batch: camera (Camera::init, src/render/camera.h:
 * 128-166), image size, samples and shader settings (the matching
 * spray_gpu_config fields).  Views of one call share the scene, the lights,
 * ks/shininess and every queue of the wavefront. */
typedef struct spray_gpu_view {
  float position[3];
  float lookat[3];
  float up[3];
  float vfov;
  int32_t image_w;
  int32_t image_h;
  int32_t pixel_samples;
  int32_t ao_mode;
  int32_t ao_samples;
  int32_t bounces;
  int32_t rr_depth;
  int32_t ao_light_shadow;
  float ao_max_distance;
} spray_gpu_view;

/* Per-frame counters.  A "ray" is one logical ray counted once, whatever the
 * number of domains it visits; a "visit" is one (ray, domain) pair traced. */
typedef struct spray_gpu_stats {
  int64_t rays_primary;
  int64_t rays_shadow;      /* AO and light-shadow rays */
  int64_t rays_bounce;
  int64_t visits_radiance;
  int64_t visits_shadow;
  int64_t visits_culled;    /* pairs skipped by entry-distance culling */
  int64_t domain_loads;     /* domain-cache misses (host-to-device domain copies) */
  int64_t h2d_bytes;        /* bytes copied host-to-device during the frame */
  int64_t d2h_bytes;
  int64_t kernel_launches;  /* kernels this library launched during the frame */
  int64_t list_overflows;   /* rays whose domain list exceeded list_size */
  double frame_ms;          /* device time of the frame (CUDA events) */
  double trace_ms;          /* device time inside the closest-hit kernel */
  double occlude_ms;        /* device time inside the occlusion kernel */
  double schedule_ms;       /* device time inside the scheduling kernels */
  int64_t trace_launches;
  int64_t occlude_launches;
  int64_t nodes_radiance;   /* BVH nodes fetched by closest-hit traversal */
  int64_t tris_radiance;    /* triangles tested by closest-hit traversal */
  int64_t nodes_shadow;     /* BVH nodes fetched by occlusion traversal */
  int64_t tris_shadow;      /* triangles tested by occlusion traversal */
  int64_t scene_triangles;  /* triangles in the scene */
  int64_t scene_bytes;      /* device bytes of BVH nodes, triangles and shading data */
  double h2d_ms;            /* device time of the out-of-core domain copies (copy stream) */
  int64_t learn_pairs;      /* policy 3: training pairs collected so far */
  int64_t learn_trained;    /* policy 3: 1 once the proposal has been trained */
  double learn_ms;          /* policy 3: device time spent training after this frame */
  double learn_loss;        /* policy 3: mean loss of the last training batch */
  int64_t inplace_domains;  /* out of core: (domain, batch) pairs traced in place from host memory */
  int64_t inplace_bytes;    /* out of core: bytes those traversals requested from pinned host memory
                               (128 per BVH node, 48 per triangle, 60 per closest hit's faces,
                               colours and normals); not included in h2d_bytes */
  int64_t cache_slots;      /* out of core: device domain-cache capacity in domains (0 in core) */
  int64_t cache_slot_bytes; /* out of core: bytes of one cache slot (sized by the largest domain) */
  int64_t learn_eval_pairs; /* policy 3: held-out pairs (>= 2 candidates) the proposal was scored on */
  double learn_top1;        /* policy 3: share of them whose predicted candidate holds the hit */
  double learn_top1_nearest;/* policy 3: share whose hit is in the nearest candidate (the
                               front-to-back order's guess) */
  int64_t exchange_bytes;   /* domain-parallel: bytes this rank passed to the reductions */
  int64_t rounds;           /* policy 5: rounds (domains run, one per round) */
  int64_t visits_shade;     /* policy 5: rays run in the domain of their hit for shading only */
  int64_t eyes_culled;      /* primary rays (counted in rays_primary) resolved as misses at
                               generation: their pixel's 16x16 screen bin touches no domain
                               box's projection, so every slab test fails for them; frames
                               without debug_capture */
} spray_gpu_stats;

/* ---------------------------------------------------------------- setup */
void spray_gpu_config_defaults(spray_gpu_config* cfg);
const char* spray_gpu_last_error(void);

/* Tracer::init (src/ooc/ooc_tracer.inl:28-82) without the scene/camera. */
int spray_gpu_create(const spray_gpu_config* cfg, spray_gpu_tracer** out);
int spray_gpu_destroy(spray_gpu_tracer* t);

/* Scene::init + domain cache warm-up (src/render/scene.inl:30-100).  Builds
 * each domain's BVH and uploads every domain when the cache holds them all. */
int spray_gpu_set_scene(spray_gpu_tracer* t, const spray_gpu_domain* domains, int32_t num_domains,
                        const spray_gpu_light* lights, int32_t num_lights);

/* Prepared-domain blobs (the on-disk side of the out-of-core path): what
 * set_scene builds per domain -- vertex normals (TriMeshBuffer::computeNormals,
 * src/render/trimesh_buffer.cc:267-326), the BVH and the leaf-ordered
 * triangles that replace SpRay's per-load PLY parse and Embree build
 * (TriMeshBuffer::load, trimesh_buffer.cc:117-169) -- written once, one file
 * `dir/domain_NNNNN.sdom` per domain.  spray_scene_prepare needs no GPU. */
int spray_scene_prepare(const spray_gpu_domain* domains, int32_t num_domains, const char* dir);
/* set_scene from blobs in `dir` (domains 0..num_domains-1): no normal or BVH
 * build; SPRAY_GPU_EIO for a missing, truncated or foreign file. */
int spray_gpu_set_scene_prepared(spray_gpu_tracer* t, const char* dir, int32_t num_domains,
                                 const spray_gpu_light* lights, int32_t num_lights);

/* Camera::init (src/render/camera.h:128-166); vfov in degrees. */
int spray_gpu_set_camera(spray_gpu_tracer* t, const float pos[3], const float lookat[3],
                         const float up[3], float vfov);

/* Tracer::trace (src/ooc/ooc_tracer.inl:184-234): renders one frame and
 * writes W*H RGBA floats to rgba_out (host memory) with HdrImage semantics:
 * the buffer is cleared, then every unoccluded, history-consistent shadow ray
 * adds w / pixel_samples to its pixel (src/ooc/ooc_tcontext.inl:123-135). */
int spray_gpu_trace(spray_gpu_tracer* t, float* rgba_out, spray_gpu_stats* stats);

/* Same frame, result left in device memory (W*H*4 floats at rgba_dev), for
 * callers that keep the image on the GPU.  No host copy. */
int spray_gpu_trace_device(spray_gpu_tracer* t, float* rgba_dev, spray_gpu_stats* stats);

/* Several views traced in the same wavefronts (no counterpart in SpRay,
 * which renders one camera per run): each view's float4 image, view after
 * view, into `images` (host memory, sum of W*H*4 floats); the _device
 * variant writes device memory.  Each view's image equals what a tracer
 * configured with that view's settings renders. */
int spray_gpu_trace_views(spray_gpu_tracer* t, const spray_gpu_view* views, int32_t num_views, float* images,
                          spray_gpu_stats* stats);
int spray_gpu_trace_views_device(spray_gpu_tracer* t, const spray_gpu_view* views, int32_t num_views,
                                 float* images, spray_gpu_stats* stats);

/* ---------------------------------------------------------------- host scene
 * SceneLoader::load + PlyLoader (src/io/scene_loader.cc:315-358,
 * src/io/ply_loader.cc:179-324): parse a .spray file and load every domain's
 * PLY with its transform applied.  The loaded scene can be handed to
 * spray_gpu_set_scene through spray_scene_domains/lights. */
int spray_scene_load(const char* spray_file, const char* ply_path, spray_scene** out);
int spray_scene_free(spray_scene* s);
int spray_scene_counts(const spray_scene* s, int32_t* num_domains, int32_t* num_lights);
/* Fills caller arrays; the domain pointers stay valid until spray_scene_free. */
int spray_scene_domains(const spray_scene* s, spray_gpu_domain* out, int32_t capacity);
int spray_scene_lights(const spray_scene* s, spray_gpu_light* out, int32_t capacity);

/* Writes a binary little endian PLY (float xyz, uchar rgb, int faces). */
int spray_write_ply(const char* path, const float* vertices, int64_t num_vertices,
                    const uint32_t* colors, const uint32_t* faces, int64_t num_faces);

/* Wavelet isosurface of f = 255 exp(-(x^2+y^2+z^2)/(2*0.5^2)) + 10 sin(60x+p0)
 * + 18 sin(30y+p1) + 5 cos(40z+p2) on [-1,1]^3 sampled on samples^3 points.
 * The caller provides the output capacities; counts are returned even when the
 * arrays are too small (then SPRAY_GPU_EOVERFLOW). */
int spray_generate_wavelet(int32_t samples, double iso, const double phase[3], float* vertices,
                           int64_t vertex_capacity, uint32_t* faces, int64_t face_capacity,
                           int64_t* num_vertices, int64_t* num_faces);

/* ---------------------------------------------------------------- test hooks
 * With cfg.debug_capture set, the first wavefront of the last traced frame is
 * kept; these copy its stage buffers out.  `bounce` selects the radiance depth.
 * Record layouts are the spray_gpu_dbg_* structs below; count is in records. */
#define SPRAY_DBG_RAYS 0        /* spray_gpu_dbg_ray, radiance rays entering the bounce */
#define SPRAY_DBG_RQUEUES 1     /* spray_gpu_dbg_entry, radiance queue entries */
#define SPRAY_DBG_HITS 2        /* spray_gpu_dbg_hit, resolved closest hits */
#define SPRAY_DBG_SHADOWS 3     /* spray_gpu_dbg_shadow, shadow rays and their occlusion */
#define SPRAY_DBG_SQUEUES 4     /* spray_gpu_dbg_entry, shadow queue entries */
#define SPRAY_DBG_SCORES 5      /* spray_gpu_dbg_score, domain scores and schedule order */
#define SPRAY_DBG_LOADS 6       /* spray_gpu_dbg_load, out of core: every domain the frame asked the
                                   cache for, in order (kept for every frame, bounce 0, no
                                   debug_capture needed; empty in core, except under
                                   schedule_policy 5, which logs every round's domain) */
#define SPRAY_DBG_NODES 7       /* the BVH of domain `bounce` as set_scene built it: BvhNode4
                                   records of 128 bytes (child boxes lo/hi x, y, z as 4 floats each,
                                   4 child references, 4 pad; child >= 0 inner node, kEmptyChild
                                   0x80000000 unused, else leaf ~((first << 3) | (count - 1))); needs
                                   no debug_capture */
#define SPRAY_DBG_TRIS 8        /* the leaf-ordered triangles of domain `bounce`: 3 x float4 (the
                                   vertices; w of the first = the domain-local face index bits) */

typedef struct spray_gpu_dbg_ray {
  uint32_t sample;   /* index of the sample in the wavefront */
  int32_t pixid;
  int32_t samid;
  float org[3];
  float dir[3];
  float w[3];
} spray_gpu_dbg_ray;

/* One (ray, domain) queue entry: RayData{ray, tdom, dom_depth} pushed to the
 * queue of `domain` (src/ooc/ooc_isector.h:126-174).  Entries are grouped by
 * domain; within a domain they are in ray order.  origin = 1 marks the test of
 * a shadow ray in the domain that spawned it (TContext::procShads2,
 * src/ooc/ooc_tcontext.inl:73-91). */
typedef struct spray_gpu_dbg_entry {
  int32_t domain;
  uint32_t ray;      /* radiance: sample index; shadow: alive index * slots + slot */
  float tdom;
  int32_t depth;
  int32_t origin;
} spray_gpu_dbg_entry;

typedef struct spray_gpu_dbg_hit {
  uint32_t sample;
  int32_t hit;
  float t;
  int32_t domain;
  int32_t prim;
  uint32_t color;
  float ns[3];
} spray_gpu_dbg_hit;

typedef struct spray_gpu_dbg_shadow {
  uint32_t sample;
  int32_t slot;
  float org[3];
  float dir[3];
  float w[3];
  float tmax;
  int32_t occluded;
} spray_gpu_dbg_shadow;

typedef struct spray_gpu_dbg_load {
  int32_t domain;
  int32_t outcome;   /* 1 cache hit (already resident), 0 miss (copied into a slot), 2 traced
                        in place from host memory (the cache is not asked) */
  int32_t evicted;   /* domain whose slot a miss took, -1 none */
  int32_t pass;      /* pass over the domains that made the request (0, 1, ... in the frame) */
} spray_gpu_dbg_load;

typedef struct spray_gpu_dbg_score {
  int32_t domain;
  int64_t score;
  int32_t order;     /* position of the domain in the processing schedule */
} spray_gpu_dbg_score;

int spray_gpu_debug_count(spray_gpu_tracer* t, int32_t what, int32_t bounce, int64_t* count);
int spray_gpu_debug_copy(spray_gpu_tracer* t, int32_t what, int32_t bounce, void* out,
                         int64_t capacity);

/* ---------------------------------------------------------------- domain-parallel
 * SpRay's in-situ tracer (insitu::MultiThreadTracer,
 * src/insitu/insitu_multithread_tracer.inl:313-442) pins each domain to one
 * MPI rank (InsituPartition::partition, src/render/data_partition.h:60-137:
 * Morton order of the domain centres, ndomains / ranks consecutive domains
 * per rank) and composites every bounce's closest-hit distances with an MPI
 * MIN all-reduce and its occlusion bits with a BOR all-reduce
 * (VBuf::compositeTbuf / compositeObuf, src/insitu/insitu_vbuf.h:109-129).
 * With spray_gpu_set_insitu each rank's tracer holds and traverses only the
 * domains the same partition gives it; every rank keeps the whole ray state
 * (camera rays, shading, compaction and retirement run on each), and per
 * depth the tracer calls, in this order, on every rank:
 *   min_u64  over every sample's packed hit key (t bits << 32 | triangle):
 *            element-wise minimum of unsigned 64-bit values across ranks;
 *   max_u8   over the resolved hit records (16 bytes per sample; the rank
 *            holding the winning hit wrote it, the others zeros);
 *   max_u8   over the shadow rays' occlusion flags (0 or 1).
 * Each call reduces `n` elements in place and returns 0 (nonzero aborts the
 * frame with SPRAY_GPU_ECUDA).  With host_buffers = 1 the tracer copies the
 * data to pinned host memory first and passes host pointers (MPI, gloo; the
 * stream argument is NULL); with 0 it passes device pointers and its stream,
 * on which the call must order its work (NCCL).  Every rank ends the frame
 * with the single-rank image.  Call before spray_gpu_set_scene (the partition
 * needs the domain boxes, and only owned domains are built); the scene must
 * fit each rank's device (no out-of-core cache) and schedule_policy must be 0
 * or 1.  num_ranks = 1 switches it off. */
typedef struct spray_gpu_reduce_ops {
  void* user;
  int32_t host_buffers;
  int (*min_u64)(void* user, uint64_t* data, int64_t n, void* stream);
  int (*max_u8)(void* user, uint8_t* data, int64_t n, void* stream);
} spray_gpu_reduce_ops;

int spray_gpu_set_insitu(spray_gpu_tracer* t, int32_t num_ranks, int32_t rank,
                         const spray_gpu_reduce_ops* ops);
/* The partition itself (host only, no device needed): rank of each of the
 * num_domains domains given their world boxes (6 floats each). */
int spray_gpu_insitu_partition(const float* domain_bounds, int32_t num_domains, int32_t num_ranks,
                               int32_t* owner);

/* ---------------------------------------------------------------- no allocation
 * No counterpart in the reference.  The scheduler (slab test of every ray
 * against every domain AABB, (t, id)-sorted domain lists, stable partition
 * into per-domain queues, as Isector::isectAll builds them) for callers that
 * cannot allocate device memory while they run -- a renderer holding a fixed
 * device budget reserved at start-up, a host runtime that hands out GPU
 * memory from its own pool (a cudaMalloc behind its back breaks its
 * accounting; cudaFree synchronises the device).  All scratch lives in one
 * static device array (about 13 MB, kept on each device that used it until
 * exit); this call allocates nothing.
 *   domain_bounds  device, 6 floats per domain (min xyz, max xyz), <= 256 domains
 *   ray_org/dir    device, 4 floats per ray (xyz + unused), 16-byte aligned,
 *                  <= 262144 rays, tnear 1e-3, tfar infinity
 *   list_size      checked to lie in [1, 32]; it does not cap the lists (it
 *                  only sizes the domain statistics, which this call does not
 *                  keep): a ray's list holds up to 32 domains, and a ray that
 *                  overlaps more fails the call with SPRAY_GPU_EOVERFLOW
 *   entries        device output, 2 words per entry: ray | depth << 26, tdom
 *                  bits; grouped by domain, ray order inside a domain
 *   entry_capacity entries the output holds; fewer than the rays produce
 *                  fails with SPRAY_GPU_EOVERFLOW ("entry_capacity")
 *   domain_start   device output, num_domains + 1 entry offsets
 *   num_entries    host output
 *   stream         cudaStream_t to run on (NULL = legacy default stream)
 * At most 1048576 entries; larger requests fail with SPRAY_GPU_EINVAL or
 * SPRAY_GPU_EOVERFLOW.  The call reads its entry count back and synchronises
 * `stream` before it returns, so it must not be made while that stream or the
 * device is being captured into a CUDA graph.  The first call on a device
 * looks up the scratch array's device address and keeps it for the process;
 * after cudaDeviceReset on that device the kept address is stale, so a
 * process that resets a device must not call this again on it.  Calls share
 * the scratch: calls that overlap on the GPU race. */
int spray_gpu_schedule_static(const float* domain_bounds, int32_t num_domains, const float* ray_org,
                              const float* ray_dir, int32_t num_rays, int32_t list_size,
                              uint32_t* entries, int64_t entry_capacity, uint32_t* domain_start,
                              int64_t* num_entries, void* stream);

/* ---------------------------------------------------------------- learned proposal
 * The learned domain-order proposal (schedule_policy 3) is a 54-64-64-64-8
 * MLP with BF16 weights and FP32 accumulation on the tensor cores.  SpRay has
 * no learned component, so these entry points have no reference counterpart;
 * they expose the network's kernels on caller-owned device buffers (testing,
 * offline training).  All pointers are device pointers; every call blocks
 * until its work has finished.  `params` holds spray_mlp_param_count() floats
 * (W1 b1 W2 b2 W3 b3 W4 b4, weights [out][in], W1 64x64 with input columns
 * 54..63 zero, W4 16x64 with rows 8..15 zero); `boxes` 6 floats per domain;
 * `norm` = centre xyz and scale, features are (p - centre) * scale. */
typedef struct spray_mlp_sample {
  float org[3];
  float dir[3];
  uint16_t cand[8];   /* candidate domains in (entry t, id) order */
  int32_t ncand;      /* 0..8 */
  int32_t label;      /* position of the candidate holding the closest hit, -1 none */
} spray_mlp_sample;

int32_t spray_mlp_param_count(void);
/* logits [n][8] (absent candidates -inf) and their argmax per sample */
int spray_mlp_forward_dev(const float* params, const float* boxes, const float norm[4],
                          const spray_mlp_sample* samples, int64_t n, float* logits, int32_t* pred,
                          int32_t device);
/* gradient of the mean cross-entropy over the labelled samples:
 * grad[param_count + 2] = gradient, loss sum, labelled count */
int spray_mlp_grad_dev(const float* params, const float* boxes, const float norm[4],
                       const spray_mlp_sample* samples, int64_t n, float* grad, int32_t device);
/* `steps` Adam steps (lr; beta1 0.9, beta2 0.999, eps 1e-8) over consecutive
 * batches of `batch` samples (wrapping), Adam step numbers first_step,
 * first_step + 1, ...; losses[steps] receives each step's mean loss (may be NULL) */
int spray_mlp_train_dev(float* params, float* adam_m, float* adam_v, const float* boxes,
                        const float norm[4], const spray_mlp_sample* samples, int64_t n, int32_t batch,
                        float lr, int32_t steps, int32_t first_step, float* losses, int32_t device);

#ifdef __cplusplus
}
#endif

#endif /* SPRAY_GPU_H_ */
