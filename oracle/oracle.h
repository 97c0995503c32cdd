/*
 * CPU oracle for the speculative domain-parallel ray-tracing loop of SpRay.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C++, the
 * reference's CPU algorithm for the hot path so the CUDA path can be checked
 * against it.  Only tests, the smoke check and bench.py's CPU-baseline leg
 * call it.  It shares no code with the product.
 *
 * Pinning: the reference binary cannot be built (Embree 2.17, MPI and GLFW
 * are absent) and it ships no golden vectors, but many of its hot-path
 * functions compile alone (oracle/build_ref.sh, with stand-ins for the glm,
 * glog and MPI headers).  The oracle equals them function by function --
 * sampler, slab test, camera, disk and cosine sampling, lights, Blinn-Phong,
 * reflection and refraction, colour unpack, LRU cache, tiles, domain scores
 * (tests/test_reference_vectors.py and tests/golden/).  Traversal and the
 * loop as a whole stay unpinned: the oracle substitutes its own BVH and the
 * published watertight triangle test (Woop, Benthin, Wald, JCGT 2013) for
 * Embree.
 *
 * Three modes:
 *   A  orc_render_speculative: the reference's loop itself -- per-thread
 *      queues, DomainStats score order, VBuf speculation history, pending
 *      queue, LRU/infinite domain cache, OpenMP threads with the same barriers.
 *   B  stage functions (eye rays, scheduling, closest hit, shading, occlusion)
 *      and orc_render_wavefront, which applies them bounce by bounce.
 *   C  orc_render_baseline: the reference's non-speculative image tracer
 *      (src/baseline/): one domain per round, the one with the most queued
 *      rays (LoadAnyOnceImageSched), each ray moving on to its next domain
 *      only when no hit lies in front of it.
 */
#ifndef SPRAY_ORACLE_H_
#define SPRAY_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_config {
  int32_t image_w, image_h;
  int32_t ao_mode, ao_samples, pixel_samples, bounces;
  float ks[3];
  float shininess;
  float fov;
  int32_t cache_size;          /* <0 infinite cache, else LRU capacity in domains */
  int32_t max_samples_per_rank;
  int32_t list_size;           /* SPRAY_RAY_DOMAIN_LIST_SIZE */
  int32_t history_size;        /* SPRAY_SPECU_HISTORY_SIZE (<= 8) */
  int32_t num_ranks, rank;
  /* extensions (0 = reference behaviour) */
  int32_t ao_light_shadow;
  float ao_max_distance;
  int32_t rr_depth;
} orc_config;

typedef struct orc_stats {
  int64_t rays_primary, rays_shadow, rays_bounce;
  int64_t visits_radiance, visits_shadow;
  int64_t domain_loads;
  int64_t rounds;
  int64_t visits_shade;  /* mode C: rays sent back to the domain of their hit for shading */
  /* mode B with orc_set_bvh4 on every domain: the ordered front-to-back walk
   * of the radiance rays over those hierarchies (domains visited after
   * culling, inner nodes expanded, triangles tested) and the rays whose hit
   * differed from the oracle's own (0 when the hierarchies are sound) */
  int64_t bvh4_visits, bvh4_nodes, bvh4_tris, bvh4_mismatches;
} orc_stats;

void* orc_create(const orc_config* cfg, int32_t num_domains);
void orc_destroy(void* o);
/* world-space mesh of domain d (copied); bounds = world AABB min xyz, max xyz */
int orc_set_domain(void* o, int32_t d, const float* vertices, int64_t nv, const uint32_t* faces,
                   int64_t nf, const uint32_t* colors, const float bounds[6], int32_t bsdf,
                   const float params[3]);
/* lights: 13 floats each: type, position[3], radiance[3], edge1[3], edge2[3] */
int orc_set_lights(void* o, int32_t nl, const float* lights);
int orc_build(void* o);  /* vertex normals and per-domain BVHs */
/* the product's 4-wide BVH of domain d (32 floats per node, 12 per
 * leaf-ordered triangle, one per face), for counting the work of an ordered
 * traversal of it in orc_render_wavefront; after orc_build */
int orc_set_bvh4(void* o, int32_t d, const float* nodes, int64_t num_nodes, const float* tris, int64_t num_tris);
int orc_set_camera(void* o, const float pos[3], const float lookat[3], const float up[3], float vfov);
int orc_normals(void* o, int32_t d, float* out);  /* 3 * nv */

/* blocking tiles: writes 4 ints (x, y, w, h) per tile, returns count */
int32_t orc_tiles(void* o, int32_t* out, int32_t capacity);

/* eye rays of tiles [first, first + count): org/dir 3 floats, pixid, samid */
int64_t orc_gen_eyes(void* o, int32_t first_tile, int32_t num_tiles, float* org, float* dir,
                     int32_t* pixid, int32_t* samid);

/* Scheduling of n rays.  Radiance (origin == NULL): Isector::isectAll.
 * Shadow (origin != NULL, tmax per ray): the test in the origin domain plus
 * Isector::isectWithoutCurrentDomain.  Entries (5 ints each: domain, ray,
 * tdom bits, depth, origin flag) are written queue by queue in push order;
 * dstats [D][list_size] counts pushes per (domain, depth).  Returns the
 * number of entries or -1 when capacity is too small. */
int64_t orc_schedule(void* o, int64_t n, const float* org, const float* dir, const float* tmax,
                     const int32_t* origin, int32_t* entries, int64_t capacity, int64_t* dstats);

/* DomainStats::schedule on dstats: scores[D], order[D] (ties by id). */
int orc_scores(void* o, const int64_t* dstats, int64_t* scores, int32_t* order);

/* Closest hit over the AABB-overlapped domains of each ray.  Per ray: hit,
 * t, domain, prim, u, v, colour, Ns[3]. */
int orc_closest(void* o, int64_t n, const float* org, const float* dir, int32_t* hit, float* t,
                int32_t* domain, int32_t* prim, float* u, float* v, uint32_t* color, float* ns);

/* Occlusion of shadow rays (origin domain always tested). */
int orc_occluded(void* o, int64_t n, const float* org, const float* dir, const float* tmax,
                 const int32_t* origin, uint8_t* occluded);

/* Shader at actual depth `depth` for n rays with hits.  Per ray input: org,
 * dir, w (3 floats each), pixid, samid, hit t, domain, colour, Ns[3].
 * Output per ray: `slots` shadow rays (dir[3], w[3], tmax, valid) and one
 * bounce ray (dir[3], w[3], valid). */
int32_t orc_slots(void* o);
int orc_shade(void* o, int32_t depth, int64_t n, const float* org, const float* dir, const float* w,
              const int32_t* pixid, const int32_t* samid, const float* t, const int32_t* domain,
              const uint32_t* color, const float* ns, float* sdir, float* sw, float* stmax,
              uint8_t* svalid, float* bdir, float* bw, uint8_t* bvalid);

/* Known-answer hooks: RandomSampler stream, slab test, triangle test, LRU. */
int orc_rng(int32_t seed, int32_t n, float* out);
int orc_sincos(int64_t n, const float* x, float* s, float* c);
int orc_slab(const float bounds[6], const float org[3], const float dir[3], float t0, float t1,
             float* tmin, float* tmax);
int orc_triangle(const float org[3], const float dir[3], const float v[9], float tnear, float tfar,
                 float* t, float* u, float* v_out);
/* replays domain loads through LruCache; hits[i] = 1 on a cache hit;
 * evicted[i] (may be NULL) = the domain a miss displaced, -1 otherwise */
int orc_lru_trace(int32_t num_domains, int32_t cache_size, int64_t n, const int32_t* ids, uint8_t* hits,
                  int32_t* evicted);

/* Per-function hooks, n cases each, for the comparison with the reference's
 * own code (oracle/build_ref.sh).  Vectors are packed float triples.
 *   camera_rays: Camera::init + generateRay at image coordinates xy[2n]
 *   disk: ConcentricDiskSampling of u[2n]; local_to_world: localToWorld(N, v)
 *   cosine_sample: getCosineHemisphereSample(u1, u2, N) -> wi, pdf
 *   point_light: normalize(light - p), the point-light shadow direction
 *   blinn_phong: 20 floats per case (costheta, kd, ks, shininess, li, wi,
 *     n_hat, wo) -> 3
 *   unpack_color: util::unpack -> rgb
 *   reflect: Reflect(wo, n); fr_dielectric / refract: 9 floats per case
 *     (cos_theta_i, eta_i, eta_t, wo, n) -> fr or ok, and wt (0 if unset) */
int orc_camera_rays(const float pos[3], const float lookat[3], const float up[3], float vfov, int32_t w,
                    int32_t h, int64_t n, const float* xy, float* dir);
int orc_disk(int64_t n, const float* u, float* d);
int orc_local_to_world(int64_t n, const float* normal, const float* v, float* out);
int orc_cosine_sample(int64_t n, const float* u, const float* normal, float* wi, float* pdf);
int orc_point_light(int64_t n, const float* light, const float* p, float* wi);
int orc_blinn_phong(int64_t n, const float* args, float* out);
int orc_unpack_color(int64_t n, const uint32_t* color, float* rgb);
int orc_reflect(int64_t n, const float* wo, const float* normal, float* out);
int orc_fr_dielectric(int64_t n, const float* args, float* fr, float* wt);
int orc_refract(int64_t n, const float* args, uint8_t* ok, float* wt);
/* VBuf over nsamples samples of history H: op 0 = update(t[i], ray),
 * op 1 = correct(ray), for rays (samid, depth, hist[H * i ...]); result[i]
 * is the returned flag, hist the ray's history afterwards */
int orc_vbuf_trace(int32_t nsamples, int32_t H, int64_t n, const uint8_t* op, const int32_t* samid,
                   const int32_t* depth, float* hist, const float* t, uint8_t* result);
/* DomainList::sort (rays.h:71-79) of n (id, tnear) pairs in push order */
int orc_domain_list_sort(int32_t n, const int32_t* ids, const float* ts, int32_t* ids_out, float* ts_out);
/* TriMeshBuffer::computeNormals + updateIntersection (trimesh_buffer.cc:267-360)
 * on a mesh: n (triangle, u, v) queries -> interpolated colour and shading
 * normal; normals (may be NULL) receives the 3 * nv vertex normals */
int orc_mesh_attributes(const float* vertices, int64_t nv, const uint32_t* faces, int64_t nf,
                        const uint32_t* colors, int64_t n, const uint32_t* prim, const float* u, const float* v,
                        uint32_t* color, float* ns, float* normals);
/* HdrImage::add in order: rgba[4 * pixid[i] + c] += scale * rgb[3 * i + c] */
int orc_hdr_add(int64_t n, const int32_t* pixid, const float* rgb, double scale, float* rgba);

/* Full frames: W*H*4 floats. */
int orc_render_wavefront(void* o, float* rgba, orc_stats* stats);
int orc_render_speculative(void* o, int32_t nthreads, float* rgba, orc_stats* stats);
/* Mode C (one process).  visits_radiance counts closest-hit tests in a
 * domain, visits_shadow occlusion tests (including the one in the shading
 * domain), visits_shade the shading-only visits; rounds is the number of
 * scheduled domains; domain_loads the misses of an LRU of cache_size domains
 * over that sequence, from an empty cache. */
int orc_render_baseline(void* o, float* rgba, orc_stats* stats);
/* the domain of every round of the last orc_render_baseline frame: copies
 * min(capacity, rounds) ids, returns rounds */
int64_t orc_baseline_schedule(void* o, int32_t* out, int64_t capacity);
/* LoadAnyOnceSched::scheduleImage on per-domain queue counts: the domain to
 * process next and whether every count is zero */
int orc_load_any_once(int32_t num_domains, const int64_t* counts, int32_t* id, uint8_t* done);

#ifdef __cplusplus
}
#endif

#endif
