// TEST INFRASTRUCTURE ONLY.  Exposes hot-path functions of the reference,
// compiled from its own sources where they lie (oracle/build_ref.sh), through
// a C ABI, so that the oracle's restatement of each can be compared with the
// reference's code value for value.  Nothing of the reference is copied: this
// file only includes its headers and calls the functions they define.
//
// The reference's third-party headers are absent, so oracle/ref_shim stands in
// for them: glm (float vector arithmetic restated in glm's operation order),
// glog (CHECK aborts), the CMake-generated config header (the CMake cache
// defaults) and the MPI profiler header.  render/aabb.cc is not compiled (it
// includes OpenGL); the slab test reads only Aabb::bounds, so the default
// constructor it would provide is defined empty below.
//
// render/rays.h and render/trimesh_buffer.cc name Embree 2's ray, scene and
// mesh declarations; oracle/ref_shim/embree2 declares them, with set-up calls
// that do nothing (the pinned functions trace no rays).
//
// Include order follows src/apps/spray_ooc.cc: the shader headers (light.h,
// reflection.h, hence sampler.h and <math.h>) come before camera.h, so the
// unqualified tan() in Camera::init resolves as it does in that program.
#include <cstdint>
#include <cstring>

#include "render/light.h"
#include "render/reflection.h"
#include "render/aabb.h"
#include "render/camera.h"
#include "display/image.h"
#include "io/ply_loader.h"
#include "io/scene_loader.h"
#include "render/lru_cache.h"
#include "render/tile.h"
#include "ooc/ooc_domain_stats.h"
#include "ooc/ooc_vbuf.h"
#include "utils/comm.h"
#include "utils/util.h"
#include "render/rays.h"
#include "render/trimesh_buffer.h"
#include "render/data_partition.h"
#include "baseline/baseline_qstats.h"
#include "baseline/baseline_schedulers.h"

namespace spray {
Aabb::Aabb() {}
// The reference's process-wide MPI descriptor (defined with its main
// programs): one process, rank 0.
MpiComm global_mpi_comm;
}  // namespace spray

// LoadAnyOnceSched::scheduleMulti (baseline_schedulers.cc) sums counts over
// processes; with one process it is never called.
extern "C" int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 1; }

using namespace spray;

namespace {
glm::vec3 v3(const float* p) { return glm::vec3(p[0], p[1], p[2]); }
void put3(const glm::vec3& v, float* p) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}
}  // namespace

extern "C" {

// intersectAabb, float-array form (render/aabb.h:139-169).  tmin/tmax are
// written only when the slabs overlap; they start at 0 here, as in the oracle.
int ref_slab(const float b[6], const float org[3], const float dir[3], float t0, float t1, float* tmin,
             float* tmax) {
  Aabb box;
  box.bounds[0] = v3(b);
  box.bounds[1] = v3(b + 3);
  float o[3] = {org[0], org[1], org[2]};
  float d[3] = {dir[0], dir[1], dir[2]};
  *tmin = *tmax = 0.f;
  return intersectAabb(box, o, d, t0, t1, tmin, tmax) ? 1 : 0;
}

// Camera::init then Camera::generateRay(x, y, org, dir) (render/camera.h:128-209)
int ref_camera_rays(const float pos[3], const float lookat[3], const float up[3], float vfov, int32_t w,
                    int32_t h, int64_t n, const float* xy, float* dir) {
  Camera cam;
  cam.init(v3(pos), v3(lookat), v3(up), vfov, w, h);
  for (int64_t i = 0; i < n; ++i) {
    float org[3];
    cam.generateRay(xy[2 * i], xy[2 * i + 1], org, dir + 3 * i);
  }
  return 0;
}

// ConcentricDiskSampling (render/sampler.h:49-92)
int ref_disk(int64_t n, const float* u, float* d) {
  ConcentricDiskSampling disk;
  for (int64_t i = 0; i < n; ++i) disk(u[2 * i], u[2 * i + 1], &d[2 * i], &d[2 * i + 1]);
  return 0;
}

// localToWorld (render/sampler.h:101-110)
int ref_local_to_world(int64_t n, const float* N, const float* v, float* out) {
  for (int64_t i = 0; i < n; ++i) put3(localToWorld(v3(N + 3 * i), v3(v + 3 * i)), out + 3 * i);
  return 0;
}

// getCosineHemisphereSample (render/sampler.cc:54-60)
int ref_cosine_sample(int64_t n, const float* u, const float* N, float* wi, float* pdf) {
  for (int64_t i = 0; i < n; ++i) {
    glm::vec3 d;
    getCosineHemisphereSample(u[2 * i], u[2 * i + 1], v3(N + 3 * i), &d, &pdf[i]);
    put3(d, wi + 3 * i);
  }
  return 0;
}

// DiffuseHemisphereLight::sampleArea (render/light.h:80-85) with a sampler
// seeded by RandomSampler_init(seed[i])
int ref_diffuse_light(int64_t n, const int32_t* seed, const float* N, float* wi, float* pdf) {
  DiffuseHemisphereLight light(glm::vec3(1, 1, 1));
  for (int64_t i = 0; i < n; ++i) {
    RandomSampler s;
    RandomSampler_init(s, seed[i]);
    glm::vec3 d;
    light.sampleArea(s, v3(N + 3 * i), &d, &pdf[i]);
    put3(d, wi + 3 * i);
  }
  return 0;
}

// PointLight::sample (render/light.h:47-52): wi toward the light
int ref_point_light(int64_t n, const float* light_pos, const float* p, float* wi) {
  for (int64_t i = 0; i < n; ++i) {
    PointLight light(v3(light_pos + 3 * i), glm::vec3(1, 1, 1));
    glm::vec3 d;
    float pdf;
    light.sample(v3(p + 3 * i), &d, &pdf);
    put3(d, wi + 3 * i);
  }
  return 0;
}

// blinnPhong (render/reflection.h:202-214); 20 floats per case: costheta, kd,
// ks, shininess, li, wi, n_hat, wo
int ref_blinn_phong(int64_t n, const float* a, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 20 * i;
    put3(blinnPhong(p[0], v3(p + 1), v3(p + 4), p[7], v3(p + 8), v3(p + 11), v3(p + 14), v3(p + 17)),
         out + 3 * i);
  }
  return 0;
}

// Reflect (render/reflection.h:126-128)
int ref_reflect(int64_t n, const float* wo, const float* N, float* out) {
  for (int64_t i = 0; i < n; ++i) put3(Reflect(v3(wo + 3 * i), v3(N + 3 * i)), out + 3 * i);
  return 0;
}

// FrDielectric (render/reflection.h:134-158); 9 floats per case:
// cos_theta_i, eta_i, eta_t, wo, n.  wt stays 0 on total internal reflection.
int ref_fr_dielectric(int64_t n, const float* a, float* fr, float* wt) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 9 * i;
    glm::vec3 t(0, 0, 0);
    fr[i] = FrDielectric(p[0], p[1], p[2], v3(p + 3), v3(p + 6), &t);
    put3(t, wt + 3 * i);
  }
  return 0;
}

// Refract (render/reflection.h:160-174), same layout as ref_fr_dielectric
int ref_refract(int64_t n, const float* a, uint8_t* ok, float* wt) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 9 * i;
    glm::vec3 t(0, 0, 0);
    ok[i] = Refract(p[0], p[1], p[2], v3(p + 3), v3(p + 6), &t) ? 1 : 0;
    put3(t, wt + 3 * i);
  }
  return 0;
}

// util::unpack(uint32_t, float[3]) (utils/util.h:75-79)
int ref_unpack_color(int64_t n, const uint32_t* color, float* rgb) {
  for (int64_t i = 0; i < n; ++i) util::unpack(color[i], rgb + 3 * i);
  return 0;
}

// LruCache::init + LruCache::load (render/lru_cache.cc); hits[i] = 1 on a hit
int ref_lru_trace(int32_t num_domains, int32_t cache_size, int64_t n, const int32_t* ids, uint8_t* hits) {
  LruCache c;
  c.init(num_domains, cache_size);
  for (int64_t i = 0; i < n; ++i) {
    int block = -1;
    hits[i] = c.load(ids[i], &block) ? 1 : 0;
  }
  return 0;
}

// ImageScheduleTileList::init (render/tile.cc:317-391): the blocking tiles of
// rank `rank` of `num_ranks`, four ints (x, y, w, h) each; returns the count.
// The caller keeps the tile height above 0 (the reference divides by it).
int32_t ref_tiles(int64_t image_w, int64_t image_h, int64_t spp, int64_t num_ranks, int32_t rank,
                  int64_t max_samples_per_rank, int32_t* out, int32_t capacity) {
  global_mpi_comm.size = (int)num_ranks;
  global_mpi_comm.rank = rank;
  ImageScheduleTileList list;
  list.init(image_w, image_h, spp, num_ranks, rank, max_samples_per_rank);
  int32_t n = 0;
  for (; !list.empty(); list.pop(), ++n) {
    if (n < capacity) {
      const Tile& t = list.front();
      out[4 * n] = t.x;
      out[4 * n + 1] = t.y;
      out[4 * n + 2] = t.w;
      out[4 * n + 3] = t.h;
    }
  }
  return n;
}

// LoadAnyOnceImageSched::init + schedule (baseline/baseline_schedulers.cc:31-62)
// on one round's per-domain queue counts: the domain processed next and
// whether the frame is done.
int ref_load_any_once(int32_t num_domains, const int64_t* counts, int32_t* id, uint8_t* done) {
  global_mpi_comm.size = 1;
  global_mpi_comm.rank = 0;
  baseline::QStats stats;
  stats.init(num_domains);
  for (int32_t d = 0; d < num_domains; ++d) stats.set(d, counts[d]);
  InsituPartition partition;
  baseline::LoadAnyOnceImageSched sched;
  sched.init(num_domains, partition);
  sched.schedule(stats);
  int out = -1;
  *done = sched.getSchedule(&out) ? 1 : 0;
  *id = out;
  return 0;
}

// DomainStats::resize + increment + schedule (ooc/ooc_domain_stats.cc:34-111)
// over counts[num_domains * 16] (16 = the list size of the CMake defaults):
// order[i] = the i-th domain of the schedule.
int ref_domain_order(int32_t num_domains, const int64_t* counts, int32_t* order) {
  global_mpi_comm.size = 1;
  global_mpi_comm.rank = 0;
  ooc::DomainStats s;
  s.resize(num_domains, false);
  s.reset();
  for (int32_t d = 0; d < num_domains; ++d)
    for (int k = 0; k < SPRAY_RAY_DOMAIN_LIST_SIZE; ++k)
      for (int64_t c = 0; c < counts[(int64_t)d * SPRAY_RAY_DOMAIN_LIST_SIZE + k]; ++c) s.increment(d, k);
  s.schedule();
  for (int32_t i = 0; i < num_domains; ++i) order[i] = s.getDomainId(i);
  return 0;
}

// SceneLoader::load (io/scene_loader.cc:311-358), then per domain: its
// transform (16 floats, column-major), object and world bounds (min xyz, max
// xyz), vertex and face counts and material kind (-1 none, 0 diffuse,
// 1 mirror, 2 glass, 3 transmission); per light: kind (0 point, 1 diffuse)
// and radiance.  Returns the domain count, or -1 when `cap` or `light_cap` is
// too small.
int32_t ref_scene_load(const char* spray, const char* ply_dir, int32_t cap, float* transform, float* obj_bounds,
                       float* world_bounds, int64_t* counts, int32_t* bsdf_kind, int32_t light_cap,
                       int32_t* num_lights, int32_t* light_kind, float* light_radiance) {
  std::vector<Domain> doms;
  std::vector<Light*> lights;
  SceneLoader loader;
  loader.load(spray, ply_dir ? ply_dir : "", &doms, &lights);
  int32_t n = (int32_t)doms.size();
  *num_lights = (int32_t)lights.size();
  int32_t ret = (n > cap || *num_lights > light_cap) ? -1 : n;
  if (ret >= 0) {
    for (int32_t i = 0; i < n; ++i) {
      const Domain& d = doms[i];
      for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) transform[16 * i + 4 * c + k] = d.transform[c][k];
      for (int b = 0; b < 2; ++b) {
        put3(d.object_aabb.bounds[b], obj_bounds + 6 * i + 3 * b);
        put3(d.world_aabb.bounds[b], world_bounds + 6 * i + 3 * b);
      }
      counts[2 * i] = (int64_t)d.num_vertices;
      counts[2 * i + 1] = (int64_t)d.num_faces;
      const Bsdf* b = d.bsdf;
      bsdf_kind[i] = !b ? -1
                     : dynamic_cast<const DiffuseBsdf*>(b)      ? 0
                     : dynamic_cast<const MirrorBsdf*>(b)       ? 1
                     : dynamic_cast<const GlassBsdf*>(b)        ? 2
                     : dynamic_cast<const TransmissionBsdf*>(b) ? 3
                                                                : -2;
    }
    for (int32_t l = 0; l < *num_lights; ++l) {
      glm::vec3 wi, rad;
      float pdf;
      if (lights[l]->isAreaLight()) {
        RandomSampler s;
        RandomSampler_init(s, 1);
        rad = lights[l]->sampleArea(s, glm::vec3(0, 0, 1), &wi, &pdf);
        light_kind[l] = 1;
      } else {
        rad = lights[l]->sample(glm::vec3(0, 0, 0), &wi, &pdf);
        light_kind[l] = 0;
      }
      put3(rad, light_radiance + 3 * l);
    }
  }
  for (Light* l : lights) delete l;
  return ret;
}

// PlyLoader::load (io/ply_loader.cc:179-204): vertices (3 floats), faces
// (3 indices) and packed RGB colours of a PLY file.  Returns the vertex count
// and writes the face count, or -1 when the capacities are too small.
int64_t ref_ply_load(const char* file, int64_t vcap, int64_t fcap, float* vertices, uint32_t* faces,
                     uint32_t* colors, int64_t* num_faces) {
  PlyLoader::Header h;
  PlyLoader::quickHeaderRead(file, &h);
  if ((int64_t)h.num_vertices > vcap || (int64_t)h.num_faces > fcap) return -1;
  PlyLoader loader;
  PlyLoader::Data d;
  d.vertices_capacity = (size_t)vcap * 3;
  d.faces_capacity = (size_t)fcap * 3;
  d.colors_capacity = (size_t)vcap;
  d.vertices = vertices;
  d.faces = faces;
  d.colors = colors;
  loader.load(file, &d);
  *num_faces = (int64_t)d.num_faces;
  return (int64_t)d.num_vertices;
}

// The vertex loop of TriMeshBuffer::load (render/trimesh_buffer.cc:141-153,
// which needs Embree to compile): v = transform * vec4(v, 1), in place.
int ref_transform_points(const float* m16, int64_t n, float* v) {
  glm::mat4 x;
  for (int c = 0; c < 4; ++c) x[c] = glm::vec4(m16[4 * c], m16[4 * c + 1], m16[4 * c + 2], m16[4 * c + 3]);
  for (int64_t i = 0; i < 3 * n; i += 3) {
    glm::vec4 r = x * glm::vec4(v[i], v[i + 1], v[i + 2], 1.0f);
    v[i] = r.x;
    v[i + 1] = r.y;
    v[i + 2] = r.z;
  }
  return 0;
}

// VBuf::update / VBuf::correct (ooc/ooc_vbuf.cc:41-112) over nsamples samples
// (one tile of nsamples x 1 pixels, one sample each) with the history size of
// the CMake defaults; same layout as the oracle's orc_vbuf_trace
int ref_vbuf_trace(int32_t nsamples, int64_t n, const uint8_t* op, const int32_t* samid, const int32_t* depth,
                   float* hist, const float* t, uint8_t* result) {
  const int H = SPRAY_SPECU_HISTORY_SIZE;
  ooc::VBuf vb;
  vb.resize(Tile(0, 0, nsamples, 1), 1);
  for (int64_t i = 0; i < n; ++i) {
    ooc::Ray r;
    std::memset(&r, 0, sizeof(r));
    r.samid = samid[i];
    r.depth = depth[i];
    for (int k = 0; k < H; ++k) r.history[k] = hist[H * i + k];
    result[i] = (op[i] == 0 ? vb.update(t[i], &r) : vb.correct(r)) ? 1 : 0;
    for (int k = 0; k < H; ++k) hist[H * i + k] = r.history[k];
  }
  return 0;
}

// HdrImage::add(pixid, rgb, double scale) (display/image.h:99-109), n times
// in order, on a w x h image that starts as `rgba` (4 floats per pixel)
int ref_hdr_add(int32_t w, int32_t h, int64_t n, const int32_t* pixid, const float* rgb, double scale,
                float* rgba) {
  HdrImage img;
  img.resize(w, h);
  std::memcpy(img.buf, rgba, sizeof(float) * 4 * (size_t)w * h);
  for (int64_t i = 0; i < n; ++i) img.add(pixid[i], rgb + 3 * i, scale);
  std::memcpy(rgba, img.buf, sizeof(float) * 4 * (size_t)w * h);
  return 0;
}

// HdrImage::writePpm (display/image.h:183-204) of a w x h float4 image
int ref_write_ppm(int32_t w, int32_t h, const float* rgba, const char* filename) {
  HdrImage img;
  img.resize(w, h);
  std::memcpy(img.buf, rgba, sizeof(float) * 4 * (size_t)w * h);
  img.writePpm(filename);
  return 0;
}

// DomainList::push then DomainList::sort (render/rays.h:57-93) of n (id,
// tnear) pairs, pushed in the given order; the sorted pairs come back.
int ref_domain_list_sort(int32_t n, const int32_t* ids, const float* ts, int32_t* ids_out, float* ts_out) {
  DomainList l;
  l.resize((std::size_t)n);
  l.reset();
  for (int32_t i = 0; i < n; ++i) l.push(ids[i], ts[i]);
  l.sort();
  for (int32_t i = 0; i < n; ++i) {
    ids_out[i] = l.getId((std::size_t)i);
    ts_out[i] = l.getTnear((std::size_t)i);
  }
  return 0;
}

// TriMeshBuffer::load of a PLY file (no transform; vertex normals by
// computeNormals, render/trimesh_buffer.cc:117-169,288-326), then
// updateIntersection (trimesh_buffer.cc:328-360) for n (triangle, u, v):
// interpolated colour and shading normal.
int ref_mesh_attributes(const char* ply, int64_t max_nv, int64_t max_nf, int64_t n, const uint32_t* prim,
                        const float* u, const float* v, uint32_t* color, float* ns) {
  TriMeshBuffer mesh;
  mesh.init(1, (std::size_t)max_nv, (std::size_t)max_nf, true);
  mesh.load(ply, 0, glm::mat4(1.0f), false);
  for (int64_t i = 0; i < n; ++i) {
    RTCRayIntersection isect;
    std::memset(&isect, 0, sizeof(isect));
    isect.primID = prim[i];
    isect.u = u[i];
    isect.v = v[i];
    mesh.updateIntersection(0, &isect);
    color[i] = isect.color;
    for (int k = 0; k < 3; ++k) ns[3 * i + k] = isect.Ns[k];
  }
  return 0;
}

}  // extern "C"
