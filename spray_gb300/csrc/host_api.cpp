// C ABI of the host-side scene helpers: .spray/PLY loading, PLY writing and
// the wavelet generator.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spray_gpu.h"
#include "host_scene.h"

namespace spray {
int fail(int code, const std::string& msg);
}

struct spray_scene {
  sg::SceneDesc desc;
  std::vector<sg::Mesh> meshes;
};

extern "C" {

int spray_scene_load(const char* spray_file, const char* ply_path, spray_scene** out) {
  if (!spray_file || !out) return spray::fail(SPRAY_GPU_EINVAL, "null argument");
  *out = nullptr;
  try {
    auto s = std::make_unique<spray_scene>();
    s->desc = sg::loadSceneFile(spray_file, ply_path ? ply_path : "");
    s->meshes.resize(s->desc.domains.size());
    std::vector<std::string> errs(s->meshes.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int d = 0; d < (int)s->meshes.size(); ++d) {
      try {
        sg::loadDomainMesh(s->desc.domains[d], &s->meshes[d]);
      } catch (const std::exception& e) {
        errs[d] = e.what();
      }
    }
    for (auto& e : errs)
      if (!e.empty()) return spray::fail(SPRAY_GPU_EIO, e);
    *out = s.release();
    return SPRAY_GPU_OK;
  } catch (const std::exception& e) {
    return spray::fail(SPRAY_GPU_EIO, e.what());
  }
}

int spray_scene_free(spray_scene* s) {
  delete s;
  return SPRAY_GPU_OK;
}

int spray_scene_counts(const spray_scene* s, int32_t* num_domains, int32_t* num_lights) {
  if (!s) return spray::fail(SPRAY_GPU_EINVAL, "null scene");
  if (num_domains) *num_domains = (int32_t)s->desc.domains.size();
  if (num_lights) *num_lights = (int32_t)s->desc.lights.size();
  return SPRAY_GPU_OK;
}

int spray_scene_domains(const spray_scene* s, spray_gpu_domain* out, int32_t capacity) {
  if (!s || !out) return spray::fail(SPRAY_GPU_EINVAL, "null argument");
  if (capacity < (int32_t)s->desc.domains.size()) return spray::fail(SPRAY_GPU_EINVAL, "capacity too small");
  for (size_t d = 0; d < s->desc.domains.size(); ++d) {
    const sg::Domain& dd = s->desc.domains[d];
    const sg::Mesh& m = s->meshes[d];
    spray_gpu_domain& o = out[d];
    std::memset(&o, 0, sizeof(o));
    o.vertices = m.vertices.data();
    o.faces = m.faces.data();
    o.colors = m.colors.data();
    o.num_vertices = (int64_t)(m.vertices.size() / 3);
    o.num_faces = (int64_t)(m.faces.size() / 3);
    std::memcpy(o.world_bounds, dd.world_bounds, sizeof(o.world_bounds));
    o.bsdf_type = dd.bsdf_type;
    std::memcpy(o.bsdf_params, dd.bsdf_params, sizeof(o.bsdf_params));
  }
  return SPRAY_GPU_OK;
}

int spray_scene_lights(const spray_scene* s, spray_gpu_light* out, int32_t capacity) {
  if (!s || (!out && !s->desc.lights.empty())) return spray::fail(SPRAY_GPU_EINVAL, "null argument");
  if (capacity < (int32_t)s->desc.lights.size()) return spray::fail(SPRAY_GPU_EINVAL, "capacity too small");
  for (size_t l = 0; l < s->desc.lights.size(); ++l) {
    const sg::Light& L = s->desc.lights[l];
    spray_gpu_light& o = out[l];
    std::memset(&o, 0, sizeof(o));
    o.type = L.type;
    std::memcpy(o.position, L.position, 12);
    std::memcpy(o.radiance, L.radiance, 12);
    std::memcpy(o.edge1, L.edge1, 12);
    std::memcpy(o.edge2, L.edge2, 12);
  }
  return SPRAY_GPU_OK;
}

int spray_write_ply(const char* path, const float* vertices, int64_t num_vertices,
                    const uint32_t* colors, const uint32_t* faces, int64_t num_faces) {
  if (!path || !vertices || !faces) return spray::fail(SPRAY_GPU_EINVAL, "null argument");
  try {
    sg::writePly(path, vertices, (uint64_t)num_vertices, colors, faces, (uint64_t)num_faces);
    return SPRAY_GPU_OK;
  } catch (const std::exception& e) {
    return spray::fail(SPRAY_GPU_EIO, e.what());
  }
}

int spray_generate_wavelet(int32_t samples, double iso, const double phase[3], float* vertices,
                           int64_t vertex_capacity, uint32_t* faces, int64_t face_capacity,
                           int64_t* num_vertices, int64_t* num_faces) {
  try {
    sg::WaveletSpec spec;
    spec.samples = samples;
    spec.iso = iso;
    if (phase)
      for (int k = 0; k < 3; ++k) spec.phase[k] = phase[k];
    std::vector<float> v;
    std::vector<uint32_t> f;
    sg::generateWavelet(spec, &v, &f);
    int64_t nv = (int64_t)v.size() / 3, nf = (int64_t)f.size() / 3;
    if (num_vertices) *num_vertices = nv;
    if (num_faces) *num_faces = nf;
    if (nv > vertex_capacity || nf > face_capacity || !vertices || !faces)
      return spray::fail(SPRAY_GPU_EOVERFLOW, "output arrays too small");
    std::memcpy(vertices, v.data(), v.size() * 4);
    std::memcpy(faces, f.data(), f.size() * 4);
    return SPRAY_GPU_OK;
  } catch (const std::exception& e) {
    return spray::fail(SPRAY_GPU_EINVAL, e.what());
  }
}

}  // extern "C"
