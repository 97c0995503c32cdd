// spray_gpu_film: film-mode driver over the C ABI, with the command line of
// SpRay's spray_ooc (src/apps/spray_ooc.cc:32-111, options of Config::parse,
// src/render/config.cc:107-281).  It loads the .spray scene, sets the camera
// (SprayRenderer::initCamera, src/render/spray_renderer.inl:87-105), renders
// --frames frames (SprayRenderer::renderFilm, spray_renderer.inl:352-380) and
// writes the PPM of the last one (HdrImage::writePpm, src/display/image.h:183-204).
// The interactive GLFW/OpenGL modes are unavailable: there is no graphics stack.
#include <getopt.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spray_gpu.h"

namespace {

struct Options {
  spray_gpu_config cfg;
  std::string scene_file, ply_path, output = "spray.ppm", mode = "glfw";
  bool has_camera = false;
  float cam[6] = {0, 0, 0, 0, 0, 0};
  float up[3] = {0.f, 1.f, 0.f};
  long frames = -1;
};

void usage(const char* argv0) {
  std::printf(
      "Usage: %s [options] <scene.spray>\n"
      "  --output, -o <filename (spray.ppm)>\n  --ply-path <path to ply files>\n"
      "  --mode, -m <film>\n  --cache-size <max. number of domains>\n"
      "  --width, -w <image_width>\n  --height, -h <image_height>\n  --frames <number of frames>\n"
      "  --bounces <number of bounces (1)>\n  --camera-up <upx upy upz>\n"
      "  --camera <posx posy posz lookx looky lookz>\n  --fov <vertical degrees (90)>\n"
      "  --ao-samples <n (8)>\n  --ao-mode\n  --pixel-samples <n (4)>\n"
      "  --max-samples-per-rank <n (1048576)>\n  --blinn ks_r ks_g ks_b shininess\n"
      "  --nthreads <n>, --light-samples <n>, --partition image, --shading <lambert|blinn>,\n"
      "  --local-disk <path>, --num-partitions <n>, --dev-mode: accepted for compatibility\n",
      argv0);
}

// util::parseTuple (src/utils/util.h:45-51): values start at optarg.
void parseTuple(char** argv, int len, float* out) {
  int index = optind - 1;
  for (int i = 0; i < len; ++i) out[i] = (float)std::atof(argv[index + i]);
  optind = index + len;
}

int parse(int argc, char** argv, Options* o) {
  spray_gpu_config_defaults(&o->cfg);
  static struct option longopts[] = {
      {"output", required_argument, 0, 'o'},       {"local-disk", required_argument, 0, 'l'},
      {"mode", required_argument, 0, 'm'},         {"width", required_argument, 0, 'w'},
      {"height", required_argument, 0, 'h'},       {"frames", required_argument, 0, 300},
      {"nthreads", required_argument, 0, 302},     {"camera-up", required_argument, 0, 308},
      {"light-samples", required_argument, 0, 309}, {"bounces", required_argument, 0, 310},
      {"camera", required_argument, 0, 311},       {"cache-size", required_argument, 0, 313},
      {"fov", required_argument, 0, 314},          {"partition", required_argument, 0, 324},
      {"num-partitions", required_argument, 0, 325}, {"ao-samples", required_argument, 0, 400},
      {"ao-mode", no_argument, 0, 402},            {"pixel-samples", required_argument, 0, 403},
      {"shading", required_argument, 0, 404},      {"blinn", required_argument, 0, 405},
      {"max-samples-per-rank", required_argument, 0, 406}, {"ply-path", required_argument, 0, 408},
      {"dev-mode", no_argument, 0, 1000},          {0, 0, 0, 0}};
  int c, idx = 0;
  while ((c = getopt_long(argc, argv, "o:t:m:r:w:h:x", longopts, &idx)) != -1) {
    switch (c) {
      case 'o': o->output = optarg; break;
      case 'l': break;
      case 'm': o->mode = optarg; break;
      case 'w': o->cfg.image_w = std::atoi(optarg); break;
      case 'h': o->cfg.image_h = std::atoi(optarg); break;
      case 300: o->frames = std::atol(optarg); break;
      case 302: o->cfg.nthreads = std::atoi(optarg); break;
      case 308: parseTuple(argv, 3, o->up); break;
      case 309: break;
      case 310: o->cfg.bounces = std::atoi(optarg); break;
      case 311: parseTuple(argv, 6, o->cam); o->has_camera = true; break;
      case 313: o->cfg.cache_size = std::atoi(optarg); break;
      case 314: o->cfg.fov = (float)std::atof(optarg); break;
      case 324:
        if (std::string(optarg) != "image") {
          std::fprintf(stderr, "unsupported partition %s (only image partitioning is on this path)\n", optarg);
          return 1;
        }
        break;
      case 325: break;
      case 400: o->cfg.ao_samples = std::atoi(optarg); break;
      case 402: o->cfg.ao_mode = 1; break;
      case 403: o->cfg.pixel_samples = std::atoi(optarg); break;
      case 404: break;
      case 405: {
        float d[4];
        parseTuple(argv, 4, d);
        for (int k = 0; k < 3; ++k) o->cfg.ks[k] = d[k];
        o->cfg.shininess = d[3];
      } break;
      case 406: o->cfg.max_samples_per_rank = std::atoi(optarg); break;
      case 408: o->ply_path = optarg; break;
      case 1000: break;
      default: usage(argv[0]); return 1;
    }
  }
  if (optind >= argc) {
    std::fprintf(stderr, "input file not found\n");
    return 1;
  }
  o->scene_file = argv[optind];
  std::string ext = o->scene_file.substr(o->scene_file.find_last_of('.') + 1);
  if (ext != "spray") {
    std::fprintf(stderr, "scene file must end in .spray\n");
    return 1;
  }
  return 0;
}

int check(int code, const char* what) {
  if (code != SPRAY_GPU_OK) std::fprintf(stderr, "%s failed (%d): %s\n", what, code, spray_gpu_last_error());
  return code;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  if (parse(argc, argv, &o)) return 2;
  if (o.mode != "film") {
    std::fprintf(stderr, "mode %s is unavailable: only film mode (headless) is supported\n", o.mode.c_str());
    return 2;
  }
  if (o.frames < 1) {
    std::fprintf(stderr, "film mode needs --frames N with N >= 1\n");
    return 2;
  }
  spray_scene* scene = nullptr;
  if (check(spray_scene_load(o.scene_file.c_str(), o.ply_path.empty() ? nullptr : o.ply_path.c_str(), &scene),
            "scene load"))
    return 1;
  int32_t nd = 0, nl = 0;
  spray_scene_counts(scene, &nd, &nl);
  std::vector<spray_gpu_domain> doms(nd);
  std::vector<spray_gpu_light> lights(nl > 0 ? nl : 1);
  spray_scene_domains(scene, doms.data(), nd);
  spray_scene_lights(scene, lights.data(), nl);
  std::printf("[INFO] number of domains: %d\n[INFO] number of lights: %d\n", nd, nl);

  spray_gpu_tracer* t = nullptr;
  if (check(spray_gpu_create(&o.cfg, &t), "create")) return 1;
  if (check(spray_gpu_set_scene(t, doms.data(), nd, lights.data(), nl), "set_scene")) return 1;
  float pos[3], look[3];
  if (o.has_camera) {
    for (int k = 0; k < 3; ++k) {
      pos[k] = o.cam[k];
      look[k] = o.cam[3 + k];
    }
  } else {
    // scene bound centre, pushed back along +z by half the extent's length
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (auto& d : doms)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::fmin(lo[k], d.world_bounds[k]);
        hi[k] = std::fmax(hi[k], d.world_bounds[3 + k]);
      }
    float ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    float len = std::sqrt((ext[0] * ext[0] + ext[1] * ext[1]) + ext[2] * ext[2]);
    for (int k = 0; k < 3; ++k) look[k] = (float)(0.5 * (lo[k] + hi[k]));
    pos[0] = look[0];
    pos[1] = look[1];
    pos[2] = look[2] + len * 0.5f;
    o.up[0] = 0.f;
    o.up[1] = 1.f;
    o.up[2] = 0.f;
  }
  if (check(spray_gpu_set_camera(t, pos, look, o.up, o.cfg.fov), "set_camera")) return 1;
  const int W = o.cfg.image_w, H = o.cfg.image_h;
  std::vector<float> img((size_t)W * H * 4);
  double total_ms = 0.0, rays = 0.0;
  for (long f = 0; f < o.frames; ++f) {
    spray_gpu_stats st;
    auto t0 = std::chrono::steady_clock::now();
    if (check(spray_gpu_trace(t, img.data(), &st), "trace")) return 1;
    auto t1 = std::chrono::steady_clock::now();
    total_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
    rays += (double)(st.rays_primary + st.rays_shadow + st.rays_bounce);
  }
  std::printf("frames %ld  %.3f ms/frame  %.1f Mrays/s\n", o.frames, total_ms / o.frames,
              rays / (total_ms * 1e-3) / 1e6);
  FILE* fp = std::fopen(o.output.c_str(), "w");
  if (!fp) {
    std::fprintf(stderr, "cannot write %s\n", o.output.c_str());
    return 1;
  }
  std::fprintf(fp, "P3\n%d %d\n1023\n", W, H);
  for (int y = H - 1; y > -1; --y)
    for (int x = 0; x < W; ++x) {
      const float* p = &img[4 * ((size_t)y * W + x)];
      float r = p[0] * 1023.f, g = p[1] * 1023.f, b = p[2] * 1023.f;
      r = r < 0.0f ? 0.0f : (r > 1023.0f ? 1023.0f : r);
      g = g < 0.0f ? 0.0f : (g > 1023.0f ? 1023.0f : g);
      b = b < 0.0f ? 0.0f : (b > 1023.0f ? 1023.0f : b);
      std::fprintf(fp, "%u %u %u\n", (unsigned)r, (unsigned)g, (unsigned)b);
    }
  std::fclose(fp);
  spray_gpu_destroy(t);
  spray_scene_free(scene);
  return 0;
}
