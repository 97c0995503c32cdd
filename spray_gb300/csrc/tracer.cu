// Host side of the GPU tracer: scene upload, blocking tiles, wavefront
// orchestration on one CUDA stream, and the C ABI declared in spray_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spray_gpu.h"
#include "bvh.h"
#include "kernels.cuh"
#include "spray_math.cuh"
#include "tracer_internal.h"

namespace spray {

// Blocks per SM of the compaction passes and of the grid-stride streaming
// kernels (resolve, shade, retire); 8 measured best against 4, 6, 12, 16, 24
// on a GB300 (C2 frame 13.18 -> 12.69 ms).
constexpr int kCompactBlocksPerSm = 8;
constexpr int kStreamBlocksPerSm = 8;

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

// ---------------------------------------------------------------- tiles
// ImageScheduleTileList::init (src/render/tile.cc:317-391) on the vertical
// stripe of this rank (makeVerticalStripe, tile.cc:214-235).
std::vector<HostTile> makeTiles(int W, int H, int spp, int num_ranks, int rank,
                                int64_t max_samples) {
  std::vector<HostTile> tiles;
  int sw = std::max(W / num_ranks, 1);
  int sx = rank * sw;
  if (sx >= W) return tiles;
  int w = ((sx + sw > W) || (rank == num_ranks - 1)) ? W - sx : sw;
  int h = H;
  int64_t num_samples = (int64_t)w * h * spp;
  int64_t est = (num_samples + max_samples - 1) / max_samples;
  if (est < 1) est = 1;
  int tile_h = h / (int)est;
  if (tile_h < 1) throw std::invalid_argument("max_samples_per_rank smaller than one image row");
  for (int y = 0; y < h; y += tile_h) {
    HostTile t;
    t.x = sx;
    t.y = y;
    t.w = w;
    t.h = std::min(tile_h, h - y);
    tiles.push_back(t);
  }
  return tiles;
}

// ---------------------------------------------------------------- normals
// TriMeshBuffer::computeNormals (src/render/trimesh_buffer.cc:267-326):
// unnormalised sum of face cross products, faces in file order.
void computeVertexNormals(const float* v, int64_t nv, const uint32_t* f, int64_t nf, float* n) {
  for (int64_t i = 0; i < 3 * nv; ++i) n[i] = 0.0f;
  for (int64_t i = 0; i < nf; ++i) {
    size_t a = 3 * (size_t)f[3 * i], b = 3 * (size_t)f[3 * i + 1], c = 3 * (size_t)f[3 * i + 2];
    float ux = v[b] - v[a], uy = v[b + 1] - v[a + 1], uz = v[b + 2] - v[a + 2];
    float vx = v[c] - v[a], vy = v[c + 1] - v[a + 1], vz = v[c + 2] - v[a + 2];
    float nx = uy * vz - uz * vy;
    float ny = uz * vx - ux * vz;
    float nz = ux * vy - uy * vx;
    for (size_t k : {a, b, c}) {
      n[k] += nx;
      n[k + 1] += ny;
      n[k + 2] += nz;
    }
  }
}

// ---------------------------------------------------------------- camera
// Camera::init (src/render/camera.h:128-166).
CameraDev makeCamera(const float p[3], const float l[3], const float up[3], float vfov, int W, int H) {
  CameraDev c;
  float aspect = (float)W / (float)H;
  float theta = vfov * M_PI / 180.0f;
  float half_h = std::tan(theta / 2.0f);
  float half_w = aspect * half_h;
  V3 campos = v3(p[0], p[1], p[2]), lookat = v3(l[0], l[1], l[2]), upv = v3(up[0], up[1], up[2]);
  V3 w = campos - lookat;
  V3 u = cross(upv, w);
  V3 v = cross(w, u);
  w = normalize(w);
  u = normalize(u);
  v = normalize(v);
  V3 center = campos - w;
  V3 ll = (center - (half_w * u)) - (half_h * v);
  V3 wv = (2.0f * half_w) * u;
  V3 hv = (2.0f * half_h) * v;
  float* dst[4] = {c.pos, c.ll, c.wv, c.hv};
  V3 src[4] = {campos, ll, wv, hv};
  for (int k = 0; k < 4; ++k) {
    dst[k][0] = src[k].x;
    dst[k][1] = src[k].y;
    dst[k][2] = src[k].z;
  }
  c.image_w = (float)W;
  c.image_h = (float)H;
  return c;
}

// ---------------------------------------------------------------- domain preparation
void buildPack(const spray_gpu_domain& src, int d, DomainPack& p, bool bvh) {
  if (src.num_faces <= 0 || src.num_vertices <= 0 || !src.vertices || !src.faces)
    throw std::invalid_argument("domain " + std::to_string(d) + " has no geometry");
  if (src.num_faces >= (1ll << 28)) throw std::invalid_argument("domain too large");
  for (int64_t i = 0; i < 3 * src.num_faces; ++i)
    if ((int64_t)src.faces[i] >= src.num_vertices)
      throw std::invalid_argument("domain " + std::to_string(d) + ": face index out of range");
  p.nv = src.num_vertices;
  p.nf = src.num_faces;
  p.normals.resize(3 * (size_t)p.nv);
  computeVertexNormals(src.vertices, p.nv, src.faces, p.nf, p.normals.data());
  if (bvh) {
    BvhBuildResult b;
    buildBvh4(src.vertices, src.faces, (uint32_t)p.nf, &b);
    p.nodes = std::move(b.nodes);
    p.bvh_depth = b.depth;
    p.tris.resize(3 * (size_t)p.nf);
    for (size_t k = 0; k < b.tri_order.size(); ++k) {
      uint32_t prim = b.tri_order[k];
      const uint32_t* fi = src.faces + 3 * (size_t)prim;
      for (int c = 0; c < 3; ++c) {
        const float* vp = src.vertices + 3 * (size_t)fi[c];
        float w = 0.f;
        if (c == 0) std::memcpy(&w, &prim, 4);
        p.tris[3 * k + c] = make_float4(vp[0], vp[1], vp[2], w);
      }
    }
  }
  p.faces.assign(src.faces, src.faces + 3 * p.nf);
  if (src.colors) p.colors.assign(src.colors, src.colors + p.nv);
  else p.colors.assign(p.nv, 0u);
  for (int c = 0; c < 6; ++c) p.bounds[c] = src.world_bounds[c];
  p.bsdf = src.bsdf_type;
  for (int c = 0; c < 3; ++c) p.bsdf_p[c] = src.bsdf_params[c];
}

// Blob layout (little-endian, version 1): a 128-byte header, then the arrays
// at the 256-byte-aligned offsets it records: BVH nodes (128 B each),
// leaf-ordered triangles (3 float4 each), faces (3 uint32 each), colours (one
// uint32 per vertex), normals (3 floats per vertex).
namespace {
struct BlobHeader {
  char magic[8];
  uint32_t version;
  int32_t bsdf_type;
  float world_bounds[6];
  float bsdf_params[3];
  int32_t bvh_depth;
  int64_t num_vertices, num_faces, num_nodes;
  uint64_t off_nodes, off_tris, off_faces, off_colors, off_normals, file_bytes;
};
static_assert(sizeof(BlobHeader) <= 128, "blob header");
constexpr char kBlobMagic[8] = {'S', 'P', 'R', 'A', 'Y', 'D', 'O', 'M'};

uint64_t align256(uint64_t x) { return (x + 255) & ~(uint64_t)255; }
}  // namespace

std::string domainBlobPath(const std::string& dir, int d) {
  char name[32];
  std::snprintf(name, sizeof(name), "domain_%05d.sdom", d);
  return dir + "/" + name;
}

void writeDomainBlob(const std::string& path, const DomainPack& p) {
  BlobHeader h{};
  std::memcpy(h.magic, kBlobMagic, 8);
  h.version = 1;
  h.bsdf_type = p.bsdf;
  for (int c = 0; c < 6; ++c) h.world_bounds[c] = p.bounds[c];
  for (int c = 0; c < 3; ++c) h.bsdf_params[c] = p.bsdf_p[c];
  h.bvh_depth = p.bvh_depth;
  h.num_vertices = p.nv;
  h.num_faces = p.nf;
  h.num_nodes = (int64_t)p.nodes.size();
  uint64_t at = 256;
  h.off_nodes = at;
  at = align256(at + p.nodes.size() * sizeof(BvhNode4));
  h.off_tris = at;
  at = align256(at + p.tris.size() * sizeof(float4));
  h.off_faces = at;
  at = align256(at + p.faces.size() * 4);
  h.off_colors = at;
  at = align256(at + p.colors.size() * 4);
  h.off_normals = at;
  at += p.normals.size() * 4;
  h.file_bytes = at;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw IoError("cannot write " + path);
  bool ok = true;
  auto put = [&](uint64_t off, const void* src, size_t n) {
    ok = ok && std::fseek(f, (long)off, SEEK_SET) == 0 && (n == 0 || std::fwrite(src, 1, n, f) == n);
  };
  unsigned char head[256] = {0};
  std::memcpy(head, &h, sizeof(h));
  put(0, head, sizeof(head));
  put(h.off_nodes, p.nodes.data(), p.nodes.size() * sizeof(BvhNode4));
  put(h.off_tris, p.tris.data(), p.tris.size() * sizeof(float4));
  put(h.off_faces, p.faces.data(), p.faces.size() * 4);
  put(h.off_colors, p.colors.data(), p.colors.size() * 4);
  put(h.off_normals, p.normals.data(), p.normals.size() * 4);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw IoError("short write to " + path);
}

void readDomainBlob(const std::string& path, DomainPack* p) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw IoError("cannot open " + path);
  BlobHeader h{};
  bool ok = std::fread(&h, 1, sizeof(h), f) == sizeof(h);
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  auto fail_io = [&](const std::string& why) {
    std::fclose(f);
    throw IoError(path + ": " + why);
  };
  if (!ok || std::memcmp(h.magic, kBlobMagic, 8) != 0) fail_io("not a prepared-domain blob");
  if (h.version != 1) fail_io("unsupported blob version " + std::to_string(h.version));
  if (h.num_vertices <= 0 || h.num_faces <= 0 || h.num_faces >= (1ll << 28) || h.num_nodes <= 0 ||
      h.num_nodes >= (1ll << 31))
    fail_io("bad counts");
  const uint64_t nv = (uint64_t)h.num_vertices, nf = (uint64_t)h.num_faces, nn = (uint64_t)h.num_nodes;
  if (h.off_nodes < 256 || h.off_tris < h.off_nodes + nn * sizeof(BvhNode4) ||
      h.off_faces < h.off_tris + 3 * nf * sizeof(float4) || h.off_colors < h.off_faces + 3 * nf * 4 ||
      h.off_normals < h.off_colors + nv * 4 || h.file_bytes != h.off_normals + 3 * nv * 4 ||
      (uint64_t)size != h.file_bytes)
    fail_io("inconsistent layout or truncated file");
  p->nv = (int64_t)nv;
  p->nf = (int64_t)nf;
  p->bsdf = h.bsdf_type;
  for (int c = 0; c < 6; ++c) p->bounds[c] = h.world_bounds[c];
  for (int c = 0; c < 3; ++c) p->bsdf_p[c] = h.bsdf_params[c];
  p->bvh_depth = h.bvh_depth;
  p->nodes.resize(nn);
  p->tris.resize(3 * nf);
  p->faces.resize(3 * nf);
  p->colors.resize(nv);
  p->normals.resize(3 * nv);
  auto get = [&](uint64_t off, void* dst, size_t n) {
    ok = ok && std::fseek(f, (long)off, SEEK_SET) == 0 && std::fread(dst, 1, n, f) == n;
  };
  get(h.off_nodes, p->nodes.data(), nn * sizeof(BvhNode4));
  get(h.off_tris, p->tris.data(), 3 * nf * sizeof(float4));
  get(h.off_faces, p->faces.data(), 3 * nf * 4);
  get(h.off_colors, p->colors.data(), nv * 4);
  get(h.off_normals, p->normals.data(), 3 * nv * 4);
  std::fclose(f);
  if (!ok) throw IoError(path + ": read failed");
  for (uint64_t i = 0; i < 3 * nf; ++i)
    if (p->faces[i] >= nv) throw IoError(path + ": face index out of range");
}

// Builds and writes every domain's blob (domains in parallel).
void prepareScene(const spray_gpu_domain* domains, int nd, const std::string& dir) {
  std::vector<std::string> errors(nd);
  std::vector<char> io(nd, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int d = 0; d < nd; ++d) {
    try {
      DomainPack p;
      buildPack(domains[d], d, p);
      writeDomainBlob(domainBlobPath(dir, d), p);
    } catch (const IoError& e) {
      errors[d] = e.what();
      io[d] = 1;
    } catch (const std::exception& e) {
      errors[d] = e.what();
    }
  }
  for (int d = 0; d < nd; ++d) {
    if (errors[d].empty()) continue;
    if (io[d]) throw IoError(errors[d]);
    throw std::invalid_argument(errors[d]);
  }
}

// ---------------------------------------------------------------- tracer
Tracer::Tracer(const spray_gpu_config& c) : cfg(c) {
  if (cfg.image_w <= 0 || cfg.image_h <= 0) throw std::invalid_argument("image size must be positive");
  if (cfg.pixel_samples <= 0) throw std::invalid_argument("pixel_samples must be positive");
  if (cfg.bounces <= 0) throw std::invalid_argument("bounces must be positive");
  if (cfg.ao_samples <= 0) throw std::invalid_argument("ao_samples must be positive");
  if (cfg.list_size <= 0 || cfg.list_size > kMaxList)
    throw std::invalid_argument("list_size must be in [1, 32]");
  if (cfg.max_samples_per_rank <= 0) throw std::invalid_argument("max_samples_per_rank must be positive");
  if (cfg.num_ranks <= 0 || cfg.rank < 0 || cfg.rank >= cfg.num_ranks)
    throw std::invalid_argument("rank must be in [0, num_ranks)");
  if (cfg.schedule_policy < 0 || cfg.schedule_policy > 5)
    throw std::invalid_argument("schedule_policy must be 0, 1, 2, 3, 4 or 5");
  if (cfg.schedule_policy == 5 && cfg.num_ranks != 1)
    throw std::invalid_argument("schedule_policy 5 traces the whole image on one rank");
  if (cfg.schedule_policy == 3 &&
      (cfg.learn_samples < 0 || cfg.learn_batch <= 0 || cfg.learn_epochs < 0 || !(cfg.learn_lr > 0.0f) ||
       cfg.learn_frames < 1))
    throw std::invalid_argument(
        "learned proposal needs learn_samples >= 0, learn_batch > 0, learn_epochs >= 0, learn_lr > 0, "
        "learn_frames >= 1");
  if (cfg.ooc_batch < 0) throw std::invalid_argument("ooc_batch must be >= 0");
  if (cfg.ooc_inplace < 0) throw std::invalid_argument("ooc_inplace must be >= 0");
  if (cfg.bucket_launches != 0 && cfg.bucket_launches != 1 && cfg.bucket_launches != kDepthBuckets)
    throw std::invalid_argument("bucket_launches must be 0, 1 or 4");
  if (cfg.trace_blocks_per_sm < 0 || cfg.trace_blocks_per_sm > 32)
    throw std::invalid_argument("trace_blocks_per_sm must be in [0, 32]");
  if (cfg.sched_chunks_per_warp < 0 || cfg.sched_chunks_per_warp > 64)
    throw std::invalid_argument("sched_chunks_per_warp must be in [0, 64]");
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (cfg.device < 0 || cfg.device >= ndev) throw CudaError("no CUDA device " + std::to_string(cfg.device));
  CK(cudaSetDevice(cfg.device));
  CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, cfg.device));
  CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&cstream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ev_start));
  CK(cudaEventCreate(&ev_stop));
  devAlloc(&d_ctr, 1);
  initShadeTables();
}

Tracer::~Tracer() {
  cudaSetDevice(cfg.device);
  freeScene();
  freeBuffers();
  dropGraph();
  devFree(d_ctr);
  devFree(d_views);
  for (auto& e : ev_pool) cudaEventDestroy(e);
  if (ev_start) cudaEventDestroy(ev_start);
  if (ev_stop) cudaEventDestroy(ev_stop);
  if (stream) cudaStreamDestroy(stream);
  if (cstream) cudaStreamDestroy(cstream);
  if (h_reduce) cudaFreeHost(h_reduce);
}

void Tracer::freeScene() {
  freeProposal();
  if (h_pinned) cudaFreeHost(h_pinned);
  h_pinned = nullptr;
  if (h_stage) cudaFreeHost(h_stage);
  h_stage = nullptr;
  if (h_live) cudaFreeHost(h_live);
  h_live = nullptr;
  devFree(d_live);
  devFree(d_live_doms);
  ooc = false;
  devFree(d_segs);
  devFree(d_dnodes);
  devFree(d_dboxes);
  freeRounds();  // sized by the domain count
  bvh_dump.clear();
  dnode_count = 0;
  devFree(d_bin_start);
  devFree(d_bin_ids);
  bin_start_cap = bin_ids_cap = 0;
  bins_key.clear();  // new domain boxes
  devFree(d_domains);
  devFree(d_nodes);
  devFree(d_tris);
  devFree(d_faces);
  devFree(d_colors);
  devFree(d_normals);
  devFree(d_lights);
}

void Tracer::dropGraph() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  graph_exec = nullptr;
  graph_gen = 0;
}

void Tracer::freeBuffers() {
  ++buf_gen;
  for (int k = 0; k < 2; ++k) {
    devFree(rays[k].org);
    devFree(rays[k].dir);
    devFree(rays[k].wgt);
  }
  devFree(d_pixid);
  devFree(d_samid);
  devFree(d_view);
  devFree(d_views);
  devFree(d_alive_list);
  devFree(d_alive_list2);
  devFree(d_alive_count2);
  devFree(d_alive_count);
  devFree(d_next_flag);
  devFree(d_ray_key);
  devFree(d_hit_ns);
  devFree(sh.dir);
  devFree(sh.wgt);
  devFree(sh.hitpos);
  devFree(sh.occluded);
  devFree(d_shadow_flag);
  devFree(d_shadow_list);
  devFree(d_shadow_count);
  devFree(d_arena);
  devFree(d_arena_top);
  devFree(d_list_off);
  devFree(d_list_cnt);
  devFree(d_hist);
  devFree(d_dstats);
  devFree(d_entries);
  devFree(d_dbg_depth);
  devFree(d_key_start);
  devFree(d_num_entries);
  devFree(d_pred);
  devFree(d_lab);
  devFree(d_lflag);
  devFree(d_lsel);
  devFree(d_lnsel);
  devFree(d_sentries);
  devFree(d_skey_start);
  devFree(d_snum_entries);
  devFree(d_rec_key);
  devFree(d_rec_attr);
  devFree(d_work);
  devFree(d_scan_tmp);
  devFree(d_block_tmp);
  devFree(d_block_tmp2);
  devFree(d_image);
  devFree(d_scores);
  devFree(d_order);
  devFree(d_tiles);
  cap_samples = 0;
}

int Tracer::slotsFor(int ao_mode, int ao_samples, int ao_light_shadow) const {
  if (ao_mode) return ao_samples + (ao_light_shadow ? 1 : 0);
  int s = 0;
  for (const auto& l : lights) s += (l.type == 0) ? 1 : ao_samples;
  return s;
}

// Shadow slots per alive ray: the most any view of the frame needs.
int Tracer::slots() const {
  if (fviews.empty()) return slotsFor(cfg.ao_mode, cfg.ao_samples, cfg.ao_light_shadow);
  int s = 0;
  for (const FrameView& v : fviews) s = std::max(s, slotsFor(v.ao_mode, v.ao_samples, v.ao_light_shadow));
  return s;
}

// CTAs of a traversal launch: a multiple of the SM count (persistent warps pull work).
int Tracer::traceBlocks() const { return num_sms * (cfg.trace_blocks_per_sm > 0 ? cfg.trace_blocks_per_sm : 4); }

int Tracer::maxBounces() const {
  if (fviews.empty()) return cfg.bounces;
  int b = 0;
  for (const FrameView& v : fviews) b = std::max(b, v.bounces);
  return b;
}

void Tracer::setScene(const spray_gpu_domain* doms, int nd, const spray_gpu_light* ls, int nl) {
  if (nd <= 0) throw std::invalid_argument("scene needs at least one domain");
  if (nd > 65535) throw std::invalid_argument("at most 65535 domains");
  if (!cfg.ao_mode && nl <= 0) throw std::invalid_argument("path tracing needs at least one light");
  if (cfg.cache_size == 0) throw std::invalid_argument("cache_size must not be 0");
  CK(cudaSetDevice(cfg.device));
  freeScene();
  D = nd;
  lights.assign(ls, ls + nl);
  if (slots() > kMaxSlots) throw std::invalid_argument("too many shadow rays per hit (max 64)");
  std::vector<DomainPack> packs(nd);
  std::vector<std::string> errors(nd);
  if (situ()) {
    std::vector<float> b(6 * (size_t)nd);
    for (int d = 0; d < nd; ++d)
      for (int c = 0; c < 6; ++c) b[6 * d + c] = doms[d].world_bounds[c];
    owner = insituPartition(b.data(), nd, insitu_ranks);
  } else {
    owner.assign(nd, 0);
  }
  const bool dev_bvh = cfg.bvh_device != 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int d = 0; d < nd; ++d) {
    try {
      if (owner[d] == insitu_rank) {
        buildPack(doms[d], d, packs[d], !dev_bvh);
      } else {
        // another rank's domain: its box, material and triangle count only
        DomainPack& p = packs[d];
        if (doms[d].num_faces <= 0) throw std::invalid_argument("domain " + std::to_string(d) + " has no geometry");
        for (int c = 0; c < 6; ++c) p.bounds[c] = doms[d].world_bounds[c];
        p.bsdf = doms[d].bsdf_type;
        for (int c = 0; c < 3; ++c) p.bsdf_p[c] = doms[d].bsdf_params[c];
        p.prim_count = doms[d].num_faces;
      }
    } catch (const std::exception& e) {
      errors[d] = e.what();
    }
  }
  for (int d = 0; d < nd; ++d)
    if (!errors[d].empty()) throw std::invalid_argument(errors[d]);
  if (dev_bvh) {
    std::vector<int> mine;
    for (int d = 0; d < nd; ++d)
      if (owner[d] == insitu_rank) mine.push_back(d);
    // batches of at most 16 M triangles bound the build's device memory (~5 GB)
    buildBvhsOnDevice(doms, mine, packs, stream, 16ull << 20);
  }
  installScene(packs, ls, nl);
}

void Tracer::setScenePrepared(const std::string& dir, int nd, const spray_gpu_light* ls, int nl) {
  if (nd <= 0) throw std::invalid_argument("a scene needs at least one domain");
  freeScene();
  D = nd;
  lights.assign(ls, ls + nl);
  if (slots() > kMaxSlots) throw std::invalid_argument("too many shadow rays per hit (max 64)");
  std::vector<DomainPack> packs(nd);
  std::vector<std::string> errors(nd);
#pragma omp parallel for schedule(dynamic, 1)
  for (int d = 0; d < nd; ++d) {
    try {
      readDomainBlob(domainBlobPath(dir, d), &packs[d]);
    } catch (const std::exception& e) {
      errors[d] = e.what();
    }
  }
  for (int d = 0; d < nd; ++d)
    if (!errors[d].empty()) throw IoError(errors[d]);
  if (situ()) {
    std::vector<float> b(6 * (size_t)nd);
    for (int d = 0; d < nd; ++d)
      for (int c = 0; c < 6; ++c) b[6 * d + c] = packs[d].bounds[c];
    owner = insituPartition(b.data(), nd, insitu_ranks);
    for (int d = 0; d < nd; ++d)
      if (owner[d] != insitu_rank) {
        DomainPack& p = packs[d];
        p.prim_count = p.nf;
        p.nv = p.nf = 0;
        p.nodes.clear();
        p.tris.clear();
        p.faces.clear();
        p.colors.clear();
        p.normals.clear();
        p.bvh_depth = 0;
      }
  } else {
    owner.assign(nd, 0);
  }
  installScene(packs, ls, nl);
}

// Concatenates the prepared domains (in-core) or moves them to the pinned
// arena (out of core), then builds the domain hierarchy and the light table.
void Tracer::installScene(std::vector<DomainPack>& packs, const spray_gpu_light* ls, int nl) {
  const int nd = (int)packs.size();
  domain_verts.assign(nd, 0);
  for (int d = 0; d < nd; ++d) domain_verts[d] = (size_t)packs[d].nv;
  // concatenate in domain order
  hdoms.assign(nd, DomainDev{});
  size_t nn = 0, nt = 0, nvv = 0;
  uint64_t gp = 0;
  max_bvh_depth = 0;
  for (int d = 0; d < nd; ++d) {
    DomainDev& dd = hdoms[d];
    for (int c = 0; c < 3; ++c) {
      dd.bmin[c] = packs[d].bounds[c];
      dd.bmax[c] = packs[d].bounds[3 + c];
    }
    dd.node_base = (int32_t)nn;
    dd.tri_base = (int32_t)nt;
    dd.gprim_base = (uint32_t)gp;
    dd.vert_base = (int32_t)nvv;
    dd.face_base = (int32_t)nt;
    dd.bsdf = packs[d].bsdf;
    for (int c = 0; c < 3; ++c) dd.bsdf_p[c] = packs[d].bsdf_p[c];
    dd.resident = 1;
    dd.num_nodes = (int32_t)packs[d].nodes.size();
    dd.num_tris = (int32_t)packs[d].nf;
    nn += packs[d].nodes.size();
    nt += (size_t)packs[d].nf;
    nvv += (size_t)packs[d].nv;
    gp += (uint64_t)(packs[d].prim_count >= 0 ? packs[d].prim_count : packs[d].nf);
    max_bvh_depth = std::max(max_bvh_depth, packs[d].bvh_depth);
    if (gp >= 0xffffffffull || nt >= (1ull << 31) || nn >= (1ull << 31))
      throw std::invalid_argument("scene too large for 32-bit triangle numbering");
  }
  if (max_bvh_depth * 3 + 4 > 64) throw std::runtime_error("BVH deeper than the traversal stack");
  total_tris = nt;
  scene_bytes = nn * sizeof(BvhNode4) + 3 * nt * sizeof(float4) + 3 * nt * 4 + nvv * 4 + 3 * nvv * 4;
  // out-of-core when the cache holds fewer domains than the scene has
  size_t max_nodes = 0, max_tris = 0, max_verts = 0;
  for (int d = 0; d < nd; ++d) {
    max_nodes = std::max(max_nodes, packs[d].nodes.size());
    max_tris = std::max(max_tris, (size_t)packs[d].nf);
    max_verts = std::max(max_verts, (size_t)packs[d].nv);
  }
  const size_t slot_bytes = max_nodes * sizeof(BvhNode4) + max_tris * (3 * sizeof(float4) + 12) + max_verts * 16;
  int capacity = nd;
  if (cfg.cache_bytes > 0) capacity = (int)std::max<int64_t>(1, std::min<int64_t>(nd, cfg.cache_bytes / (int64_t)slot_bytes));
  else if (cfg.cache_size > 0 && cfg.cache_size < nd) capacity = cfg.cache_size;
  ooc = capacity < nd;
  if (ooc && situ()) throw std::invalid_argument("domain-parallel tracing keeps each rank's domains in core");
  if (ooc) {
    setupOutOfCore(packs, capacity, max_nodes, max_tris, max_verts, slot_bytes);
    packs.clear();
  } else {
  devAlloc(&d_domains, nd);
  devAlloc(&d_nodes, nn);
  devAlloc(&d_tris, 3 * nt);
  devAlloc(&d_faces, 3 * nt);
  devAlloc(&d_colors, nvv);
  devAlloc(&d_normals, 3 * nvv);
  for (int d = 0; d < nd; ++d) {
    const DomainPack& p = packs[d];
    const DomainDev& dd = hdoms[d];
    CK(cudaMemcpy(d_nodes + dd.node_base, p.nodes.data(), p.nodes.size() * sizeof(BvhNode4),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_tris + 3 * (size_t)dd.tri_base, p.tris.data(), p.tris.size() * sizeof(float4),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_faces + 3 * (size_t)dd.face_base, p.faces.data(), p.faces.size() * 4,
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_colors + dd.vert_base, p.colors.data(), p.colors.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_normals + 3 * (size_t)dd.vert_base, p.normals.data(), p.normals.size() * 4,
                  cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(d_domains, hdoms.data(), nd * sizeof(DomainDev), cudaMemcpyHostToDevice));
  }
  // hierarchy over the domain boxes for the scheduler (all domains are tested
  // directly when there are few)
  dnode_count = 0;
  std::vector<float> boxes(6 * (size_t)nd);
  for (int d = 0; d < nd; ++d)
    for (int c = 0; c < 3; ++c) {
      boxes[6 * d + c] = hdoms[d].bmin[c];
      boxes[6 * d + 3 + c] = hdoms[d].bmax[c];
    }
  devAlloc(&d_dboxes, boxes.size());
  CK(cudaMemcpy(d_dboxes, boxes.data(), boxes.size() * 4, cudaMemcpyHostToDevice));
  if (nd >= kDomainBvhMin) {
    std::vector<BvhNode4> dn;
    buildDomainBvh4(boxes.data(), nd, &dn);
    dnode_count = (int)dn.size();
    devAlloc(&d_dnodes, dn.size());
    CK(cudaMemcpy(d_dnodes, dn.data(), dn.size() * sizeof(BvhNode4), cudaMemcpyHostToDevice));
  }
  std::vector<float> lf(13 * std::max(nl, 1), 0.f);
  for (int l = 0; l < nl; ++l) {
    float* q = &lf[13 * l];
    q[0] = (float)ls[l].type;
    for (int c = 0; c < 3; ++c) {
      q[1 + c] = ls[l].position[c];
      q[4 + c] = ls[l].radiance[c];
      q[7 + c] = ls[l].edge1[c];
      q[10 + c] = ls[l].edge2[c];
    }
  }
  devAlloc(&d_lights, lf.size());
  CK(cudaMemcpy(d_lights, lf.data(), lf.size() * 4, cudaMemcpyHostToDevice));
  if (situ()) devAlloc(&d_segs, 2 * (size_t)D + 2);  // one segment table over the owned domains
  freeBuffers();  // sizes depend on the domain count and slots
  if (learned()) setupProposal();
  has_scene = true;
}

// ---------------------------------------------------------------- out of core
// Domains stay in pinned host memory, prepared (BVH, leaf-ordered triangles,
// shading data) once; the device holds `capacity` fixed-size slots managed by
// an LRU with the reference's policy (LruCache::load, src/render/lru_cache.cc:
// 65-171: promote on hit, evict the least recently used block on a miss).
void Tracer::setupOutOfCore(std::vector<DomainPack>& packs, int capacity, size_t max_nodes,
                            size_t max_tris, size_t max_verts, size_t slot_bytes) {
  cache_capacity = capacity;
  slot_nodes = max_nodes;
  slot_tris = max_tris;
  slot_verts = max_verts;
  cache_slot_bytes = slot_bytes;
  // one pinned arena: per domain nodes | tris | faces | colours | normals
  host_off.assign(D, 0);
  size_t total = 0;
  for (int d = 0; d < D; ++d) {
    host_off[d] = total;
    const DomainPack& p = packs[d];
    total += p.nodes.size() * sizeof(BvhNode4) + p.tris.size() * sizeof(float4) + p.faces.size() * 4 +
             p.colors.size() * 4 + p.normals.size() * 4;
    total = (total + 255) & ~(size_t)255;
  }
  // mapped, so that a domain can also be traced in place over the host link
  CK(cudaHostAlloc((void**)&h_pinned, std::max<size_t>(total, 256), cudaHostAllocMapped));
  char* dev_pinned = nullptr;
  CK(cudaHostGetDevicePointer((void**)&dev_pinned, h_pinned, 0));
  for (int d = 0; d < D; ++d) {
    const DomainPack& p = packs[d];
    char* q = h_pinned + host_off[d];
    DomainDev& dd = hdoms[d];
    auto put = [&](const void* src, size_t n) {
      const char* at = dev_pinned + (q - h_pinned);
      std::memcpy(q, src, n);
      q += n;
      return at;
    };
    dd.src_nodes = reinterpret_cast<const BvhNode4*>(put(p.nodes.data(), p.nodes.size() * sizeof(BvhNode4)));
    dd.src_tris = reinterpret_cast<const float4*>(put(p.tris.data(), p.tris.size() * sizeof(float4)));
    dd.src_faces = reinterpret_cast<const uint32_t*>(put(p.faces.data(), p.faces.size() * 4));
    dd.src_colors = reinterpret_cast<const uint32_t*>(put(p.colors.data(), p.colors.size() * 4));
    dd.src_normals = reinterpret_cast<const float*>(put(p.normals.data(), p.normals.size() * 4));
    dd.resident = 0;
    dd.node_base = dd.tri_base = dd.vert_base = dd.face_base = 0;
  }
  devAlloc(&d_domains, D);
  devAlloc(&d_nodes, (size_t)capacity * max_nodes);
  devAlloc(&d_tris, 3 * (size_t)capacity * max_tris);
  devAlloc(&d_faces, 3 * (size_t)capacity * max_tris);
  devAlloc(&d_colors, (size_t)capacity * max_verts);
  devAlloc(&d_normals, 3 * (size_t)capacity * max_verts);
  // segment tables (one per radiance depth bucket, one for shadows) of D + 1
  // begins and D + 1 prefixes each
  devAlloc(&d_segs, (kDepthBuckets + 1) * (2 * (size_t)D + 2));
  CK(cudaHostAlloc((void**)&h_stage, D * sizeof(DomainDev) + (kDepthBuckets + 1) * (2 * (size_t)D + 2) * 4,
                   cudaHostAllocDefault));
  devAlloc(&d_live, 2 * (size_t)D);
  devAlloc(&d_live_doms, D);
  CK(cudaHostAlloc((void**)&h_live, 3 * (size_t)D * 4, cudaHostAllocDefault));
  CK(cudaMemcpy(d_domains, hdoms.data(), D * sizeof(DomainDev), cudaMemcpyHostToDevice));
  lru.init(capacity);
}

void LruSlots::init(int cap) {
  capacity = cap;
  blocks.clear();
  where.clear();
}

bool LruSlots::load(int domain, int* slot, int* evicted) {
  *evicted = -1;
  auto it = where.find(domain);
  if (it != where.end()) {
    std::pair<int, int> b = *it->second;
    blocks.erase(it->second);
    blocks.push_back(b);
    where[domain] = std::prev(blocks.end());
    *slot = b.first;
    return true;
  }
  int s;
  if ((int)blocks.size() < capacity) {
    s = (int)blocks.size();
  } else {
    std::pair<int, int> old = blocks.front();
    blocks.pop_front();
    where.erase(old.second);
    *evicted = old.second;
    s = old.first;
  }
  blocks.push_back({s, domain});
  where[domain] = std::prev(blocks.end());
  *slot = s;
  return false;
}

// Copies a domain into a device slot (ordered on stream s, from pinned memory).
void Tracer::loadDomain(int d, int slot, cudaStream_t s) {
  DomainDev& dd = hdoms[d];
  const size_t nn = (size_t)dd.num_nodes, nt = (size_t)dd.num_tris;
  // vertex count: colours + normals follow the faces in the pinned block
  const char* q = h_pinned + host_off[d];
  size_t nv = domain_verts[d];
  dd.node_base = (int32_t)(slot * slot_nodes);
  dd.tri_base = (int32_t)(slot * slot_tris);
  dd.face_base = (int32_t)(slot * slot_tris);
  dd.vert_base = (int32_t)(slot * slot_verts);
  dd.resident = 1;
  size_t b_nodes = nn * sizeof(BvhNode4), b_tris = 3 * nt * sizeof(float4), b_faces = 3 * nt * 4;
  CK(cudaMemcpyAsync(d_nodes + dd.node_base, q, b_nodes, cudaMemcpyHostToDevice, s));
  q += b_nodes;
  CK(cudaMemcpyAsync(d_tris + 3 * (size_t)dd.tri_base, q, b_tris, cudaMemcpyHostToDevice, s));
  q += b_tris;
  CK(cudaMemcpyAsync(d_faces + 3 * (size_t)dd.face_base, q, b_faces, cudaMemcpyHostToDevice, s));
  q += b_faces;
  CK(cudaMemcpyAsync(d_colors + dd.vert_base, q, nv * 4, cudaMemcpyHostToDevice, s));
  q += nv * 4;
  CK(cudaMemcpyAsync(d_normals + 3 * (size_t)dd.vert_base, q, 3 * nv * 4, cudaMemcpyHostToDevice, s));
  h2d_bytes += b_nodes + b_tris + b_faces + nv * 16;
  ++domain_loads;
}

// Traces the queues of an out-of-core scene: domains in `order` that have
// entries are made resident in batches of at most the cache capacity (so a
// batch never evicts its own domains), and each batch is traced in one launch
// over its entry segments.
// Request log of the frame (SPRAY_DBG_LOADS): domain, outcome, evicted, pass.
void Tracer::logLoad(int d, int outcome, int evicted) {
  const spray_gpu_dbg_load r{d, outcome, evicted, load_pass};
  std::vector<char>& v = dbg[{SPRAY_DBG_LOADS, 0}];
  const char* b = reinterpret_cast<const char*>(&r);
  v.insert(v.end(), b, b + sizeof(r));
}

void Tracer::traceOutOfCore(bool shadow, const std::vector<int>& order, int S) {
  ++load_pass;
  std::vector<uint32_t> ks(D + 1);
  CK(cudaMemcpyAsync(ks.data(), d_key_start, (D + 1) * 4, cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  std::vector<int> todo;
  for (int d : order)
    if (ks[d + 1] > ks[d]) todo.push_back(d);
  size_t i = 0;
  while (i < todo.size()) {
    size_t j = std::min(todo.size(), i + (size_t)cache_capacity);
    for (size_t k = i; k < j; ++k) {
      int slot, evicted;
      const bool hit = lru.load(todo[k], &slot, &evicted);
      logLoad(todo[k], hit ? 1 : 0, hit ? -1 : evicted);
      if (!hit) {
        if (evicted >= 0) hdoms[evicted].resident = 0;
        loadDomain(todo[k], slot, stream);
      }
    }
    // stage the domain table and the segment table (begin, prefix) of this batch
    DomainDev* sd = reinterpret_cast<DomainDev*>(h_stage);
    std::memcpy(sd, hdoms.data(), D * sizeof(DomainDev));
    uint32_t* seg = reinterpret_cast<uint32_t*>(h_stage + D * sizeof(DomainDev));
    const int nseg = (int)(j - i);
    uint32_t run = 0;
    for (int k = 0; k < nseg; ++k) {
      int d = todo[i + k];
      seg[k] = ks[d];
      seg[D + 1 + k] = run;
      run += ks[d + 1] - ks[d];
    }
    seg[D + 1 + nseg] = run;
    CK(cudaMemcpyAsync(d_domains, sd, D * sizeof(DomainDev), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_segs, seg, (2 * (size_t)D + 2) * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(d_work, 0, 4, stream));
    TraceArgs ta = traceArgs(0, S);
    ta.seg_begin = d_segs;
    ta.seg_prefix = d_segs + D + 1;
    ta.nseg = nseg;
    cudaEvent_t e0 = poolEvent(), e1 = poolEvent();
    CK(cudaEventRecord(e0, stream));
    if (shadow) launchTraceOccluded(stream, ta, traceBlocks());
    else launchTraceClosest(stream, ta, traceBlocks());
    CK(cudaEventRecord(e1, stream));
    (shadow ? occl_events : trace_events).push_back({e0, e1});
    launches += 1;
    // the staging buffer is reused by the next batch
    CK(cudaStreamSynchronize(stream));
    i = j;
  }
}

// Domain processing order: DomainStats::schedule on the counts of the last
// radiance scheduling (descending score, ties by id).
std::vector<int> Tracer::scoreOrder() {
  std::vector<long long> st((size_t)D * cfg.list_size);
  CK(cudaMemcpyAsync(st.data(), d_dstats, st.size() * 8, cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  std::vector<std::pair<long long, int>> sc(D);
  const int L = cfg.list_size;
  for (int d = 0; d < D; ++d) {
    long long v = 0;
    for (int k = 0; k < L; ++k) v += st[(size_t)d * L + k] * (long long)(L - k);
    sc[d] = {v, d};
  }
  std::sort(sc.begin(), sc.end(), [](const std::pair<long long, int>& a, const std::pair<long long, int>& b) {
    return a.first > b.first || (a.first == b.first && a.second < b.second);
  });
  std::vector<int> order(D);
  for (int k = 0; k < D; ++k) order[k] = sc[k].second;
  return order;
}

void Tracer::setCamera(const float p[3], const float l[3], const float up[3], float vfov) {
  cam = makeCamera(p, l, up, vfov, cfg.image_w, cfg.image_h);
  has_camera = true;
}

void Tracer::planWaves() {
  // every view's blocking tiles, views in order (ImageScheduleTileList::init per view)
  tiles.clear();
  for (size_t v = 0; v < fviews.size(); ++v) {
    std::vector<HostTile> t = makeTiles(fviews[v].w, fviews[v].h, fviews[v].spp, cfg.num_ranks, cfg.rank,
                                        cfg.max_samples_per_rank);
    for (HostTile& h : t) h.view = (int)v;
    tiles.insert(tiles.end(), t.begin(), t.end());
  }
  const int S = std::max(slots(), 1);
  int64_t cap = cfg.wave_samples > 0 ? cfg.wave_samples : (int64_t)64 << 20;
  // shadow ray ids (alive index x slots + slot) stay below the entry's id
  // field and the wavefront's shadow buffers below kMaxWaveShadowRays
  const int64_t lim = std::min<int64_t>((int64_t)kRayIdMask, kMaxWaveShadowRays) / S;
  cap = std::min<int64_t>(cap, lim - 1);
  waves.clear();
  size_t k = 0;
  while (k < tiles.size()) {
    Wave w;
    w.first_tile = (int)k;
    w.num_tiles = 0;
    w.samples = 0;
    w.pixels = 0;
    while (k < tiles.size()) {
      const int64_t tp = (int64_t)tiles[k].w * tiles[k].h;
      const int64_t ts = tp * fviews[tiles[k].view].spp;
      if (w.num_tiles > 0 && w.samples + ts > cap) break;
      if (ts >= lim)
        throw std::invalid_argument("a blocking tile holds more rays than one wavefront can address");
      w.samples += ts;
      w.pixels += tp;
      ++w.num_tiles;
      ++k;
    }
    waves.push_back(w);
  }
  wave_tiles.assign(tiles.size(), TileDev{});
  uint64_t sig = 1469598103934665603ull;
  auto mix = [&](uint64_t x) { sig = (sig ^ x) * 1099511628211ull; };
  for (const Wave& w : waves) {
    int64_t base = 0, pbase = 0;
    for (int q = 0; q < w.num_tiles; ++q) {
      const HostTile& t = tiles[w.first_tile + q];
      const int spp = fviews[t.view].spp;
      TileDev& td = wave_tiles[w.first_tile + q];
      td = TileDev{};
      td.x = t.x;
      td.y = t.y;
      td.w = t.w;
      td.h = t.h;
      td.sample_base = base;
      td.pix_base = pbase;
      td.view = t.view;
      td.spp = spp;
      base += (int64_t)t.w * t.h * spp;
      pbase += (int64_t)t.w * t.h;
      mix((uint64_t)t.x | ((uint64_t)t.y << 32));
      mix((uint64_t)t.w | ((uint64_t)t.h << 32));
      mix((uint64_t)t.view | ((uint64_t)spp << 32));
    }
    mix((uint64_t)w.num_tiles);
  }
  // the view table: image slots back to back, shader settings
  hviews.assign(fviews.size(), ViewDev{});
  frame_pixels = 0;
  for (size_t v = 0; v < fviews.size(); ++v) {
    const FrameView& f = fviews[v];
    ViewDev& d = hviews[v];
    d.cam = f.cam;
    d.image_w = f.w;
    d.image_h = f.h;
    d.spp = f.spp;
    d.ao_mode = f.ao_mode;
    d.ao_samples = f.ao_samples;
    d.bounces = f.bounces;
    d.rr_depth = f.rr_depth;
    d.ao_light_shadow = f.ao_light_shadow;
    d.ao_max_distance = f.ao_max_distance;
    d.pixel_base = frame_pixels;
    d.scale = 1.0 / (double)f.spp;
    frame_pixels += (int64_t)f.w * f.h;
    mix((uint64_t)f.ao_mode | ((uint64_t)f.bounces << 8) | ((uint64_t)f.ao_samples << 16));
  }
  if (sig != plan_sig) {
    plan_sig = sig;
    ++buf_gen;  // the captured frame no longer matches
  }
}

void Tracer::ensureBuffers(int64_t nsamples) {
  const int S = std::max(slots(), 1);
  const int nkeys = kDepthBuckets * D;
  // one resident wave: each warp owns a contiguous chunk of rays
  sched_blocks = num_sms * schedBlocksPerSm(D, kDepthBuckets * D, dnode_count);
  sched_warps = sched_blocks * (kSchedThreads / 32);
  // up to eight ray chunks per scheduling warp, so that uneven rays balance
  // out (a wave uses about one chunk per 1024 rays of these, see chunksFor);
  // a chunk's per-key counts must fit 16 bits
  sched_chunks = (cfg.sched_chunks_per_warp > 0 ? cfg.sched_chunks_per_warp : 8) * sched_warps;
  if (chunkSize((uint64_t)std::max<int64_t>(nsamples, 1024) * S, sched_chunks) >= 65536)
    throw std::runtime_error("too few scheduling chunks for 16-bit histogram counters");
  if (nsamples <= cap_samples && cap_entries >= needed_entries && frame_pixels <= image_cap &&
      (int64_t)tiles.size() <= tiles_cap && fviews.size() <= views_cap)
    return;
  freeBuffers();
  ++buf_gen;
  int64_t N = std::max<int64_t>(nsamples, 1024);
  int64_t NS = N * S;
  if (needed_entries == 0) needed_entries = (uint64_t)std::max<int64_t>(4 * N, 2 * NS);
  uint64_t E = needed_entries;
  for (int k = 0; k < 2; ++k) {
    devAlloc(&rays[k].org, N);
    devAlloc(&rays[k].dir, N);
    devAlloc(&rays[k].wgt, N);
  }
  devAlloc(&d_pixid, N);
  devAlloc(&d_samid, N);
  devAlloc(&d_view, N);
  for (int k = 0; k < 2; ++k) {
    rays[k].pixid = d_pixid;
    rays[k].samid = d_samid;
    rays[k].view = d_view;
  }
  devAlloc(&d_alive_list, N);
  devAlloc(&d_alive_list2, N);
  devAlloc(&d_alive_count2, 1);
  devAlloc(&d_alive_count, 1);
  devAlloc(&d_next_flag, N);
  devAlloc(&d_ray_key, N);
  devAlloc(&d_hit_ns, N);
  devAlloc(&sh.dir, NS);
  devAlloc(&sh.wgt, NS);
  devAlloc(&sh.hitpos, N);
  devAlloc(&sh.occluded, NS);
  devAlloc(&d_shadow_flag, NS);
  devAlloc(&d_shadow_list, NS);
  devAlloc(&d_shadow_count, 1);
  devAlloc(&d_arena, E);
  devAlloc(&d_arena_top, 1);
  devAlloc(&d_list_off, NS);
  devAlloc(&d_list_cnt, NS);
  devAlloc(&d_hist, (size_t)nkeys * sched_chunks);
  devAlloc(&d_dstats, (size_t)D * cfg.list_size);
  devAlloc(&d_entries, E);
  if (cfg.debug_capture) devAlloc(&d_dbg_depth, E);  // list positions of the captured queues
  devAlloc(&d_key_start, nkeys + 1);
  devAlloc(&d_num_entries, 1);
  if (learned()) {
    devAlloc(&d_pred, N);
    devAlloc(&d_lab, N);
    devAlloc(&d_lflag, N);
    devAlloc(&d_lsel, N);
    devAlloc(&d_lnsel, 1);
  }
  if (ooc && cfg.schedule_policy >= 2) {
    devAlloc(&d_sentries, E);
    devAlloc(&d_skey_start, nkeys + 1);
    devAlloc(&d_snum_entries, 1);
  }
  devAlloc(&d_rec_key, E);
  devAlloc(&d_rec_attr, E);
  devAlloc(&d_work, kDepthBuckets);
  scan_words = scanTmpWords(nkeys, sched_chunks);
  devAlloc(&d_scan_tmp, scan_words);
  compact_blocks = num_sms * kCompactBlocksPerSm;
  devAlloc(&d_block_tmp, compact_blocks);
  devAlloc(&d_block_tmp2, compact_blocks);  // the shader's bounce counts per block
  devAlloc(&d_image, (size_t)std::max<int64_t>(frame_pixels, 1));
  image_cap = frame_pixels;
  devAlloc(&d_views, std::max<size_t>(fviews.size(), 1));
  views_cap = fviews.size();
  devAlloc(&d_scores, D);
  devAlloc(&d_order, D);
  devAlloc(&d_tiles, tiles.size() + 1);
  tiles_cap = (int64_t)tiles.size();
  cap_samples = N;
  cap_entries = E;
}

void Tracer::schedule(bool shadow, int order_by_depth, uint32_t* count, uint32_t* list, int S,
                      bool primary, bool into_shadow_queues, bool predicted) {
  SchedArgs a{};
  a.shadow = shadow;
  a.count = count;
  a.list = list;
  a.rays = rays[cur];
  a.sh = sh;
  a.slots = S;
  a.order_by_depth = order_by_depth;
  a.list_size = cfg.list_size;
  a.ray_key = d_ray_key;
  a.dnodes = d_dnodes;
  a.dboxes = d_dboxes;
  a.dnode_count = dnode_count;
  if (primary && use_bins) {
    a.bin_start = d_bin_start;
    a.bin_ids = d_bin_ids;
    a.views = d_views;
    a.bin_shift = kBinShift;
  }
  a.arena = d_arena;
  a.arena_top = d_arena_top;
  a.arena_cap = cap_entries;
  a.list_off = d_list_off;
  a.list_cnt = d_list_cnt;
  a.hist = d_hist;
  a.nchunks = sched_chunks;
  a.dstats = d_dstats;
  a.want_stats = (ooc || cfg.debug_capture) ? 1 : 0;
  a.entries = into_shadow_queues ? d_sentries : d_entries;
  a.entry_cap = cap_entries;
  a.key_start = into_shadow_queues ? d_skey_start : d_key_start;
  a.dbg_depth = into_shadow_queues ? nullptr : d_dbg_depth;
  a.num_entries = into_shadow_queues ? d_snum_entries : d_num_entries;
  a.ctr = d_ctr;
  CK(cudaMemsetAsync(d_arena_top, 0, sizeof(unsigned long long), stream));
  if (predicted) {
    // lists, then the proposal's bucket boundary per ray, then the partition
    a.defer_hist = 1;
    launchSchedLists(stream, a, d_domains, D, sched_warps, sched_blocks);
    mlp::ArenaSource src = arenaSource();
    src.count = count;
    src.list = list;
    mlp::launchPredictArena(stream, proposalNet(), src, d_pred, num_sms * 5);  // 5 CTAs per SM
    a.pred = d_pred;
    launchSchedPartition(stream, a, D, sched_warps, d_scan_tmp, scan_words);
    launches += 7;
  } else {
    launchSchedule(stream, a, d_domains, D, sched_warps, sched_blocks, d_scan_tmp, scan_words);
    launches += 5;
  }
}

TraceArgs Tracer::traceArgs(int order_by_depth, int S) {
  TraceArgs t{};
  t.scene = sceneDev();
  t.entries = d_entries;
  t.num_entries = d_num_entries;
  t.key_start = d_key_start;
  t.nkeys = order_by_depth ? kDepthBuckets * D : D;
  t.work = d_work;
  t.bucket = -1;
  t.seg_begin = nullptr;
  t.seg_prefix = nullptr;
  t.nseg = 0;
  t.rays = rays[cur];
  t.sh = sh;
  t.slots = S;
  t.ray_key = d_ray_key;
  t.rec_key = d_rec_key;
  t.rec_attr = d_rec_attr;
  t.cull = cfg.cull;
  // AO frames: short, bounded shadow rays whose walks end unevenly suit the
  // refilling occlusion walk; path-traced frames the batched one (measured)
  bool ao = fviews.empty() ? cfg.ao_mode != 0 : true;
  for (const FrameView& v : fviews) ao = ao && v.ao_mode != 0;
  t.refill = ao ? 1 : 0;
  t.ctr = d_ctr;
  return t;
}

SceneDev Tracer::sceneDev() const {
  SceneDev s;
  s.domains = d_domains;
  s.num_domains = D;
  s.nodes = d_nodes;
  s.tris = d_tris;
  s.faces = d_faces;
  s.colors = d_colors;
  s.normals = d_normals;
  return s;
}

// Timing event on the work stream; during graph capture it becomes an event
// record node of the graph, so replays still time their kernels.
void Tracer::record(cudaEvent_t e) {
  CK(cudaEventRecordWithFlags(e, stream, capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
}

cudaEvent_t Tracer::poolEvent() {
  if (ev_used == ev_pool.size()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    ev_pool.push_back(e);
  }
  return ev_pool[ev_used++];
}

// Generates the wave's primary rays (tiles and camera are already on the device).
//
// The eye rays are culled by the screen bins: the samples of pixels in bins
// that no domain box's projection touches have an empty domain list, so they
// stop here (no record, not in the alive list) instead of passing through
// the depth-0 scheduling, shading, compaction and retire; a compaction of the
// live flags makes the alive list in sample order.  The debug capture keeps every sample
// alive (its ray and hit records cover every eye ray).
void Tracer::beginWave(const Wave& w) {
  cur = 0;
  EyeCull cull;
  if (use_bins && !cfg.debug_capture && d_bin_start) {
    cull.bin_start = d_bin_start;
    cull.bin_shift = kBinShift;
    cull.live = d_next_flag;
  }
  launchGenPrimary(stream, d_views, d_tiles + w.first_tile, w.num_tiles, w.samples, rays[0], d_alive_list,
                   d_alive_count, cull, d_ctr);
  launches += 1;
  if (cull.live) {
    launchCompact(stream, d_next_flag, nullptr, 1, (uint64_t)w.samples, d_alive_list, d_alive_count, nullptr,
                  d_block_tmp, compact_blocks);
    launchCountCulled(stream, d_alive_count, w.samples, d_ctr);
    launches += 4;
  }
}

ShadeArgs Tracer::shadeArgs(int b, int S) {
  ShadeArgs sa{};
  sa.scene = sceneDev();
  sa.count = d_alive_count;
  sa.list = d_alive_list;
  sa.rays = rays[cur];
  sa.next = rays[cur ^ 1];
  sa.next_flag = d_next_flag;
  sa.ray_key = d_ray_key;
  sa.hit_ns = d_hit_ns;
  sa.sh = sh;
  sa.shadow_flag = d_shadow_flag;
  sa.slots = S;
  sa.depth = b;
  sa.views = d_views;
  for (int c = 0; c < 3; ++c) sa.ks[c] = cfg.ks[c];
  sa.shininess = cfg.shininess;
  sa.lights = d_lights;
  sa.num_lights = (int)lights.size();
  sa.ctr = d_ctr;
  return sa;
}

void Tracer::traceWave(const Wave& w, bool capture) {
  const int S = std::max(slots(), 1);
  const int nb_total = maxBounces();
  beginWave(w);
  // non-speculative (policy 4): one pass per list position, so radiance
  // queues are keyed by depth bucket out of core as well
  const bool nonspec = ooc && cfg.schedule_policy == 4;
  // domain-parallel: radiance keys are domains, each rank traces its own in one launch
  const int order_by_depth = (cfg.cull && (!ooc || nonspec) && !situ()) ? 1 : 0;
  const int nblk = num_sms * kStreamBlocksPerSm;
  for (int b = 0; b < nb_total; ++b) {
    if (capture) captureRays(b);
    // radiance rays -> per-domain queues
    if (b == 0 || capture || ooc) {
      CK(cudaMemsetAsync(d_dstats, 0, (size_t)D * cfg.list_size * sizeof(long long), stream));
    }
    cudaEvent_t s0 = poolEvent(), s1 = poolEvent();
    record(s0);
    schedule(false, order_by_depth, d_alive_count, d_alive_list, S, b == 0, false,
             learned() && proposal_trained && order_by_depth && !capture && cfg.learn_buckets);
    record(s1);
    sched_events.push_back({s0, s1});
    if (capture) {
      launchScores(stream, d_dstats, D, cfg.list_size, d_scores, d_order);
      launches += 1;
      captureQueues(SPRAY_DBG_RQUEUES, b, order_by_depth);
      captureScores(b);
    }
    // closest hits; with culling, one launch per depth bucket so that every
    // entry sees the hits of all nearer domain lists (front-to-back waves)
    TraceArgs ta = traceArgs(order_by_depth, S);
    std::vector<int> order;
    if (nonspec) {
      // LoadAnyOnce restated: a ray waits in the queue of its next domain only
      // (list position k in pass k), and continues only when no hit lies in
      // front of that domain; each pass takes the domains with the most
      // pending rays first
      const int rb = order_by_depth ? kDepthBuckets : 1;
      for (int k = 0; k < rb; ++k) oocPass(true, false, S, rb, k, 1, true);
    } else if (situ()) {
      // this rank's domains, then the t-buffer composite: every rank's
      // closest hit per ray, the minimum of the packed keys
      traceOwned(false, S);
      reduceCall(true, d_ray_key, w.samples, sizeof(uint64_t));
      CK(cudaMemsetAsync(d_hit_ns, 0, (size_t)w.samples * sizeof(float4), stream));
    } else if (ooc) {
      order = scoreOrder();
      if (cfg.schedule_policy == 1) {
        traceOutOfCore(false, residentFirst(order), S);
      } else {
        traceOutOfCore(false, order, S);
      }
    } else {
      CK(cudaMemsetAsync(d_work, 0, 4 * kDepthBuckets, stream));
      // entries are sorted bucket-major, so one launch that walks them in order
      // still traces nearer list positions first; a launch per bucket makes
      // every nearer hit visible to the culling test, so visit counts repeat
      // exactly from frame to frame (the image is the same either way)
      const int nb = (order_by_depth && cfg.bucket_launches == kDepthBuckets) ? kDepthBuckets : 1;
      for (int k = 0; k < nb; ++k) {
        ta.bucket = nb == kDepthBuckets ? k : -1;
        ta.work = d_work + k;
        cudaEvent_t t0 = poolEvent(), t1 = poolEvent();
        record(t0);
        launchTraceClosest(stream, ta, traceBlocks());
        record(t1);
        trace_events.push_back({t0, t1});
      }
      launches += nb;
    }
    // in core the closest-hit launch left barycentrics for resolve to interpolate
    launchResolve(stream, ta, d_hit_ns, nblk, !ooc && !situ());
    launches += 1;
    // the winning entry's rank published the hit's normal and colour, the
    // other ranks left zeros: the bytewise maximum is the winner's record
    if (situ()) reduceCall(false, d_hit_ns, w.samples * (int64_t)sizeof(float4), 1);
    if (learned() && !proposal_trained) collectPairs();
    if (capture) captureHits(b);
    // shade
    // the shader writes the next-depth flag of every alive ray and, per block,
    // the kept counts of the two compactions below (same partition)
    ShadeArgs sa = shadeArgs(b, S);
    sa.blk_shadow = d_block_tmp;
    sa.blk_next = d_block_tmp2;
    launchShade(stream, sa, compact_blocks);
    launches += 1;
    // shadow rays -> queues -> occlusion
    launchCompactCounted(stream, d_shadow_flag, d_alive_count, (uint32_t)S, d_shadow_list, d_shadow_count,
                         nullptr, nullptr, d_block_tmp, compact_blocks);
    launches += 1;
    // In core the shadow entries are sorted by list position (the ray's own
    // domain first): the occlusion walk takes them in that order, so an
    // occluder found near the ray culls its entries in farther domains.
    const int sorder = (!ooc && !nonspec && !situ()) ? 1 : 0;
    schedule(true, sorder, d_shadow_count, d_shadow_list, S, false, nonspec);
    if (capture) captureQueues(SPRAY_DBG_SQUEUES, b, sorder);
    if (nonspec) {
      oocPass(false, true, S, 1, 0, 0, true);
    } else if (situ()) {
      // occlusion in this rank's domains, then the occlusion composite
      traceOwned(true, S);
      reduceCall(false, sh.occluded, w.samples * (int64_t)S, 1);
    } else if (ooc && cfg.schedule_policy == 0) {
      traceOutOfCore(true, order, S);
    } else if (ooc) {
      traceOutOfCore(true, residentFirst(order), S);
    } else {
      CK(cudaMemsetAsync(d_work, 0, 4, stream));
      TraceArgs to = traceArgs(sorder, S);
      cudaEvent_t o0 = poolEvent(), o1 = poolEvent();
      record(o0);
      launchTraceOccluded(stream, to, traceBlocks());
      record(o1);
      occl_events.push_back({o0, o1});
      launches += 1;
    }
    if (capture) captureShadows(b, S);
    // retire
    launchRetire(stream, d_image, d_views, d_alive_list, d_alive_count, rays[cur], sh, d_shadow_flag, S, nblk);
    launches += 1;
    // next depth
    if (b + 1 < nb_total) {
      // compact this depth's alive list (not every sample of the wave)
      launchCompactCounted(stream, d_next_flag, d_alive_count, 1, d_alive_list2, d_alive_count2, nullptr,
                           d_alive_list, d_block_tmp2, compact_blocks);
      std::swap(d_alive_list, d_alive_list2);
      std::swap(d_alive_count, d_alive_count2);
      launches += 1;
      cur ^= 1;
    }
  }
}

// Resident domains first (most recently used first), then the rest of `order`.
std::vector<int> Tracer::residentFirst(const std::vector<int>& order) const {
  std::vector<int> ro;
  std::vector<char> seen(D, 0);
  for (auto it = lru.blocks.rbegin(); it != lru.blocks.rend(); ++it) {
    ro.push_back(it->second);
    seen[it->second] = 1;
  }
  for (int d : order)
    if (!seen[d]) ro.push_back(d);
  return ro;
}

// Out of core, batched: one pass over the domains traces the radiance queues
// and/or the shadow queues while each domain is resident.  Before each batch
// the live entries of every remaining domain are counted on the device; a
// domain none of whose entries is still live (all culled by nearer hits, or
// all of its shadow rays already occluded) is dropped without being loaded.
// Dropping changes neither hit nor occlusion: a culled entry cannot beat its
// ray's hit, and an occluded shadow ray stays occluded.
void Tracer::oocPass(bool with_r, bool with_s, int S, int rb, int rb_first, int rb_count, bool by_live) {
  ++load_pass;
  if (rb_count < 0) rb_count = rb - rb_first;
  const int rb_end = rb_first + rb_count;
  const int nrk = rb * D;  // radiance keys: bucket * D + domain
  std::vector<uint32_t> rk(nrk + 1, 0), sk(D + 1, 0);
  uint32_t rn = 0, sn = 0;
  if (with_r) {
    CK(cudaMemcpyAsync(rk.data(), d_key_start, (nrk + 1) * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&rn, d_num_entries, 4, cudaMemcpyDeviceToHost, stream));
  }
  if (with_s) {
    CK(cudaMemcpyAsync(sk.data(), d_skey_start, (D + 1) * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&sn, d_snum_entries, 4, cudaMemcpyDeviceToHost, stream));
  }
  CK(cudaStreamSynchronize(stream));
  // a queue that overflowed holds no entries; the frame is traced again with larger queues
  if (with_r && rk[nrk] != rn) with_r = false;
  if (with_s && sk[D] != sn) with_s = false;
  if (!with_r && !with_s) return;
  auto rcount = [&](int d) {
    uint32_t c = 0;
    for (int b = rb_first; b < rb_end; ++b) c += rk[b * D + d + 1] - rk[b * D + d];
    return c;
  };
  std::vector<int> order = scoreOrder();
  std::vector<uint32_t> pc;
  if (use_pred_order) {
    // resident domains first (most recently used first), then the domains that
    // hold more predicted hits
    pc.resize(D);
    CK(cudaMemcpyAsync(pc.data(), d_predcount, D * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    auto more = [&](int x, int y) { return pc[x] > pc[y]; };
    std::stable_sort(order.begin(), order.end(), more);
    order = residentFirst(order);
  } else {
    order = residentFirst(order);
  }
  std::vector<int> remaining;
  for (int d : order)
    if ((with_r && rcount(d) > 0) || (with_s && sk[d + 1] > sk[d])) remaining.push_back(d);
  // a batch's copies run on the copy stream while the previous batch traces;
  // two batches fit the cache together, so a copy never evicts a domain that
  // the running trace reads (and the batch before it has finished)
  const int half = std::max(1, cache_capacity / 2);
  const int B = std::min(cfg.ooc_batch > 0 ? cfg.ooc_batch : half, half);
  // domains whose live entries are counted before a batch is chosen: enough to
  // fill it after drops; with in-place tracing every remaining domain may join
  const int window_n = (cfg.ooc_inplace > 0 || by_live) ? D : 2 * B;
  int32_t* hdoms_list = reinterpret_cast<int32_t*>(h_live);
  uint32_t* hlive = h_live + D;
  // live counts of `doms`, written to hlive when `done` has completed
  auto countLive = [&](const std::vector<int>& doms, cudaEvent_t done) {
    if (!doms.empty()) {
      std::memcpy(hdoms_list, doms.data(), doms.size() * 4);
      CK(cudaMemcpyAsync(d_live_doms, hdoms_list, doms.size() * 4, cudaMemcpyHostToDevice, stream));
      LiveArgs la{};
      la.rentries = with_r ? d_entries : nullptr;
      la.rkey_start = d_key_start;
      la.rbucket0 = rb_first;
      la.rbuckets = rb_count;
      la.ray_key = d_ray_key;
      la.rec_key = d_rec_key;
      la.sentries = with_s ? d_sentries : nullptr;
      la.skey_start = d_skey_start;
      la.occluded = sh.occluded;
      la.domains = d_live_doms;
      la.ndomains = (int)doms.size();
      la.D = D;
      la.cull = cfg.cull;
      la.live = d_live;
      // the batched orders compare counts only with ooc_inplace and 0; the
      // most-pending-first order of the non-speculative policy sorts by them
      la.cap = by_live ? 0u : (uint32_t)std::max<int64_t>(cfg.ooc_inplace, 0);
      launchCountLive(stream, la);
      launches += 1;
      CK(cudaMemcpyAsync(hlive, d_live, 2 * (size_t)D * 4, cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaEventRecord(done, stream));
  };
  // the next batch: the first B domains of `remaining` with live entries; the
  // rest stay in `remaining`, domains without live entries are dropped
  // traced in place: not resident, and few live entries (by the counts in hlive)
  auto inPlace = [&](int d) {
    return hdoms[d].resident != 1 && cfg.ooc_inplace > 0 &&
           (uint64_t)(with_r ? hlive[d] : 0) + (with_s ? hlive[D + d] : 0) <= (uint64_t)cfg.ooc_inplace;
  };
  // B bounds the domains that go through the cache (resident or copied); those
  // traced in place take no slot and join the batch freely
  auto select = [&](std::vector<int>& remaining, std::vector<int>& batch) {
    std::vector<int> rest;
    batch.clear();
    int cached = 0;
    const size_t counted_n = std::min(remaining.size(), (size_t)window_n);
    for (size_t k = 0; k < remaining.size(); ++k) {
      const int d = remaining[k];
      if (k < counted_n) {
        const bool lr = with_r && hlive[d] > 0, ls = with_s && hlive[D + d] > 0;
        if (!lr && !ls) continue;  // nothing left to trace here: not loaded
        if (inPlace(d)) {
          batch.push_back(d);
          continue;
        }
        if (cached < B) {
          batch.push_back(d);
          ++cached;
          continue;
        }
      }
      rest.push_back(d);
    }
    remaining.swap(rest);
  };
  // a domain that is not resident and has at most ooc_inplace live entries in
  // this batch is traced in place from pinned host memory instead of copied
  std::vector<int> inplace;
  auto issueLoads = [&](const std::vector<int>& batch, cudaEvent_t loaded) {
    cudaEvent_t c0 = poolEvent();
    CK(cudaEventRecord(c0, cstream));
    inplace.clear();
    for (int d : batch) {
      if (inPlace(d)) {
        hdoms[d].resident = 2;
        inplace.push_back(d);
        logLoad(d, 2, -1);
        continue;
      }
      int slot, evicted;
      const bool hit = lru.load(d, &slot, &evicted);
      logLoad(d, hit ? 1 : 0, hit ? -1 : evicted);
      if (!hit) {
        if (evicted >= 0) hdoms[evicted].resident = 0;
        loadDomain(d, slot, cstream);
      }
    }
    CK(cudaEventRecord(loaded, cstream));
    copy_events.push_back({c0, loaded});
  };
  // live counts cover a window of the next 2 B remaining domains: enough to
  // fill a batch after drops, and each domain is counted about once
  auto window = [&](const std::vector<int>& rem) {
    return std::vector<int>(rem.begin(), rem.begin() + std::min(rem.size(), (size_t)window_n));
  };
  // after a count: select, and while a whole window was dropped, count on
  auto nextBatch = [&](std::vector<int>& batch) {
    select(remaining, batch);
    while (batch.empty() && !remaining.empty()) {
      cudaEvent_t c = poolEvent();
      countLive(window(remaining), c);
      CK(cudaEventSynchronize(c));
      select(remaining, batch);
    }
  };
  std::vector<int> batch, next;
  cudaEvent_t counted = poolEvent();
  countLive(window(remaining), counted);
  CK(cudaEventSynchronize(counted));
  if (by_live) {
    // LoadAnyOnceImageSched::schedule (src/baseline/baseline_schedulers.cc): the
    // domain holding the most pending rays first
    std::stable_sort(remaining.begin(), remaining.end(), [&](int x, int y) {
      return (uint64_t)hlive[x] + hlive[D + x] > (uint64_t)hlive[y] + hlive[D + y];
    });
  }
  nextBatch(batch);
  cudaEvent_t loaded = poolEvent();
  if (!batch.empty()) issueLoads(batch, loaded);
  const size_t tbl = 2 * (size_t)D + 2;  // words per segment table
  while (!batch.empty()) {
    // domain table, then segment tables: radiance bucket 0..rb-1, shadows
    DomainDev* sd = reinterpret_cast<DomainDev*>(h_stage);
    std::memcpy(sd, hdoms.data(), D * sizeof(DomainDev));
    // the device table of this batch marks them in place; later batches decide anew
    inplace_domains += (int64_t)inplace.size();
    for (int d : inplace) hdoms[d].resident = 0;
    uint32_t* seg = reinterpret_cast<uint32_t*>(h_stage + D * sizeof(DomainDev));
    std::vector<int> nseg(rb + 1, 0);
    for (int q = 0; q <= rb; ++q) {
      const bool shadow = q == rb;
      const bool on = shadow ? with_s : (with_r && q >= rb_first && q < rb_end);
      uint32_t* beg = seg + q * tbl;
      uint32_t* pre = beg + D + 1;
      uint32_t run = 0;
      if (on)
        for (int d : batch) {
          if (hlive[(shadow ? D : 0) + d] == 0) continue;
          const uint32_t b0 = shadow ? sk[d] : rk[q * D + d], b1 = shadow ? sk[d + 1] : rk[q * D + d + 1];
          if (b1 == b0) continue;
          beg[nseg[q]] = b0;
          pre[nseg[q]] = run;
          run += b1 - b0;
          ++nseg[q];
        }
      pre[nseg[q]] = run;
    }
    CK(cudaMemcpyAsync(d_domains, sd, D * sizeof(DomainDev), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_segs, seg, (rb + 1) * tbl * 4, cudaMemcpyHostToDevice, stream));
    // counts for the batch after this one, taken before this one traces
    counted = poolEvent();
    countLive(window(remaining), counted);
    CK(cudaStreamWaitEvent(stream, loaded, 0));
    // radiance buckets front to back (or predicted first), then the shadows
    for (int q = 0; q <= rb; ++q) {
      if (nseg[q] == 0) continue;
      const bool shadow = q == rb;
      CK(cudaMemsetAsync(d_work, 0, 4, stream));
      TraceArgs ta = traceArgs(shadow ? 0 : (rb > 1 ? 1 : 0), S);
      if (shadow) {
        ta.entries = d_sentries;
        ta.key_start = d_skey_start;
        ta.num_entries = d_snum_entries;
      }
      ta.seg_begin = d_segs + q * tbl;
      ta.seg_prefix = ta.seg_begin + D + 1;
      ta.nseg = nseg[q];
      cudaEvent_t e0 = poolEvent(), e1 = poolEvent();
      CK(cudaEventRecord(e0, stream));
      if (shadow) launchTraceOccluded(stream, ta, traceBlocks());
      else launchTraceClosest(stream, ta, traceBlocks());
      CK(cudaEventRecord(e1, stream));
      (shadow ? occl_events : trace_events).push_back({e0, e1});
      launches += 1;
    }
    // the counts (and every trace before this batch's) have completed: the
    // staging buffers are free and the next batch's copies can start
    CK(cudaEventSynchronize(counted));
    nextBatch(next);
    batch.swap(next);
    if (!batch.empty()) {
      // a cache too small for two batches copies only after the trace has finished
      if (2 * B > cache_capacity) CK(cudaStreamSynchronize(stream));
      loaded = poolEvent();
      issueLoads(batch, loaded);
    }
  }
  CK(cudaStreamSynchronize(stream));
}

// Out of core, batched (schedule_policy 2): the shadow rays of depth b and the
// radiance rays of depth b + 1 are both spawned by the shader at depth b and
// are independent of each other, so they are queued together and traced in
// one pass over the domains; depth b is retired after that pass.  The image is
// the same as the unbatched order's: only the order of the traced entries
// changes, and hits fold through the order-independent packed atomicMin.
void Tracer::traceWaveBatched(const Wave& w) {
  const int S = std::max(slots(), 1);
  const int nb_total = maxBounces();
  const int nblk = num_sms * kStreamBlocksPerSm;
  beginWave(w);
  // radiance queues keyed by depth bucket when culling, so each batch traces
  // its entries front to back (learned: predicted domain and those in front
  // of it first)
  const int order_by_depth = cfg.cull ? 1 : 0;
  const int rb = order_by_depth ? kDepthBuckets : 1;
  auto scheduleRadiance = [&](bool primary) {
    CK(cudaMemsetAsync(d_dstats, 0, (size_t)D * cfg.list_size * sizeof(long long), stream));
    cudaEvent_t s0 = poolEvent(), s1 = poolEvent();
    record(s0);
    const bool pred = learned() && proposal_trained;
    // with learn_buckets the schedule already ran the prediction (bucket
    // boundaries); otherwise the prediction only orders the domain loads
    const bool buckets = pred && order_by_depth && cfg.learn_buckets;
    schedule(false, order_by_depth, d_alive_count, d_alive_list, S, primary, false, buckets);
    record(s1);
    sched_events.push_back({s0, s1});
    if (pred) predictDomainCounts(!buckets);
  };
  scheduleRadiance(true);
  oocPass(true, false, S, rb);
  for (int b = 0; b < nb_total; ++b) {
    TraceArgs ta = traceArgs(0, S);
    launchResolve(stream, ta, d_hit_ns, nblk, false);
    if (learned() && !proposal_trained) collectPairs();
    CK(cudaMemsetAsync(d_next_flag, 0, (size_t)w.samples, stream));
    launchShade(stream, shadeArgs(b, S), nblk);
    launchCompact(stream, d_shadow_flag, d_alive_count, (uint32_t)S, 0, d_shadow_list, d_shadow_count,
                  nullptr, d_block_tmp, compact_blocks);
    launches += 5;
    schedule(true, 0, d_shadow_count, d_shadow_list, S, false, true);
    // this depth's alive list stays for the retire below (the next depth's
    // list goes to the other buffer)
    const uint32_t* retire_list = d_alive_list;
    const uint32_t* retire_count = d_alive_count;
    const bool more = b + 1 < nb_total;
    if (more) {
      launchCompact(stream, d_next_flag, nullptr, 1, (uint64_t)w.samples, d_alive_list2, d_alive_count2, nullptr,
                    d_block_tmp, compact_blocks);
      std::swap(d_alive_list, d_alive_list2);
      std::swap(d_alive_count, d_alive_count2);
      launches += 3;
      cur ^= 1;
      scheduleRadiance(false);
    }
    oocPass(more, true, S, rb);
    launchRetire(stream, d_image, d_views, retire_list, retire_count, rays[cur], sh, d_shadow_flag, S, nblk);
    launches += 1;
  }
}

// ---------------------------------------------------------------- proposal
// The learned domain-order proposal: parameters initialised He-uniform from
// a fixed seed, trained online on the (ray, candidates, winning position)
// pairs the exact tracer produces during its first frames, then consulted to
// order the trace.  It never decides a hit: every candidate entry is still
// traced or culled by a hit that is nearer than its domain.
namespace {
uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
}  // namespace

void Tracer::freeProposal() {
  devFree(d_mlp);
  devFree(d_mlp_partial);
  devFree(d_boxes);
  devFree(d_pairs);
  devFree(d_pairs_filled);
  devFree(d_predcount);
  devFree(d_mlp_err);
  devFree(d_mlp_eval);
  proposal_trained = false;
  frames_collected = 0;
  adam_step = 0;
  pairs_filled = 0;
}

void Tracer::setupProposal() {
  freeProposal();
  namespace ml = mlp;
  std::vector<float> p(3 * ml::kParams + ml::kPartial, 0.0f);
  uint64_t st = (uint64_t)cfg.learn_seed * 0x2545F4914F6CDD1Dull + 1;
  auto put = [&](int off, int rows, int cols, int real_rows, int real_cols, int fan_in) {
    const double lim = std::sqrt(6.0 / fan_in);
    for (int r = 0; r < real_rows; ++r)
      for (int c = 0; c < real_cols; ++c) {
        const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
        p[off + r * cols + c] = (float)((2.0 * u - 1.0) * lim);
      }
    (void)rows;
  };
  put(ml::kW1, ml::kHid, ml::kK, ml::kHid, ml::kIn, ml::kIn);
  put(ml::kW2, ml::kHid, ml::kHid, ml::kHid, ml::kHid, ml::kHid);
  put(ml::kW3, ml::kHid, ml::kHid, ml::kHid, ml::kHid, ml::kHid);
  put(ml::kW4, ml::kOutPad, ml::kHid, ml::kCand, ml::kHid, ml::kHid);
  devAlloc(&d_mlp, p.size());
  CK(cudaMemcpy(d_mlp, p.data(), p.size() * 4, cudaMemcpyHostToDevice));
  devAlloc(&d_mlp_partial, (size_t)ml::gradBlocks(num_sms) * ml::kPartial);
  // domain boxes and the normalisation of positions to the scene box
  std::vector<float> bx(6 * (size_t)D);
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int d = 0; d < D; ++d)
    for (int c = 0; c < 3; ++c) {
      bx[6 * d + c] = hdoms[d].bmin[c];
      bx[6 * d + 3 + c] = hdoms[d].bmax[c];
      lo[c] = std::min(lo[c], hdoms[d].bmin[c]);
      hi[c] = std::max(hi[c], hdoms[d].bmax[c]);
    }
  float half = 0.0f;
  for (int c = 0; c < 3; ++c) {
    mlp_norm.centre[c] = 0.5f * (lo[c] + hi[c]);
    half = std::max(half, 0.5f * (hi[c] - lo[c]));
  }
  mlp_norm.scale = half > 0.0f ? 1.0f / half : 1.0f;
  devAlloc(&d_boxes, bx.size());
  CK(cudaMemcpy(d_boxes, bx.data(), bx.size() * 4, cudaMemcpyHostToDevice));
  pairs_cap = (uint64_t)cfg.learn_samples;
  if (pairs_cap) devAlloc(&d_pairs, pairs_cap);
  devAlloc(&d_pairs_filled, 1);
  CK(cudaMemset(d_pairs_filled, 0, sizeof(unsigned long long)));
  devAlloc(&d_predcount, D);
  devAlloc(&d_mlp_err, 1);
  CK(cudaMemset(d_mlp_err, 0, sizeof(int)));
  devAlloc(&d_mlp_eval, 3);
}

mlp::ArenaSource Tracer::arenaSource() const {
  mlp::ArenaSource a;
  a.count = d_alive_count;
  a.list = d_alive_list;
  a.org = rays[cur].org;
  a.dir = rays[cur].dir;
  a.arena = d_arena;
  a.list_off = d_list_off;
  a.list_cnt = d_list_cnt;
  return a;
}

mlp::Net Tracer::proposalNet() const {
  mlp::Net n;
  n.params = d_mlp;
  n.boxes = d_boxes;
  n.norm = mlp_norm;
  n.error = d_mlp_err;
  return n;
}

// Training pairs of the radiance rays just resolved (their lists are still in
// the arena); the pair buffer fills in alive order up to its capacity.
void Tracer::collectPairs() {
  if (!pairs_cap) return;
  mlp::launchCollect(stream, arenaSource(), d_ray_key, d_domains, d_pairs, d_pairs_filled, pairs_cap, d_lab,
                     d_lflag, d_lsel, d_lnsel, d_block_tmp, compact_blocks);
  launches += 6;
}

// Predicted hits per domain for the out-of-core order (the prediction itself
// is already in d_pred when the schedule used it).
void Tracer::predictDomainCounts(bool run_predict) {
  CK(cudaMemsetAsync(d_predcount, 0, (size_t)D * 4, stream));
  // (atomics folded into the inference epilogue measured slower: they stall
  // the tensor-core tile loop more than this pass costs)
  if (run_predict) {
    mlp::launchPredictArena(stream, proposalNet(), arenaSource(), d_pred, num_sms * 5);
    launches += 1;
  }
  mlp::launchPredCount(stream, arenaSource(), d_pred, d_predcount, num_sms * 4);
  launches += 1;
  use_pred_order = true;
}

// learn_epochs passes of Adam (batch learn_batch) over the collected pairs.
void Tracer::trainProposal() {
  namespace ml = mlp;
  const int64_t all = std::min<int64_t>(pairs_filled, (int64_t)pairs_cap);
  // the last sixteenth of the pairs (at most 2^18) is held out to score the
  // trained proposal; the rest trains it
  const int64_t held = all >= 64 ? std::min<int64_t>(all / 16, 1 << 18) : 0;
  const int64_t n = all - held;
  cudaEvent_t e0 = poolEvent(), e1 = poolEvent();
  CK(cudaEventRecord(e0, stream));
  float* params = d_mlp;
  float* m = d_mlp + ml::kParams;
  float* v = d_mlp + 2 * ml::kParams;
  float* grad = d_mlp + 3 * ml::kParams;
  if (n > 0) {
    const int64_t B = std::min<int64_t>(cfg.learn_batch, n);
    const int64_t per_epoch = (n + B - 1) / B;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((B + ml::kTile - 1) / ml::kTile,
                                                                  ml::gradBlocks(num_sms)));
    for (int64_t k = 0; k < per_epoch * cfg.learn_epochs; ++k) {
      const int64_t start = (k % per_epoch) * B;
      const int64_t len = std::min<int64_t>(B, n - start);
      ml::launchGrad(stream, proposalNet(), d_pairs + start, len, 1.0f / (float)len, d_mlp_partial, grid);
      ml::launchReduceAdam(stream, d_mlp_partial, grid, grad, params, m, v, cfg.learn_lr, ++adam_step);
    }
  }
  CK(cudaEventRecord(e1, stream));
  unsigned long long ev[3] = {0ull, 0ull, 0ull};
  if (held > 0) {
    CK(cudaMemsetAsync(d_mlp_eval, 0, 3 * sizeof(unsigned long long), stream));
    ml::launchEvaluate(stream, proposalNet(), d_pairs + n, held, d_mlp_eval, num_sms * 5);
    CK(cudaMemcpyAsync(ev, d_mlp_eval, sizeof(ev), cudaMemcpyDeviceToHost, stream));
  }
  CK(cudaStreamSynchronize(stream));
  CK(cudaGetLastError());
  int err = 0;
  CK(cudaMemcpy(&err, d_mlp_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) throw std::runtime_error("a tensor-core wait of the learned proposal gave up");
  learn_eval_pairs = (int64_t)ev[0];
  learn_top1 = ev[0] ? (double)ev[1] / (double)ev[0] : 0.0;
  learn_top1_nearest = ev[0] ? (double)ev[2] / (double)ev[0] : 0.0;
  float tail[2] = {0.f, 0.f};
  if (n > 0) CK(cudaMemcpy(tail, grad + ml::kParams, sizeof(tail), cudaMemcpyDeviceToHost));
  learn_loss = tail[1] > 0.f ? tail[0] / tail[1] : 0.0;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  learn_ms = ms;
  proposal_trained = true;
  // the pair buffer is no longer needed
  devFree(d_pairs);
}

// Records every launch of an in-core frame (counter and image clears, all
// waves) into a CUDA graph.  Nothing in that sequence waits on the host: ray
// and entry counts stay on the device, the camera and tiles are read from
// device memory, so replaying the graph renders whatever camera was uploaded.
void Tracer::captureFrame() {
  dropGraph();
  const int64_t l0 = launches;
  sched_events.clear();
  trace_events.clear();
  occl_events.clear();
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed));
  capturing = true;
  try {
    CK(cudaMemsetAsync(d_ctr, 0, sizeof(Counters), stream));
    CK(cudaMemsetAsync(d_image, 0, (size_t)frame_pixels * sizeof(float4), stream));
    for (const Wave& w : waves) traceWave(w, false);
  } catch (...) {
    capturing = false;
    cudaStreamEndCapture(stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  capturing = false;
  CK(cudaStreamEndCapture(stream, &g));
  cudaError_t e = cudaGraphInstantiate(&graph_exec, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  graph_gen = buf_gen;
  graph_launches = launches - l0;
  graph_sched = sched_events;
  graph_trace = trace_events;
  graph_occl = occl_events;
}

// The bins of one view (bins_x per row) in lists[0 ..]: the domains whose
// projected, widened box touches each bin, nearest box first.
void Tracer::binView(const FrameView& f, std::vector<uint16_t>* lists, int bins_x) const {
  const int W = f.w, H = f.h;
  const CameraDev& cam = f.cam;
  // camera frame in double: P(u, v) = ll + u wv + v hv, viewing along -w
  double pos[3], ll[3], wv[3], hv[3], fw[3];
  for (int k = 0; k < 3; ++k) {
    pos[k] = cam.pos[k];
    ll[k] = cam.ll[k];
    wv[k] = cam.wv[k];
    hv[k] = cam.hv[k];
  }
  // forward = (centre of the image plane) - pos
  for (int k = 0; k < 3; ++k) fw[k] = (ll[k] + 0.5 * wv[k] + 0.5 * hv[k]) - pos[k];
  auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  const double fw2 = dot(fw, fw), wv2 = dot(wv, wv), hv2 = dot(hv, hv);
  // domains by distance from the camera to their boxes, so that each bin's
  // list is close to the entry order of its rays
  std::vector<std::pair<double, int>> near(D);
  for (int d = 0; d < D; ++d) {
    double q2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double c = std::min(std::max(pos[k], (double)hdoms[d].bmin[k]), (double)hdoms[d].bmax[k]);
      q2 += (c - pos[k]) * (c - pos[k]);
    }
    near[d] = {q2, d};
  }
  std::sort(near.begin(), near.end());
  for (const auto& nd : near) {
    const int d = nd.second;
    const DomainDev& dd = hdoms[d];
    double umin = 1e300, umax = -1e300, vmin = 1e300, vmax = -1e300;
    bool everywhere = false;
    for (int c = 0; c < 8 && !everywhere; ++c) {
      double q[3] = {((c & 1) ? dd.bmax[0] : dd.bmin[0]) - pos[0], ((c & 2) ? dd.bmax[1] : dd.bmin[1]) - pos[1],
                     ((c & 4) ? dd.bmax[2] : dd.bmin[2]) - pos[2]};
      double depth = dot(q, fw) / fw2;  // 1 on the image plane
      if (!(depth > 1e-6)) {
        everywhere = true;
        break;
      }
      double p[3];
      for (int k = 0; k < 3; ++k) p[k] = pos[k] + q[k] / depth - ll[k];
      double u = dot(p, wv) / wv2, v = dot(p, hv) / hv2;
      umin = std::min(umin, u);
      umax = std::max(umax, u);
      vmin = std::min(vmin, v);
      vmax = std::max(vmax, v);
    }
    int x0 = 0, x1 = W - 1, y0 = 0, y1 = H - 1;
    if (!everywhere) {
      double fx0 = umin * W - 2.0, fx1 = umax * W + 2.0, fy0 = vmin * H - 2.0, fy1 = vmax * H + 2.0;
      if (fx1 < 0.0 || fy1 < 0.0 || fx0 > W || fy0 > H) continue;
      x0 = (int)std::max(0.0, std::floor(fx0));
      x1 = (int)std::min((double)(W - 1), std::ceil(fx1));
      y0 = (int)std::max(0.0, std::floor(fy0));
      y1 = (int)std::min((double)(H - 1), std::ceil(fy1));
    }
    for (int by = y0 / kBinSize; by <= y1 / kBinSize; ++by)
      for (int bx = x0 / kBinSize; bx <= x1 / kBinSize; ++bx) lists[by * bins_x + bx].push_back((uint16_t)d);
  }
}

// Screen bins of the primary rays, per view.  Each domain box is projected
// through the view's camera onto its image plane; the pixel rectangle of its 8
// corners, widened by two pixels, lists the domain in every bin it touches.  A
// box with a corner at or behind the camera plane is listed everywhere.  A ray
// can only pass the exact slab test of a box whose projection contains its
// pixel, so the per-bin lists are supersets of what the full test would find.
// The views' bins lie back to back in one table (ViewDev::bin_base, bins_x).
void Tracer::buildScreenBins() {
  // the bins depend only on the cameras, the image sizes and the domain boxes:
  // unchanged since the last build, the device copy is still current
  const size_t vk = sizeof(CameraDev) + 2 * sizeof(int);
  std::vector<unsigned char> key(fviews.size() * vk);
  for (size_t v = 0; v < fviews.size(); ++v) {
    std::memcpy(key.data() + v * vk, &fviews[v].cam, sizeof(CameraDev));
    std::memcpy(key.data() + v * vk + sizeof(CameraDev), &fviews[v].w, sizeof(int));
    std::memcpy(key.data() + v * vk + sizeof(CameraDev) + sizeof(int), &fviews[v].h, sizeof(int));
  }
  const bool current = key == bins_key && d_bin_start && d_bin_ids;
  if (!current) {
    bins_key = key;
    bin_view_base.assign(fviews.size(), 0);
    bin_view_x.assign(fviews.size(), 0);
  }
  int nb = 0;
  for (size_t v = 0; v < fviews.size(); ++v) {
    if (!current) {
      bin_view_base[v] = nb;
      bin_view_x[v] = (fviews[v].w + kBinSize - 1) / kBinSize;
    }
    hviews[v].bin_base = bin_view_base[v];
    hviews[v].bins_x = bin_view_x[v];
    nb += bin_view_x[v] * ((fviews[v].h + kBinSize - 1) / kBinSize);
  }
  if (current) return;
  std::vector<std::vector<uint16_t>> lists(nb);
  for (size_t v = 0; v < fviews.size(); ++v) binView(fviews[v], lists.data() + bin_view_base[v], bin_view_x[v]);
  std::vector<uint32_t> start(nb + 1, 0);
  for (int b = 0; b < nb; ++b) start[b + 1] = start[b] + (uint32_t)lists[b].size();
  std::vector<uint16_t> ids(std::max<uint32_t>(start[nb], 1));
  for (int b = 0; b < nb; ++b) std::copy(lists[b].begin(), lists[b].end(), ids.begin() + start[b]);
  if ((size_t)(nb + 1) > bin_start_cap) {
    devFree(d_bin_start);
    bin_start_cap = nb + 1;
    devAlloc(&d_bin_start, bin_start_cap);
    ++buf_gen;
  }
  if (ids.size() > bin_ids_cap) {
    // headroom, so that camera moves rarely reallocate (and recapture)
    devFree(d_bin_ids);
    bin_ids_cap = ids.size() + ids.size() / 2;
    devAlloc(&d_bin_ids, bin_ids_cap);
    ++buf_gen;
  }
  CK(cudaMemcpyAsync(d_bin_start, start.data(), start.size() * 4, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(d_bin_ids, ids.data(), ids.size() * 2, cudaMemcpyHostToDevice, stream));
  CK(cudaStreamSynchronize(stream));  // the host vectors are freed on return
  h2d_bytes += start.size() * 4 + ids.size() * 2;
}

// One frame of the configured view (Tracer::trace, ooc_tracer.inl:184-234).
void Tracer::trace(float* out, bool out_is_device, spray_gpu_stats* st) {
  if (!has_scene) throw StateError("trace before set_scene");
  if (!has_camera) throw StateError("trace before set_camera");
  FrameView v;
  v.cam = cam;
  v.w = cfg.image_w;
  v.h = cfg.image_h;
  v.spp = cfg.pixel_samples;
  v.ao_mode = cfg.ao_mode;
  v.ao_samples = cfg.ao_samples;
  v.bounces = cfg.bounces;
  v.rr_depth = cfg.rr_depth;
  v.ao_light_shadow = cfg.ao_light_shadow;
  v.ao_max_distance = cfg.ao_max_distance;
  fviews.assign(1, v);
  traceFrame(out, out_is_device, st);
}

// Several views in one frame: their tiles share the wavefronts, so every
// stage runs once per depth for all of them (multi-view batch).
void Tracer::traceViews(const spray_gpu_view* views, int n, float* out, bool out_is_device, spray_gpu_stats* st) {
  if (!has_scene) throw StateError("trace before set_scene");
  if (n <= 0 || n > 65535) throw std::invalid_argument("num_views must be in [1, 65535]");
  std::vector<FrameView> fv(n);
  for (int k = 0; k < n; ++k) {
    const spray_gpu_view& s = views[k];
    if (s.image_w <= 0 || s.image_h <= 0 || s.pixel_samples <= 0 || s.bounces <= 0 || s.ao_samples <= 0)
      throw std::invalid_argument("view " + std::to_string(k) + ": sizes, samples and bounces must be positive");
    if (!s.ao_mode && lights.empty())
      throw std::invalid_argument("view " + std::to_string(k) + ": path tracing needs at least one light");
    FrameView& v = fv[k];
    v.cam = makeCamera(s.position, s.lookat, s.up, s.vfov, s.image_w, s.image_h);
    v.w = s.image_w;
    v.h = s.image_h;
    v.spp = s.pixel_samples;
    v.ao_mode = s.ao_mode;
    v.ao_samples = s.ao_samples;
    v.bounces = s.bounces;
    v.rr_depth = s.rr_depth;
    v.ao_light_shadow = s.ao_light_shadow;
    v.ao_max_distance = s.ao_max_distance;
    if (slotsFor(v.ao_mode, v.ao_samples, v.ao_light_shadow) > kMaxSlots)
      throw std::invalid_argument("view " + std::to_string(k) + ": too many shadow rays per hit (max 64)");
  }
  fviews.swap(fv);
  traceFrame(out, out_is_device, st);
}

void Tracer::traceFrame(float* out, bool out_is_device, spray_gpu_stats* st) {
  CK(cudaSetDevice(cfg.device));
  planWaves();
  int64_t maxw = 0;
  for (auto& w : waves) maxw = std::max(maxw, w.samples);
  for (int attempt = 0; attempt < 4; ++attempt) {
    ensureBuffers(maxw);
    launches = 0;
    h2d_bytes = 0;
    d2h_bytes = 0;
    domain_loads = 0;
    inplace_domains = 0;
    reduce_bytes = 0;
    ev_used = 0;
    sched_events.clear();
    trace_events.clear();
    occl_events.clear();
    copy_events.clear();
    dbg.clear();
    dbg[{SPRAY_DBG_LOADS, 0}];  // the request log exists for every frame (empty in core)
    load_pass = 0;
    rounds = 0;
    visits_shade = 0;
    use_pred_order = false;
    CK(cudaEventRecord(ev_start, stream));
    if (use_bins) buildScreenBins();
    CK(cudaMemcpyAsync(d_views, hviews.data(), hviews.size() * sizeof(ViewDev), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tiles, wave_tiles.data(), wave_tiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice,
                       stream));
    h2d_bytes += hviews.size() * sizeof(ViewDev) + wave_tiles.size() * sizeof(TileDev);
    const bool graphed = cfg.graphs && !ooc && !cfg.debug_capture && !learned() && !situ() && !rounded();
    if (graphed) {
      if (!graph_exec || graph_gen != buf_gen) captureFrame();
      CK(cudaGraphLaunch(graph_exec, stream));
      launches = graph_launches;
      sched_events = graph_sched;
      trace_events = graph_trace;
      occl_events = graph_occl;
    } else {
      CK(cudaMemsetAsync(d_ctr, 0, sizeof(Counters), stream));
      CK(cudaMemsetAsync(d_image, 0, (size_t)frame_pixels * sizeof(float4), stream));
      if (rounded()) {
        traceRounds();
      } else {
        for (size_t k = 0; k < waves.size(); ++k) {
          const bool capture = cfg.debug_capture && k == 0;
          if (ooc && (cfg.schedule_policy == 2 || cfg.schedule_policy == 3) && !capture)
            traceWaveBatched(waves[k]);
          else traceWave(waves[k], capture);
        }
      }
    }
    CK(cudaEventRecord(ev_stop, stream));
    Counters ctr;
    CK(cudaMemcpyAsync(&ctr, d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    if (ctr.arena_overflows || ctr.entry_overflows) {
      dropGraph();
      needed_entries = cap_entries * 2;
      continue;  // retrace with larger queues
    }
    if (ctr.list_overflows) throw OverflowError("a ray overlapped more than 32 domains");
    if (ctr.error_flags & (kErrBadNode | kErrTraversalBound))
      throw std::runtime_error("BVH traversal left its bounds (corrupt hierarchy)");
    learn_ms = 0.0;
    if (learned() && !proposal_trained) {
      unsigned long long filled = 0;
      CK(cudaMemcpy(&filled, d_pairs_filled, sizeof(filled), cudaMemcpyDeviceToHost));
      pairs_filled = (int64_t)filled;
      if (++frames_collected >= cfg.learn_frames || filled >= pairs_cap) trainProposal();
    }
    size_t img_bytes = (size_t)frame_pixels * sizeof(float4);
    if (out) {
      if (out_is_device) {
        CK(cudaMemcpyAsync(out, d_image, img_bytes, cudaMemcpyDeviceToDevice, stream));
      } else {
        CK(cudaMemcpyAsync(out, d_image, img_bytes, cudaMemcpyDeviceToHost, stream));
        d2h_bytes += img_bytes;
      }
      CK(cudaStreamSynchronize(stream));
    }
    if (st) {
      std::memset(st, 0, sizeof(*st));
      st->rays_primary = (int64_t)ctr.rays_primary;
      st->rays_shadow = (int64_t)ctr.rays_shadow;
      st->rays_bounce = (int64_t)ctr.rays_bounce;
      st->visits_radiance = (int64_t)ctr.visits_radiance;
      st->visits_shadow = (int64_t)ctr.visits_shadow;
      st->visits_culled = (int64_t)ctr.visits_culled;
      st->domain_loads = domain_loads;
      st->h2d_bytes = (int64_t)h2d_bytes;
      st->d2h_bytes = (int64_t)d2h_bytes;
      st->kernel_launches = launches;
      st->list_overflows = (int64_t)ctr.list_overflows;
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ev_start, ev_stop));
      st->frame_ms = ms;
      auto sum = [](const std::vector<std::pair<cudaEvent_t, cudaEvent_t>>& v) {
        double acc = 0.0;
        for (auto& p : v) {
          float m = 0.f;
          if (cudaEventElapsedTime(&m, p.first, p.second) == cudaSuccess) acc += m;
        }
        return acc;
      };
      st->trace_ms = sum(trace_events);
      st->occlude_ms = sum(occl_events);
      st->schedule_ms = sum(sched_events);
      st->trace_launches = (int64_t)trace_events.size();
      st->occlude_launches = (int64_t)occl_events.size();
      st->nodes_radiance = (int64_t)ctr.nodes_radiance;
      st->tris_radiance = (int64_t)ctr.tris_radiance;
      st->nodes_shadow = (int64_t)ctr.nodes_shadow;
      st->tris_shadow = (int64_t)ctr.tris_shadow;
      st->scene_triangles = (int64_t)total_tris;
      st->scene_bytes = (int64_t)scene_bytes;
      st->h2d_ms = sum(copy_events);
      st->learn_pairs = pairs_filled;
      st->learn_trained = proposal_trained ? 1 : 0;
      st->learn_ms = learn_ms;
      st->learn_loss = learn_loss;
      st->inplace_domains = inplace_domains;
      st->inplace_bytes = (int64_t)(ctr.nodes_inplace * sizeof(BvhNode4) + ctr.tris_inplace * 3 * sizeof(float4) +
                                    ctr.hits_inplace * (3 * 4 + 3 * 4 + 9 * 4));
      st->cache_slots = ooc ? cache_capacity : 0;
      st->cache_slot_bytes = ooc ? (int64_t)cache_slot_bytes : 0;
      st->learn_eval_pairs = learn_eval_pairs;
      st->learn_top1 = learn_top1;
      st->learn_top1_nearest = learn_top1_nearest;
      st->exchange_bytes = reduce_bytes;
      st->rounds = rounds;
      st->visits_shade = visits_shade;
      st->eyes_culled = (int64_t)ctr.eyes_culled;
    }
    return;
  }
  throw std::runtime_error("queue capacity could not be grown enough");
}

// ---------------------------------------------------------------- debug
template <class T>
static std::vector<T> fetch(const T* d, size_t n, cudaStream_t s) {
  std::vector<T> h(n);
  if (n) {
    CK(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  return h;
}
static uint32_t fetch1(const uint32_t* d, cudaStream_t s) { return fetch(d, 1, s)[0]; }

void Tracer::captureRays(int b) {
  uint32_t n = fetch1(d_alive_count, stream);
  auto list = fetch(d_alive_list, n, stream);
  auto org = fetch(rays[cur].org, cap_samples, stream);
  auto dir = fetch(rays[cur].dir, cap_samples, stream);
  auto wgt = fetch(rays[cur].wgt, cap_samples, stream);
  auto pix = fetch(d_pixid, cap_samples, stream);
  auto sam = fetch(d_samid, cap_samples, stream);
  std::vector<char>& out = dbg[{SPRAY_DBG_RAYS, b}];
  out.resize(n * sizeof(spray_gpu_dbg_ray));
  auto* r = (spray_gpu_dbg_ray*)out.data();
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t s = list[i];
    r[i].sample = s;
    r[i].pixid = pix[s];
    r[i].samid = sam[s];
    // primary rays carry weight 1 (not stored: the shader knows depth 0)
    float4 o = org[s], d = dir[s], w = b == 0 ? make_float4(1.f, 1.f, 1.f, 0.f) : wgt[s];
    float ov[3] = {o.x, o.y, o.z}, dv[3] = {d.x, d.y, d.z}, wv[3] = {w.x, w.y, w.z};
    std::memcpy(r[i].org, ov, 12);
    std::memcpy(r[i].dir, dv, 12);
    std::memcpy(r[i].w, wv, 12);
  }
}

void Tracer::captureQueues(int what, int b, int order_by_depth) {
  uint32_t E = fetch1(d_num_entries, stream);
  const int nkeys = order_by_depth ? kDepthBuckets * D : D;
  auto ks = fetch(d_key_start, nkeys + 1, stream);
  auto ent = fetch(d_entries, E, stream);
  std::vector<uint8_t> dep = d_dbg_depth ? fetch(d_dbg_depth, E, stream) : std::vector<uint8_t>(E, 0xff);
  std::vector<char>& out = dbg[{what, b}];
  out.resize(E * sizeof(spray_gpu_dbg_entry));
  auto* r = (spray_gpu_dbg_entry*)out.data();
  int key = 0;
  for (uint32_t e = 0; e < E; ++e) {
    while (key + 1 < nkeys && ks[key + 1] <= e) ++key;
    r[e].domain = key % D;
    r[e].ray = ent[e].x & kRayIdMask;
    float t;
    std::memcpy(&t, &ent[e].y, 4);
    r[e].tdom = t;
    r[e].depth = dep[e] == 0xff ? -1 : (int32_t)dep[e];
    r[e].origin = (int32_t)(ent[e].x >> 31);
  }
}

void Tracer::captureScores(int b) {
  auto sc = fetch(d_scores, D, stream);
  auto od = fetch(d_order, D, stream);
  std::vector<char>& out = dbg[{SPRAY_DBG_SCORES, b}];
  out.resize(D * sizeof(spray_gpu_dbg_score));
  auto* r = (spray_gpu_dbg_score*)out.data();
  for (int d = 0; d < D; ++d) {
    r[d].domain = d;
    r[d].score = sc[d];
    r[d].order = -1;
  }
  for (int k = 0; k < D; ++k) r[od[k]].order = k;
}

void Tracer::captureHits(int b) {
  uint32_t n = fetch1(d_alive_count, stream);
  auto list = fetch(d_alive_list, n, stream);
  auto key = fetch(d_ray_key, cap_samples, stream);
  auto ns = fetch(d_hit_ns, cap_samples, stream);
  std::vector<char>& out = dbg[{SPRAY_DBG_HITS, b}];
  out.resize(n * sizeof(spray_gpu_dbg_hit));
  auto* r = (spray_gpu_dbg_hit*)out.data();
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t s = list[i];
    r[i].sample = s;
    uint64_t k = key[s];
    if (k == kNoHit) {
      r[i].hit = 0;
      r[i].t = INFINITY;
      r[i].domain = -1;
      r[i].prim = -1;
      r[i].color = 0;
      r[i].ns[0] = r[i].ns[1] = r[i].ns[2] = 0.f;
      continue;
    }
    r[i].hit = 1;
    r[i].t = hitKeyT(k);
    uint32_t g = (uint32_t)k;
    int d = 0;
    while (d + 1 < D && hdoms[d + 1].gprim_base <= g) ++d;
    r[i].domain = d;
    r[i].prim = (int32_t)(g - hdoms[d].gprim_base);
    float4 h = ns[s];
    std::memcpy(&r[i].color, &h.w, 4);
    r[i].ns[0] = h.x;
    r[i].ns[1] = h.y;
    r[i].ns[2] = h.z;
  }
}

void Tracer::captureShadows(int b, int S) {
  uint32_t n = fetch1(d_alive_count, stream);
  auto list = fetch(d_alive_list, n, stream);
  size_t ns = (size_t)n * S;
  auto flag = fetch(d_shadow_flag, ns, stream);
  auto dir = fetch(sh.dir, ns, stream);
  auto wgt = fetch(sh.wgt, ns, stream);
  auto occ = fetch(sh.occluded, ns, stream);
  auto hp = fetch(sh.hitpos, n, stream);
  std::vector<char>& out = dbg[{SPRAY_DBG_SHADOWS, b}];
  out.clear();
  for (uint32_t a = 0; a < n; ++a)
    for (int k = 0; k < S; ++k) {
      size_t sid = (size_t)a * S + k;
      if (!flag[sid]) continue;
      spray_gpu_dbg_shadow r;
      r.sample = list[a];
      r.slot = k;
      r.org[0] = hp[a].x;
      r.org[1] = hp[a].y;
      r.org[2] = hp[a].z;
      r.dir[0] = dir[sid].x;
      r.dir[1] = dir[sid].y;
      r.dir[2] = dir[sid].z;
      r.tmax = dir[sid].w;
      r.w[0] = wgt[sid].x;
      r.w[1] = wgt[sid].y;
      r.w[2] = wgt[sid].z;
      r.occluded = occ[sid];
      const char* p = (const char*)&r;
      out.insert(out.end(), p, p + sizeof(r));
    }
}

int64_t Tracer::debugCount(int what, int bounce) const {
  auto it = dbg.find({what, bounce});
  if (it == dbg.end()) return -1;
  static const size_t sizes[] = {sizeof(spray_gpu_dbg_ray), sizeof(spray_gpu_dbg_entry),
                                 sizeof(spray_gpu_dbg_hit), sizeof(spray_gpu_dbg_shadow),
                                 sizeof(spray_gpu_dbg_entry), sizeof(spray_gpu_dbg_score),
                                 sizeof(spray_gpu_dbg_load)};
  return (int64_t)(it->second.size() / sizes[what]);
}

const std::vector<char>* Tracer::debugData(int what, int bounce) const {
  auto it = dbg.find({what, bounce});
  return it == dbg.end() ? nullptr : &it->second;
}

// The BVH nodes (SPRAY_DBG_NODES) or the leaf-ordered triangles
// (SPRAY_DBG_TRIS) of domain d as set_scene built them: from the device in
// core, from the pinned host copy out of core.  Null for a domain this tracer
// did not build (another rank's, in situ).
const std::vector<char>* Tracer::domainBvh(int what, int d) {
  if (!has_scene || d < 0 || d >= D) return nullptr;
  const DomainDev& dd = hdoms[d];
  if (dd.num_nodes <= 0) return nullptr;
  const bool nodes = what == SPRAY_DBG_NODES;
  const size_t nb = nodes ? (size_t)dd.num_nodes * sizeof(BvhNode4) : (size_t)dd.num_tris * 3 * sizeof(float4);
  std::vector<char>& v = bvh_dump[{what, d}];
  v.resize(nb);
  if (ooc) {
    const char* q = h_pinned + host_off[d] + (nodes ? 0 : (size_t)dd.num_nodes * sizeof(BvhNode4));
    std::memcpy(v.data(), q, nb);
  } else {
    const void* src = nodes ? (const void*)(d_nodes + dd.node_base) : (const void*)(d_tris + 3 * (size_t)dd.tri_base);
    CK(cudaMemcpy(v.data(), src, nb, cudaMemcpyDeviceToHost));
  }
  return &v;
}

}  // namespace spray

// ====================================================================== C ABI
using spray::fail;

#define API_GUARD(body)                                                  \
  try {                                                                  \
    body                                                                 \
  } catch (const spray::CudaError& e) {                                  \
    return fail(SPRAY_GPU_ECUDA, e.what());                              \
  } catch (const spray::StateError& e) {                                 \
    return fail(SPRAY_GPU_ESTATE, e.what());                             \
  } catch (const spray::OverflowError& e) {                              \
    return fail(SPRAY_GPU_EOVERFLOW, e.what());                          \
  } catch (const spray::IoError& e) {                                    \
    return fail(SPRAY_GPU_EIO, e.what());                                \
  } catch (const std::invalid_argument& e) {                             \
    return fail(SPRAY_GPU_EINVAL, e.what());                             \
  } catch (const std::bad_alloc&) {                                      \
    return fail(SPRAY_GPU_ENOMEM, "host allocation failed");             \
  } catch (const std::exception& e) {                                    \
    return fail(SPRAY_GPU_ECUDA, e.what());                              \
  }

struct spray_gpu_tracer {
  std::unique_ptr<spray::Tracer> impl;
};

extern "C" {

void spray_gpu_config_defaults(spray_gpu_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->image_w = 400;
  c->image_h = 400;
  c->ao_mode = 0;
  c->ao_samples = 8;
  c->pixel_samples = 4;
  c->bounces = 1;
  c->fov = 90.0f;
  c->cache_size = -1;
  c->max_samples_per_rank = 1024 * 1024;
  c->list_size = 16;
  c->history_size = 4;
  c->nthreads = 1;
  c->num_ranks = 1;
  c->rank = 0;
  c->cull = 1;
  c->learn_samples = (int64_t)1 << 24;
  c->learn_batch = 65536;
  c->learn_epochs = 2;
  c->learn_lr = 1e-3f;
  c->learn_seed = 1;
  c->learn_frames = 4;
  c->graphs = 1;
  c->ooc_inplace = 16384;
  c->bvh_device = 1;
}

const char* spray_gpu_last_error(void) { return spray::g_last_error.c_str(); }

int spray_gpu_create(const spray_gpu_config* cfg, spray_gpu_tracer** out) {
  if (!cfg || !out) return fail(SPRAY_GPU_EINVAL, "null argument");
  *out = nullptr;
  API_GUARD({
    auto t = std::make_unique<spray_gpu_tracer>();
    t->impl = std::make_unique<spray::Tracer>(*cfg);
    *out = t.release();
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_destroy(spray_gpu_tracer* t) {
  if (!t) return SPRAY_GPU_OK;
  delete t;
  return SPRAY_GPU_OK;
}

int spray_gpu_set_scene(spray_gpu_tracer* t, const spray_gpu_domain* domains, int32_t num_domains,
                        const spray_gpu_light* lights, int32_t num_lights) {
  if (!t || !domains || (num_lights > 0 && !lights)) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    t->impl->setScene(domains, num_domains, lights, num_lights);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_set_scene_prepared(spray_gpu_tracer* t, const char* dir, int32_t num_domains,
                                 const spray_gpu_light* lights, int32_t num_lights) {
  if (!t || !dir || (num_lights > 0 && !lights)) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    t->impl->setScenePrepared(dir, num_domains, lights, num_lights);
    return SPRAY_GPU_OK;
  })
}

int spray_scene_prepare(const spray_gpu_domain* domains, int32_t num_domains, const char* dir) {
  if (!domains || !dir) return fail(SPRAY_GPU_EINVAL, "null argument");
  if (num_domains <= 0) return fail(SPRAY_GPU_EINVAL, "a scene needs at least one domain");
  API_GUARD({
    spray::prepareScene(domains, num_domains, dir);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_set_camera(spray_gpu_tracer* t, const float pos[3], const float lookat[3],
                         const float up[3], float vfov) {
  if (!t || !pos || !lookat || !up) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    t->impl->setCamera(pos, lookat, up, vfov);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_set_insitu(spray_gpu_tracer* t, int32_t num_ranks, int32_t rank,
                         const spray_gpu_reduce_ops* ops) {
  if (!t) return fail(SPRAY_GPU_EINVAL, "null tracer");
  API_GUARD({
    t->impl->setInsitu(num_ranks, rank, ops);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_insitu_partition(const float* domain_bounds, int32_t num_domains, int32_t num_ranks,
                               int32_t* owner) {
  if (!domain_bounds || !owner) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    std::vector<int> o = spray::insituPartition(domain_bounds, num_domains, num_ranks);
    for (int d = 0; d < num_domains; ++d) owner[d] = o[d];
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_trace(spray_gpu_tracer* t, float* rgba_out, spray_gpu_stats* stats) {
  if (!t) return fail(SPRAY_GPU_EINVAL, "null tracer");
  API_GUARD({
    t->impl->trace(rgba_out, false, stats);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_trace_device(spray_gpu_tracer* t, float* rgba_dev, spray_gpu_stats* stats) {
  if (!t) return fail(SPRAY_GPU_EINVAL, "null tracer");
  API_GUARD({
    t->impl->trace(rgba_dev, true, stats);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_trace_views(spray_gpu_tracer* t, const spray_gpu_view* views, int32_t num_views, float* images,
                          spray_gpu_stats* stats) {
  if (!t || !views) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    t->impl->traceViews(views, num_views, images, false, stats);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_trace_views_device(spray_gpu_tracer* t, const spray_gpu_view* views, int32_t num_views,
                                 float* images, spray_gpu_stats* stats) {
  if (!t || !views) return fail(SPRAY_GPU_EINVAL, "null argument");
  API_GUARD({
    t->impl->traceViews(views, num_views, images, true, stats);
    return SPRAY_GPU_OK;
  })
}

int spray_gpu_debug_count(spray_gpu_tracer* t, int32_t what, int32_t bounce, int64_t* count) {
  if (!t || !count) return fail(SPRAY_GPU_EINVAL, "null argument");
  if (what == SPRAY_DBG_NODES || what == SPRAY_DBG_TRIS) {
    API_GUARD({
      const std::vector<char>* d = t->impl->domainBvh(what, bounce);
      if (!d) return fail(SPRAY_GPU_EINVAL, "no BVH for that domain here");
      *count = (int64_t)(d->size() / (what == SPRAY_DBG_NODES ? sizeof(spray::BvhNode4) : 3 * sizeof(float4)));
      return SPRAY_GPU_OK;
    })
  }
  if (what < 0 || what > SPRAY_DBG_LOADS) return fail(SPRAY_GPU_EINVAL, "unknown debug buffer");
  int64_t n = t->impl->debugCount(what, bounce);
  if (n < 0) return fail(SPRAY_GPU_ESTATE, "no captured buffer (set debug_capture and trace)");
  *count = n;
  return SPRAY_GPU_OK;
}

int spray_gpu_debug_copy(spray_gpu_tracer* t, int32_t what, int32_t bounce, void* out, int64_t capacity) {
  if (!t || !out) return fail(SPRAY_GPU_EINVAL, "null argument");
  const bool bvh = what == SPRAY_DBG_NODES || what == SPRAY_DBG_TRIS;
  if (!bvh && (what < 0 || what > SPRAY_DBG_LOADS)) return fail(SPRAY_GPU_EINVAL, "unknown debug buffer");
  const std::vector<char>* d = nullptr;
  if (bvh) {
    API_GUARD({ d = t->impl->domainBvh(what, bounce); })
    if (!d) return fail(SPRAY_GPU_EINVAL, "no BVH for that domain here");
  } else {
    d = t->impl->debugData(what, bounce);
  }
  if (!d) return fail(SPRAY_GPU_ESTATE, "no captured buffer (set debug_capture and trace)");
  if ((int64_t)d->size() > capacity) return fail(SPRAY_GPU_EINVAL, "output buffer too small");
  std::memcpy(out, d->data(), d->size());
  return SPRAY_GPU_OK;
}

}  // extern "C"
