// CPU oracle: restatement of SpRay's speculative domain-parallel ray-tracing
// loop.  TEST INFRASTRUCTURE ONLY -- see oracle.h.  Compile with
// -ffp-contract=off so that every float expression rounds once per operation,
// like the CUDA path compiled with -fmad=false.
#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <queue>
#include <stdexcept>
#include <vector>

namespace orc {

const float kInf = std::numeric_limits<float>::infinity();
const float kEps = 0.001f;                       // SPRAY_RAY_EPSILON (src/render/spray.h:51)
const float kOneOverPi = 0.3183098861837907f;    // SPRAY_ONE_OVER_PI (spray.h:55)
const double kOneOver255 = 0.00392156862745098;  // SPRAY_1_OVER_255 (spray.h:59)
const int kMaxHistory = 8;

// ---------------------------------------------------------------- vectors
struct F3 {
  float x, y, z;
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
inline F3 add(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 neg(F3 a) { return F3{-a.x, -a.y, -a.z}; }
inline F3 mul(F3 a, F3 b) { return F3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline F3 muls(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
inline F3 smul(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }
inline F3 divs(F3 a, float s) { return F3{a.x / s, a.y / s, a.z / s}; }
// glm::dot for vec3: (x*x' + y*y') + z*z'
inline float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline F3 cross(F3 a, F3 b) {
  return F3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
// glm::normalize = v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt
inline F3 normalize(F3 v) { return muls(v, 1.0f / std::sqrt(dot(v, v))); }
inline float gmax(float x, float y) { return (x < y) ? y : x; }
inline float gmin(float x, float y) { return (y < x) ? y : x; }
inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
inline bool hasPositive(F3 v) { return v.x > 0.0f || v.y > 0.0f || v.z > 0.0f; }  // utils/math.h:76

// ---------------------------------------------------------------- RNG
// RandomSampler (deps/embree/random_sampler.h:34-108)
struct RandomSampler {
  uint32_t s;
};
inline uint32_t murmurMix(uint32_t hash, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  hash ^= k;
  hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
  return hash;
}
inline uint32_t murmurFinalize(uint32_t hash) {
  hash ^= hash >> 16;
  hash *= 0x85ebca6bu;
  hash ^= hash >> 13;
  hash *= 0xc2b2ae35u;
  hash ^= hash >> 16;
  return hash;
}
inline void samplerInit(RandomSampler& r, int id) { r.s = murmurFinalize(murmurMix(0u, (uint32_t)id)); }
inline float samplerGet1D(RandomSampler& r) {
  r.s = r.s * 1664525u + 1013904223u;
  return (float)(int)(r.s >> 1) * 4.656612873077392578125e-10f;
}

// ---------------------------------------------------------------- sin/cos
// Taylor polynomials after Cody-Waite reduction by pi/2; the same operation
// sequence as the CUDA path so both agree bit for bit (glm's cos/sin are not
// pinned by any test of the reference).
void sinCos(float x, float* so, float* co) {
  float q = x * 0.636619772367581343f;
  int k = (int)(q >= 0.0f ? q + 0.5f : q - 0.5f);
  float kf = (float)k;
  float r = x - kf * 1.5703125f;
  r = r - kf * 4.838267923332751e-4f;
  r = r - kf * 2.5632829192545614e-12f;
  float r2 = r * r;
  float sp = 2.75573192e-6f;
  sp = sp * r2 + -1.98412698e-4f;
  sp = sp * r2 + 8.33333333e-3f;
  sp = sp * r2 + -1.66666667e-1f;
  float sn = r + (r * r2) * sp;
  float cp = -2.75573192e-7f;
  cp = cp * r2 + 2.48015873e-5f;
  cp = cp * r2 + -1.38888889e-3f;
  cp = cp * r2 + 4.16666667e-2f;
  cp = cp * r2 + -0.5f;
  float cs = 1.0f + r2 * cp;
  switch (k & 3) {
    case 0: *so = sn; *co = cs; break;
    case 1: *so = cs; *co = -sn; break;
    case 2: *so = -sn; *co = -cs; break;
    default: *so = -cs; *co = sn; break;
  }
}

float powInt(float x, float e) {
  if (e >= 0.0f && e <= 256.0f && (float)(int)e == e) {
    int n = (int)e;
    float r = 1.0f, b = x;
    while (n) {
      if (n & 1) r = r * b;
      b = b * b;
      n >>= 1;
    }
    return r;
  }
  return std::pow(x, e);
}

// ---------------------------------------------------------------- sampling
// ConcentricDiskSampling (src/render/sampler.h:49-92)
void concentricDisk(float u1, float u2, float* dx, float* dy) {
  float r, theta;
  float sx = 2 * u1 - 1;
  float sy = 2 * u2 - 1;
  if (sx == 0.0 && sy == 0.0) {
    *dx = 0.0;
    *dy = 0.0;
    return;
  }
  if (sx >= -sy) {
    if (sx > sy) {
      r = sx;
      if (sy > 0.0) theta = sy / r;
      else theta = 8.0f + sy / r;
    } else {
      r = sy;
      theta = 2.0f - sx / r;
    }
  } else {
    if (sx <= sy) {
      r = -sx;
      theta = 4.0f - sy / r;
    } else {
      r = -sy;
      theta = 6.0f + sx / r;
    }
  }
  theta = (float)((double)theta * (M_PI / 4.f));  // theta *= SPRAY_PI / 4.f
  float s, c;
  sinCos(theta, &s, &c);
  *dx = r * c;
  *dy = r * s;
}

// localToWorld (sampler.h:101-110), getCosineHemisphereSample (sampler.cc:54-60)
F3 localToWorld(F3 N, F3 v) {
  F3 dx0 = f3(0, N.z, -N.y);
  F3 dx1 = f3(-N.z, 0, N.x);
  F3 dx = normalize(dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1);
  F3 dy = normalize(cross(N, dx));
  F3 r;
  for (int i = 0; i < 3; ++i) r[i] = (dx[i] * v.x + dy[i] * v.y) + N[i] * v.z;
  return r;
}

void cosineSample(float u1, float u2, F3 N, F3* wi, float* pdf) {
  F3 v;
  concentricDisk(u1, u2, &v.x, &v.y);
  v.z = std::sqrt(gmax(0.f, 1.f - v.x * v.x - v.y * v.y));
  v = normalize(v);
  *wi = normalize(localToWorld(N, v));
  *pdf = v.z * kOneOverPi;
}

// ---------------------------------------------------------------- geometry
// intersectAabb, float-array form (src/render/aabb.h:139-169)
bool intersectAabb(const float lo[3], const float hi[3], const float org[3], const float dir[3],
                   float t0, float t1, float* tmin_o, float* tmax_o) {
  const float* bounds[2] = {lo, hi};
  float inv[3];
  inv[0] = 1.0f / dir[0];
  inv[1] = 1.0f / dir[1];
  inv[2] = 1.0f / dir[2];
  int sign[3];
  sign[0] = (inv[0] < 0.0f);
  sign[1] = (inv[1] < 0.0f);
  sign[2] = (inv[2] < 0.0f);
  float tmin, tmax, tymin, tymax, tzmin, tzmax;
  tmin = (bounds[sign[0]][0] - org[0]) * inv[0];
  tmax = (bounds[1 - sign[0]][0] - org[0]) * inv[0];
  tymin = (bounds[sign[1]][1] - org[1]) * inv[1];
  tymax = (bounds[1 - sign[1]][1] - org[1]) * inv[1];
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  tzmin = (bounds[sign[2]][2] - org[2]) * inv[2];
  tzmax = (bounds[1 - sign[2]][2] - org[2]) * inv[2];
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  *tmin_o = tmin;
  *tmax_o = tmax;
  return ((tmin < t1) && (tmax > t0));
}

// Watertight ray/triangle intersection (Woop, Benthin, Wald, JCGT 2(1), 2013)
struct Shear {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
Shear makeShear(F3 d) {
  Shear s;
  int kz = 0;
  float m = std::fabs(d.x);
  if (std::fabs(d.y) > m) {
    kz = 1;
    m = std::fabs(d.y);
  }
  if (std::fabs(d.z) > m) kz = 2;
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (d[kz] < 0.0f) std::swap(kx, ky);
  s.kx = kx;
  s.ky = ky;
  s.kz = kz;
  s.Sx = d[kx] / d[kz];
  s.Sy = d[ky] / d[kz];
  s.Sz = 1.0f / d[kz];
  return s;
}

bool triangleHit(const Shear& sh, F3 org, F3 p0, F3 p1, F3 p2, float tnear, float tfar, float* t_o,
                 float* u_o, float* v_o) {
  F3 A = sub(p0, org), B = sub(p1, org), C = sub(p2, org);
  float Ax = A[sh.kx] - sh.Sx * A[sh.kz];
  float Ay = A[sh.ky] - sh.Sy * A[sh.kz];
  float Bx = B[sh.kx] - sh.Sx * B[sh.kz];
  float By = B[sh.ky] - sh.Sy * B[sh.kz];
  float Cx = C[sh.kx] - sh.Sx * C[sh.kz];
  float Cy = C[sh.ky] - sh.Sy * C[sh.kz];
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = U + V + W;
  if (det == 0.0f) return false;
  float Az = sh.Sz * A[sh.kz], Bz = sh.Sz * B[sh.kz], Cz = sh.Sz * C[sh.kz];
  float T = U * Az + V * Bz + W * Cz;
  float rcp = 1.0f / det;
  float t = T * rcp;
  if (!(t > tnear && t < tfar)) return false;
  *t_o = t;
  *u_o = V * rcp;
  *v_o = W * rcp;
  return true;
}

// ---------------------------------------------------------------- BVH
// A binary median-split BVH, unrelated to the product's; conservative box
// test so the closest hit it finds is the exact minimum over all triangles.
struct BNode {
  float lo[3], hi[3];
  int left, right;  // children, or -1
  int first, count;
};

struct MeshBvh {
  std::vector<BNode> nodes;
  std::vector<uint32_t> prims;
};

void buildBvh(const std::vector<float>& v, const std::vector<uint32_t>& f, MeshBvh* out) {
  size_t nf = f.size() / 3;
  std::vector<float> cen(3 * nf), lo(3 * nf), hi(3 * nf);
  for (size_t t = 0; t < nf; ++t)
    for (int k = 0; k < 3; ++k) {
      float a = v[3 * f[3 * t] + k], b = v[3 * f[3 * t + 1] + k], c = v[3 * f[3 * t + 2] + k];
      lo[3 * t + k] = std::min(a, std::min(b, c));
      hi[3 * t + k] = std::max(a, std::max(b, c));
      cen[3 * t + k] = lo[3 * t + k] + hi[3 * t + k];
    }
  out->prims.resize(nf);
  for (size_t t = 0; t < nf; ++t) out->prims[t] = (uint32_t)t;
  out->nodes.clear();
  struct Job {
    int node, first, count;
  };
  std::vector<Job> stack;
  out->nodes.push_back(BNode{});
  stack.push_back({0, 0, (int)nf});
  while (!stack.empty()) {
    Job j = stack.back();
    stack.pop_back();
    BNode nd;
    for (int k = 0; k < 3; ++k) {
      nd.lo[k] = kInf;
      nd.hi[k] = -kInf;
    }
    for (int i = j.first; i < j.first + j.count; ++i) {
      uint32_t t = out->prims[i];
      for (int k = 0; k < 3; ++k) {
        nd.lo[k] = std::min(nd.lo[k], lo[3 * t + k]);
        nd.hi[k] = std::max(nd.hi[k], hi[3 * t + k]);
      }
    }
    nd.first = j.first;
    nd.count = j.count;
    nd.left = nd.right = -1;
    if (j.count > 4) {
      int axis = 0;
      float ext = nd.hi[0] - nd.lo[0];
      for (int k = 1; k < 3; ++k)
        if (nd.hi[k] - nd.lo[k] > ext) {
          ext = nd.hi[k] - nd.lo[k];
          axis = k;
        }
      int mid = j.first + j.count / 2;
      std::nth_element(out->prims.begin() + j.first, out->prims.begin() + mid,
                       out->prims.begin() + j.first + j.count, [&](uint32_t a, uint32_t b) {
                         float ca = cen[3 * a + axis], cb = cen[3 * b + axis];
                         return ca < cb || (ca == cb && a < b);
                       });
      nd.left = (int)out->nodes.size();
      nd.right = nd.left + 1;
      out->nodes.push_back(BNode{});
      out->nodes.push_back(BNode{});
      stack.push_back({nd.left, j.first, mid - j.first});
      stack.push_back({nd.right, mid, j.first + j.count - mid});
    }
    out->nodes[j.node] = nd;
  }
}

inline bool boxHit(const BNode& n, F3 org, F3 inv, float tnear, float tfar, float* tn) {
  float t0 = tnear, t1 = tfar;
  for (int k = 0; k < 3; ++k) {
    float a = (n.lo[k] - org[k]) * inv[k], b = (n.hi[k] - org[k]) * inv[k];
    float mn = std::fmin(a, b), mx = std::fmax(a, b);
    t0 = std::fmax(t0, mn);
    t1 = std::fmin(t1, mx);
  }
  *tn = t0;
  return t0 <= t1 * 1.0000004f;
}

// ---------------------------------------------------------------- scene
// A 4-wide BVH in the product's layout (128-byte nodes: child boxes lo/hi x,
// lo/hi y, lo/hi z as four floats each, then four child references: >= 0 an
// inner node, 0x80000000 an empty slot, otherwise a leaf ~((first << 3) |
// (count - 1)) into the leaf-ordered triangles, three float4 each, the first
// vertex's w holding the domain-local face index bits), given to the oracle
// only to count the work of an ordered traversal of that same hierarchy.
struct Bvh4 {
  std::vector<float> nodes;  // 32 floats per node (the references as int bits)
  std::vector<float> tris;   // 12 floats per triangle
};

struct Domain {
  std::vector<float> v;
  std::vector<uint32_t> f;
  std::vector<uint32_t> colors;
  std::vector<float> normals;
  float lo[3], hi[3];
  int bsdf = 0;
  float params[3] = {1, 1, 1};
  MeshBvh bvh;
  Bvh4 b4;
  uint32_t prim_base = 0;  // faces of the domains before this one
};

struct Light {
  int type;
  F3 pos, radiance, e1, e2;
};

struct Hit {
  float t, u, v;
  uint32_t prim;
};

void sortDomainList(std::vector<std::pair<float, int>>* l);

// Closest hit in a domain, tnear = 1e-3, tfar = inf (Scene::intersect,
// src/render/scene.inl:189-199).  Ties keep the lowest primitive id.
bool closestInDomain(const Domain& d, F3 org, F3 dir, Hit* h) {
  Shear sh = makeShear(dir);
  F3 inv = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  float best = kInf;
  uint32_t bprim = 0xffffffffu;
  bool found = false;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = d.bvh.nodes[stack[--sp]];
    float tn;
    if (!boxHit(n, org, inv, kEps, best, &tn)) continue;
    if (n.left < 0) {
      for (int i = n.first; i < n.first + n.count; ++i) {
        uint32_t p = d.bvh.prims[i];
        const uint32_t* fi = &d.f[3 * (size_t)p];
        F3 a = f3(d.v[3 * fi[0]], d.v[3 * fi[0] + 1], d.v[3 * fi[0] + 2]);
        F3 b = f3(d.v[3 * fi[1]], d.v[3 * fi[1] + 1], d.v[3 * fi[1] + 2]);
        F3 c = f3(d.v[3 * fi[2]], d.v[3 * fi[2] + 1], d.v[3 * fi[2] + 2]);
        float t, u, vv;
        if (triangleHit(sh, org, a, b, c, kEps, kInf, &t, &u, &vv)) {
          if (t < best || (t == best && p < bprim)) {
            best = t;
            bprim = p;
            h->t = t;
            h->u = u;
            h->v = vv;
            h->prim = p;
            found = true;
          }
        }
      }
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.right;
    }
  }
  return found;
}

// Any hit in (1e-3, tfar) (Scene::occluded, scene.inl:201-209).
bool occludedInDomain(const Domain& d, F3 org, F3 dir, float tfar) {
  Shear sh = makeShear(dir);
  F3 inv = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = d.bvh.nodes[stack[--sp]];
    float tn;
    if (!boxHit(n, org, inv, kEps, tfar, &tn)) continue;
    if (n.left < 0) {
      for (int i = n.first; i < n.first + n.count; ++i) {
        uint32_t p = d.bvh.prims[i];
        const uint32_t* fi = &d.f[3 * (size_t)p];
        F3 a = f3(d.v[3 * fi[0]], d.v[3 * fi[0] + 1], d.v[3 * fi[0] + 2]);
        F3 b = f3(d.v[3 * fi[1]], d.v[3 * fi[1] + 1], d.v[3 * fi[1] + 2]);
        F3 c = f3(d.v[3 * fi[2]], d.v[3 * fi[2] + 1], d.v[3 * fi[2] + 2]);
        float t, u, vv;
        if (triangleHit(sh, org, a, b, c, kEps, tfar, &t, &u, &vv)) return true;
      }
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.right;
    }
  }
  return false;
}

// TriMeshBuffer::updateIntersection (src/render/trimesh_buffer.cc:328-360)
void shadingAttributes(const Domain& d, const Hit& h, uint32_t* color, F3* ns) {
  const uint32_t* fi = &d.f[3 * (size_t)h.prim];
  uint32_t c[3] = {d.colors[fi[0]], d.colors[fi[1]], d.colors[fi[2]]};
  uint32_t rgb[9];
  for (int k = 0; k < 3; ++k) {
    rgb[3 * k] = (c[k] >> 16) & 0xff;
    rgb[3 * k + 1] = (c[k] >> 8) & 0xff;
    rgb[3 * k + 2] = c[k] & 0xff;
  }
  float w = 1.f - h.u - h.v;
  uint32_t out = 0;
  for (int ch = 0; ch < 3; ++ch) {
    float x = (rgb[ch] * w) + (rgb[3 + ch] * h.u) + (rgb[6 + ch] * h.v);
    uint32_t q = x > 0.0f ? (uint32_t)x : 0u;  // rounding noise below zero clamps to 0
    if (q > 255u) q = 255u;
    out |= q << (16 - 8 * ch);
  }
  *color = out;
  const float* n0 = &d.normals[3 * (size_t)fi[0]];
  const float* n1 = &d.normals[3 * (size_t)fi[1]];
  const float* n2 = &d.normals[3 * (size_t)fi[2]];
  for (int k = 0; k < 3; ++k) (*ns)[k] = (n0[k] * w) + (n1[k] * h.u) + (n2[k] * h.v);
}

// util::unpack (src/utils/util.h:69-73)
F3 unpack(uint32_t color) {
  F3 r;
  r.x = (float)(((color >> 16) & 0xff) * kOneOver255);
  r.y = (float)(((color >> 8) & 0xff) * kOneOver255);
  r.z = (float)((color & 0xff) * kOneOver255);
  return r;
}

// blinnPhong (src/render/reflection.h:202-214)
F3 blinnPhong(float costheta, F3 kd, F3 ks, float shininess, F3 li, F3 wi, F3 n_hat, F3 wo) {
  F3 half_hat = normalize(add(wi, wo));
  float n_dot_h = gclamp(dot(n_hat, half_hat), 0.0f, 1.0f);
  F3 cs = muls(ks, powInt(n_dot_h, shininess));
  F3 cd = muls(kd, costheta);
  return mul(li, add(cd, cs));
}

// HdrImage::add(pixid, rgb, double scale) (src/display/image.h:99-109): each
// channel += scale * rgb in double, rounded once to float
inline void hdrAdd(float* px, F3 rgb, double scale) {
  px[0] = (float)((double)px[0] + scale * (double)rgb.x);
  px[1] = (float)((double)px[1] + scale * (double)rgb.y);
  px[2] = (float)((double)px[2] + scale * (double)rgb.z);
}

// Reflect (src/render/reflection.h:126-128)
F3 reflect(F3 wo, F3 normal_ff) { return add(neg(wo), muls(normal_ff, 2.0f * dot(wo, normal_ff))); }

// FrDielectric (src/render/reflection.h:134-158): reflectance, and the
// transmitted direction unless the reflection is total (then 1, wt untouched)
float frDielectric(float cosThetaI, float etaI, float etaT, F3 wo, F3 normal_ff, F3* wt) {
  float sin2ThetaI = gmax(0.0f, 1.0f - (cosThetaI * cosThetaI));
  float eta = etaI / etaT;
  float sin2ThetaT = eta * eta * sin2ThetaI;
  if (sin2ThetaT >= 1.0f) return 1.0f;
  float cosThetaT = std::sqrt(1.0f - sin2ThetaT);
  float Rparl = ((etaT * cosThetaI) - (etaI * cosThetaT)) / ((etaT * cosThetaI) + (etaI * cosThetaT));
  float Rperp = ((etaI * cosThetaI) - (etaT * cosThetaT)) / ((etaI * cosThetaI) + (etaT * cosThetaT));
  float fr = (Rparl * Rparl + Rperp * Rperp) / 2.0f;
  *wt = add(smul(eta, neg(wo)), muls(normal_ff, eta * cosThetaI - cosThetaT));
  return fr;
}

// Refract (src/render/reflection.h:160-174): false on total internal reflection
bool refract(float cosThetaI, float etaI, float etaT, F3 wo, F3 normal_ff, F3* wt) {
  float sin2ThetaI = gmax(0.0f, 1.0f - (cosThetaI * cosThetaI));
  float eta = etaI / etaT;
  float sin2ThetaT = eta * eta * sin2ThetaI;
  if (sin2ThetaT >= 1.0f) return false;
  float cosThetaT = std::sqrt(1.0f - sin2ThetaT);
  *wt = add(smul(eta, neg(wo)), muls(normal_ff, eta * cosThetaI - cosThetaT));
  return true;
}

// Closest hit in one domain through its Bvh4, counting inner nodes expanded
// and triangles tested.  The walk is the product's ordered traversal: the
// four child boxes tested with t1 widened by kBoxSlack, children ordered near
// to far by their entry distance (its two low bits replaced by the slot), the
// nearest one continued when it starts within the best hit, the others pushed
// far to near, and stack entries beyond the best hit dropped on pop; a leaf's
// triangles are tested with an infinite tfar and kept by the (t, global face)
// key.  best_key enters as the key to beat.
constexpr float kBoxSlack = 1.0000004f;
constexpr int32_t kEmpty4 = (int32_t)0x80000000;

bool closestBvh4(const Domain& d, F3 org, F3 dir, uint64_t* best_key, float* best_t, int64_t* nodes,
                 int64_t* tris) {
  const float* N = d.b4.nodes.data();
  const int nn = (int)(d.b4.nodes.size() / 32);
  const float* T = d.b4.tris.data();
  const int nt = (int)(d.b4.tris.size() / 12);
  Shear sh = makeShear(dir);
  const float inv[3] = {1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z};
  const float o[3] = {org.x, org.y, org.z};
  const int s[3] = {inv[0] < 0.0f, inv[1] < 0.0f, inv[2] < 0.0f};
  int32_t sref[128];
  float st[128];
  int sp = 0;
  bool found = false;
  auto pop = [&]() -> int32_t {
    while (sp > 0) {
      --sp;
      if (st[sp] <= *best_t) return sref[sp];
    }
    return kEmpty4;
  };
  int32_t cur = 0;
  while (cur != kEmpty4) {
    while (cur >= 0) {
      if (cur >= nn) throw std::runtime_error("bvh4: node index out of range");
      ++*nodes;
      const float* q = N + 32 * (size_t)cur;
      int32_t ch[4];
      std::memcpy(ch, q + 24, 16);
      uint32_t k[4];
      for (int c = 0; c < 4; ++c) {
        float t0 = kEps, t1 = *best_t;
        float a[3], b[3];
        for (int x = 0; x < 3; ++x) {
          const float nearp = q[8 * x + 4 * s[x] + c], farp = q[8 * x + 4 * (s[x] ^ 1) + c];
          a[x] = (nearp - o[x]) * inv[x];
          b[x] = (farp - o[x]) * inv[x];
        }
        t0 = std::fmax(std::fmax(a[0], a[1]), std::fmax(a[2], kEps));
        t1 = std::fmin(std::fmin(b[0], b[1]), std::fmin(b[2], *best_t)) * kBoxSlack;
        uint32_t bits;
        std::memcpy(&bits, &t0, 4);
        k[c] = (t0 <= t1 && ch[c] != kEmpty4) ? ((bits & ~3u) | (uint32_t)c) : 0xffffffffu;
      }
      std::sort(k, k + 4);
      float k0t;
      const uint32_t k0b = k[0] & ~3u;
      std::memcpy(&k0t, &k0b, 4);
      if (k[0] != 0xffffffffu && k0t <= *best_t) {
        for (int j = 3; j >= 1; --j) {
          if (k[j] == 0xffffffffu) continue;
          if (sp == 128) throw std::runtime_error("bvh4: traversal stack overflow");
          const uint32_t kb = k[j] & ~3u;
          sref[sp] = ch[k[j] & 3u];
          std::memcpy(&st[sp], &kb, 4);
          ++sp;
        }
        cur = ch[k[0] & 3u];
      } else {
        cur = pop();
      }
    }
    if (cur == kEmpty4) break;
    const uint32_t v = ~(uint32_t)cur;
    const uint32_t first = v >> 3, cnt = (v & 7u) + 1u;
    if ((int)(first + cnt) > nt) throw std::runtime_error("bvh4: leaf out of range");
    *tris += cnt;
    for (uint32_t j = 0; j < cnt; ++j) {
      const float* t3 = T + 12 * (size_t)(first + j);
      float t, u, vv;
      if (triangleHit(sh, org, f3(t3[0], t3[1], t3[2]), f3(t3[4], t3[5], t3[6]), f3(t3[8], t3[9], t3[10]), kEps,
                      kInf, &t, &u, &vv)) {
        uint32_t prim, tb;
        std::memcpy(&prim, &t3[3], 4);
        std::memcpy(&tb, &t, 4);
        const uint64_t key = ((uint64_t)tb << 32) | (uint64_t)(d.prim_base + prim);
        if (key < *best_key) {
          *best_key = key;
          *best_t = t;
          found = true;
        }
      }
    }
    cur = pop();
  }
  return found;
}

struct Tile {
  int x, y, w, h;
};

struct Oracle {
  orc_config cfg;
  std::vector<Domain> doms;
  std::vector<Light> lights;
  // camera (src/render/camera.h:128-166)
  F3 cam_pos, cam_ll, cam_wv, cam_hv;
  float img_w = 1, img_h = 1;

  int D() const { return (int)doms.size(); }

  void setCamera(const float p[3], const float l[3], const float up[3], float vfov) {
    int W = cfg.image_w, H = cfg.image_h;
    float aspect_ratio = static_cast<float>(W) / static_cast<float>(H);
    float theta = vfov * M_PI / 180.0f;
    float image_half_h = std::tan(theta / 2.0f);
    float image_half_w = aspect_ratio * image_half_h;
    F3 campos = f3(p[0], p[1], p[2]), lookat = f3(l[0], l[1], l[2]), upvec = f3(up[0], up[1], up[2]);
    F3 w = sub(campos, lookat);
    F3 u = cross(upvec, w);
    F3 v = cross(w, u);
    w = normalize(w);
    u = normalize(u);
    v = normalize(v);
    F3 image_center = sub(campos, w);
    cam_ll = sub(sub(image_center, smul(image_half_w, u)), smul(image_half_h, v));
    cam_wv = smul(2.0f * image_half_w, u);
    cam_hv = smul(2.0f * image_half_h, v);
    cam_pos = campos;
    img_w = (float)W;
    img_h = (float)H;
  }

  // Camera::generateRay (camera.h:173-209)
  F3 generateRay(float x, float y) const {
    float u = x / img_w;
    float v = y / img_h;
    return normalize(sub(add(add(cam_ll, smul(u, cam_wv)), smul(v, cam_hv)), cam_pos));
  }

  // ImageScheduleTileList::init with makeVerticalStripe (src/render/tile.cc:214-235, 317-391)
  std::vector<Tile> tiles() const {
    std::vector<Tile> out;
    int W = cfg.image_w, H = cfg.image_h;
    int R = cfg.num_ranks, r = cfg.rank;
    int w = std::max(W / R, 1);
    int x = r * w;
    if (x >= W) return out;
    int vw = ((x + w > W) || (r == R - 1)) ? W - x : w;
    int64_t num_samples = (int64_t)vw * H * cfg.pixel_samples;
    int64_t est = (num_samples + cfg.max_samples_per_rank - 1) / cfg.max_samples_per_rank;
    int ntiles = (int)est;
    int tile_h = H / ntiles;
    if (tile_h <= 0) throw std::invalid_argument("tile height 0");
    for (int y = 0; y < H; y += tile_h) out.push_back(Tile{x, y, vw, std::min(tile_h, H - y)});
    return out;
  }

  // genSingleEyes / genMultiEyes (src/ooc/ooc_tracer.inl:84-172), tile-local ids
  void eye(const Tile& t, int64_t bufid, F3* dir, int* pixid) const {
    int spp = cfg.pixel_samples;
    int64_t lp = spp > 1 ? bufid / spp : bufid;
    int x = t.x + (int)(lp % t.w), y = t.y + (int)(lp / t.w);
    *pixid = y * cfg.image_w + x;
    if (spp > 1) {
      RandomSampler s;
      samplerInit(s, (int)bufid);
      float fx = (float)(x) + samplerGet1D(s);
      float fy = (float)(y) + samplerGet1D(s);
      *dir = generateRay(fx, fy);
    } else {
      *dir = generateRay((float)x, (float)y);
    }
  }

  // Domain list of a ray: every AABB hit with t0 = 1e-3, t1 = tmax, sorted by
  // (t, id) (WbvhEmbree::cbIntersect1 wbvh_embree.cc:126-148, DomainList::sort
  // rays.h:71-79).
  void domainList(F3 org, F3 dir, float tmax, std::vector<std::pair<float, int>>* out) const {
    out->clear();
    float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
    for (int i = 0; i < D(); ++i) {
      float tmin, tmx;
      if (intersectAabb(doms[i].lo, doms[i].hi, o, d, kEps, tmax, &tmin, &tmx)) out->push_back({tmin, i});
    }
    sortDomainList(out);
  }

  int slots() const {
    if (cfg.ao_mode) return cfg.ao_samples + (cfg.ao_light_shadow ? 1 : 0);
    int s = 0;
    for (auto& l : lights) s += l.type == 0 ? 1 : cfg.ao_samples;
    return s;
  }

  // Shadow rays and the bounce ray of one hit.  Restates ShaderAo::operator()
  // (src/ooc/ooc_shader_ao.h:92-197) and ShaderPt::operator()
  // (src/ooc/ooc_shader_pt.h:93-227); next_depth is the actual depth of the
  // bounce ray (ray_depth + rayin.depth + 1 in the reference).
  struct ShadowOut {
    F3 dir, w;
    float tmax;
    bool valid;
    int light;
  };
  struct BounceOut {
    F3 dir, w;
    bool valid;
  };
  void shade(int next_depth, F3 org, F3 dir, F3 Lin, int pixid, int samid, float t, int dom,
             uint32_t color, F3 normal, std::vector<ShadowOut>* sh, BounceOut* bo, F3* pos_out) const {
    const Domain& D_ = doms[dom];
    F3 pos = f3(dir.x * t + org.x, dir.y * t + org.y, dir.z * t + org.z);  // hitPosition, rays.h:437-441
    *pos_out = pos;
    F3 surf = unpack(color);
    F3 wo = neg(dir);
    float cos_theta_i = dot(wo, normal);
    bool entering = (cos_theta_i > 0.0f);
    F3 normal_ff = entering ? normal : neg(normal);
    normal_ff = normalize(normal_ff);
    bool delta = D_.bsdf != 0;
    sh->clear();
    bo->valid = false;
    if (cfg.ao_mode) {
      const float ao_weight = 1.0f / static_cast<float>(cfg.ao_samples);
      float tmax = cfg.ao_max_distance > 0.0f ? cfg.ao_max_distance : kInf;
      for (int l = 0; l < cfg.ao_samples; ++l) {
        ShadowOut s{};
        s.light = l;
        if (!delta) {
          RandomSampler ls;
          samplerInit(ls, (int)((uint32_t)pixid * (uint32_t)(l + 1)));
          float u1 = samplerGet1D(ls), u2 = samplerGet1D(ls);
          float pdf;
          cosineSample(u1, u2, normal_ff, &s.dir, &pdf);
          float costheta = gclamp(dot(normal_ff, s.dir), 0.0f, 1.0f);
          s.w = muls(mul(Lin, surf), kOneOverPi * costheta * ao_weight / pdf);
          s.valid = hasPositive(s.w);
        }
        s.tmax = tmax;
        sh->push_back(s);
      }
      if (cfg.ao_light_shadow) {
        ShadowOut s{};
        s.light = cfg.ao_samples;
        if (!lights.empty()) {
          const Light& L = lights[0];
          s.dir = normalize(sub(L.pos, pos));
          float costheta = gclamp(dot(normal_ff, s.dir), 0.0f, 1.0f);
          s.w = muls(mul(mul(Lin, surf), L.radiance), kOneOverPi * costheta);
          s.valid = hasPositive(s.w);
        }
        s.tmax = kInf;
        sh->push_back(s);
      }
    } else if (!delta) {
      F3 ks = f3(cfg.ks[0], cfg.ks[1], cfg.ks[2]);
      RandomSampler ls;
      samplerInit(ls, (int)((uint32_t)samid * (uint32_t)next_depth));
      for (size_t l = 0; l < lights.size(); ++l) {
        const Light& L = lights[l];
        if (L.type == 1) {
          for (int s = 0; s < cfg.ao_samples; ++s) {
            ShadowOut so{};
            so.light = (int)l;
            float u1 = samplerGet1D(ls), u2 = samplerGet1D(ls);
            float pdf;
            cosineSample(u1, u2, normal_ff, &so.dir, &pdf);
            if (pdf > 0.0f) {
              float costheta = gclamp(dot(normal_ff, so.dir), 0.0f, 1.0f);
              so.w = muls(mul(Lin, blinnPhong(costheta, surf, ks, cfg.shininess, L.radiance, so.dir,
                                              normal_ff, wo)),
                          (1.0f / (pdf * cfg.ao_samples)));
              so.valid = hasPositive(so.w);
            }
            so.tmax = kInf;
            sh->push_back(so);
          }
        } else if (L.type == 0) {
          ShadowOut so{};
          so.light = (int)l;
          so.dir = normalize(sub(L.pos, pos));
          float pdf = 1.0;
          float costheta = gclamp(dot(normal_ff, so.dir), 0.0f, 1.0f);
          so.w = muls(mul(Lin, blinnPhong(costheta, surf, ks, cfg.shininess, L.radiance, so.dir,
                                          normal_ff, wo)),
                      (1.0f / pdf));
          so.valid = hasPositive(so.w);
          so.tmax = kInf;
          sh->push_back(so);
        } else {  // emissive quad, an extension of the reference's light set
          F3 nq = cross(L.e1, L.e2);
          float area = std::sqrt(dot(nq, nq));
          F3 nqn = normalize(nq);
          for (int s = 0; s < cfg.ao_samples; ++s) {
            ShadowOut so{};
            so.light = (int)l;
            float u1 = samplerGet1D(ls), u2 = samplerGet1D(ls);
            F3 q = add(add(L.pos, muls(L.e1, u1)), muls(L.e2, u2));
            F3 dv = sub(q, pos);
            float dist2 = dot(dv, dv);
            float dist = std::sqrt(dist2);
            so.dir = divs(dv, dist);
            float cos_l = std::fabs(dot(nqn, so.dir));
            if (cos_l > 0.0f && dist > 0.0f) {
              float pdf = dist2 / (area * cos_l);
              float costheta = gclamp(dot(normal_ff, so.dir), 0.0f, 1.0f);
              so.w = muls(mul(Lin, blinnPhong(costheta, surf, ks, cfg.shininess, L.radiance, so.dir,
                                              normal_ff, wo)),
                          (1.0f / (pdf * (float)cfg.ao_samples)));
              so.valid = hasPositive(so.w);
            }
            so.tmax = dist;
            sh->push_back(so);
          }
        }
      }
    }
    if (next_depth < cfg.bounces) {
      wo = normalize(wo);
      if (delta) {
        if (cos_theta_i != 0.0f) {
          cos_theta_i = gclamp(cos_theta_i, -1.0f, 1.0f);
          float abs_cos_theta_i = std::fabs(cos_theta_i);
          if (!entering) cos_theta_i = abs_cos_theta_i;
          float fr = 1.0f;
          bool refl = false, trans = false;
          F3 wt = f3(0, 0, 0);
          if (D_.bsdf == 1) {
            fr = 1.0f;
            refl = true;
          } else {
            float etaI = entering ? D_.params[0] : D_.params[1];
            float etaT = entering ? D_.params[1] : D_.params[0];
            if (D_.bsdf == 2) {  // GlassBsdf + FrDielectric (reflection.h:134-158, 288-326)
              fr = frDielectric(cos_theta_i, etaI, etaT, wo, normal_ff, &wt);
              if (fr == 1.0f) refl = true;
              else if (fr == 0.0f) trans = true;
              else refl = true;  // the reference aborts here (CHECK in the shader)
            } else if (refract(cos_theta_i, etaI, etaT, wo, normal_ff, &wt)) {
              // TransmissionBsdf + Refract (reflection.h:160-174, 331-364)
              fr = 0.0f;
              trans = true;
            } else {
              fr = 1.0f;
              refl = true;
            }
          }
          if (refl) {
            F3 wr = reflect(wo, normal_ff);
            bo->dir = normalize(wr);
            bo->w = muls(Lin, fr / abs_cos_theta_i);
            bo->valid = hasPositive(bo->w);
          } else if (trans) {
            bo->dir = normalize(wt);
            bo->w = muls(Lin, (1.0f - fr) / abs_cos_theta_i);
            bo->valid = hasPositive(bo->w);
          }
        }
      } else {
        RandomSampler s;
        samplerInit(s, (int)((uint32_t)samid * (uint32_t)next_depth));
        float u1 = samplerGet1D(s), u2 = samplerGet1D(s);
        float pdf;
        cosineSample(u1, u2, normal_ff, &bo->dir, &pdf);
        float costheta = gclamp(dot(normal_ff, bo->dir), 0.0f, 1.0f);
        bo->w = divs(muls(muls(mul(Lin, surf), kOneOverPi), costheta), pdf);
        bo->valid = hasPositive(bo->w);
      }
      if (bo->valid && cfg.rr_depth > 0 && next_depth >= cfg.rr_depth) {
        float q = gmin(1.0f, gmax(bo->w.x, gmax(bo->w.y, bo->w.z)));
        RandomSampler rs;
        samplerInit(rs, (int)(((uint32_t)samid * (uint32_t)next_depth) ^ 0x2545f491u));
        float ur = samplerGet1D(rs);
        if (ur >= q) bo->valid = false;
        else bo->w = divs(bo->w, q);
      }
    }
  }

  // ------------------------------------------------------------ mode B
  struct WRay {
    F3 org, dir, w;
    int pixid, samid;
  };

  bool closest(F3 org, F3 dir, Hit* h, int* dom, int64_t* visits) const {
    std::vector<std::pair<float, int>> list;
    domainList(org, dir, kInf, &list);
    bool found = false;
    float bt = kInf;
    int bd = -1;
    uint32_t bp = 0;
    for (auto& e : list) {
      Hit hh;
      if (visits) ++*visits;
      if (closestInDomain(doms[e.second], org, dir, &hh)) {
        // (t, domain, prim) order: domains are visited in (t, id) order, so
        // compare explicitly
        if (!found || hh.t < bt || (hh.t == bt && (e.second < bd || (e.second == bd && hh.prim < bp)))) {
          *h = hh;
          bt = hh.t;
          bd = e.second;
          bp = hh.prim;
          found = true;
        }
      }
    }
    *dom = bd;
    return found;
  }

  // The work of the ordered front-to-back walk of a ray over the Bvh4s: its
  // domains in (entry t, id) order, a domain skipped when its entry lies
  // beyond the best hit so far, each walk starting from that hit.  Returns the
  // key (t bits << 32 | global face) of the closest hit, ~0 for none.
  uint64_t countBvh4(F3 org, F3 dir, int64_t* visits, int64_t* nodes, int64_t* tris) const {
    std::vector<std::pair<float, int>> list;
    domainList(org, dir, kInf, &list);
    uint64_t key = ~0ull;
    float best = kInf;
    for (auto& e : list) {
      if (key != ~0ull && e.first > best) continue;
      ++*visits;
      closestBvh4(doms[e.second], org, dir, &key, &best, nodes, tris);
    }
    return key;
  }

  bool occluded(F3 org, F3 dir, float tmax, int origin, int64_t* visits) const {
    if (visits) ++*visits;
    if (occludedInDomain(doms[origin], org, dir, tmax)) return true;
    std::vector<std::pair<float, int>> list;
    domainList(org, dir, tmax, &list);
    for (auto& e : list) {
      if (e.second == origin) continue;
      if (visits) ++*visits;
      if (occludedInDomain(doms[e.second], org, dir, tmax)) return true;
    }
    return false;
  }

  void renderWavefront(float* rgba, orc_stats* st) const {
    int W = cfg.image_w, H = cfg.image_h, spp = cfg.pixel_samples;
    std::fill(rgba, rgba + (size_t)W * H * 4, 0.0f);
    orc_stats s{};
    double scale = 1.0 / (double)spp;
    for (const Tile& t : tiles()) {
      int64_t n = (int64_t)t.w * t.h * spp;
      std::vector<WRay> rays(n);
      std::vector<char> alive(n, 1);
      std::vector<int> sample_pixid(n);
      for (int64_t i = 0; i < n; ++i) {
        rays[i].org = cam_pos;
        eye(t, i, &rays[i].dir, &rays[i].pixid);
        rays[i].w = f3(1.f, 1.f, 1.f);
        rays[i].samid = (int)i;
        sample_pixid[i] = rays[i].pixid;
      }
      s.rays_primary += n;
      for (int b = 0; b < cfg.bounces; ++b) {
        std::vector<WRay> next(n);
        std::vector<char> nalive(n, 0);
        // per-sample shadow contributions, added per pixel in sample order
        std::vector<std::vector<std::pair<F3, bool>>> contrib(n);
        int64_t vis_r = 0, vis_s = 0, nsh = 0, nb = 0, v4 = 0, n4 = 0, t4 = 0, bad4 = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : vis_r, vis_s, nsh, nb, v4, n4, t4, bad4)
        for (int64_t i = 0; i < n; ++i) {
          if (!alive[i]) continue;
          const WRay& r = rays[i];
          Hit h;
          int dom;
          const bool hit = closest(r.org, r.dir, &h, &dom, &vis_r);
          if (has_bvh4) {
            // the same hit through the product's hierarchy, and its work
            const uint64_t k4 = countBvh4(r.org, r.dir, &v4, &n4, &t4);
            uint32_t tb;
            std::memcpy(&tb, &h.t, 4);
            const uint64_t want = hit ? (((uint64_t)tb << 32) | (uint64_t)(doms[dom].prim_base + h.prim)) : ~0ull;
            if (k4 != want) ++bad4;
          }
          if (!hit) continue;
          uint32_t color;
          F3 ns;
          shadingAttributes(doms[dom], h, &color, &ns);
          std::vector<ShadowOut> sh;
          BounceOut bo;
          F3 pos;
          shade(b + 1, r.org, r.dir, r.w, r.pixid, r.samid, h.t, dom, color, ns, &sh, &bo, &pos);
          for (auto& so : sh) {
            if (!so.valid) continue;
            ++nsh;
            bool occ = occluded(pos, so.dir, so.tmax, dom, &vis_s);
            contrib[i].push_back({so.w, !occ});
          }
          if (bo.valid) {
            next[i] = WRay{pos, bo.dir, bo.w, r.pixid, r.samid};
            nalive[i] = 1;
            ++nb;
          }
        }
        s.visits_radiance += vis_r;
        s.visits_shadow += vis_s;
        s.bvh4_visits += v4;
        s.bvh4_nodes += n4;
        s.bvh4_tris += t4;
        s.bvh4_mismatches += bad4;
        s.rays_shadow += nsh;
        if (b + 1 < cfg.bounces) s.rays_bounce += nb;
        for (int64_t p = 0; p < n / spp; ++p) {
          int pixid = sample_pixid[p * spp];
          float* px = rgba + 4 * (size_t)pixid;
          for (int k = 0; k < spp; ++k)
            for (auto& c : contrib[p * spp + k]) {
              if (!c.second) continue;
              hdrAdd(px, c.first, scale);
            }
        }
        if (b + 1 < cfg.bounces) {
          rays.swap(next);
          alive.swap(nalive);
        }
      }
    }
    if (st) *st = s;
  }

  // ------------------------------------------------------------ mode A
  void renderSpeculative(int nthreads, float* rgba, orc_stats* st);

  // ------------------------------------------------------------ mode C
  void renderBaseline(float* rgba, orc_stats* st, std::vector<int>* schedule);
  std::vector<int> baseline_schedule;  // the domains of the last mode C frame, one per round
  bool has_bvh4 = false;               // every domain holds a Bvh4 (orc_set_bvh4)
};

// =================================================================== mode A
// The reference's speculative loop: ooc::Tracer::trace
// (src/ooc/ooc_tracer.inl:184-234), PContext::isectPrims
// (src/ooc/ooc_pcontext.h:91-181), TContext (ooc_tcontext.h/.inl), VBuf
// (ooc_vbuf.cc:41-112), DomainStats (ooc_domain_stats.cc:60-111), and the
// domain caches (infinite_cache.cc:47-60, lru_cache.cc:65-171).

struct Ray {  // src/ooc/ooc_ray.h:28-40
  float org[3];
  int pixid;
  float dir[3];
  int samid;
  float w[3];
  int depth;
  float history[kMaxHistory];
  float tdom;
  int committed;
  int light;
  int occluded;
  float tmax;  // end of shadow rays; infinity in the reference
};

struct RayData {  // ooc_ray.h:42-46
  Ray* ray;
  float tdom;
  int dom_depth;
};

// Chunked bump allocator with stable addresses (pbrt MemoryArena role).
struct Arena {
  std::vector<std::unique_ptr<Ray[]>> chunks;
  size_t used = 0;  // rays handed out
  static const size_t kChunk = 1 << 16;
  Ray* alloc() {
    size_t c = used / kChunk, o = used % kChunk;
    if (c == chunks.size()) chunks.emplace_back(new Ray[kChunk]);
    ++used;
    return &chunks[c][o];
  }
  Ray* allocN(size_t n, std::vector<Ray*>* out) {
    out->resize(n);
    for (size_t i = 0; i < n; ++i) (*out)[i] = alloc();
    return n ? (*out)[0] : nullptr;
  }
  void reset() { used = 0; }
};

struct DomainStats {
  int nd = 0, L = 0;
  std::vector<int64_t> stats;
  std::vector<std::pair<int64_t, int>> scores;
  std::vector<int> schedule_;
  void resize(int ndomains, int list_size) {
    nd = ndomains;
    L = list_size;
    stats.assign((size_t)nd * L, 0);
    schedule_.assign(nd, 0);
  }
  void reset() { std::fill(stats.begin(), stats.end(), 0); }
  // ooc_domain_stats.h:68-77; indices past the list size are dropped here
  // (the reference writes into the next domain's counters)
  void increment(int id, int depth) {
    if (depth < L) ++stats[(size_t)id * L + depth];
  }
  void decrement(int id, int depth) {
    if (depth < L) --stats[(size_t)id * L + depth];
  }
  void add(const DomainStats& o, int id) {
    for (int d = 0; d < L; ++d) stats[(size_t)id * L + d] += o.stats[(size_t)id * L + d];
  }
  void schedule() {
    scores.resize(nd);
    for (int id = 0; id < nd; ++id) {
      int64_t score = 0;
      for (int depth = 0; depth < L; ++depth) score += stats[(size_t)id * L + depth] * (L - depth);
      scores[id] = {score, id};
    }
    // descending score; ties by id (the reference's std::sort leaves them unordered)
    std::sort(scores.begin(), scores.end(), [](const std::pair<int64_t, int>& a, const std::pair<int64_t, int>& b) {
      return a.first > b.first || (a.first == b.first && a.second < b.second);
    });
    for (int i = 0; i < nd; ++i) schedule_[i] = scores[i].second;
  }
};

struct VBuf {  // ooc_vbuf.cc
  std::vector<float> tbuf;
  int H = 4;
  void resize(size_t nsamples, int h) {
    H = h;
    tbuf.assign(nsamples * H, kInf);
  }
  void reset() { std::fill(tbuf.begin(), tbuf.end(), kInf); }
  bool correct(const Ray& ray) const {
    size_t off = (size_t)ray.samid * H;
    for (int i = 0; i < ray.depth; ++i)
      if (ray.history[i] != tbuf[off + i]) return false;
    return true;
  }
  bool update(float t, Ray* ray) {
    const int ray_depth = ray->depth;
    int update_pos = ray_depth;
    const size_t off = (size_t)ray->samid * H;
    for (int i = 0; i < ray_depth; ++i) {
      float local_t = ray->history[i], global_t = tbuf[off + i];
      if (local_t < global_t) {
        update_pos = i;
        break;
      } else if (local_t > global_t) {
        update_pos = -1;
        break;
      }
    }
    bool updated;
    if (update_pos == -1) {
      updated = false;
    } else if (update_pos < ray_depth) {
      updated = true;
      ray->history[ray_depth] = t;
      for (int i = update_pos; i <= ray_depth; ++i) tbuf[off + i] = ray->history[i];
    } else {
      if (t < tbuf[off + ray_depth]) {
        updated = true;
        tbuf[off + ray_depth] = t;
        ray->history[ray_depth] = t;
      } else {
        updated = false;
      }
    }
    if (updated)
      for (int i = ray_depth + 1; i < H; ++i) tbuf[off + i] = kInf;
    return updated;
  }
};

struct LruCache {  // lru_cache.cc:41-171
  int capacity = 0, size = 0, nd = 0;
  std::list<std::pair<int, int>> blocks;  // (block, domain), front = LRU
  std::map<int, std::list<std::pair<int, int>>::iterator> id_to_block;
  std::vector<int> hit;
  int last_evicted = -1;  // domain the last miss displaced, -1 when a block was free
  void init(int ndomains, int cache_size) {
    nd = ndomains;
    capacity = (cache_size < 0 || cache_size >= ndomains) ? ndomains : cache_size;
    size = 0;
    blocks.clear();
    id_to_block.clear();
    hit.assign(nd, 0);
  }
  bool load(int domid) {
    if (hit[domid]) {
      auto it = id_to_block[domid];
      auto b = *it;
      blocks.erase(it);
      blocks.push_back(b);
      id_to_block[domid] = std::prev(blocks.end());
      return true;
    }
    hit[domid] = 1;
    last_evicted = -1;
    if (size < capacity) {
      blocks.push_back({size, domid});
      id_to_block[domid] = std::prev(blocks.end());
      ++size;
    } else {
      auto old = blocks.front();
      blocks.pop_front();
      id_to_block.erase(old.second);
      hit[old.second] = 0;
      last_evicted = old.second;
      blocks.push_back({old.first, domid});
      id_to_block[domid] = std::prev(blocks.end());
    }
    return false;
  }
};

struct TContext {
  const Oracle* o = nullptr;
  int H = 4;
  Arena mem0, mem1;
  Arena* mem_in = &mem0;
  Arena* mem_out = &mem1;
  VBuf vbuf;
  DomainStats rstats;
  std::vector<std::queue<RayData>> rqs, sqs0, sqs1;
  std::vector<std::queue<RayData>>* sqs_in = &sqs0;
  std::vector<std::queue<RayData>>* sqs_out = &sqs1;
  std::queue<Ray*> sq2, rq2, pending_q, frq, fsq_in, fsq_out, cr0, cr1;
  std::queue<Ray*>* commit_q = &cr0;
  std::queue<Ray*>* retire_q = &cr1;
  std::vector<std::pair<float, int>> list;
  float* image = nullptr;
  int W = 0;
  double scale = 1.0;
  orc_stats st{};

  void init(const Oracle* oo, size_t tile_samples, float* img) {
    o = oo;
    H = o->cfg.history_size;
    int D = o->D();
    vbuf.resize(tile_samples, H);
    rstats.resize(D, o->cfg.list_size);
    rqs.assign(D, {});
    sqs0.assign(D, {});
    sqs1.assign(D, {});
    image = img;
    W = o->cfg.image_w;
    scale = 1.0 / (double)o->cfg.pixel_samples;
  }

  // Isector::isectAll (ooc_isector.h:126-145)
  void isectAll(Ray* r, std::vector<std::queue<RayData>>* qs) {
    o->domainList(f3(r->org[0], r->org[1], r->org[2]), f3(r->dir[0], r->dir[1], r->dir[2]), kInf, &list);
    for (size_t i = 0; i < list.size(); ++i) {
      (*qs)[list[i].second].push(RayData{r, list[i].first, (int)i});
      rstats.increment(list[i].second, (int)i);
    }
  }
  // Isector::isectWithoutCurrentDomain (ooc_isector.h:147-174)
  bool isectExcept(int exclude, Ray* r, std::vector<std::queue<RayData>>* qs) {
    o->domainList(f3(r->org[0], r->org[1], r->org[2]), f3(r->dir[0], r->dir[1], r->dir[2]), r->tmax, &list);
    int n = 0;
    for (size_t i = 0; i < list.size(); ++i) {
      int id = list[i].second;
      if (id != exclude) {
        ++n;
        (*qs)[id].push(RayData{r, list[i].first, (int)i});
        rstats.increment(id, (int)i);
      }
    }
    return n > 0;
  }
  bool sqsInEmpty() const {
    for (auto& q : *sqs_in)
      if (!q.empty()) return false;
    return true;
  }
  bool rqsEmpty() const {
    for (auto& q : rqs)
      if (!q.empty()) return false;
    return true;
  }
  void filterQs(int id) {
    auto& rq = rqs[id];
    while (!rq.empty()) {
      RayData& d = rq.front();
      Ray* r = d.ray;
      rstats.decrement(id, d.dom_depth);
      if (d.tdom <= r->history[r->depth] && vbuf.correct(*r)) frq.push(r);
      rq.pop();
    }
    filterSqs(id, sqs_in, &fsq_in);
    filterSqs(id, sqs_out, &fsq_out);
  }
  void filterSqs(int id, std::vector<std::queue<RayData>>* sqs, std::queue<Ray*>* fsq) {
    auto& sq = (*sqs)[id];
    while (!sq.empty()) {
      RayData& d = sq.front();
      Ray* r = d.ray;
      rstats.decrement(id, d.dom_depth);
      if (!r->occluded && vbuf.correct(*r)) fsq->push(r);
      sq.pop();
    }
  }
  bool allFilterQsEmpty() const { return frq.empty() && fsq_in.empty() && fsq_out.empty(); }

  void makeShadow(const Ray& ray, int light, F3 pos, F3 dir, F3 w, float t, Ray* s) {  // ooc_ray.h:54-83
    s->org[0] = pos.x;
    s->org[1] = pos.y;
    s->org[2] = pos.z;
    s->pixid = ray.pixid;
    s->dir[0] = dir.x;
    s->dir[1] = dir.y;
    s->dir[2] = dir.z;
    s->samid = ray.samid;
    s->w[0] = w.x;
    s->w[1] = w.y;
    s->w[2] = w.z;
    s->depth = ray.depth + 1;
    for (int d = 0; d < ray.depth; ++d) s->history[d] = ray.history[d];
    s->history[ray.depth] = t;
    s->committed = 0;
    s->light = light;
    s->occluded = 0;
    s->tmax = kInf;
  }
  void makeRay(const Ray& in, F3 pos, F3 dir, F3 w, float t, Ray* out, int depth) {  // ooc_ray.h:85-112
    out->org[0] = pos.x;
    out->org[1] = pos.y;
    out->org[2] = pos.z;
    out->pixid = in.pixid;
    out->dir[0] = dir.x;
    out->dir[1] = dir.y;
    out->dir[2] = dir.z;
    out->samid = in.samid;
    out->w[0] = w.x;
    out->w[1] = w.y;
    out->w[2] = w.z;
    out->depth = depth;
    for (int d = 0; d < in.depth; ++d) out->history[d] = in.history[d];
    out->history[in.depth] = t;
    // The reference leaves history[depth] of the new ray unset (stale arena
    // memory) although filterRqs culls against it (ooc_tcontext.inl:147);
    // the intended value, that of every fresh ray (ooc_tracer.inl:118), is +inf.
    if (depth > 0) out->history[depth] = kInf;
    out->committed = 0;
    out->occluded = 0;
    out->tmax = kInf;
  }

  void procFilterQs(int id, int ray_depth) {
    const Domain& dom = o->doms[id];
    // procRads (ooc_tcontext.inl:28-49)
    while (!frq.empty()) {
      Ray* r = frq.front();
      frq.pop();
      ++st.visits_radiance;
      Hit h;
      F3 org = f3(r->org[0], r->org[1], r->org[2]), dir = f3(r->dir[0], r->dir[1], r->dir[2]);
      if (closestInDomain(dom, org, dir, &h)) {
        if (vbuf.update(h.t, r)) {
          uint32_t color;
          F3 ns;
          shadingAttributes(dom, h, &color, &ns);
          std::vector<Oracle::ShadowOut> shs;
          Oracle::BounceOut bo;
          F3 pos;
          int next_actual = ray_depth + r->depth + 1;
          o->shade(next_actual, org, dir, f3(r->w[0], r->w[1], r->w[2]), r->pixid, r->samid, h.t, id,
                   color, ns, &shs, &bo, &pos);
          for (auto& s : shs) {
            if (!s.valid) continue;
            Ray* sr = mem_out->alloc();
            makeShadow(*r, s.light, pos, s.dir, s.w, h.t, sr);
            sr->tmax = s.tmax;
            sq2.push(sr);
            ++st.rays_shadow;
          }
          if (bo.valid) {  // genR2 (ooc_shader_ao.h:73-89)
            Ray* r2 = mem_out->alloc();
            int nvd = r->depth + 1;
            if (nvd == H) {
              makeRay(*r, pos, bo.dir, bo.w, h.t, r2, 0);
              pending_q.push(r2);
            } else {
              makeRay(*r, pos, bo.dir, bo.w, h.t, r2, nvd);
              rq2.push(r2);
            }
            ++st.rays_bounce;
          }
          // procShads2 (ooc_tcontext.inl:72-91)
          while (!sq2.empty()) {
            Ray* s = sq2.front();
            sq2.pop();
            ++st.visits_shadow;
            if (!occludedInDomain(dom, f3(s->org[0], s->org[1], s->org[2]),
                                  f3(s->dir[0], s->dir[1], s->dir[2]), s->tmax)) {
              if (!isectExcept(id, s, sqs_out)) {
                s->committed = 1;
                commit_q->push(s);
              }
            }
          }
          // procRads2 (ooc_tcontext.inl:93-100)
          while (!rq2.empty()) {
            Ray* r2 = rq2.front();
            rq2.pop();
            isectAll(r2, &rqs);
          }
        }
      }
    }
    procShads(dom, &fsq_in, retire_q);
    procShads(dom, &fsq_out, commit_q);
  }
  // procShads (ooc_tcontext.inl:51-70)
  void procShads(const Domain& dom, std::queue<Ray*>* qin, std::queue<Ray*>* qout) {
    while (!qin->empty()) {
      Ray* r = qin->front();
      qin->pop();
      ++st.visits_shadow;
      bool occ = occludedInDomain(dom, f3(r->org[0], r->org[1], r->org[2]),
                                  f3(r->dir[0], r->dir[1], r->dir[2]), r->tmax);
      if (occ) r->occluded = 1;
      if (!occ && !r->committed) {
        r->committed = 1;
        qout->push(r);
      }
    }
  }
  // retire (ooc_tcontext.inl:123-135)
  void retire() {
    while (!retire_q->empty()) {
      Ray* r = retire_q->front();
      retire_q->pop();
      if (!r->occluded && vbuf.correct(*r)) {
        float* px = image + 4 * (size_t)r->pixid;
        hdrAdd(px, f3(r->w[0], r->w[1], r->w[2]), scale);
      }
    }
  }
  void swapQs() {
    std::swap(commit_q, retire_q);
    std::swap(sqs_in, sqs_out);
  }
  // procPendingQ (ooc_tcontext.h:206-216)
  void procPendingQ() {
    while (!pending_q.empty()) {
      Ray* r = pending_q.front();
      pending_q.pop();
      if (vbuf.correct(*r)) {
        r->depth = 0;
        r->history[0] = kInf;
        isectAll(r, &rqs);
      }
    }
  }
};

void Oracle::renderSpeculative(int T, float* rgba, orc_stats* out) {
  if (cfg.history_size < 1 || cfg.history_size > kMaxHistory)
    throw std::invalid_argument("history_size out of range");
  int W = cfg.image_w, Hh = cfg.image_h;
  std::fill(rgba, rgba + (size_t)W * Hh * 4, 0.0f);
  std::vector<Tile> tl = tiles();
  size_t largest = 0;
  for (auto& t : tl) largest = std::max(largest, (size_t)t.w * t.h * cfg.pixel_samples);
  std::vector<TContext> tcs(T);
  for (auto& tc : tcs) tc.init(this, largest, rgba);
  LruCache cache;
  cache.init(D(), cfg.cache_size);
  int64_t loads = 0, rounds = 0;
  if (cfg.cache_size < 0)  // Scene::init warms every domain (scene.inl:85-93)
    for (int d = 0; d < D(); ++d) cache.load(d);
  DomainStats pstats;
  pstats.resize(D(), cfg.list_size);
  std::vector<int> flag(T);
  std::vector<Ray*> eyes;
  int64_t primaries = 0;
  for (const Tile& tile : tl) {
    int64_t n = (int64_t)tile.w * tile.h * cfg.pixel_samples;
    primaries += n;
    for (auto& tc : tcs) {
      tc.mem_in->reset();
      tc.mem_out->reset();
    }
    tcs[0].mem_in->allocN(n, &eyes);
#pragma omp parallel num_threads(T)
    {
      int tid = omp_get_thread_num();
      TContext& tc = tcs[tid];
      for (int64_t i = tid; i < n; i += T) {  // genSingleEyes/genMultiEyes, schedule(static, 1)
        Ray* r = eyes[i];
        r->org[0] = cam_pos.x;
        r->org[1] = cam_pos.y;
        r->org[2] = cam_pos.z;
        F3 d;
        eye(tile, i, &d, &r->pixid);
        r->dir[0] = d.x;
        r->dir[1] = d.y;
        r->dir[2] = d.z;
        r->samid = (int)i;
        r->w[0] = r->w[1] = r->w[2] = 1.f;
        r->depth = 0;
        r->history[0] = kInf;
        r->committed = 0;
        r->occluded = 0;
        r->tmax = kInf;
      }
#pragma omp barrier
      tc.rstats.reset();
      for (int64_t i = tid; i < n; i += T) tc.isectAll(eyes[i], &tc.rqs);  // isectDomsRads
#pragma omp barrier
      int ray_depth = 0;
      while (true) {  // PContext::isectPrims
        tc.procPendingQ();
        tc.vbuf.reset();
        while (true) {
          bool sqs_in_empty = tc.sqsInEmpty(), rqs_empty = tc.rqsEmpty(),
               retire_empty = tc.retire_q->empty();
          flag[tid] = sqs_in_empty && rqs_empty && retire_empty;
#pragma omp barrier
          bool all_empty = true;
          for (int k = 0; k < T; ++k) all_empty = all_empty && flag[k];
#pragma omp barrier
          if (all_empty) break;
          flag[tid] = sqs_in_empty && rqs_empty;
#pragma omp barrier
          bool inputs_empty = true;
          for (int k = 0; k < T; ++k) inputs_empty = inputs_empty && flag[k];
#pragma omp barrier
          if (!inputs_empty) {
#pragma omp single
            {
              pstats.reset();
              ++rounds;
            }
#pragma omp critical(orc_merge)
            for (int id = 0; id < D(); ++id) pstats.add(tc.rstats, id);
#pragma omp barrier
#pragma omp single
            pstats.schedule();
            for (int i = 0; i < D(); ++i) {
              int id = pstats.schedule_[i];
              tc.filterQs(id);
              flag[tid] = tc.allFilterQsEmpty();
#pragma omp barrier
              bool none = true;
              for (int k = 0; k < T; ++k) none = none && flag[k];
#pragma omp barrier
              if (!none) {
#pragma omp single
                {
                  if (!cache.load(id)) ++loads;
                }
                tc.procFilterQs(id, ray_depth);
              }
#pragma omp barrier
            }
          }
#pragma omp critical(orc_retire)
          tc.retire();
          tc.swapQs();
#pragma omp barrier
        }
        tc.mem_in->reset();
        std::swap(tc.mem_in, tc.mem_out);
        ray_depth += cfg.history_size;
        flag[tid] = tc.pending_q.empty();
#pragma omp barrier
        bool pend_empty = true;
        for (int k = 0; k < T; ++k) pend_empty = pend_empty && flag[k];
#pragma omp barrier
        if (pend_empty) break;
      }
    }
  }
  orc_stats s{};
  s.rays_primary = primaries;
  for (auto& tc : tcs) {
    s.rays_shadow += tc.st.rays_shadow;
    s.rays_bounce += tc.st.rays_bounce;
    s.visits_radiance += tc.st.visits_radiance;
    s.visits_shadow += tc.st.visits_shadow;
  }
  s.domain_loads = loads;
  s.rounds = rounds;
  if (out) *out = s;
}

// =================================================================== mode C
// The reference's non-speculative image tracer on one process:
//   baseline::ImageTracer::trace (src/baseline/baseline_image_tracer.inl:28-131):
//     all eye rays queued in their first domain, then rounds until every
//     queue is empty; each round takes one domain from the scheduler, loads
//     it, runs its shadow queue, its radiance queue and the rays its shaders
//     spawned (temp_q), and adds the round's retired contributions;
//   ImageTracer::schedule (baseline_image_tracer.inl:134-157): the count of a
//     domain is its radiance plus shadow queue length;
//   LoadAnyOnceSched::scheduleImage (baseline_schedulers.cc:43-62);
//   InsituTracer::genEyeRays, isectEyeDomains, processRays, processShadow,
//     processRay2 (baseline_insitu_tracer.inl:407-497, 545-766);
//   DomainIntersector::intersect (baseline_isector.h:44-98);
//   baseline::ShaderPt / ShaderAo (baseline_shader_pt.h:55-196,
//     baseline_shader_ao.h:54-98): the light and bounce samples and their
//     seeds are the speculative shaders', so Oracle::shade computes them; the
//     shadow ray is tested in the shading domain when it is made.
// One thread: what a round queues follows from each ray's own state, so the
// per-domain counts that drive the schedule do not depend on the order in
// which the round's rays run; only the order of the image additions does.

// LoadAnyOnceSched::scheduleImage: the domain with the most queued rays;
// equal counts stay in the order std::sort leaves them (ids ascending in).
int loadAnyOnceSchedule(int nd, const int64_t* counts, bool* done) {
  std::vector<std::pair<int, int64_t>> rc(nd);
  for (int i = 0; i < nd; ++i) rc[i] = {i, counts[i]};
  std::sort(rc.begin(), rc.end(),
            [](const std::pair<int, int64_t>& a, const std::pair<int, int64_t>& b) { return a.second > b.second; });
  *done = rc[0].second == 0;
  return rc[0].first;
}

namespace {
constexpr int kNone = std::numeric_limits<int>::max();  // INT_MAX in the reference's DRay

struct BRay {  // baseline::DRay (baseline_ray.h) with the hit it carries
  F3 org, dir, w;
  int pixid, samid, depth;
  float t;           // closest hit so far
  int domid;         // its domain, kNone without one
  Hit hit;
  bool shade_only;   // DRAY_FLAG_SHADE: queued back to domid for shading
  int domain_pos;    // position in the ray's domain list, kNone when not traversing
  float next_tdom;   // entry distance of the domain after domain_pos
  float tmax;        // occlusion range of shadow rays (infinite in the reference)
};

struct Commit {  // CommitB (baseline_commit_buffer.h)
  int pixid;
  F3 rgb;
};
}  // namespace

void Oracle::renderBaseline(float* rgba, orc_stats* out, std::vector<int>* schedule) {
  if (cfg.num_ranks != 1) throw std::invalid_argument("the baseline loop runs on one process");
  const int W = cfg.image_w, H = cfg.image_h, spp = cfg.pixel_samples, nd = D();
  std::fill(rgba, rgba + (size_t)W * H * 4, 0.0f);
  orc_stats s{};
  std::vector<BRay> rays;
  std::vector<std::vector<int>> qs(nd), sqs(nd);
  std::deque<int> temp_q;
  std::vector<Commit> commits;
  std::vector<std::pair<float, int>> list;

  // DomainIntersector::intersect: advance the ray to the next domain of its
  // list (a new ray starts past the current domain when that domain is the
  // list's first) and queue it there; kNone when the list is exhausted
  auto advance = [&](int current, int idx, std::vector<std::vector<int>>* q) {
    BRay& r = rays[idx];
    domainList(r.org, r.dir, r.tmax, &list);
    const int n = (int)list.size();
    if (r.domain_pos < kNone) r.domain_pos += 1;
    else r.domain_pos = (n && list[0].second == current) ? 1 : 0;
    if (r.domain_pos < n) {
      r.next_tdom = r.domain_pos + 1 < n ? list[r.domain_pos + 1].first : kInf;
      if (q) (*q)[list[r.domain_pos].second].push_back(idx);
    } else {
      r.domain_pos = kNone;
      r.next_tdom = kInf;
    }
  };

  // the shader of a hit in domain id: shadow rays tested here first, then
  // queued in their next domain or retired; the bounce ray joins temp_q
  auto shadeHit = [&](int id, int idx, const Hit& h) {
    const BRay r = rays[idx];
    uint32_t color;
    F3 ns;
    shadingAttributes(doms[id], h, &color, &ns);
    std::vector<ShadowOut> sh;
    BounceOut bo;
    F3 pos;
    shade(r.depth + 1, r.org, r.dir, r.w, r.pixid, r.samid, h.t, id, color, ns, &sh, &bo, &pos);
    for (const ShadowOut& so : sh) {
      if (!so.valid) continue;
      ++s.rays_shadow;
      ++s.visits_shadow;
      if (occludedInDomain(doms[id], pos, so.dir, so.tmax)) continue;
      BRay sr{};
      sr.org = pos;
      sr.dir = so.dir;
      sr.w = so.w;
      sr.pixid = r.pixid;
      sr.samid = r.samid;
      sr.depth = r.depth + 1;
      sr.t = kInf;
      sr.domid = kNone;
      sr.domain_pos = kNone;
      sr.next_tdom = kInf;
      sr.tmax = so.tmax;
      rays.push_back(sr);
      const int si = (int)rays.size() - 1;
      advance(id, si, &sqs);
      if (rays[si].domain_pos == kNone) commits.push_back({r.pixid, so.w});
    }
    if (bo.valid) {
      ++s.rays_bounce;
      BRay br{};
      br.org = pos;
      br.dir = bo.dir;
      br.w = bo.w;
      br.pixid = r.pixid;
      br.samid = r.samid;
      br.depth = r.depth + 1;
      br.t = kInf;
      br.domid = kNone;
      br.domain_pos = kNone;
      br.next_tdom = kInf;
      br.tmax = kInf;
      rays.push_back(br);
      temp_q.push_back((int)rays.size() - 1);
    }
  };

  // processShadow: not occluded here -> next domain, or retired at the end
  auto processShadow = [&](int id, int idx) {
    ++s.visits_shadow;
    const BRay& r = rays[idx];
    if (occludedInDomain(doms[id], r.org, r.dir, r.tmax)) return;
    advance(id, idx, &sqs);
    if (rays[idx].domain_pos == kNone) commits.push_back({rays[idx].pixid, rays[idx].w});
  };

  // processRay2: shade a hit that is known to be the closest, move on, or
  // send the ray back to the domain of its closest hit for shading
  auto processRay = [&](int id, int idx) {
    BRay& r = rays[idx];
    if (r.shade_only) {
      ++s.visits_shade;
      shadeHit(id, idx, r.hit);
      return;
    }
    ++s.visits_radiance;
    Hit h;
    if (closestInDomain(doms[id], r.org, r.dir, &h)) {
      if (h.t < r.t) {
        r.t = h.t;
        r.domid = id;
        r.hit = h;
        if (std::isinf(r.next_tdom) || r.t < r.next_tdom) shadeHit(id, idx, h);
        else advance(id, idx, &qs);
      } else {
        r.shade_only = true;
        qs[r.domid].push_back(idx);
      }
    } else if (std::isinf(r.next_tdom)) {
      if (r.domid < nd) {
        r.shade_only = true;
        qs[r.domid].push_back(idx);
      }
    } else {
      advance(id, idx, &qs);
    }
  };

  // genEyeRays + isectEyeDomains over the single tile of the image (ImgSchedNop)
  rays.reserve((size_t)W * H * spp);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x)
      for (int k = 0; k < spp; ++k) {
        BRay r{};
        const int pixid = y * W + x;
        r.pixid = pixid;
        r.org = cam_pos;
        if (spp > 1) {
          r.samid = spp * pixid + k;
          RandomSampler rs;
          samplerInit(rs, r.samid);
          float fx = (float)x + samplerGet1D(rs);
          float fy = (float)y + samplerGet1D(rs);
          r.dir = generateRay(fx, fy);
        } else {
          r.samid = pixid;
          r.dir = generateRay((float)x, (float)y);
        }
        r.w = f3(1.f, 1.f, 1.f);
        r.t = kInf;
        r.domid = kNone;
        r.tmax = kInf;
        r.next_tdom = kInf;
        rays.push_back(r);
        const int idx = (int)rays.size() - 1;
        domainList(r.org, r.dir, kInf, &list);
        if (!list.empty()) {
          rays[idx].domain_pos = 0;
          rays[idx].next_tdom = list.size() > 1 ? list[1].first : kInf;
          qs[list[0].second].push_back(idx);
        } else {
          rays[idx].domain_pos = kNone;
        }
      }
  s.rays_primary = (int64_t)rays.size();

  LruCache cache;
  cache.init(nd, cfg.cache_size);
  std::vector<int64_t> counts(nd);
  const double scale = 1.0 / (double)spp;
  while (true) {
    for (int i = 0; i < nd; ++i) counts[i] = (int64_t)qs[i].size() + (int64_t)sqs[i].size();
    bool done;
    const int id = loadAnyOnceSchedule(nd, counts.data(), &done);
    if (done) break;
    ++s.rounds;
    if (schedule) schedule->push_back(id);
    if (!cache.load(id)) ++s.domain_loads;
    std::vector<int> shadows, radiance;
    shadows.swap(sqs[id]);
    radiance.swap(qs[id]);
    for (int idx : shadows) processShadow(id, idx);
    for (int idx : radiance) processRay(id, idx);
    while (!temp_q.empty()) {
      const int idx = temp_q.front();
      temp_q.pop_front();
      advance(kNone, idx, nullptr);  // list position only; the ray runs here first
      processRay(id, idx);
    }
    for (const Commit& c : commits) hdrAdd(rgba + 4 * (size_t)c.pixid, c.rgb, scale);
    commits.clear();
  }
  if (out) *out = s;
}

}  // namespace orc

// =================================================================== C API
using orc::F3;
using orc::Oracle;
using orc::f3;

extern "C" {

void* orc_create(const orc_config* cfg, int32_t nd) {
  if (!cfg || nd <= 0) return nullptr;
  Oracle* o = new Oracle();
  o->cfg = *cfg;
  o->doms.resize(nd);
  return o;
}

void orc_destroy(void* o) { delete (Oracle*)o; }

int orc_set_domain(void* ov, int32_t d, const float* v, int64_t nv, const uint32_t* f, int64_t nf,
                   const uint32_t* colors, const float b[6], int32_t bsdf, const float params[3]) {
  Oracle* o = (Oracle*)ov;
  if (!o || d < 0 || d >= o->D()) return 1;
  orc::Domain& D = o->doms[d];
  D.v.assign(v, v + 3 * nv);
  D.f.assign(f, f + 3 * nf);
  if (colors) D.colors.assign(colors, colors + nv);
  else D.colors.assign(nv, 0u);
  for (int k = 0; k < 3; ++k) {
    D.lo[k] = b[k];
    D.hi[k] = b[3 + k];
    D.params[k] = params ? params[k] : 1.f;
  }
  D.bsdf = bsdf;
  return 0;
}

int orc_set_lights(void* ov, int32_t nl, const float* L) {
  Oracle* o = (Oracle*)ov;
  o->lights.clear();
  for (int l = 0; l < nl; ++l) {
    const float* q = L + 13 * l;
    orc::Light li;
    li.type = (int)q[0];
    li.pos = f3(q[1], q[2], q[3]);
    li.radiance = f3(q[4], q[5], q[6]);
    li.e1 = f3(q[7], q[8], q[9]);
    li.e2 = f3(q[10], q[11], q[12]);
    o->lights.push_back(li);
  }
  return 0;
}

extern "C++" {
namespace orc {
// TriMeshBuffer::computeNormals (src/render/trimesh_buffer.cc:267-326):
// unnormalised face normals (u x v) summed into each vertex in face order.
void computeNormals(Domain& D) {
  size_t nv = D.v.size() / 3, nf = D.f.size() / 3;
  D.normals.assign(3 * nv, 0.0f);
  for (size_t i = 0; i < nf; ++i) {
    size_t vid[3] = {D.f[3 * i] * 3ull, D.f[3 * i + 1] * 3ull, D.f[3 * i + 2] * 3ull};
    F3 v0 = f3(D.v[vid[0]], D.v[vid[0] + 1], D.v[vid[0] + 2]);
    F3 v1 = f3(D.v[vid[1]], D.v[vid[1] + 1], D.v[vid[1] + 2]);
    F3 v2 = f3(D.v[vid[2]], D.v[vid[2] + 1], D.v[vid[2] + 2]);
    F3 u = sub(v1, v0), v = sub(v2, v0);
    F3 n;
    n.x = u.y * v.z - u.z * v.y;
    n.y = u.z * v.x - u.x * v.z;
    n.z = u.x * v.y - u.y * v.x;
    for (int k = 0; k < 3; ++k) {
      D.normals[vid[k]] += n.x;
      D.normals[vid[k] + 1] += n.y;
      D.normals[vid[k] + 2] += n.z;
    }
  }
}

// DomainList::sort (src/render/rays.h:71-79): by entry distance, ties by id.
void sortDomainList(std::vector<std::pair<float, int>>* l) {
  std::sort(l->begin(), l->end(), [](const std::pair<float, int>& a, const std::pair<float, int>& b) {
    return (a.first < b.first) || ((a.first == b.first) && (a.second < b.second));
  });
}
}  // namespace orc
}  // extern "C++"

int orc_set_bvh4(void* ov, int32_t d, const float* nodes, int64_t num_nodes, const float* tris,
                 int64_t num_tris) {
  Oracle* o = (Oracle*)ov;
  if (d < 0 || d >= o->D() || num_nodes <= 0 || num_tris < 0 || !nodes || (!tris && num_tris)) return 1;
  orc::Domain& D = o->doms[d];
  if ((uint64_t)num_tris != D.f.size() / 3) return 2;  // one leaf slot per face
  D.b4.nodes.assign(nodes, nodes + 32 * num_nodes);
  D.b4.tris.assign(tris, tris + 12 * num_tris);
  bool all = true;
  for (const auto& x : o->doms) all = all && !x.b4.nodes.empty();
  o->has_bvh4 = all;
  return 0;
}

int orc_build(void* ov) {
  Oracle* o = (Oracle*)ov;
  uint32_t base = 0;
  for (auto& x : o->doms) {
    x.prim_base = base;
    base += (uint32_t)(x.f.size() / 3);
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int d = 0; d < o->D(); ++d) {
    orc::Domain& D = o->doms[d];
    orc::computeNormals(D);
    orc::buildBvh(D.v, D.f, &D.bvh);
  }
  return 0;
}

int orc_domain_list_sort(int32_t n, const int32_t* ids, const float* ts, int32_t* ids_out, float* ts_out) {
  std::vector<std::pair<float, int>> l;
  for (int32_t i = 0; i < n; ++i) l.push_back({ts[i], ids[i]});
  orc::sortDomainList(&l);
  for (int32_t i = 0; i < n; ++i) {
    ids_out[i] = l[i].second;
    ts_out[i] = l[i].first;
  }
  return 0;
}

int orc_mesh_attributes(const float* vertices, int64_t nv, const uint32_t* faces, int64_t nf,
                        const uint32_t* colors, int64_t n, const uint32_t* prim, const float* u, const float* v,
                        uint32_t* color, float* ns, float* normals) {
  orc::Domain D;
  D.v.assign(vertices, vertices + 3 * nv);
  D.f.assign(faces, faces + 3 * nf);
  D.colors.assign(colors, colors + nv);
  orc::computeNormals(D);
  if (normals) std::memcpy(normals, D.normals.data(), D.normals.size() * 4);
  for (int64_t i = 0; i < n; ++i) {
    orc::Hit h;
    h.prim = prim[i];
    h.u = u[i];
    h.v = v[i];
    F3 nn;
    orc::shadingAttributes(D, h, &color[i], &nn);
    ns[3 * i] = nn.x;
    ns[3 * i + 1] = nn.y;
    ns[3 * i + 2] = nn.z;
  }
  return 0;
}

int orc_normals(void* ov, int32_t d, float* out) {
  Oracle* o = (Oracle*)ov;
  std::memcpy(out, o->doms[d].normals.data(), o->doms[d].normals.size() * 4);
  return 0;
}

int orc_set_camera(void* ov, const float p[3], const float l[3], const float up[3], float vfov) {
  ((Oracle*)ov)->setCamera(p, l, up, vfov);
  return 0;
}

int32_t orc_tiles(void* ov, int32_t* out, int32_t cap) {
  auto t = ((Oracle*)ov)->tiles();
  for (int32_t i = 0; i < (int32_t)t.size() && i < cap; ++i) {
    out[4 * i] = t[i].x;
    out[4 * i + 1] = t[i].y;
    out[4 * i + 2] = t[i].w;
    out[4 * i + 3] = t[i].h;
  }
  return (int32_t)t.size();
}

int64_t orc_gen_eyes(void* ov, int32_t first, int32_t count, float* org, float* dir, int32_t* pixid,
                     int32_t* samid) {
  Oracle* o = (Oracle*)ov;
  auto tl = o->tiles();
  int64_t k = 0;
  for (int32_t t = first; t < first + count && t < (int32_t)tl.size(); ++t) {
    int64_t n = (int64_t)tl[t].w * tl[t].h * o->cfg.pixel_samples;
    for (int64_t i = 0; i < n; ++i, ++k) {
      F3 d;
      int pid;
      o->eye(tl[t], i, &d, &pid);
      org[3 * k] = o->cam_pos.x;
      org[3 * k + 1] = o->cam_pos.y;
      org[3 * k + 2] = o->cam_pos.z;
      dir[3 * k] = d.x;
      dir[3 * k + 1] = d.y;
      dir[3 * k + 2] = d.z;
      pixid[k] = pid;
      samid[k] = (int32_t)i;
    }
  }
  return k;
}

int64_t orc_schedule(void* ov, int64_t n, const float* org, const float* dir, const float* tmax,
                     const int32_t* origin, int32_t* entries, int64_t cap, int64_t* dstats) {
  Oracle* o = (Oracle*)ov;
  const int D = o->D(), L = o->cfg.list_size;
  struct E {
    int ray;
    float t;
    int depth;
    int origin;
  };
  std::vector<std::vector<E>> q(D);
  std::vector<std::pair<float, int>> list;
  if (dstats) std::fill(dstats, dstats + (size_t)D * L, 0);
  for (int64_t i = 0; i < n; ++i) {
    F3 og = f3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    F3 dr = f3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    float tm = tmax ? tmax[i] : orc::kInf;
    o->domainList(og, dr, tm, &list);
    if (origin) {
      int od = origin[i];
      float ot = 0.f;
      for (auto& e : list)
        if (e.second == od) ot = e.first;
      q[od].push_back(E{(int)i, ot, 0, 1});
    }
    for (size_t k = 0; k < list.size(); ++k) {
      int id = list[k].second;
      if (origin && id == origin[i]) continue;
      q[id].push_back(E{(int)i, list[k].first, (int)k, 0});
      if (dstats && (int)k < L) ++dstats[(size_t)id * L + k];
    }
  }
  int64_t total = 0;
  for (auto& v : q) total += (int64_t)v.size();
  if (total > cap) return -1;
  int64_t k = 0;
  for (int d = 0; d < D; ++d)
    for (auto& e : q[d]) {
      entries[5 * k] = d;
      entries[5 * k + 1] = e.ray;
      std::memcpy(&entries[5 * k + 2], &e.t, 4);
      entries[5 * k + 3] = e.depth;
      entries[5 * k + 4] = e.origin;
      ++k;
    }
  return total;
}

int orc_scores(void* ov, const int64_t* dstats, int64_t* scores, int32_t* order) {
  Oracle* o = (Oracle*)ov;
  orc::DomainStats s;
  s.resize(o->D(), o->cfg.list_size);
  std::memcpy(s.stats.data(), dstats, s.stats.size() * 8);
  s.schedule();
  for (int i = 0; i < o->D(); ++i) {
    scores[s.scores[i].second] = s.scores[i].first;
    order[i] = s.schedule_[i];
  }
  return 0;
}

int orc_closest(void* ov, int64_t n, const float* org, const float* dir, int32_t* hit, float* t,
                int32_t* domain, int32_t* prim, float* u, float* v, uint32_t* color, float* ns) {
  Oracle* o = (Oracle*)ov;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    orc::Hit h;
    int d;
    F3 og = f3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    F3 dr = f3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    if (o->closest(og, dr, &h, &d, nullptr)) {
      hit[i] = 1;
      t[i] = h.t;
      domain[i] = d;
      prim[i] = (int32_t)h.prim;
      u[i] = h.u;
      v[i] = h.v;
      F3 nn;
      orc::shadingAttributes(o->doms[d], h, &color[i], &nn);
      ns[3 * i] = nn.x;
      ns[3 * i + 1] = nn.y;
      ns[3 * i + 2] = nn.z;
    } else {
      hit[i] = 0;
      t[i] = orc::kInf;
      domain[i] = -1;
      prim[i] = -1;
      u[i] = v[i] = 0.f;
      color[i] = 0;
      ns[3 * i] = ns[3 * i + 1] = ns[3 * i + 2] = 0.f;
    }
  }
  return 0;
}

int orc_occluded(void* ov, int64_t n, const float* org, const float* dir, const float* tmax,
                 const int32_t* origin, uint8_t* occ) {
  Oracle* o = (Oracle*)ov;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    F3 og = f3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    F3 dr = f3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    occ[i] = o->occluded(og, dr, tmax ? tmax[i] : orc::kInf, origin[i], nullptr) ? 1 : 0;
  }
  return 0;
}

int32_t orc_slots(void* ov) { return ((Oracle*)ov)->slots(); }

int orc_shade(void* ov, int32_t depth, int64_t n, const float* org, const float* dir, const float* w,
              const int32_t* pixid, const int32_t* samid, const float* t, const int32_t* domain,
              const uint32_t* color, const float* ns, float* sdir, float* sw, float* stmax,
              uint8_t* svalid, float* bdir, float* bw, uint8_t* bvalid) {
  Oracle* o = (Oracle*)ov;
  const int S = o->slots();
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    std::vector<Oracle::ShadowOut> sh;
    Oracle::BounceOut bo;
    F3 pos;
    o->shade(depth + 1, f3(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
             f3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), f3(w[3 * i], w[3 * i + 1], w[3 * i + 2]),
             pixid[i], samid[i], t[i], domain[i], color[i], f3(ns[3 * i], ns[3 * i + 1], ns[3 * i + 2]),
             &sh, &bo, &pos);
    for (int s = 0; s < S; ++s) {
      size_t k = (size_t)i * S + s;
      bool have = s < (int)sh.size();
      const Oracle::ShadowOut so = have ? sh[s] : Oracle::ShadowOut{};
      sdir[3 * k] = so.dir.x;
      sdir[3 * k + 1] = so.dir.y;
      sdir[3 * k + 2] = so.dir.z;
      sw[3 * k] = so.w.x;
      sw[3 * k + 1] = so.w.y;
      sw[3 * k + 2] = so.w.z;
      stmax[k] = so.tmax;
      svalid[k] = have && so.valid;
    }
    bdir[3 * i] = bo.dir.x;
    bdir[3 * i + 1] = bo.dir.y;
    bdir[3 * i + 2] = bo.dir.z;
    bw[3 * i] = bo.w.x;
    bw[3 * i + 1] = bo.w.y;
    bw[3 * i + 2] = bo.w.z;
    bvalid[i] = bo.valid;
  }
  return 0;
}

int orc_rng(int32_t seed, int32_t n, float* out) {
  orc::RandomSampler r;
  orc::samplerInit(r, seed);
  for (int32_t i = 0; i < n; ++i) out[i] = orc::samplerGet1D(r);
  return 0;
}

int orc_sincos(int64_t n, const float* x, float* s, float* c) {
  for (int64_t i = 0; i < n; ++i) orc::sinCos(x[i], &s[i], &c[i]);
  return 0;
}

int orc_slab(const float b[6], const float org[3], const float dir[3], float t0, float t1, float* tmin,
             float* tmax) {
  *tmin = *tmax = 0.f;
  return orc::intersectAabb(b, b + 3, org, dir, t0, t1, tmin, tmax) ? 1 : 0;
}

int orc_triangle(const float org[3], const float dir[3], const float v[9], float tnear, float tfar,
                 float* t, float* u, float* vv) {
  F3 d = f3(dir[0], dir[1], dir[2]);
  orc::Shear sh = orc::makeShear(d);
  return orc::triangleHit(sh, f3(org[0], org[1], org[2]), f3(v[0], v[1], v[2]), f3(v[3], v[4], v[5]),
                          f3(v[6], v[7], v[8]), tnear, tfar, t, u, vv)
             ? 1
             : 0;
}

int orc_camera_rays(const float pos[3], const float lookat[3], const float up[3], float vfov, int32_t w,
                    int32_t h, int64_t n, const float* xy, float* dir) {
  if (w <= 0 || h <= 0 || n < 0) return 1;
  Oracle o;
  o.cfg = orc_config{};
  o.cfg.image_w = w;
  o.cfg.image_h = h;
  o.setCamera(pos, lookat, up, vfov);
  for (int64_t i = 0; i < n; ++i) {
    F3 d = o.generateRay(xy[2 * i], xy[2 * i + 1]);
    for (int k = 0; k < 3; ++k) dir[3 * i + k] = d[k];
  }
  return 0;
}

int orc_disk(int64_t n, const float* u, float* d) {
  for (int64_t i = 0; i < n; ++i) orc::concentricDisk(u[2 * i], u[2 * i + 1], &d[2 * i], &d[2 * i + 1]);
  return 0;
}

int orc_local_to_world(int64_t n, const float* N, const float* v, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    F3 r = orc::localToWorld(f3(N[3 * i], N[3 * i + 1], N[3 * i + 2]), f3(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = r[k];
  }
  return 0;
}

int orc_cosine_sample(int64_t n, const float* u, const float* N, float* wi, float* pdf) {
  for (int64_t i = 0; i < n; ++i) {
    F3 d;
    orc::cosineSample(u[2 * i], u[2 * i + 1], f3(N[3 * i], N[3 * i + 1], N[3 * i + 2]), &d, &pdf[i]);
    for (int k = 0; k < 3; ++k) wi[3 * i + k] = d[k];
  }
  return 0;
}

// the shaders' point-light shadow direction, normalize(light - p)
// (PointLight::sample, src/render/light.h:47-52)
int orc_point_light(int64_t n, const float* light, const float* p, float* wi) {
  for (int64_t i = 0; i < n; ++i) {
    F3 d = orc::normalize(orc::sub(f3(light[3 * i], light[3 * i + 1], light[3 * i + 2]),
                                   f3(p[3 * i], p[3 * i + 1], p[3 * i + 2])));
    for (int k = 0; k < 3; ++k) wi[3 * i + k] = d[k];
  }
  return 0;
}

int orc_blinn_phong(int64_t n, const float* a, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 20 * i;
    auto v = [&](int o) { return f3(p[o], p[o + 1], p[o + 2]); };
    F3 r = orc::blinnPhong(p[0], v(1), v(4), p[7], v(8), v(11), v(14), v(17));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = r[k];
  }
  return 0;
}

int orc_unpack_color(int64_t n, const uint32_t* color, float* rgb) {
  for (int64_t i = 0; i < n; ++i) {
    F3 c = orc::unpack(color[i]);
    for (int k = 0; k < 3; ++k) rgb[3 * i + k] = c[k];
  }
  return 0;
}

int orc_reflect(int64_t n, const float* wo, const float* N, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    F3 r = orc::reflect(f3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), f3(N[3 * i], N[3 * i + 1], N[3 * i + 2]));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = r[k];
  }
  return 0;
}

int orc_fr_dielectric(int64_t n, const float* a, float* fr, float* wt) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 9 * i;
    F3 t = f3(0, 0, 0);
    fr[i] = orc::frDielectric(p[0], p[1], p[2], f3(p[3], p[4], p[5]), f3(p[6], p[7], p[8]), &t);
    for (int k = 0; k < 3; ++k) wt[3 * i + k] = t[k];
  }
  return 0;
}

int orc_refract(int64_t n, const float* a, uint8_t* ok, float* wt) {
  for (int64_t i = 0; i < n; ++i) {
    const float* p = a + 9 * i;
    F3 t = f3(0, 0, 0);
    ok[i] = orc::refract(p[0], p[1], p[2], f3(p[3], p[4], p[5]), f3(p[6], p[7], p[8]), &t) ? 1 : 0;
    for (int k = 0; k < 3; ++k) wt[3 * i + k] = t[k];
  }
  return 0;
}

int orc_hdr_add(int64_t n, const int32_t* pixid, const float* rgb, double scale, float* rgba) {
  for (int64_t i = 0; i < n; ++i)
    orc::hdrAdd(rgba + 4 * (size_t)pixid[i], f3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]), scale);
  return 0;
}

int orc_vbuf_trace(int32_t nsamples, int32_t H, int64_t n, const uint8_t* op, const int32_t* samid,
                   const int32_t* depth, float* hist, const float* t, uint8_t* result) {
  if (H < 1 || H > orc::kMaxHistory) return 1;
  orc::VBuf vb;
  vb.resize((size_t)nsamples, H);
  for (int64_t i = 0; i < n; ++i) {
    orc::Ray r{};
    r.samid = samid[i];
    r.depth = depth[i];
    for (int k = 0; k < H; ++k) r.history[k] = hist[H * i + k];
    result[i] = (op[i] == 0 ? vb.update(t[i], &r) : vb.correct(r)) ? 1 : 0;
    for (int k = 0; k < H; ++k) hist[H * i + k] = r.history[k];
  }
  return 0;
}

int orc_lru_trace(int32_t nd, int32_t cache_size, int64_t n, const int32_t* ids, uint8_t* hits,
                  int32_t* evicted) {
  orc::LruCache c;
  c.init(nd, cache_size);
  for (int64_t i = 0; i < n; ++i) {
    const bool h = c.load(ids[i]);
    hits[i] = h ? 1 : 0;
    if (evicted) evicted[i] = h ? -1 : c.last_evicted;
  }
  return 0;
}

int orc_render_wavefront(void* ov, float* rgba, orc_stats* st) {
  try {
    ((Oracle*)ov)->renderWavefront(rgba, st);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

int orc_render_baseline(void* ov, float* rgba, orc_stats* st) {
  try {
    Oracle* o = (Oracle*)ov;
    o->baseline_schedule.clear();
    o->renderBaseline(rgba, st, &o->baseline_schedule);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

int64_t orc_baseline_schedule(void* ov, int32_t* out, int64_t capacity) {
  const std::vector<int>& s = ((Oracle*)ov)->baseline_schedule;
  if (out) std::copy(s.begin(), s.begin() + std::min<int64_t>(capacity, (int64_t)s.size()), out);
  return (int64_t)s.size();
}

int orc_load_any_once(int32_t nd, const int64_t* counts, int32_t* id, uint8_t* done) {
  if (nd <= 0 || !counts || !id || !done) return 1;
  bool d;
  *id = orc::loadAnyOnceSchedule(nd, counts, &d);
  *done = d ? 1 : 0;
  return 0;
}

int orc_render_speculative(void* ov, int32_t nthreads, float* rgba, orc_stats* st) {
  try {
    ((Oracle*)ov)->renderSpeculative(std::max(1, nthreads), rgba, st);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

}  // extern "C"
