// Scalar math shared by the CUDA kernels and the host code of the tracer.
//
// Every function here is written so that the same source compiled by nvcc
// (with -fmad=false) and by g++ (with -ffp-contract=off) produces bit-identical
// results: only IEEE add/sub/mul/div/sqrt, no fused multiply-add, no library
// transcendental on a path whose bits matter.
#pragma once

#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define SPRAY_HD __host__ __device__ __forceinline__
#else
#define SPRAY_HD inline
#endif

namespace spray {

// SpRay constants (src/render/spray.h:46-60)
constexpr float kRayEpsilon = 0.001f;          // SPRAY_RAY_EPSILON, tnear of every ray
constexpr float kOneOverPi = 0.3183098861837907f;  // SPRAY_ONE_OVER_PI
constexpr double kOneOver255 = 0.00392156862745098;  // SPRAY_1_OVER_255
constexpr double kPi = 3.14159265358979323846;

struct V3 {
  float x, y, z;
};

SPRAY_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
SPRAY_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SPRAY_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SPRAY_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
SPRAY_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
SPRAY_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
SPRAY_HD V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
SPRAY_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
SPRAY_HD float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
SPRAY_HD V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
// v * (1 / sqrt(dot(v, v)))
SPRAY_HD V3 normalize(V3 v) {
  float r = 1.0f / sqrtf(dot(v, v));
  return v * r;
}
// min/max/clamp as comparisons so that NaN propagates like the reference's
// vector library (max(x, y) = x < y ? y : x)
SPRAY_HD float fmax_ref(float x, float y) { return (x < y) ? y : x; }
SPRAY_HD float fmin_ref(float x, float y) { return (y < x) ? y : x; }
SPRAY_HD float clamp_ref(float x, float lo, float hi) { return fmin_ref(fmax_ref(x, lo), hi); }
SPRAY_HD bool hasPositive(V3 v) { return v.x > 0.0f || v.y > 0.0f || v.z > 0.0f; }

// ---------------------------------------------------------------- RNG
// Restates SpRay's RandomSampler (deps/embree/random_sampler.h:34-108):
// MurmurHash3 mix + finalize of the seed, then an LCG (1664525, 1013904223)
// whose state >> 1 is scaled by 2^-31.
SPRAY_HD uint32_t rngSeed(int32_t id) {
  uint32_t k = (uint32_t)id;
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  uint32_t h = 0u ^ k;
  h = ((h << 13) | (h >> 19)) * 5u + 0xe6546b64u;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
SPRAY_HD float rngNext(uint32_t& s) {
  s = s * 1664525u + 1013904223u;
  return (float)(int32_t)(s >> 1) * 4.656612873077392578125e-10f;
}

// ---------------------------------------------------------------- sin / cos
// sin and cos for |x| <= 2*pi: Cody-Waite reduction by pi/2 (three-part
// constant, first part exact for small multiples) and Taylor polynomials
// (coefficients 1/n!) on [-pi/4, pi/4], evaluated in a fixed order so host and
// device agree bit for bit.  Accuracy is within a few ulp of the true value.
SPRAY_HD void sincosPoly(float x, float* s_out, float* c_out) {
  const float twoOverPi = 0.636619772367581343f;
  float q = x * twoOverPi;
  int k = (int)(q >= 0.0f ? q + 0.5f : q - 0.5f);
  float kf = (float)k;
  // pi/2 = A + B + C with A holding 11 significant bits
  const float A = 1.5703125f;
  const float B = 4.838267923332751e-4f;
  const float C = 2.5632829192545614e-12f;
  float r = x - kf * A;
  r = r - kf * B;
  r = r - kf * C;
  float r2 = r * r;
  float sp = 2.75573192e-6f;            // 1/9!
  sp = sp * r2 + -1.98412698e-4f;       // -1/7!
  sp = sp * r2 + 8.33333333e-3f;        // 1/5!
  sp = sp * r2 + -1.66666667e-1f;       // -1/3!
  float sn = r + (r * r2) * sp;
  float cp = -2.75573192e-7f;           // -1/10!
  cp = cp * r2 + 2.48015873e-5f;        // 1/8!
  cp = cp * r2 + -1.38888889e-3f;       // -1/6!
  cp = cp * r2 + 4.16666667e-2f;        // 1/4!
  cp = cp * r2 + -0.5f;                 // -1/2!
  float cs = 1.0f + r2 * cp;
  int m = k & 3;
  float s, c;
  if (m == 0) { s = sn; c = cs; }
  else if (m == 1) { s = cs; c = -sn; }
  else if (m == 2) { s = -sn; c = -cs; }
  else { s = -cs; c = sn; }
  *s_out = s;
  *c_out = c;
}

// x^e for the Blinn-Phong lobe.  Integral exponents in [0, 256] use binary
// exponentiation (identical on host and device); other exponents fall back to
// powf, whose last bits may differ between host and device.
SPRAY_HD float powShininess(float x, float e) {
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
  return powf(x, e);
}

// ---------------------------------------------------------------- sampling
// Concentric disk mapping and cosine-weighted hemisphere sample about N
// (src/render/sampler.h:49-120, sampler.cc:54-60).  theta is scaled by pi/4 in
// double precision and rounded to float, as the reference's mixed-precision
// expression does.
SPRAY_HD void concentricDisk(float u1, float u2, float* dx, float* dy) {
  float sx = 2 * u1 - 1;
  float sy = 2 * u2 - 1;
  if (sx == 0.0f && sy == 0.0f) {
    *dx = 0.0f;
    *dy = 0.0f;
    return;
  }
  float r, theta;
  if (sx >= -sy) {
    if (sx > sy) {
      r = sx;
      if (sy > 0.0f) theta = sy / r;
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
  theta = (float)((double)theta * (kPi / 4.0));
  float s, c;
  sincosPoly(theta, &s, &c);
  *dx = r * c;
  *dy = r * s;
}

SPRAY_HD V3 localToWorld(V3 N, V3 v) {
  V3 dx0 = v3(0, N.z, -N.y);
  V3 dx1 = v3(-N.z, 0, N.x);
  V3 dx = normalize(dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1);
  V3 dy = normalize(cross(N, dx));
  return V3{(dx.x * v.x + dy.x * v.y) + N.x * v.z, (dx.y * v.x + dy.y * v.y) + N.y * v.z,
            (dx.z * v.x + dy.z * v.y) + N.z * v.z};
}

SPRAY_HD void cosineHemisphereSample(float u1, float u2, V3 N, V3* wi, float* pdf) {
  V3 v;
  concentricDisk(u1, u2, &v.x, &v.y);
  v.z = sqrtf(fmax_ref(0.f, (1.f - v.x * v.x) - v.y * v.y));
  v = normalize(v);
  *wi = normalize(localToWorld(N, v));
  *pdf = v.z * kOneOverPi;
}

// ---------------------------------------------------------------- slab test
// SpRay's ray/AABB slab test (src/render/aabb.h:139-169), t0 = 1e-3, used to
// build a ray's domain list.  Bit-exact: IEEE reciprocal, no contraction.
SPRAY_HD bool slabTest(const float bmin[3], const float bmax[3], V3 org, V3 inv, float t0, float t1,
                       float* tmin_o) {
  int sx = inv.x < 0.0f, sy = inv.y < 0.0f, sz = inv.z < 0.0f;
  float tmin = ((sx ? bmax[0] : bmin[0]) - org.x) * inv.x;
  float tmax = ((sx ? bmin[0] : bmax[0]) - org.x) * inv.x;
  float tymin = ((sy ? bmax[1] : bmin[1]) - org.y) * inv.y;
  float tymax = ((sy ? bmin[1] : bmax[1]) - org.y) * inv.y;
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  float tzmin = ((sz ? bmax[2] : bmin[2]) - org.z) * inv.z;
  float tzmax = ((sz ? bmin[2] : bmax[2]) - org.z) * inv.z;
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  *tmin_o = tmin;
  return (tmin < t1) && (tmax > t0);
}

// ---------------------------------------------------------------- triangles
// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013).  Per-ray shear constants, edge functions
// recomputed in double when one is exactly zero, no backface culling.
// Barycentrics follow the (u, v) convention of the reference's hit record:
// hit = (1-u-v)*v0 + u*v1 + v*v2.
struct RayShear {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

SPRAY_HD float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

SPRAY_HD RayShear makeShear(V3 d) {
  RayShear s;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = 0;
  float m = ax;
  if (ay > m) { kz = 1; m = ay; }
  if (az > m) { kz = 2; }
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (comp(d, kz) < 0.0f) {
    int t = kx;
    kx = ky;
    ky = t;
  }
  s.kx = kx;
  s.ky = ky;
  s.kz = kz;
  float dz = comp(d, kz);
  s.Sx = comp(d, kx) / dz;
  s.Sy = comp(d, ky) / dz;
  s.Sz = 1.0f / dz;
  return s;
}

// Returns true with t, u, v when the triangle is hit with tnear < t < tfar.
SPRAY_HD bool intersectTriangle(const RayShear& sh, V3 org, V3 p0, V3 p1, V3 p2, float tnear,
                                float tfar, float* t_o, float* u_o, float* v_o) {
  V3 A = p0 - org, B = p1 - org, C = p2 - org;
  float Akz = comp(A, sh.kz), Bkz = comp(B, sh.kz), Ckz = comp(C, sh.kz);
  float Ax = comp(A, sh.kx) - sh.Sx * Akz;
  float Ay = comp(A, sh.ky) - sh.Sy * Akz;
  float Bx = comp(B, sh.kx) - sh.Sx * Bkz;
  float By = comp(B, sh.ky) - sh.Sy * Bkz;
  float Cx = comp(C, sh.kx) - sh.Sx * Ckz;
  float Cy = comp(C, sh.ky) - sh.Sy * Ckz;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
    U = (float)(CxBy - CyBx);
    double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
    V = (float)(AxCy - AyCx);
    double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
    W = (float)(BxAy - ByAx);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = (U + V) + W;
  if (det == 0.0f) return false;
  float Az = sh.Sz * Akz, Bz = sh.Sz * Bkz, Cz = sh.Sz * Ckz;
  float T = (U * Az + V * Bz) + W * Cz;
  float rcp = 1.0f / det;
  float t = T * rcp;
  if (!(t > tnear && t < tfar)) return false;
  *t_o = t;
  *u_o = V * rcp;
  *v_o = W * rcp;
  return true;
}

// Packed closest-hit key: positive-float bits of t in the high word, the
// global triangle number in the low word.  Smaller key = closer hit, ties
// broken by the lower (domain, primitive).
SPRAY_HD uint64_t packHitKey(float t, uint32_t gprim) {
  union {
    float f;
    uint32_t u;
  } c;
  c.f = t;
  return ((uint64_t)c.u << 32) | (uint64_t)gprim;
}
SPRAY_HD float hitKeyT(uint64_t key) {
  union {
    float f;
    uint32_t u;
  } c;
  c.u = (uint32_t)(key >> 32);
  return c.f;
}
constexpr uint64_t kNoHit = ~0ull;

// Interpolated vertex colour with truncation to integer channels and the
// unnormalised shading normal (src/render/trimesh_buffer.cc:328-360).
SPRAY_HD uint32_t interpolateColor(uint32_t c0, uint32_t c1, uint32_t c2, float u, float v) {
  float w = 1.f - u - v;
  uint32_t out = 0;
  for (int sh = 16; sh >= 0; sh -= 8) {
    float a = (float)((c0 >> sh) & 0xffu), b = (float)((c1 >> sh) & 0xffu),
          c = (float)((c2 >> sh) & 0xffu);
    float x = (a * w + b * u) + c * v;
    uint32_t q = x > 0.0f ? (uint32_t)x : 0u;  // negative rounding noise clamps to 0
    if (q > 255u) q = 255u;
    out |= q << sh;
  }
  return out;
}

SPRAY_HD V3 interpolateNormal(V3 n0, V3 n1, V3 n2, float u, float v) {
  float w = 1.f - u - v;
  return V3{(n0.x * w + n1.x * u) + n2.x * v, (n0.y * w + n1.y * u) + n2.y * v,
            (n0.z * w + n1.z * u) + n2.z * v};
}

}  // namespace spray
