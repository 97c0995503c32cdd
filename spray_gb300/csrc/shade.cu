// AO and path-tracing shaders applied to resolved closest hits, and the
// retire step that accumulates unoccluded shadow rays into the image.
//
// The shaders restate ShaderAo::operator() (src/ooc/ooc_shader_ao.h:92-197)
// and ShaderPt::operator() (src/ooc/ooc_shader_pt.h:93-227) for the single
// hit a wavefront keeps per sample: the speculative loop only retires shadow
// rays whose history matches the sample's closest hits
// (src/ooc/ooc_vbuf.cc:41-52, ooc_tcontext.inl:123-135), which are exactly
// the rays spawned here.  Shadow ray `slot` of alive ray a lives at
// a * slots + slot.
#include <algorithm>

#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {

__constant__ float c_unpack[256];  // i * SPRAY_1_OVER_255 rounded to float

namespace {

__device__ __forceinline__ V3 unpackColor(uint32_t c) {
  return v3(c_unpack[(c >> 16) & 0xffu], c_unpack[(c >> 8) & 0xffu], c_unpack[c & 0xffu]);
}

// src/render/reflection.h:202-214
__device__ __forceinline__ V3 blinnPhong(float costheta, V3 kd, V3 ks, float shininess, V3 li,
                                         V3 wi, V3 n_hat, V3 wo) {
  V3 half_hat = normalize(wi + wo);
  float n_dot_h = clamp_ref(dot(n_hat, half_hat), 0.0f, 1.0f);
  V3 cs = ks * powShininess(n_dot_h, shininess);
  V3 cd = kd * costheta;
  return li * (cd + cs);
}

__device__ __forceinline__ void writeShadow(const ShadeArgs& a, uint32_t sid, V3 wi, V3 w, float tmax,
                                            bool valid) {
  if (valid) {
    a.sh.dir[sid] = make_float4(wi.x, wi.y, wi.z, tmax);
    a.sh.wgt[sid] = make_float4(w.x, w.y, w.z, 1.0f);
  }
  a.shadow_flag[sid] = valid ? 1 : 0;
}

__device__ __forceinline__ int domainOfPrim(const DomainDev* doms, int D, uint32_t gprim) {
  int lo = 0, hi = D - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (doms[mid].gprim_base <= gprim) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Fresnel term for dielectrics (src/render/reflection.h:134-158).
__device__ float frDielectric(float cosThetaI, float etaI, float etaT, V3 wo, V3 nff, V3* wt) {
  float sin2ThetaI = fmax_ref(0.0f, 1.0f - (cosThetaI * cosThetaI));
  float eta = etaI / etaT;
  float sin2ThetaT = eta * eta * sin2ThetaI;
  if (sin2ThetaT >= 1.0f) return 1.0f;
  float cosThetaT = sqrtf(1.0f - sin2ThetaT);
  float Rparl = ((etaT * cosThetaI) - (etaI * cosThetaT)) / ((etaT * cosThetaI) + (etaI * cosThetaT));
  float Rperp = ((etaI * cosThetaI) - (etaT * cosThetaT)) / ((etaI * cosThetaI) + (etaT * cosThetaT));
  float fr = (Rparl * Rparl + Rperp * Rperp) / 2.0f;
  *wt = (eta * -wo) + (nff * (eta * cosThetaI - cosThetaT));
  return fr;
}

}  // namespace

// Domains whose first global face number the shader keeps in shared memory
// for the hit's domain search (more domains search the device table).
constexpr int kShadeSmemDomains = 4096;

// Four resident blocks per SM (64 registers): the shader is latency-bound,
// and occupancy pays more than the few spills (measured against 94 registers).
__global__ void __launch_bounds__(256, 4) kShade(ShadeArgs a) {
  __shared__ uint32_t sprim[kShadeSmemDomains];
  const int D = a.scene.num_domains;
  const bool stab = D <= kShadeSmemDomains;
  if (stab)
    for (int k = threadIdx.x; k < D; k += blockDim.x) sprim[k] = a.scene.domains[k].gprim_base;
  __syncthreads();
  const uint32_t n = *a.count;
  const int S = a.slots;
  unsigned long long nshadow = 0, nbounce = 0;
  // a contiguous range of alive rays per block (the compaction's partition)
  const uint64_t per = ((uint64_t)n + gridDim.x - 1) / gridDim.x;
  const uint64_t i0 = min((uint64_t)n, per * blockIdx.x), i1 = min((uint64_t)n, i0 + per);
  for (uint64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const uint32_t sample = a.list[i];
    const uint64_t key = a.ray_key[sample];
    a.next_flag[sample] = 0;  // set below when a bounce ray is emitted
    const uint32_t sbase = (uint32_t)i * S;
    if (key == kNoHit) {
      for (int s = 0; s < S; ++s) a.shadow_flag[sbase + s] = 0;
      continue;
    }
    const float t = hitKeyT(key);
    // the sample's loads first: they do not depend on the domain search
    // primary rays (depth 0) carry weight 1, which kGenPrimary does not store
    const float4 o4 = a.rays.org[sample], d4 = a.rays.dir[sample];
    const float4 w4 = a.depth == 0 ? make_float4(1.f, 1.f, 1.f, 0.f) : a.rays.wgt[sample];
    const float4 hn = a.hit_ns[sample];
    int d;
    if (stab) {
      // last domain whose first global face is <= the hit's
      const uint32_t gprim = (uint32_t)key;
      int lo = 0, hi = D - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sprim[mid] <= gprim) lo = mid;
        else hi = mid - 1;
      }
      d = lo;
    } else {
      d = domainOfPrim(a.scene.domains, D, (uint32_t)key);
    }
    const DomainDev dom = a.scene.domains[d];
    const V3 org = v3(o4.x, o4.y, o4.z), dir = v3(d4.x, d4.y, d4.z);
    const V3 Lin = v3(w4.x, w4.y, w4.z);
    const V3 pos = v3(dir.x * t + org.x, dir.y * t + org.y, dir.z * t + org.z);
    const V3 normal = v3(hn.x, hn.y, hn.z);
    const V3 surf = unpackColor(__float_as_uint(hn.w));
    V3 wo = -dir;
    float cos_theta_i = dot(wo, normal);
    const bool entering = cos_theta_i > 0.0f;
    const V3 nff = normalize(entering ? normal : -normal);
    const bool delta = dom.bsdf != 0;
    const int pixid = a.rays.pixid[sample];
    const int samid = a.rays.samid[sample];
    const ViewDev& vw = a.views[a.rays.view[sample]];
    const int ao_mode = vw.ao_mode, ao_samples = vw.ao_samples, bounces = vw.bounces;
    const int rr_depth = vw.rr_depth, ao_light_shadow = vw.ao_light_shadow;
    const float ao_max_distance = vw.ao_max_distance;
    const int next_depth = a.depth + 1;
    a.sh.hitpos[i] = make_float4(pos.x, pos.y, pos.z, __int_as_float(d));
    int slot = 0;
    if (ao_mode) {
      const float ao_weight = 1.0f / (float)ao_samples;
      const float tmax = ao_max_distance > 0.0f ? ao_max_distance : __int_as_float(0x7f800000);
      for (int l = 0; l < ao_samples; ++l, ++slot) {
        bool valid = false;
        V3 wi = v3(0, 0, 0), Lr = v3(0, 0, 0);
        if (!delta) {
          uint32_t st = rngSeed((int32_t)((uint32_t)pixid * (uint32_t)(l + 1)));
          float u1 = rngNext(st), u2 = rngNext(st);
          float pdf;
          cosineHemisphereSample(u1, u2, nff, &wi, &pdf);
          float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
          Lr = (Lin * surf) * (((kOneOverPi * costheta) * ao_weight) / pdf);
          valid = hasPositive(Lr);
        }
        writeShadow(a, sbase + slot, wi, Lr, tmax, valid);
        nshadow += valid;
      }
      if (ao_light_shadow) {
        bool valid = false;
        V3 wi = v3(0, 0, 0), Lr = v3(0, 0, 0);
        if (a.num_lights > 0) {
          const float* L = a.lights;
          wi = normalize(v3(L[1], L[2], L[3]) - pos);
          float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
          Lr = ((Lin * surf) * v3(L[4], L[5], L[6])) * (kOneOverPi * costheta);
          valid = hasPositive(Lr);
        }
        writeShadow(a, sbase + slot, wi, Lr, __int_as_float(0x7f800000), valid);
        nshadow += valid;
        ++slot;
      }
    } else if (!delta) {
      const V3 ks = v3(a.ks[0], a.ks[1], a.ks[2]);
      uint32_t st = rngSeed((int32_t)((uint32_t)samid * (uint32_t)next_depth));
      for (int l = 0; l < a.num_lights; ++l) {
        const float* L = a.lights + 13 * l;
        const int type = (int)L[0];
        const V3 radiance = v3(L[4], L[5], L[6]);
        if (type == 1) {  // hemisphere "diffuse" light (light.h:67-89)
          for (int s = 0; s < ao_samples; ++s, ++slot) {
            float u1 = rngNext(st), u2 = rngNext(st);
            V3 wi;
            float pdf;
            cosineHemisphereSample(u1, u2, nff, &wi, &pdf);
            bool valid = false;
            V3 Lr = v3(0, 0, 0);
            if (pdf > 0.0f) {
              float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
              Lr = (Lin * blinnPhong(costheta, surf, ks, a.shininess, radiance, wi, nff, wo)) *
                   (1.0f / (pdf * (float)ao_samples));
              valid = hasPositive(Lr);
            }
            writeShadow(a, sbase + slot, wi, Lr, __int_as_float(0x7f800000), valid);
            nshadow += valid;
          }
        } else if (type == 0) {  // point light (light.h:41-65)
          V3 wi = normalize(v3(L[1], L[2], L[3]) - pos);
          float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
          V3 Lr = (Lin * blinnPhong(costheta, surf, ks, a.shininess, radiance, wi, nff, wo)) *
                  (1.0f / 1.0f);
          bool valid = hasPositive(Lr);
          writeShadow(a, sbase + slot, wi, Lr, __int_as_float(0x7f800000), valid);
          nshadow += valid;
          ++slot;
        } else {  // emissive quad (extension): uniform area sampling
          const V3 p0 = v3(L[1], L[2], L[3]);
          const V3 e1 = v3(L[7], L[8], L[9]), e2 = v3(L[10], L[11], L[12]);
          const V3 nq = cross(e1, e2);
          const float area = sqrtf(dot(nq, nq));
          const V3 nqn = normalize(nq);
          for (int s = 0; s < ao_samples; ++s, ++slot) {
            float u1 = rngNext(st), u2 = rngNext(st);
            V3 q = (p0 + e1 * u1) + e2 * u2;
            V3 dv = q - pos;
            float dist2 = dot(dv, dv);
            float dist = sqrtf(dist2);
            V3 wi = dv / dist;
            float cos_l = fabsf(dot(nqn, wi));
            bool valid = false;
            V3 Lr = v3(0, 0, 0);
            if (cos_l > 0.0f && dist > 0.0f) {
              float pdf = dist2 / (area * cos_l);
              float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
              Lr = (Lin * blinnPhong(costheta, surf, ks, a.shininess, radiance, wi, nff, wo)) *
                   (1.0f / (pdf * (float)ao_samples));
              valid = hasPositive(Lr);
            }
            writeShadow(a, sbase + slot, wi, Lr, dist, valid);
            nshadow += valid;
          }
        }
      }
    }
    for (; slot < S; ++slot) a.shadow_flag[sbase + slot] = 0;

    // bounce ray (genR2); the speculation-history wrap of the reference
    // (pending queue at SPRAY_HISTORY_SIZE) does not change the depth count
    if (next_depth < bounces) {
      wo = normalize(wo);
      bool emit = false;
      V3 wi = v3(0, 0, 0), Lr = v3(0, 0, 0);
      if (delta) {
        if (cos_theta_i != 0.0f) {
          cos_theta_i = clamp_ref(cos_theta_i, -1.0f, 1.0f);
          float abs_cos = fabsf(cos_theta_i);
          if (!entering) cos_theta_i = abs_cos;
          float fr;
          int reflect = 0, transmit = 0;
          V3 wt = v3(0, 0, 0);
          if (dom.bsdf == 1) {  // mirror
            fr = 1.0f;
            reflect = 1;
          } else {
            float etaI = entering ? dom.bsdf_p[0] : dom.bsdf_p[1];
            float etaT = entering ? dom.bsdf_p[1] : dom.bsdf_p[0];
            if (dom.bsdf == 2) {  // glass
              fr = frDielectric(cos_theta_i, etaI, etaT, wo, nff, &wt);
              if (fr == 1.0f) reflect = 1;
              else if (fr == 0.0f) transmit = 1;
              else {
                // the reference aborts on a glass hit with both lobes; keep reflection
                reflect = 1;
                atomicOr((unsigned long long*)&a.ctr->error_flags, kErrGlassBothLobes);
              }
            } else {  // transmission
              float sin2ThetaI = fmax_ref(0.0f, 1.0f - (cos_theta_i * cos_theta_i));
              float eta = etaI / etaT;
              float sin2ThetaT = eta * eta * sin2ThetaI;
              if (sin2ThetaT >= 1.0f) {
                fr = 1.0f;
                reflect = 1;
              } else {
                float cosThetaT = sqrtf(1.0f - sin2ThetaT);
                wt = (eta * -wo) + (nff * (eta * cos_theta_i - cosThetaT));
                fr = 0.0f;
                transmit = 1;
              }
            }
          }
          if (reflect) {
            V3 wr = -wo + ((2.0f * dot(wo, nff)) * nff);
            wi = normalize(wr);
            Lr = Lin * (fr / abs_cos);
            emit = hasPositive(Lr);
          } else if (transmit) {
            wi = normalize(wt);
            Lr = Lin * ((1.0f - fr) / abs_cos);
            emit = hasPositive(Lr);
          }
        }
      } else {
        uint32_t st = rngSeed((int32_t)((uint32_t)samid * (uint32_t)next_depth));
        float u1 = rngNext(st), u2 = rngNext(st);
        float pdf;
        cosineHemisphereSample(u1, u2, nff, &wi, &pdf);
        float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
        Lr = (((Lin * surf) * kOneOverPi) * costheta) / pdf;
        emit = hasPositive(Lr);
      }
      if (emit && rr_depth > 0 && next_depth >= rr_depth) {
        // Russian roulette (extension): survive with q = min(1, max(Lr)),
        // drawn from its own stream so the reference streams stay untouched
        float q = fmin_ref(1.0f, fmax_ref(Lr.x, fmax_ref(Lr.y, Lr.z)));
        uint32_t rs = rngSeed((int32_t)(((uint32_t)samid * (uint32_t)next_depth) ^ 0x2545f491u));
        float ur = rngNext(rs);
        if (ur >= q) emit = false;
        else Lr = Lr / q;
      }
      if (emit) {
        a.next.org[sample] = make_float4(pos.x, pos.y, pos.z, 0.f);
        a.next.dir[sample] = make_float4(wi.x, wi.y, wi.z, 0.f);
        a.next.wgt[sample] = make_float4(Lr.x, Lr.y, Lr.z, 0.f);
        a.next_flag[sample] = 1;
        ++nbounce;
      }
    }
  }
  for (int o = 16; o; o >>= 1) {
    nshadow += __shfl_down_sync(0xffffffffu, nshadow, o);
    nbounce += __shfl_down_sync(0xffffffffu, nbounce, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nshadow) atomicAdd(&a.ctr->rays_shadow, nshadow);
    if (nbounce) atomicAdd(&a.ctr->rays_bounce, nbounce);
  }
  if (a.blk_shadow) {
    // this block's kept counts for the two compactions that follow
    __shared__ unsigned int bsum[2];
    if (threadIdx.x == 0) bsum[0] = bsum[1] = 0u;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&bsum[0], (unsigned int)nshadow);
      atomicAdd(&bsum[1], (unsigned int)nbounce);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      a.blk_shadow[blockIdx.x] = bsum[0];
      a.blk_next[blockIdx.x] = bsum[1];
    }
  }
}

void initShadeTables() {
  float lut[256];
  for (int i = 0; i < 256; ++i) lut[i] = (float)(i * kOneOver255);
  cudaMemcpyToSymbol(c_unpack, lut, sizeof(lut));
}

void launchShade(cudaStream_t s, const ShadeArgs& a, int nblocks) {
  kShade<<<nblocks, 256, 0, s>>>(a);
}

// Per pixel of the wave: samples in order, slots in order, each unoccluded
// shadow ray adds w * (1 / spp) with the double-precision scale of
// HdrImage::add (src/display/image.h:99-109).
// Per pixel of the wave: its tile (binary search on pix_base), its samples
// (tile-local pixel lp holds samples lp * spp .. lp * spp + spp - 1), its view's
// image slot and scale; samples and slots in order, the sum in double.
//
// A block takes 256 consecutive pixels, whose samples are one contiguous
// range: their alive indices are staged in shared memory with coalesced loads
// (one pad word per 32, so that each thread's run of spp indices is read
// without bank conflicts) when the range fits kRetireStage, else read directly.
constexpr int kRetireStage = 4096;

__global__ void __launch_bounds__(256) kRetire(float4* image, const TileDev* __restrict__ tiles, int ntiles,
                                               int64_t npix, const ViewDev* __restrict__ views,
                                               const int32_t* __restrict__ alive_idx, ShadowBuf sh,
                                               const uint8_t* __restrict__ flag, int S) {
  __shared__ int32_t sidx[kRetireStage + kRetireStage / 32];
  __shared__ int64_t range[2];
  for (int64_t p0 = (int64_t)blockIdx.x * blockDim.x; p0 < npix; p0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = p0 + threadIdx.x;
    const bool valid = p < npix;
    int lo = 0;
    if (valid) {
      int hi = ntiles - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tiles[mid].pix_base <= p) lo = mid;
        else hi = mid - 1;
      }
    }
    const TileDev tl = tiles[lo];
    const int spp = tl.spp;
    const int64_t lp = p - tl.pix_base;
    const int64_t s0 = tl.sample_base + lp * spp;
    if (threadIdx.x == 0) range[0] = s0;
    if (p == min(npix, p0 + (int64_t)blockDim.x) - 1) range[1] = s0 + spp;
    __syncthreads();
    const int64_t sbeg = range[0], nstage = range[1] - range[0];
    const bool staged = nstage <= kRetireStage;
    if (staged) {
      // 8 loads in flight per thread before their shared-memory stores
      for (int j0 = threadIdx.x; j0 < (int)nstage; j0 += 8 * blockDim.x) {
        int32_t v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = j0 + u * (int)blockDim.x;
          v[u] = j < (int)nstage ? alive_idx[sbeg + j] : 0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = j0 + u * (int)blockDim.x;
          if (j < (int)nstage) sidx[j + (j >> 5)] = v[u];
        }
      }
    }
    __syncthreads();
    if (valid) {
      const ViewDev& vw = views[tl.view];
      const double scale = vw.scale;
      const int lpi = (int)lp;  // tile-local pixel (32-bit division)
      const int x = tl.x + lpi % tl.w, y = tl.y + lpi / tl.w;
      float4* px = image + vw.pixel_base + (int64_t)y * vw.image_w + x;
      float4 acc = *px;
      bool touched = false;
      const int f0 = (int)(s0 - sbeg);
      for (int s = 0; s < spp; ++s) {
        const int f = f0 + s;
        const int32_t ai = staged ? sidx[f + (f >> 5)] : alive_idx[s0 + s];
        if (ai < 0) continue;
        for (int k = 0; k < S; ++k) {
          uint32_t sid = (uint32_t)ai * S + k;
          if (!flag[sid] || sh.occluded[sid]) continue;
          float4 w = sh.wgt[sid];
          acc.x = (float)((double)acc.x + scale * (double)w.x);
          acc.y = (float)((double)acc.y + scale * (double)w.y);
          acc.z = (float)((double)acc.z + scale * (double)w.z);
          touched = true;
        }
      }
      if (touched) *px = acc;
    }
    __syncthreads();  // the next group restages sidx and range
  }
}

void launchRetireImpl(cudaStream_t s, float4* image, const TileDev* tiles, int ntiles, int64_t npix,
                      const ViewDev* views, const int32_t* alive_idx, const ShadowBuf sh,
                      const uint8_t* flag, int slots, int nblocks) {
  // one 256-pixel group per block where the grid allows (the staged loads of
  // many blocks overlap), at least nblocks
  const int64_t groups = (npix + 255) / 256;
  const int64_t blocks = std::max<int64_t>(nblocks, std::min<int64_t>(groups, 1 << 24));
  kRetire<<<(unsigned)blocks, 256, 0, s>>>(image, tiles, ntiles, npix, views, alive_idx, sh, flag, slots);
}

}  // namespace spray
