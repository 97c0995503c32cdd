// The AO and path-tracing shaders of one closest hit, shared by the
// wavefront shader (kShade, shade.cu) and the round loop of the
// non-speculative tracer (rounds.cu).  Restates ShaderAo::operator()
// (src/ooc/ooc_shader_ao.h:92-197) and ShaderPt::operator()
// (src/ooc/ooc_shader_pt.h:93-227); the non-speculative shaders
// (src/baseline/baseline_shader_ao.h:54-98, baseline_shader_pt.h:55-196)
// draw the same samples from the same seeds.
#pragma once

#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {
namespace {

// src/render/reflection.h:202-214
__device__ __forceinline__ V3 blinnPhong(float costheta, V3 kd, V3 ks, float shininess, V3 li,
                                         V3 wi, V3 n_hat, V3 wo) {
  V3 half_hat = normalize(wi + wo);
  float n_dot_h = clamp_ref(dot(n_hat, half_hat), 0.0f, 1.0f);
  V3 cs = ks * powShininess(n_dot_h, shininess);
  V3 cd = kd * costheta;
  return li * (cd + cs);
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

// Frame-wide inputs of the shaders.
struct ShadeEnv {
  const float* lights;  // 13 floats per light: type, pos, radiance, e1, e2
  int num_lights;
  float ks[3], shininess;
  Counters* ctr;
};

// Shades a hit at `pos` seen along `dir` with weight Lin (normal and surface
// colour interpolated at the hit; next_depth = the depth of the rays it
// spawns).  Calls shadow(slot, wi, w, tmax, valid) for every shadow slot in
// order and bounce(wi, w) for a surviving bounce ray; returns the number of
// slots it emitted.
template <class ShadowFn, class BounceFn>
__device__ __forceinline__ int shadeHit(const ShadeEnv& env, const ViewDev& vw, V3 dir, V3 Lin, V3 pos,
                                        V3 normal, V3 surf, int bsdf, const float* bsdf_p, int pixid,
                                        int samid, int next_depth, ShadowFn&& shadow, BounceFn&& bounce) {
  const int ao_mode = vw.ao_mode, ao_samples = vw.ao_samples, bounces = vw.bounces;
  const int rr_depth = vw.rr_depth, ao_light_shadow = vw.ao_light_shadow;
  const float ao_max_distance = vw.ao_max_distance;
  V3 wo = -dir;
  float cos_theta_i = dot(wo, normal);
  const bool entering = cos_theta_i > 0.0f;
  const V3 nff = normalize(entering ? normal : -normal);
  const bool delta = bsdf != 0;
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
      shadow(slot, wi, Lr, tmax, valid);
    }
    if (ao_light_shadow) {
      bool valid = false;
      V3 wi = v3(0, 0, 0), Lr = v3(0, 0, 0);
      if (env.num_lights > 0) {
        const float* L = env.lights;
        wi = normalize(v3(L[1], L[2], L[3]) - pos);
        float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
        Lr = ((Lin * surf) * v3(L[4], L[5], L[6])) * (kOneOverPi * costheta);
        valid = hasPositive(Lr);
      }
      shadow(slot, wi, Lr, __int_as_float(0x7f800000), valid);
      ++slot;
    }
  } else if (!delta) {
    const V3 ks = v3(env.ks[0], env.ks[1], env.ks[2]);
    uint32_t st = rngSeed((int32_t)((uint32_t)samid * (uint32_t)next_depth));
    for (int l = 0; l < env.num_lights; ++l) {
      const float* L = env.lights + 13 * l;
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
            Lr = (Lin * blinnPhong(costheta, surf, ks, env.shininess, radiance, wi, nff, wo)) *
                 (1.0f / (pdf * (float)ao_samples));
            valid = hasPositive(Lr);
          }
          shadow(slot, wi, Lr, __int_as_float(0x7f800000), valid);
        }
      } else if (type == 0) {  // point light (light.h:41-65)
        V3 wi = normalize(v3(L[1], L[2], L[3]) - pos);
        float costheta = clamp_ref(dot(nff, wi), 0.0f, 1.0f);
        V3 Lr = (Lin * blinnPhong(costheta, surf, ks, env.shininess, radiance, wi, nff, wo)) *
                (1.0f / 1.0f);
        bool valid = hasPositive(Lr);
        shadow(slot, wi, Lr, __int_as_float(0x7f800000), valid);
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
            Lr = (Lin * blinnPhong(costheta, surf, ks, env.shininess, radiance, wi, nff, wo)) *
                 (1.0f / (pdf * (float)ao_samples));
            valid = hasPositive(Lr);
          }
          shadow(slot, wi, Lr, dist, valid);
        }
      }
    }
  }

  // bounce ray (genR2)
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
        if (bsdf == 1) {  // mirror
          fr = 1.0f;
          reflect = 1;
        } else {
          float etaI = entering ? bsdf_p[0] : bsdf_p[1];
          float etaT = entering ? bsdf_p[1] : bsdf_p[0];
          if (bsdf == 2) {  // glass
            fr = frDielectric(cos_theta_i, etaI, etaT, wo, nff, &wt);
            if (fr == 1.0f) reflect = 1;
            else if (fr == 0.0f) transmit = 1;
            else {
              // the reference aborts on a glass hit with both lobes; keep reflection
              reflect = 1;
              atomicOr((unsigned long long*)&env.ctr->error_flags, kErrGlassBothLobes);
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
    if (emit) bounce(wi, Lr);
  }
  return slot;
}

}  // namespace
}  // namespace spray
