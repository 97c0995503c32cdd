// TEST INFRASTRUCTURE ONLY.  Exposes the reference's own random sampler
// (deps/embree/random_sampler.h, compiled from where it lies by
// oracle/build_ref.sh) through a C ABI, so that the oracle's restatement of
// the sampler can be compared with the reference's code, value for value.
#include <cstdint>

#define __forceinline inline
#include "random_sampler.h"

using namespace spray;

extern "C" {

// n floats of RandomSampler_init(id) followed by RandomSampler_get1D
// (the eye-ray jitter and shader streams, src/ooc/ooc_tracer.inl,
// src/ooc/ooc_shader_ao.h, src/ooc/ooc_shader_pt.h).
int ref_rng(int32_t id, int32_t n, float* out) {
  RandomSampler r;
  RandomSampler_init(r, id);
  for (int32_t i = 0; i < n; ++i) out[i] = RandomSampler_get1D(r);
  return 0;
}

// The raw 32-bit states behind those floats.
int ref_rng_uint(int32_t id, int32_t n, uint32_t* out) {
  RandomSampler r;
  RandomSampler_init(r, id);
  for (int32_t i = 0; i < n; ++i) out[i] = RandomSampler_getUInt(r);
  return 0;
}

}  // extern "C"
