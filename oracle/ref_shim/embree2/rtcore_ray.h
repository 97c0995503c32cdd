// TEST INFRASTRUCTURE ONLY.  The single-ray record of the Embree 2 compile
// shim (see embree2/rtcore.h), with the fields render/rays.h sets.
#pragma once

#include "embree2/rtcore.h"

struct alignas(16) RTCRay {
  float org[3];
  float align0;
  float dir[3];
  float align1;
  float tnear;
  float tfar;
  float time;
  unsigned mask;
  float Ng[3];
  float align2;
  float u;
  float v;
  unsigned geomID;
  unsigned primID;
  unsigned instID;
};
