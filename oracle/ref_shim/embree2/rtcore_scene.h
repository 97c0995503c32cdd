// TEST INFRASTRUCTURE ONLY.  Scene declarations of the Embree 2 compile shim
// (see embree2/rtcore.h): no-op scene handles.
#pragma once

#include "embree2/rtcore.h"

enum RTCSceneFlags { RTC_SCENE_STATIC = 0, RTC_SCENE_DYNAMIC = 1 };
enum RTCAlgorithmFlags { RTC_INTERSECT1 = 1 };

inline RTCScene rtcDeviceNewScene(RTCDevice, RTCSceneFlags, RTCAlgorithmFlags) {
  return reinterpret_cast<RTCScene>(spray_embree_shim::handle() + 1);
}
inline void rtcDeleteScene(RTCScene) {}
inline void rtcCommit(RTCScene) {}
