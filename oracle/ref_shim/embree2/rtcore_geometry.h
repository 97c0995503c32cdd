// TEST INFRASTRUCTURE ONLY.  Geometry declarations of the Embree 2 compile
// shim (see embree2/rtcore.h): the mesh buffer's calls are accepted and ignored.
#pragma once

#include <cstddef>

#include "embree2/rtcore.h"

enum RTCGeometryFlags { RTC_GEOMETRY_STATIC = 0, RTC_GEOMETRY_DEFORMABLE = 1, RTC_GEOMETRY_DYNAMIC = 2 };
enum RTCBufferType { RTC_INDEX_BUFFER = 0, RTC_VERTEX_BUFFER = 1 };

inline unsigned rtcNewTriangleMesh(RTCScene, RTCGeometryFlags, size_t, size_t, size_t = 1) { return 0; }
inline void rtcSetBuffer2(RTCScene, unsigned, RTCBufferType, const void*, size_t, size_t, size_t = (size_t)-1) {}
inline void rtcUpdate(RTCScene, unsigned) {}
inline void rtcEnable(RTCScene, unsigned) {}
