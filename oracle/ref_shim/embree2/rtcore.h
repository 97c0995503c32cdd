// TEST INFRASTRUCTURE ONLY.  Compile shim for the Embree 2 declarations that
// the reference's render/rays.h and render/trimesh_buffer.{h,cc} name.  Embree
// is absent here.  The functions pinned through them (DomainList::sort,
// TriMeshBuffer::computeNormals and updateIntersection) trace nothing, so the
// set-up calls the mesh buffer makes (device, scene, mesh, buffer mapping,
// commit) are no-ops that hand back placeholder handles.  None of this is
// Embree's code; only the names and argument lists are kept so the
// reference's sources compile unchanged.
#pragma once

#include <cstddef>

struct __RTCDevice;
struct __RTCScene;
typedef __RTCDevice* RTCDevice;
typedef __RTCScene* RTCScene;

#define RTC_INVALID_GEOMETRY_ID ((unsigned)-1)

namespace spray_embree_shim {
inline char* handle() {
  static char tag[16];
  return tag;
}
}  // namespace spray_embree_shim

inline RTCDevice rtcNewDevice(const char* = nullptr) {
  return reinterpret_cast<RTCDevice>(spray_embree_shim::handle());
}
inline void rtcDeleteDevice(RTCDevice) {}

#include "embree2/rtcore_scene.h"
#include "embree2/rtcore_geometry.h"
