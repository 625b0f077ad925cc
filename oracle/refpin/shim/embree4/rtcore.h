// rtcore.h -- TEST INFRASTRUCTURE ONLY: declarations standing in for the
// embree 4 API header (the embree submodule is empty in the reference
// checkout).  The reference's embree backend headers name these handle
// types; the pin harness never creates an embree device, scene or geometry,
// so no embree function is declared.
#pragma once
namespace embree_for_barney {
typedef struct RTCDeviceTy *RTCDevice;
typedef struct RTCSceneTy *RTCScene;
typedef struct RTCGeometryTy *RTCGeometry;
typedef struct RTCBufferTy *RTCBuffer;
// the published embree 4 ray, hit and ray-query-context records, whose
// fields the reference's trace interface reads
struct RTCRay {
  float org_x, org_y, org_z, tnear;
  float dir_x, dir_y, dir_z, time;
  float tfar;
  unsigned int mask, id, flags;
};
struct RTCHit {
  float Ng_x, Ng_y, Ng_z;
  float u, v;
  unsigned int primID, geomID;
  unsigned int instID[1];
};
struct RTCRayHit {
  RTCRay ray;
  RTCHit hit;
};
struct RTCRayQueryContext {
  unsigned int instID[1];
};
}  // namespace embree_for_barney
