// Oracle stand-in for the Embree 3 API subset the reference calls
// (core/src/Scene.cpp:60-61,122-191,196-200,281-303). The implementation
// (oracle/ref_harness.cpp) answers rtcIntersect1 with the oracle's binary
// BVH and Moeller-Trumbore test in Embree's conventions.
#pragma once
#include <stddef.h>
#include <limits.h>

#define RTC_INVALID_GEOMETRY_ID ((unsigned int)-1)

struct RTCDeviceTy; struct RTCSceneTy; struct RTCGeometryTy;
typedef RTCDeviceTy* RTCDevice;
typedef RTCSceneTy* RTCScene;
typedef RTCGeometryTy* RTCGeometry;

enum RTCGeometryType { RTC_GEOMETRY_TYPE_TRIANGLE = 0 };
enum RTCBufferType { RTC_BUFFER_TYPE_INDEX = 0, RTC_BUFFER_TYPE_VERTEX = 1 };
enum RTCFormat { RTC_FORMAT_UINT3 = 0x5003, RTC_FORMAT_FLOAT3 = 0x9003 };

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
struct RTCRayHit { struct RTCRay ray; struct RTCHit hit; };
struct RTCIntersectContext { unsigned int flags; void* filter; unsigned int instID[1]; };

RTCDevice rtcNewDevice(const char* config);
void rtcReleaseDevice(RTCDevice device);
RTCScene rtcNewScene(RTCDevice device);
void rtcReleaseScene(RTCScene scene);
RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type);
void* rtcSetNewGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot,
                              enum RTCFormat format, size_t byteStride, size_t itemCount);
void rtcCommitGeometry(RTCGeometry geometry);
unsigned int rtcAttachGeometry(RTCScene scene, RTCGeometry geometry);
void rtcReleaseGeometry(RTCGeometry geometry);
void rtcCommitScene(RTCScene scene);
void rtcInitIntersectContext(struct RTCIntersectContext* context);
void rtcIntersect1(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit* rayhit);
