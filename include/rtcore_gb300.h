/*
 * rtcore_gb300.h -- C ABI of the GB300 triangle ray-query library.
 *
 * This header declares the subset of the Embree 3.12 `rtcore` API that the
 * triangle BVH build + stream ray-query path needs.  Type layouts, enum values
 * and function signatures are the ones a host program compiled against the
 * reference's headers expects, so such a program links this library in place
 * of libembree3 without source changes.  Each declaration names the reference
 * interface it replaces (paths are relative to the Embree source tree).
 *
 * Semantics (mirrors the reference unless stated):
 *   - handles are reference counted; every entry point catches its own errors
 *     and reports them through the device error code / callback
 *     (kernels/common/rtcore.h:28-122, kernels/common/device.cpp:258-318);
 *   - shared buffers are not copied until rtcCommitScene, which uploads the
 *     geometry and builds the BVH on the GPU;
 *   - rtcIntersect1M / rtcOccluded1M accept host (pageable or pinned) or CUDA
 *     device pointers and are synchronous on return.
 */
#ifndef RTCORE_GB300_H
#define RTCORE_GB300_H

#include <stddef.h>
#include <stdbool.h>
#include <sys/types.h>

#define RTC_VERSION_MAJOR 3
#define RTC_VERSION_MINOR 12
#define RTC_VERSION_PATCH 1
#define RTC_VERSION 31201
#define RTC_VERSION_STRING "3.12.1"

/* One instance level, as in the reference's default build
   (include/embree3/rtcore_config.h:12). */
#define RTC_MAX_INSTANCE_LEVEL_COUNT 1
#define RTC_MIN_WIDTH 0

#if defined(__cplusplus)
#  define RTC_API_EXTERN_C extern "C"
#else
#  define RTC_API_EXTERN_C
#endif
#define RTC_API RTC_API_EXTERN_C __attribute__((visibility("default")))
#define RTC_ALIGN(...) __attribute__((aligned(__VA_ARGS__)))
#define RTC_FORCEINLINE inline __attribute__((always_inline))

#define RTC_INVALID_GEOMETRY_ID ((unsigned int)-1)
#define RTC_MAX_TIME_STEP_COUNT 129

/* ---------------------------------------------------------------------- */
/* Common types (include/embree3/rtcore_common.h:51-224)                   */
/* ---------------------------------------------------------------------- */

enum RTCFormat {
  RTC_FORMAT_UNDEFINED = 0,
  RTC_FORMAT_UCHAR = 0x1001, RTC_FORMAT_UCHAR2, RTC_FORMAT_UCHAR3, RTC_FORMAT_UCHAR4,
  RTC_FORMAT_CHAR = 0x2001, RTC_FORMAT_CHAR2, RTC_FORMAT_CHAR3, RTC_FORMAT_CHAR4,
  RTC_FORMAT_USHORT = 0x3001, RTC_FORMAT_USHORT2, RTC_FORMAT_USHORT3, RTC_FORMAT_USHORT4,
  RTC_FORMAT_SHORT = 0x4001, RTC_FORMAT_SHORT2, RTC_FORMAT_SHORT3, RTC_FORMAT_SHORT4,
  RTC_FORMAT_UINT = 0x5001, RTC_FORMAT_UINT2, RTC_FORMAT_UINT3, RTC_FORMAT_UINT4,
  RTC_FORMAT_INT = 0x6001, RTC_FORMAT_INT2, RTC_FORMAT_INT3, RTC_FORMAT_INT4,
  RTC_FORMAT_ULLONG = 0x7001, RTC_FORMAT_ULLONG2, RTC_FORMAT_ULLONG3, RTC_FORMAT_ULLONG4,
  RTC_FORMAT_LLONG = 0x8001, RTC_FORMAT_LLONG2, RTC_FORMAT_LLONG3, RTC_FORMAT_LLONG4,
  RTC_FORMAT_FLOAT = 0x9001, RTC_FORMAT_FLOAT2, RTC_FORMAT_FLOAT3, RTC_FORMAT_FLOAT4,
  RTC_FORMAT_FLOAT5, RTC_FORMAT_FLOAT6, RTC_FORMAT_FLOAT7, RTC_FORMAT_FLOAT8,
  RTC_FORMAT_FLOAT9, RTC_FORMAT_FLOAT10, RTC_FORMAT_FLOAT11, RTC_FORMAT_FLOAT12,
  RTC_FORMAT_FLOAT13, RTC_FORMAT_FLOAT14, RTC_FORMAT_FLOAT15, RTC_FORMAT_FLOAT16,
  RTC_FORMAT_FLOAT2X2_ROW_MAJOR = 0x9122, RTC_FORMAT_FLOAT2X3_ROW_MAJOR = 0x9123,
  RTC_FORMAT_FLOAT2X4_ROW_MAJOR = 0x9124, RTC_FORMAT_FLOAT3X2_ROW_MAJOR = 0x9132,
  RTC_FORMAT_FLOAT3X3_ROW_MAJOR = 0x9133, RTC_FORMAT_FLOAT3X4_ROW_MAJOR = 0x9134,
  RTC_FORMAT_FLOAT4X2_ROW_MAJOR = 0x9142, RTC_FORMAT_FLOAT4X3_ROW_MAJOR = 0x9143,
  RTC_FORMAT_FLOAT4X4_ROW_MAJOR = 0x9144,
  RTC_FORMAT_FLOAT2X2_COLUMN_MAJOR = 0x9222, RTC_FORMAT_FLOAT2X3_COLUMN_MAJOR = 0x9223,
  RTC_FORMAT_FLOAT2X4_COLUMN_MAJOR = 0x9224, RTC_FORMAT_FLOAT3X2_COLUMN_MAJOR = 0x9232,
  RTC_FORMAT_FLOAT3X3_COLUMN_MAJOR = 0x9233, RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR = 0x9234,
  RTC_FORMAT_FLOAT4X2_COLUMN_MAJOR = 0x9242, RTC_FORMAT_FLOAT4X3_COLUMN_MAJOR = 0x9243,
  RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR = 0x9244,
  RTC_FORMAT_GRID = 0xA001
};

enum RTCBuildQuality {
  RTC_BUILD_QUALITY_LOW = 0,
  RTC_BUILD_QUALITY_MEDIUM = 1,
  RTC_BUILD_QUALITY_HIGH = 2,
  RTC_BUILD_QUALITY_REFIT = 3
};

struct RTC_ALIGN(16) RTCBounds {
  float lower_x, lower_y, lower_z, align0;
  float upper_x, upper_y, upper_z, align1;
};

struct RTC_ALIGN(16) RTCLinearBounds {
  struct RTCBounds bounds0;
  struct RTCBounds bounds1;
};

enum RTCIntersectContextFlags {
  RTC_INTERSECT_CONTEXT_FLAG_NONE = 0,
  RTC_INTERSECT_CONTEXT_FLAG_INCOHERENT = (0 << 0),
  RTC_INTERSECT_CONTEXT_FLAG_COHERENT = (1 << 0)
};

struct RTCRayN;
struct RTCHitN;
struct RTCIntersectContext;

struct RTCFilterFunctionNArguments {
  int* valid;
  void* geometryUserPtr;
  struct RTCIntersectContext* context;
  struct RTCRayN* ray;
  struct RTCHitN* hit;
  unsigned int N;
};
typedef void (*RTCFilterFunctionN)(const struct RTCFilterFunctionNArguments* args);

/* Same field order as include/embree3/rtcore_common.h:193-203 with
   RTC_MAX_INSTANCE_LEVEL_COUNT == 1 and RTC_MIN_WIDTH == 0. */
struct RTCIntersectContext {
  enum RTCIntersectContextFlags flags;
  RTCFilterFunctionN filter;
  unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};

/* Header-inline in the reference (include/embree3/rtcore_common.h:209-224). */
RTC_FORCEINLINE void rtcInitIntersectContext(struct RTCIntersectContext* context)
{
  unsigned l = 0;
  context->flags = RTC_INTERSECT_CONTEXT_FLAG_INCOHERENT;
  context->filter = NULL;
  for (; l < RTC_MAX_INSTANCE_LEVEL_COUNT; ++l)
    context->instID[l] = RTC_INVALID_GEOMETRY_ID;
}

/* ---------------------------------------------------------------------- */
/* Ray / hit records (include/embree3/rtcore_ray.h:11-49)                  */
/* RTCRay 48 B, RTCHit 32 B, RTCRayHit 80 B.                               */
/* ---------------------------------------------------------------------- */

struct RTC_ALIGN(16) RTCRay {
  float org_x, org_y, org_z;
  float tnear;
  float dir_x, dir_y, dir_z;
  float time;
  float tfar;
  unsigned int mask;
  unsigned int id;
  unsigned int flags;
};

struct RTC_ALIGN(16) RTCHit {
  float Ng_x, Ng_y, Ng_z;
  float u, v;
  unsigned int primID;
  unsigned int geomID;
  unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};

struct RTCRayHit {
  struct RTCRay ray;
  struct RTCHit hit;
};

/* Packets of K rays in SOA layout (rtcore_ray.h:51-230): every ray field is
   an array of K values, then every hit field. */
#define RTCGB_DECLARE_PACKET(K, A)                                                                   \
  struct RTC_ALIGN(A) RTCRay##K {                                                                    \
    float org_x[K], org_y[K], org_z[K], tnear[K];                                                    \
    float dir_x[K], dir_y[K], dir_z[K], time[K];                                                     \
    float tfar[K];                                                                                   \
    unsigned int mask[K], id[K], flags[K];                                                           \
  };                                                                                                 \
  struct RTC_ALIGN(A) RTCHit##K {                                                                    \
    float Ng_x[K], Ng_y[K], Ng_z[K], u[K], v[K];                                                     \
    unsigned int primID[K], geomID[K];                                                               \
    unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT][K];                                            \
  };                                                                                                 \
  struct RTCRayHit##K {                                                                              \
    struct RTCRay##K ray;                                                                            \
    struct RTCHit##K hit;                                                                            \
  };
RTCGB_DECLARE_PACKET(4, 16)
RTCGB_DECLARE_PACKET(8, 32)
RTCGB_DECLARE_PACKET(16, 64)
#undef RTCGB_DECLARE_PACKET

/* Streams of N rays in pointer-SOA layout (rtcore_ray.h:170-207). */
struct RTCRayNp {
  float* org_x; float* org_y; float* org_z; float* tnear;
  float* dir_x; float* dir_y; float* dir_z; float* time;
  float* tfar;
  unsigned int* mask; unsigned int* id; unsigned int* flags;
};
struct RTCHitNp {
  float* Ng_x; float* Ng_y; float* Ng_z; float* u; float* v;
  unsigned int* primID; unsigned int* geomID;
  unsigned int* instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};
struct RTCRayHitNp {
  struct RTCRayNp ray;
  struct RTCHitNp hit;
};
struct RTCRayHitN;  /* packets of runtime size N (SOA, rtcore_ray.h:209-230) */

#if defined(__cplusplus)
/* C++ accessors of runtime-N SOA packets (include/embree3/rtcore_ray.h:219-375), the
   form filter callbacks read their RTCRayN / RTCHitN arguments in: field f of lane i
   is element f * N + i of the packet (ray fields 0..11, hit fields 0..6, then the
   instance IDs, one row of N per level). */
#define RTCGB_SOA_ACCESSOR(PACKET, FIELD, TYPE, INDEX)                                      \
  RTC_FORCEINLINE TYPE& PACKET##_##FIELD(PACKET* p, unsigned int N, unsigned int i) {        \
    return ((TYPE*)p)[(INDEX) * N + i];                                                      \
  }
RTCGB_SOA_ACCESSOR(RTCRayN, org_x, float, 0)
RTCGB_SOA_ACCESSOR(RTCRayN, org_y, float, 1)
RTCGB_SOA_ACCESSOR(RTCRayN, org_z, float, 2)
RTCGB_SOA_ACCESSOR(RTCRayN, tnear, float, 3)
RTCGB_SOA_ACCESSOR(RTCRayN, dir_x, float, 4)
RTCGB_SOA_ACCESSOR(RTCRayN, dir_y, float, 5)
RTCGB_SOA_ACCESSOR(RTCRayN, dir_z, float, 6)
RTCGB_SOA_ACCESSOR(RTCRayN, time, float, 7)
RTCGB_SOA_ACCESSOR(RTCRayN, tfar, float, 8)
RTCGB_SOA_ACCESSOR(RTCRayN, mask, unsigned int, 9)
RTCGB_SOA_ACCESSOR(RTCRayN, id, unsigned int, 10)
RTCGB_SOA_ACCESSOR(RTCRayN, flags, unsigned int, 11)
RTCGB_SOA_ACCESSOR(RTCHitN, Ng_x, float, 0)
RTCGB_SOA_ACCESSOR(RTCHitN, Ng_y, float, 1)
RTCGB_SOA_ACCESSOR(RTCHitN, Ng_z, float, 2)
RTCGB_SOA_ACCESSOR(RTCHitN, u, float, 3)
RTCGB_SOA_ACCESSOR(RTCHitN, v, float, 4)
RTCGB_SOA_ACCESSOR(RTCHitN, primID, unsigned int, 5)
RTCGB_SOA_ACCESSOR(RTCHitN, geomID, unsigned int, 6)
#undef RTCGB_SOA_ACCESSOR
RTC_FORCEINLINE unsigned int& RTCHitN_instID(RTCHitN* hit, unsigned int N, unsigned int i, unsigned int l) {
  return ((unsigned int*)hit)[(7 + l) * N + i];
}
/* an RTCRayHitN packet: N rays (12 fields), then N hits */
RTC_FORCEINLINE RTCRayN* RTCRayHitN_RayN(RTCRayHitN* rayhit, unsigned int N) {
  (void)N;
  return (RTCRayN*)rayhit;
}
RTC_FORCEINLINE RTCHitN* RTCRayHitN_HitN(RTCRayHitN* rayhit, unsigned int N) {
  return (RTCHitN*)((float*)rayhit + 12 * N);
}

/* packets of compile-time size N */
template <int N>
struct RTCRayNt {
  float org_x[N], org_y[N], org_z[N], tnear[N];
  float dir_x[N], dir_y[N], dir_z[N], time[N];
  float tfar[N];
  unsigned int mask[N], id[N], flags[N];
};
template <int N>
struct RTCHitNt {
  float Ng_x[N], Ng_y[N], Ng_z[N], u[N], v[N];
  unsigned int primID[N], geomID[N];
  unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT][N];
};
template <int N>
struct RTCRayHitNt {
  RTCRayNt<N> ray;
  RTCHitNt<N> hit;
};

/* lane i of a packet as a single record, and back */
RTC_FORCEINLINE RTCRay rtcGetRayFromRayN(RTCRayN* rayN, unsigned int N, unsigned int i) {
  RTCRay r;
  r.org_x = RTCRayN_org_x(rayN, N, i); r.org_y = RTCRayN_org_y(rayN, N, i); r.org_z = RTCRayN_org_z(rayN, N, i);
  r.tnear = RTCRayN_tnear(rayN, N, i);
  r.dir_x = RTCRayN_dir_x(rayN, N, i); r.dir_y = RTCRayN_dir_y(rayN, N, i); r.dir_z = RTCRayN_dir_z(rayN, N, i);
  r.time = RTCRayN_time(rayN, N, i);
  r.tfar = RTCRayN_tfar(rayN, N, i);
  r.mask = RTCRayN_mask(rayN, N, i); r.id = RTCRayN_id(rayN, N, i); r.flags = RTCRayN_flags(rayN, N, i);
  return r;
}
RTC_FORCEINLINE RTCHit rtcGetHitFromHitN(RTCHitN* hitN, unsigned int N, unsigned int i) {
  RTCHit h;
  h.Ng_x = RTCHitN_Ng_x(hitN, N, i); h.Ng_y = RTCHitN_Ng_y(hitN, N, i); h.Ng_z = RTCHitN_Ng_z(hitN, N, i);
  h.u = RTCHitN_u(hitN, N, i); h.v = RTCHitN_v(hitN, N, i);
  h.primID = RTCHitN_primID(hitN, N, i); h.geomID = RTCHitN_geomID(hitN, N, i);
  for (unsigned int l = 0; l < RTC_MAX_INSTANCE_LEVEL_COUNT; l++) h.instID[l] = RTCHitN_instID(hitN, N, i, l);
  return h;
}
RTC_FORCEINLINE void rtcCopyHitToHitN(RTCHitN* hitN, const RTCHit* hit, unsigned int N, unsigned int i) {
  RTCHitN_Ng_x(hitN, N, i) = hit->Ng_x; RTCHitN_Ng_y(hitN, N, i) = hit->Ng_y; RTCHitN_Ng_z(hitN, N, i) = hit->Ng_z;
  RTCHitN_u(hitN, N, i) = hit->u; RTCHitN_v(hitN, N, i) = hit->v;
  RTCHitN_primID(hitN, N, i) = hit->primID; RTCHitN_geomID(hitN, N, i) = hit->geomID;
  for (unsigned int l = 0; l < RTC_MAX_INSTANCE_LEVEL_COUNT; l++) RTCHitN_instID(hitN, N, i, l) = hit->instID[l];
}
RTC_FORCEINLINE RTCRayHit rtcGetRayHitFromRayHitN(RTCRayHitN* rayhitN, unsigned int N, unsigned int i) {
  RTCRayHit rh;
  rh.ray = rtcGetRayFromRayN(RTCRayHitN_RayN(rayhitN, N), N, i);
  rh.hit = rtcGetHitFromHitN(RTCRayHitN_HitN(rayhitN, N), N, i);
  return rh;
}
#endif

/* ---------------------------------------------------------------------- */
/* Device (include/embree3/rtcore_device.h)                                */
/* ---------------------------------------------------------------------- */

typedef struct RTCDeviceTy* RTCDevice;
typedef struct RTCSceneTy* RTCScene;
typedef struct RTCGeometryTy* RTCGeometry;
typedef struct RTCBufferTy* RTCBuffer;

enum RTCDeviceProperty {
  RTC_DEVICE_PROPERTY_VERSION = 0,
  RTC_DEVICE_PROPERTY_VERSION_MAJOR = 1,
  RTC_DEVICE_PROPERTY_VERSION_MINOR = 2,
  RTC_DEVICE_PROPERTY_VERSION_PATCH = 3,
  RTC_DEVICE_PROPERTY_NATIVE_RAY4_SUPPORTED = 32,
  RTC_DEVICE_PROPERTY_NATIVE_RAY8_SUPPORTED = 33,
  RTC_DEVICE_PROPERTY_NATIVE_RAY16_SUPPORTED = 34,
  RTC_DEVICE_PROPERTY_RAY_STREAM_SUPPORTED = 35,
  RTC_DEVICE_PROPERTY_BACKFACE_CULLING_CURVES_ENABLED = 63,
  RTC_DEVICE_PROPERTY_RAY_MASK_SUPPORTED = 64,
  RTC_DEVICE_PROPERTY_BACKFACE_CULLING_ENABLED = 65,
  RTC_DEVICE_PROPERTY_FILTER_FUNCTION_SUPPORTED = 66,
  RTC_DEVICE_PROPERTY_IGNORE_INVALID_RAYS_ENABLED = 67,
  RTC_DEVICE_PROPERTY_COMPACT_POLYS_ENABLED = 68,
  RTC_DEVICE_PROPERTY_TRIANGLE_GEOMETRY_SUPPORTED = 96,
  RTC_DEVICE_PROPERTY_QUAD_GEOMETRY_SUPPORTED = 97,
  RTC_DEVICE_PROPERTY_SUBDIVISION_GEOMETRY_SUPPORTED = 98,
  RTC_DEVICE_PROPERTY_CURVE_GEOMETRY_SUPPORTED = 99,
  RTC_DEVICE_PROPERTY_USER_GEOMETRY_SUPPORTED = 100,
  RTC_DEVICE_PROPERTY_POINT_GEOMETRY_SUPPORTED = 101,
  RTC_DEVICE_PROPERTY_TASKING_SYSTEM = 128,
  RTC_DEVICE_PROPERTY_JOIN_COMMIT_SUPPORTED = 129,
  RTC_DEVICE_PROPERTY_PARALLEL_COMMIT_SUPPORTED = 130
};

enum RTCError {
  RTC_ERROR_NONE = 0,
  RTC_ERROR_UNKNOWN = 1,
  RTC_ERROR_INVALID_ARGUMENT = 2,
  RTC_ERROR_INVALID_OPERATION = 3,
  RTC_ERROR_OUT_OF_MEMORY = 4,
  RTC_ERROR_UNSUPPORTED_CPU = 5,
  RTC_ERROR_CANCELLED = 6
};

typedef void (*RTCErrorFunction)(void* userPtr, enum RTCError code, const char* str);
typedef bool (*RTCMemoryMonitorFunction)(void* ptr, ssize_t bytes, bool post);
typedef bool (*RTCProgressMonitorFunction)(void* ptr, double n);

/* replaces include/embree3/rtcore_device.h:14 / kernels/common/rtcore.cpp:27 */
RTC_API RTCDevice rtcNewDevice(const char* config);
/* replaces include/embree3/rtcore_device.h:17 / kernels/common/rtcore.cpp:42 */
RTC_API void rtcRetainDevice(RTCDevice device);
/* replaces include/embree3/rtcore_device.h:20 / kernels/common/rtcore.cpp:57 */
RTC_API void rtcReleaseDevice(RTCDevice device);
/* replaces include/embree3/rtcore_device.h:55 / kernels/common/rtcore.cpp:72 */
RTC_API ssize_t rtcGetDeviceProperty(RTCDevice device, enum RTCDeviceProperty prop);
/* replaces include/embree3/rtcore_device.h:58 / kernels/common/rtcore.cpp:88 */
RTC_API void rtcSetDeviceProperty(RTCDevice device, const enum RTCDeviceProperty prop, ssize_t value);
/* replaces include/embree3/rtcore_device.h:73 / kernels/common/rtcore.cpp:104 (read-and-clear, per thread) */
RTC_API enum RTCError rtcGetDeviceError(RTCDevice device);
/* replaces include/embree3/rtcore_device.h:79 / kernels/common/rtcore.cpp:115 */
RTC_API void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction error, void* userPtr);
/* replaces include/embree3/rtcore_device.h:85 / kernels/common/rtcore.cpp:125 */
RTC_API void rtcSetDeviceMemoryMonitorFunction(RTCDevice device, RTCMemoryMonitorFunction memoryMonitor, void* userPtr);

/* ---------------------------------------------------------------------- */
/* Buffers (include/embree3/rtcore_buffer.h)                               */
/* ---------------------------------------------------------------------- */

enum RTCBufferType {
  RTC_BUFFER_TYPE_INDEX = 0,
  RTC_BUFFER_TYPE_VERTEX = 1,
  RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE = 2,
  RTC_BUFFER_TYPE_NORMAL = 3,
  RTC_BUFFER_TYPE_TANGENT = 4,
  RTC_BUFFER_TYPE_NORMAL_DERIVATIVE = 5,
  RTC_BUFFER_TYPE_GRID = 8,
  RTC_BUFFER_TYPE_FACE = 16,
  RTC_BUFFER_TYPE_LEVEL = 17,
  RTC_BUFFER_TYPE_EDGE_CREASE_INDEX = 18,
  RTC_BUFFER_TYPE_EDGE_CREASE_WEIGHT = 19,
  RTC_BUFFER_TYPE_VERTEX_CREASE_INDEX = 20,
  RTC_BUFFER_TYPE_VERTEX_CREASE_WEIGHT = 21,
  RTC_BUFFER_TYPE_HOLE = 22,
  RTC_BUFFER_TYPE_FLAGS = 32
};

/* replaces include/embree3/rtcore_buffer.h:37 / kernels/common/rtcore.cpp:134 */
RTC_API RTCBuffer rtcNewBuffer(RTCDevice device, size_t byteSize);
/* replaces include/embree3/rtcore_buffer.h:40 / kernels/common/rtcore.cpp:145 */
RTC_API RTCBuffer rtcNewSharedBuffer(RTCDevice device, void* ptr, size_t byteSize);
/* replaces include/embree3/rtcore_buffer.h:43 / kernels/common/rtcore.cpp:156 */
RTC_API void* rtcGetBufferData(RTCBuffer buffer);
/* replaces include/embree3/rtcore_buffer.h:46 / kernels/common/rtcore.cpp:167 */
RTC_API void rtcRetainBuffer(RTCBuffer buffer);
/* replaces include/embree3/rtcore_buffer.h:49 / kernels/common/rtcore.cpp:177 */
RTC_API void rtcReleaseBuffer(RTCBuffer buffer);

/* ---------------------------------------------------------------------- */
/* Geometry (include/embree3/rtcore_geometry.h)                            */
/* ---------------------------------------------------------------------- */

enum RTCGeometryType {
  RTC_GEOMETRY_TYPE_TRIANGLE = 0,
  RTC_GEOMETRY_TYPE_QUAD = 1,
  RTC_GEOMETRY_TYPE_GRID = 2,
  RTC_GEOMETRY_TYPE_SUBDIVISION = 8,
  RTC_GEOMETRY_TYPE_CONE_LINEAR_CURVE = 15,
  RTC_GEOMETRY_TYPE_ROUND_LINEAR_CURVE = 16,
  RTC_GEOMETRY_TYPE_FLAT_LINEAR_CURVE = 17,
  RTC_GEOMETRY_TYPE_ROUND_BEZIER_CURVE = 24,
  RTC_GEOMETRY_TYPE_FLAT_BEZIER_CURVE = 25,
  RTC_GEOMETRY_TYPE_NORMAL_ORIENTED_BEZIER_CURVE = 26,
  RTC_GEOMETRY_TYPE_ROUND_BSPLINE_CURVE = 32,
  RTC_GEOMETRY_TYPE_FLAT_BSPLINE_CURVE = 33,
  RTC_GEOMETRY_TYPE_NORMAL_ORIENTED_BSPLINE_CURVE = 34,
  RTC_GEOMETRY_TYPE_ROUND_HERMITE_CURVE = 40,
  RTC_GEOMETRY_TYPE_FLAT_HERMITE_CURVE = 41,
  RTC_GEOMETRY_TYPE_NORMAL_ORIENTED_HERMITE_CURVE = 42,
  RTC_GEOMETRY_TYPE_SPHERE_POINT = 50,
  RTC_GEOMETRY_TYPE_DISC_POINT = 51,
  RTC_GEOMETRY_TYPE_ORIENTED_DISC_POINT = 52,
  RTC_GEOMETRY_TYPE_ROUND_CATMULL_ROM_CURVE = 58,
  RTC_GEOMETRY_TYPE_FLAT_CATMULL_ROM_CURVE = 59,
  RTC_GEOMETRY_TYPE_NORMAL_ORIENTED_CATMULL_ROM_CURVE = 60,
  RTC_GEOMETRY_TYPE_USER = 120,
  RTC_GEOMETRY_TYPE_INSTANCE = 121
};

/* replaces include/embree3/rtcore_geometry.h:135 / kernels/common/rtcore.cpp:1139 (TRIANGLE only; other
   types raise RTC_ERROR_UNKNOWN "not supported", as the reference does for a
   geometry type compiled out) */
RTC_API RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type);
/* replaces include/embree3/rtcore_geometry.h:138 / kernels/common/rtcore.cpp:1759 */
RTC_API void rtcRetainGeometry(RTCGeometry geometry);
/* replaces include/embree3/rtcore_geometry.h:141 / kernels/common/rtcore.cpp:1769 */
RTC_API void rtcReleaseGeometry(RTCGeometry geometry);
/* replaces include/embree3/rtcore_geometry.h:144 / kernels/common/rtcore.cpp:1708 */
RTC_API void rtcCommitGeometry(RTCGeometry geometry);
/* replaces include/embree3/rtcore_geometry.h:148 / kernels/common/rtcore.cpp:1503 */
RTC_API void rtcEnableGeometry(RTCGeometry geometry);
/* replaces include/embree3/rtcore_geometry.h:151 / kernels/common/rtcore.cpp:1523 */
RTC_API void rtcDisableGeometry(RTCGeometry geometry);
/* replaces include/embree3/rtcore_geometry.h:155 / kernels/common/rtcore.cpp:1328 (only one time step is supported) */
RTC_API void rtcSetGeometryTimeStepCount(RTCGeometry geometry, unsigned int timeStepCount);
/* replaces include/embree3/rtcore_geometry.h:164 / kernels/common/rtcore.cpp:1406 (mask is stored; ray masks are compiled out
   in the reference's default build, so it does not filter) */
RTC_API void rtcSetGeometryMask(RTCGeometry geometry, unsigned int mask);
/* replaces include/embree3/rtcore_geometry.h:167 / kernels/common/rtcore.cpp:1376 */
RTC_API void rtcSetGeometryBuildQuality(RTCGeometry geometry, enum RTCBuildQuality quality);
/* replaces include/embree3/rtcore_geometry.h:174 / kernels/common/rtcore.cpp:1436 */
RTC_API void rtcSetGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot, enum RTCFormat format, RTCBuffer buffer, size_t byteOffset, size_t byteStride, size_t itemCount);
/* replaces include/embree3/rtcore_geometry.h:177 / kernels/common/rtcore.cpp:1455 */
RTC_API void rtcSetSharedGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot, enum RTCFormat format, const void* ptr, size_t byteOffset, size_t byteStride, size_t itemCount);
/* replaces include/embree3/rtcore_geometry.h:180 / kernels/common/rtcore.cpp:1470 */
RTC_API void* rtcSetNewGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot, enum RTCFormat format, size_t byteStride, size_t itemCount);
/* replaces include/embree3/rtcore_geometry.h:183 / kernels/common/rtcore.cpp:1492 */
RTC_API void* rtcGetGeometryBufferData(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot);
/* replaces include/embree3/rtcore_geometry.h:186 / kernels/common/rtcore.cpp:1513 */
RTC_API void rtcUpdateGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot);
/* replaces include/embree3/rtcore_geometry.h:190 / kernels/common/rtcore.cpp:1664.  Triangle meshes only
   (RTC_ERROR_INVALID_OPERATION for instances, as geometry.cpp:136-142).  A scene that has a callback
   on some geometry, or RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION, at commit calls the callbacks (and
   RTCIntersectContext::filter) during rtcIntersect* / rtcOccluded*: the traversal runs on the GPU,
   the callbacks on the calling thread with N = 1, and each ray is traced again until its nearest
   hit is accepted.  Not with instances, batched or learned queries (RTC_ERROR_INVALID_OPERATION). */
RTC_API void rtcSetGeometryIntersectFilterFunction(RTCGeometry geometry, RTCFilterFunctionN filter);
/* replaces include/embree3/rtcore_geometry.h:193 / kernels/common/rtcore.cpp:1674 (as above, for
   rtcOccluded*: a ray is occluded iff some hit in range is accepted) */
RTC_API void rtcSetGeometryOccludedFilterFunction(RTCGeometry geometry, RTCFilterFunctionN filter);
/* replaces include/embree3/rtcore_geometry.h:224 / kernels/common/rtcore.cpp:996: the scene an
   RTC_GEOMETRY_TYPE_INSTANCE geometry instances (one instance level) */
RTC_API void rtcSetGeometryInstancedScene(RTCGeometry geometry, RTCScene scene);
/* replaces include/embree3/rtcore_geometry.h:227 / kernels/common/rtcore.cpp:1071: local-to-world
   map (RTC_FORMAT_FLOAT3X4_ROW_MAJOR, _FLOAT3X4_COLUMN_MAJOR or _FLOAT4X4_COLUMN_MAJOR) */
RTC_API void rtcSetGeometryTransform(RTCGeometry geometry, unsigned int timeStep, enum RTCFormat format, const void* xfm);
/* replaces include/embree3/rtcore_geometry.h:233 / kernels/common/rtcore.cpp:1117 */
RTC_API void rtcGetGeometryTransform(RTCGeometry geometry, float time, enum RTCFormat format, void* xfm);

/* replaces include/embree3/rtcore_geometry.h:196 / kernels/common/rtcore.cpp:1543 */
RTC_API void rtcSetGeometryUserData(RTCGeometry geometry, void* ptr);
/* replaces include/embree3/rtcore_geometry.h:199 / kernels/common/rtcore.cpp:1553 */
RTC_API void* rtcGetGeometryUserData(RTCGeometry geometry);

/* ---------------------------------------------------------------------- */
/* Scene (include/embree3/rtcore_scene.h)                                  */
/* ---------------------------------------------------------------------- */

enum RTCSceneFlags {
  RTC_SCENE_FLAG_NONE = 0,
  RTC_SCENE_FLAG_DYNAMIC = (1 << 0),
  RTC_SCENE_FLAG_COMPACT = (1 << 1),
  RTC_SCENE_FLAG_ROBUST = (1 << 2),
  RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION = (1 << 3)
};

/* replaces include/embree3/rtcore_scene.h:28 / kernels/common/rtcore.cpp:187 */
RTC_API RTCScene rtcNewScene(RTCDevice device);
/* replaces include/embree3/rtcore_scene.h:32 / kernels/common/rtcore.cpp:198 */
RTC_API RTCDevice rtcGetSceneDevice(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:35 / kernels/common/rtcore.cpp:976 */
RTC_API void rtcRetainScene(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:38 / kernels/common/rtcore.cpp:986 */
RTC_API void rtcReleaseScene(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:42 / kernels/common/rtcore.cpp:1718 */
RTC_API unsigned int rtcAttachGeometry(RTCScene scene, RTCGeometry geometry);
/* replaces include/embree3/rtcore_scene.h:45 / kernels/common/rtcore.cpp:1733 */
RTC_API void rtcAttachGeometryByID(RTCScene scene, RTCGeometry geometry, unsigned int geomID);
/* replaces include/embree3/rtcore_scene.h:48 / kernels/common/rtcore.cpp:1748 */
RTC_API void rtcDetachGeometry(RTCScene scene, unsigned int geomID);
/* replaces include/embree3/rtcore_scene.h:51 / kernels/common/rtcore.cpp:1779 */
RTC_API RTCGeometry rtcGetGeometry(RTCScene scene, unsigned int geomID);
/* replaces include/embree3/rtcore_scene.h:55 / kernels/common/rtcore.cpp:259: uploads geometry and runs
   the GPU BVH builder */
RTC_API void rtcCommitScene(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:58 / kernels/common/rtcore.cpp:269 (same as rtcCommitScene) */
RTC_API void rtcJoinCommitScene(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:65 / kernels/common/rtcore.cpp:209 (stored; the GPU build is not interruptible) */
RTC_API void rtcSetSceneProgressMonitorFunction(RTCScene scene, RTCProgressMonitorFunction progress, void* ptr);
/* replaces include/embree3/rtcore_scene.h:68 / kernels/common/rtcore.cpp:224 */
RTC_API void rtcSetSceneBuildQuality(RTCScene scene, enum RTCBuildQuality quality);
/* replaces include/embree3/rtcore_scene.h:71 / kernels/common/rtcore.cpp:238 */
RTC_API void rtcSetSceneFlags(RTCScene scene, enum RTCSceneFlags flags);
/* replaces include/embree3/rtcore_scene.h:74 / kernels/common/rtcore.cpp:248 */
RTC_API enum RTCSceneFlags rtcGetSceneFlags(RTCScene scene);
/* replaces include/embree3/rtcore_scene.h:77 / kernels/common/rtcore.cpp:279 */
RTC_API void rtcGetSceneBounds(RTCScene scene, struct RTCBounds* bounds_o);
/* replaces include/embree3/rtcore_scene.h:80 / kernels/common/rtcore.cpp:298 */
RTC_API void rtcGetSceneLinearBounds(RTCScene scene, struct RTCLinearBounds* bounds_o);

/* replaces include/embree3/rtcore_scene.h:96 / kernels/common/rtcore.cpp:479 (a stream of one ray) */
RTC_API void rtcIntersect1(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit* rayhit);
/* replaces include/embree3/rtcore_scene.h:108 / kernels/common/rtcore.cpp:595: closest hit for M rays in
   AOS layout with arbitrary byteStride (>= sizeof(RTCRayHit), 4-byte aligned) */
RTC_API void rtcIntersect1M(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride);
/* replaces include/embree3/rtcore_scene.h:111 / kernels/common/rtcore.cpp:626 (array of pointers) */
RTC_API void rtcIntersect1Mp(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit** rayhit, unsigned int M);
/* replaces include/embree3/rtcore_scene.h:99 / kernels/common/rtcore.cpp:498: lanes with
   valid[i] == -1 are traced (through the stream path); other lanes untouched */
RTC_API void rtcIntersect4(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit4* rayhit);
/* replaces include/embree3/rtcore_scene.h:102 / kernels/common/rtcore.cpp:529 */
RTC_API void rtcIntersect8(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit8* rayhit);
/* replaces include/embree3/rtcore_scene.h:105 / kernels/common/rtcore.cpp:562 */
RTC_API void rtcIntersect16(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHit16* rayhit);
/* replaces include/embree3/rtcore_scene.h:114 / kernels/common/rtcore.cpp:657: M packets of
   N SOA rays, byteStride apart (N == 1: AOS records) */
RTC_API void rtcIntersectNM(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayHitN* rayhit, unsigned int N, unsigned int M, size_t byteStride);
/* replaces include/embree3/rtcore_scene.h:117 / kernels/common/rtcore.cpp:695 */
RTC_API void rtcIntersectNp(RTCScene scene, struct RTCIntersectContext* context, const struct RTCRayHitNp* rayhit, unsigned int N);
/* replaces include/embree3/rtcore_scene.h:123 / kernels/common/rtcore.cpp:749 */
RTC_API void rtcOccluded4(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRay4* ray);
/* replaces include/embree3/rtcore_scene.h:126 / kernels/common/rtcore.cpp:780 */
RTC_API void rtcOccluded8(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRay8* ray);
/* replaces include/embree3/rtcore_scene.h:129 / kernels/common/rtcore.cpp:814 */
RTC_API void rtcOccluded16(const int* valid, RTCScene scene, struct RTCIntersectContext* context, struct RTCRay16* ray);
/* replaces include/embree3/rtcore_scene.h:138 / kernels/common/rtcore.cpp:907 */
RTC_API void rtcOccludedNM(RTCScene scene, struct RTCIntersectContext* context, struct RTCRayN* ray, unsigned int N, unsigned int M, size_t byteStride);
/* replaces include/embree3/rtcore_scene.h:141 / kernels/common/rtcore.cpp:946 */
RTC_API void rtcOccludedNp(RTCScene scene, struct RTCIntersectContext* context, const struct RTCRayNp* ray, unsigned int N);
/* replaces include/embree3/rtcore_scene.h:120 / kernels/common/rtcore.cpp:733 */
RTC_API void rtcOccluded1(RTCScene scene, struct RTCIntersectContext* context, struct RTCRay* ray);
/* replaces include/embree3/rtcore_scene.h:132 / kernels/common/rtcore.cpp:848: any hit; occluded rays get
   tfar = -inf, the others stay untouched */
RTC_API void rtcOccluded1M(RTCScene scene, struct RTCIntersectContext* context, struct RTCRay* ray, unsigned int M, size_t byteStride);
/* replaces include/embree3/rtcore_scene.h:135 / kernels/common/rtcore.cpp:877 (array of pointers) */
RTC_API void rtcOccluded1Mp(RTCScene scene, struct RTCIntersectContext* context, struct RTCRay** ray, unsigned int M);

#endif /* RTCORE_GB300_H */
