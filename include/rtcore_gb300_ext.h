/*
 * rtcore_gb300_ext.h -- GB300-specific extensions of the C ABI.
 *
 * These entry points have no counterpart in the reference.  They expose what
 * a GPU implementation adds: build statistics of the GPU BVH, per-thread
 * timing of the last query's traversal kernel (CUDA events on the stream the
 * kernel ran on), traversal work counters, the number of kernels the library
 * has launched, and the choice of CUDA stream.
 */
#ifndef RTCORE_GB300_EXT_H
#define RTCORE_GB300_EXT_H

#include "rtcore_gb300.h"

typedef struct RTCGBBuildStats {
  double sah;               /* SAH cost with the reference's bvh_statistics semantics */
  double build_ms;          /* device time of the build (CUDA events) */
  unsigned int num_nodes;   /* 8-wide nodes */
  unsigned int num_leaves;  /* leaf children (<= 3 triangles each) */
  unsigned int num_prims;   /* valid triangles in the BVH */
  unsigned int depth;       /* wide levels */
  unsigned int ploc_iterations;
  unsigned int refit;       /* 1 when the last commit refitted the BVH instead of rebuilding */
  unsigned long long bvh_bytes; /* node + triangle record bytes in HBM */
} RTCGBBuildStats;

typedef struct RTCGBQueryStats {
  double kernel_ms;              /* traversal kernel time of the last query */
  double total_ms;               /* whole call incl. host<->device copies */
  unsigned long long rays;       /* rays traversed (counting mode only) */
  unsigned long long nodes;      /* wide nodes visited (counting mode only) */
  unsigned long long tris;       /* triangle tests (counting mode only) */
  unsigned long long h2d_bytes;  /* bytes copied host->device by the call */
  unsigned long long d2h_bytes;  /* bytes copied device->host by the call */
} RTCGBQueryStats;

/* Statistics of the scene's last commit. */
RTC_API void rtcgbGetSceneBuildStats(RTCScene scene, RTCGBBuildStats* out);

/* Statistics of the calling thread's last rtcIntersect* / rtcOccluded* call. */
RTC_API void rtcgbGetLastQueryStats(RTCGBQueryStats* out);

/* When enabled (per calling thread), queries run the counting variant of the
   traversal kernels, which also fills rays/nodes/tris in the query stats. */
RTC_API void rtcgbSetQueryCounting(int enable);

/* Total number of CUDA kernels this library has launched in the process. */
RTC_API unsigned long long rtcgbGetKernelLaunchCount(void);

/* Uses `cuda_stream` (a cudaStream_t, or NULL for the library's own
   per-thread stream) for the calling thread's builds and queries. */
RTC_API void rtcgbSetThreadStream(void* cuda_stream);

/* Copies the committed BVH to host memory for inspection: up to `max_nodes`
   80-byte node records and `max_tris` 48-byte triangle records.  Returns the
   number of nodes; *num_tris receives the number of triangle records. */
RTC_API unsigned int rtcgbGetSceneBVH(RTCScene scene, void* nodes, unsigned int max_nodes, void* tris,
                                      unsigned int max_tris, unsigned int* num_tris);

/* Host-memory access of the device: bit 0 set when kernels can address
   pageable host memory (cudaDevAttrPageableMemoryAccess), bit 1 when they can
   use host pointers of pinned / registered memory directly.  With the device
   config key gpu.host_rays=direct (default), queries on such host rays are
   traced in place (other host rays use the pipeline); gpu.host_rays=pipeline
   overlaps chunked copies with the traversal; gpu.host_rays=copy copies all
   rays, traces, and copies back. */
RTC_API int rtcgbGetDeviceHostAccess(RTCDevice device);

/* Sorts n (key, value) pairs (host arrays, in place) with the builder's
   stable LSD radix sort on the GPU.  The result equals a stable host sort by
   key; exposed so that property can be tested directly.  Returns 0 on
   success. */
RTC_API int rtcgbRadixSortPairs(unsigned long long* keys, unsigned int* values, unsigned int n);

/* Closest-hit query that allocates no memory.  No counterpart in the
   reference.  For callers that cannot call cudaMalloc during a query: a
   process whose device memory is already reserved by its own allocator, a
   real-time loop that cannot afford cudaMalloc's implicit synchronisation, a
   service held to a fixed memory budget.  Same semantics as rtcIntersect1M
   on `cuda_stream` (NULL: the default stream; synchronised before return),
   but all scratch lives in a static device array that each GPU loading the
   library holds until exit: 256 bytes of query state plus
   RTCGB_NOALLOC_STAGING_BYTES (32 MiB) for staging host-resident rays.  Rays
   in device memory are traced in place at any size; host rays whose span
   ((M-1)*byteStride + 80 bytes) exceeds the staging area are rejected with
   RTC_ERROR_INVALID_ARGUMENT.  The array's device address is looked up on
   the first call on each device, so make that first call before any stream
   capture.  All calls share the array and it keeps the last call's contents:
   each call clears the state it needs, and calls whose GPU work overlaps
   (different streams or host threads at the same time) race on it. */
#define RTCGB_NOALLOC_STAGING_BYTES 33554432u
RTC_API void rtcgbIntersect1MNoAlloc(RTCScene scene, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride,
                                     void* cuda_stream);

#endif
