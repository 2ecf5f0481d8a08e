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
  unsigned int pad;
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

/* Sorts n (key, value) pairs (host arrays, in place) with the builder's
   stable LSD radix sort on the GPU.  The result equals a stable host sort by
   key; exposed so that property can be tested directly.  Returns 0 on
   success. */
RTC_API int rtcgbRadixSortPairs(unsigned long long* keys, unsigned int* values, unsigned int n);

#endif
