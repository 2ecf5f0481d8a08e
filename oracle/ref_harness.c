/*
 * ref_harness.c -- drives the reference library (oracle/_ref/libembree3_ref.so, the
 * reference's own sources compiled by oracle/ref.mk) through its public C API.
 *
 * TEST INFRASTRUCTURE ONLY: generates the reference-made golden fixtures under
 * tests/golden/, pins the oracle to the reference, and times the reference's CPU path
 * (the CPU arm of the benchmark, where the reference builds). Never linked by the
 * product.
 *
 * It is compiled against this repository's include/embree3/rtcore.h, not the
 * reference's headers: the same calls then link to the reference library unchanged,
 * which is the drop-in claim seen from the other side.
 *
 * Calls follow the reference's own usage (tutorials/minimal/minimal.cpp:60-150 and
 * tutorials/verify/verify.cpp:4867-5016): rtcNewDevice -> rtcNewScene ->
 * rtcNewGeometry(TRIANGLE) -> rtcSetSharedGeometryBuffer(VERTEX, INDEX) ->
 * rtcCommitGeometry -> rtcAttachGeometry -> rtcCommitScene, then rtcIntersect1M /
 * rtcOccluded1M on 1024-ray chunks from T host threads with an INCOHERENT context.
 */
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#if defined(__x86_64__)
#include <pmmintrin.h>
#include <xmmintrin.h>
#endif

#include "embree3/rtcore.h"

typedef struct {
  RTCDevice device;
  RTCScene scene;
  unsigned last_error;
} RefScene;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* FTZ/DAZ per thread, as the reference asks of every thread that calls it
   (its device prints a warning otherwise, kernels/common/device.cpp). */
static void set_flush_modes(void) {
#if defined(__x86_64__)
  _MM_SET_FLUSH_ZERO_MODE(_MM_FLUSH_ZERO_ON);
  _MM_SET_DENORMALS_ZERO_MODE(_MM_DENORMALS_ZERO_ON);
#endif
}

/* device_cfg: the reference's device configuration string ("threads=8,benchmark=1").
   flags: RTCSceneFlags (RTC_SCENE_FLAG_ROBUST = 4); quality: RTCBuildQuality. */
RefScene* refh_scene_new(const char* device_cfg, int flags, int quality) {
  set_flush_modes();
  RefScene* s = (RefScene*)calloc(1, sizeof(RefScene));
  s->device = rtcNewDevice(device_cfg);
  if (!s->device) { free(s); return NULL; }
  s->scene = rtcNewScene(s->device);
  rtcSetSceneFlags(s->scene, (enum RTCSceneFlags)flags);
  rtcSetSceneBuildQuality(s->scene, (enum RTCBuildQuality)quality);
  return s;
}

/* Adds one triangle mesh over caller-owned FLOAT3 vertices and UINT3 indices (shared
   buffers: they must outlive the scene). Returns the geometry ID or -1. The vertex
   buffer is read with 16-byte loads past its last element by the reference, so the
   caller pads it by 4 bytes (include/embree3/rtcore_geometry.h, rtcSetSharedGeometryBuffer). */
int refh_add_mesh(RefScene* s, const float* verts, unsigned nverts, const unsigned* idx, unsigned ntris) {
  RTCGeometry g = rtcNewGeometry(s->device, RTC_GEOMETRY_TYPE_TRIANGLE);
  rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_VERTEX, 0, RTC_FORMAT_FLOAT3, verts, 0, 12, nverts);
  rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_INDEX, 0, RTC_FORMAT_UINT3, idx, 0, 12, ntris);
  rtcCommitGeometry(g);
  unsigned id = rtcAttachGeometry(s->scene, g);
  rtcReleaseGeometry(g);
  s->last_error = (unsigned)rtcGetDeviceError(s->device);
  return s->last_error ? -1 : (int)id;
}

/* rtcCommitScene; returns its wall time in seconds (negative on an error). */
double refh_commit(RefScene* s) {
  double t0 = now_s();
  rtcCommitScene(s->scene);
  double dt = now_s() - t0;
  s->last_error = (unsigned)rtcGetDeviceError(s->device);
  return s->last_error ? -1.0 : dt;
}

void refh_bounds(RefScene* s, float out[6]) {
  struct RTCBounds b;
  rtcGetSceneBounds(s->scene, &b);
  out[0] = b.lower_x; out[1] = b.lower_y; out[2] = b.lower_z;
  out[3] = b.upper_x; out[4] = b.upper_y; out[5] = b.upper_z;
}

unsigned refh_error(RefScene* s) { return s->last_error; }

void refh_free(RefScene* s) {
  if (!s) return;
  rtcReleaseScene(s->scene);
  rtcReleaseDevice(s->device);
  free(s);
}

typedef struct {
  RefScene* s;
  char* rays;
  unsigned n;
  size_t stride;
  unsigned chunk;
  int occluded;
  int coherent;
  atomic_uint next;
} Job;

static void* worker(void* arg) {
  Job* j = (Job*)arg;
  set_flush_modes();
  struct RTCIntersectContext ctx;
  rtcInitIntersectContext(&ctx);
  if (j->coherent) ctx.flags = RTC_INTERSECT_CONTEXT_FLAG_COHERENT;
  for (;;) {
    unsigned start = atomic_fetch_add(&j->next, j->chunk);
    if (start >= j->n) break;
    unsigned m = j->n - start < j->chunk ? j->n - start : j->chunk;
    char* p = j->rays + (size_t)start * j->stride;
    if (j->occluded)
      rtcOccluded1M(j->s->scene, &ctx, (struct RTCRay*)p, m, j->stride);
    else
      rtcIntersect1M(j->s->scene, &ctx, (struct RTCRayHit*)p, m, j->stride);
  }
  return NULL;
}

/* Stream query over n records (RTCRayHit for closest hit, RTCRay for occlusion) with
   byte stride `stride`: nthreads host threads (1 runs on the caller's thread) take
   `chunk`-ray slices in turn. Returns the wall time in seconds. */
double refh_query(RefScene* s, void* rays, unsigned n, size_t stride, int nthreads, unsigned chunk,
                  int occluded, int coherent) {
  Job j;
  j.s = s; j.rays = (char*)rays; j.n = n; j.stride = stride; j.chunk = chunk ? chunk : 1024;
  j.occluded = occluded; j.coherent = coherent;
  atomic_init(&j.next, 0u);
  if (nthreads < 1) nthreads = 1;
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  double t0 = now_s();
  for (int i = 1; i < nthreads; i++) pthread_create(&th[i], NULL, worker, &j);
  worker(&j);
  for (int i = 1; i < nthreads; i++) pthread_join(th[i], NULL);
  double dt = now_s() - t0;
  free(th);
  s->last_error = (unsigned)rtcGetDeviceError(s->device);
  return dt;
}
