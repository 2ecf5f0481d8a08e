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
  double sah;               /* SAH cost with the reference's bvh_statistics semantics, on the
                               quantised child boxes traversal sees */
  double build_ms;          /* device time of the build (CUDA events) */
  unsigned int num_nodes;   /* 8-wide nodes */
  unsigned int num_leaves;  /* leaf children (<= 4 triangles each) */
  unsigned int num_prims;   /* valid triangles in the BVH */
  unsigned int depth;       /* wide levels */
  unsigned int ploc_iterations;
  unsigned int refit;       /* 1 when the last commit refitted the BVH instead of rebuilding */
  unsigned long long bvh_bytes; /* node + triangle record bytes in HBM */
  double sah_exact;         /* the same SAH on the exact (unquantised) child boxes */
  unsigned int leaf_max;    /* triangles per leaf child the build used (gpu.leaf_max, or by scene shape) */
  unsigned int reserved;
} RTCGBBuildStats;

typedef struct RTCGBQueryStats {
  double kernel_ms;              /* traversal kernel time of the last query */
  double total_ms;               /* whole call incl. host<->device copies */
  unsigned long long rays;       /* rays traversed (counting mode only) */
  unsigned long long nodes;      /* wide nodes visited (counting mode only) */
  unsigned long long tris;       /* triangle tests (counting mode only) */
  unsigned long long h2d_bytes;  /* bytes copied host->device by the call */
  unsigned long long d2h_bytes;  /* bytes copied device->host by the call */
  unsigned long long proposal_hits; /* learned queries: rays answered inside a proposed treelet */
} RTCGBQueryStats;

/* Statistics of the scene's last commit. */
RTC_API void rtcgbGetSceneBuildStats(RTCScene scene, RTCGBBuildStats* out);

/* Device time of each phase of the scene's last commit, in microseconds, when
   that commit was a replayed rebuild (rtcCommitScene of a scene whose layout is
   unchanged since its previous commit) on a device created with the config key
   gpu.build_phases=1; returns the number of phases (8) and writes up to
   max_phases of them, else returns 0.  Phases: primitive references and leaf
   records + sort keys; radix sort; PLOC set-up; PLOC rounds; PLOC finish (one
   CTA); collapse set-up; collapse levels; leaf triangle records.  The device
   timestamps are taken by one-thread kernels between the phases, which add a
   few microseconds to the build. */
RTC_API unsigned int rtcgbGetSceneBuildPhases(RTCScene scene, double* us, unsigned int max_phases);

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
   RTC_ERROR_INVALID_ARGUMENT.  The array's device address is looked up, and
   the kernels the call launches are loaded, when the device is created
   (rtcNewDevice), so the 32 MiB are taken then and no call loads anything.
   Scenes whose queries need more than the plain traversal -- filter
   callbacks, instances, batched scenes -- are refused with
   RTC_ERROR_INVALID_OPERATION.  All calls share the array and it keeps the
   last call's contents: each call clears the state it needs, and calls whose
   GPU work overlaps (different streams or host threads at the same time) race
   on it. */
#define RTCGB_NOALLOC_STAGING_BYTES 33554432u
RTC_API void rtcgbIntersect1MNoAlloc(RTCScene scene, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride,
                                     void* cuda_stream);

/* ---- Traversal launch shapes and their tuner (no counterpart in the reference)

   The plain closest-hit and any-hit traversal kernels (records 16-byte
   aligned, scenes without filter callbacks or instances; plain, robust and
   batched scenes) are compiled in several launch shapes: threads per CTA,
   resident CTAs per SM (their register budget is 65536 / (threads x CTAs)),
   traversal stack entries kept in shared memory, and the number of idle lanes
   at which a warp fetches new rays.  Shape 0 is the default.  Every shape
   returns the same hits; only the speed differs.  A scene's queries use its
   shape, which starts as the device's gpu.trace_shape (default 0); the other
   kernel variants (counting, learned, instances, filter callbacks, unaligned
   records, the no-allocation query, the path tracer) always run shape 0, and
   a batched frame keeps the shape its scene had when the frame was made. */
typedef struct RTCGBTraversalShape {
  unsigned int threads;       /* threads per CTA */
  unsigned int ctas_per_sm;   /* resident CTAs per SM the kernels are compiled for */
  unsigned int shared_stack;  /* traversal stack entries in shared memory (the rest in local memory) */
  unsigned int refill;        /* a warp fetches new rays when this many of its lanes are idle */
} RTCGBTraversalShape;

/* Writes up to max_shapes shapes; returns the number of compiled shapes. */
RTC_API unsigned int rtcgbGetTraversalShapes(RTCGBTraversalShape* shapes, unsigned int max_shapes);
RTC_API void rtcgbSetSceneTraversalShape(RTCScene scene, unsigned int shape);
RTC_API unsigned int rtcgbGetSceneTraversalShape(RTCScene scene);

/* Picks the scene's shape for a workload: times rtcIntersect1M (batched
   scenes: rtcgbIntersect1MBatched with the given batches) on a device copy of
   the M records -- and with RTCGB_TUNE_OCCLUDED also rtcOccluded1M on the
   same records -- in every shape, `repeats` rounds (0: 5) after one warm-up
   round, the shapes taking turns within each round.  The shape with the
   least median kernel time is set on the scene and returned; a shape other
   than 0 must be at least 1 % faster than shape 0.  ms_per_shape (optional,
   one entry per shape) receives the medians in milliseconds.  The records are
   not modified.  Do not query the scene from other threads meanwhile. */
#define RTCGB_TUNE_OCCLUDED 1u
RTC_API unsigned int rtcgbTuneSceneTraversal(RTCScene scene, const struct RTCRayHit* rayhit, unsigned int M,
                                             size_t byteStride, const unsigned int* batch_start,
                                             unsigned int num_batches, unsigned int flags, unsigned int repeats,
                                             double* ms_per_shape);

/* ---- Learned hit proposer (no counterpart in the reference) ----------------

   A proposer belongs to one committed scene.  It cuts the scene's BVH into up
   to 4096 treelets (subtrees) and learns, from closest-hit records the plain
   traversal produced, which treelets a ray hits: a hash-grid encoding of the
   ray origin and direction feeds a 32-64-64-64-4096 MLP (BF16 tensor cores,
   FP32 accumulation), trained on the GPU with the library's own forward,
   backward and Adam kernels.  The learned queries search the four proposed
   treelets before the whole tree, so their results are those of
   rtcIntersect1M / rtcOccluded1M; a good proposal ends an occlusion ray early
   or lowers a closest-hit ray's tfar before the full search.  After a full
   rebuild of the scene (a refit keeps the treelets) the learned queries run
   the plain traversal until a new proposer is made.  Rays, records, labels
   and outputs may be in host or device memory. */
typedef struct RTCGBProposerTy* RTCGBProposer;

typedef struct RTCGBProposerStats {
  unsigned int num_treelets;  /* treelets of the cut (<= 4096) */
  unsigned int samples;       /* labelled records of the last training call */
  unsigned int steps;         /* Adam steps taken */
  unsigned int reserved;
  double loss;                /* mean cross-entropy of the last epoch */
  double top1, top4;          /* share of the last epoch's records whose treelet ranked first / in the top 4 */
} RTCGBProposerStats;

RTC_API RTCGBProposer rtcgbNewProposer(RTCScene scene, unsigned int seed);
/* The same with a treelet budget: the cut has at most max_treelets (8..4096)
   treelets; the network keeps its 4096 outputs, the unused ones never win.
   rtcgbNewProposer(scene, seed) is rtcgbNewProposerEx(scene, seed, 4096). */
RTC_API RTCGBProposer rtcgbNewProposerEx(RTCScene scene, unsigned int seed, unsigned int max_treelets);
RTC_API void rtcgbRetainProposer(RTCGBProposer proposer);
RTC_API void rtcgbReleaseProposer(RTCGBProposer proposer);

/* Trains on M RTCRayHit records after a closest-hit query (records without a
   hit are skipped): `epochs` passes in shuffled batches of `batch` records,
   Adam with the given learning rate. */
RTC_API void rtcgbProposerTrain(RTCGBProposer proposer, const struct RTCRayHit* records, unsigned int M,
                                size_t byteStride, unsigned int epochs, unsigned int batch, float learning_rate);

/* Top-4 treelet indices (4 per ray, best first; 0xFFFFFFFF when fewer exist). */
RTC_API void rtcgbProposerPredict(RTCGBProposer proposer, const struct RTCRay* rays, unsigned int M,
                                  size_t byteStride, unsigned int* treelets);

RTC_API void rtcgbProposerGetStats(RTCGBProposer proposer, RTCGBProposerStats* out);

/* Parameter vector (FP32): hash table (16 x 2^18 x 2), then per layer the
   weights [out][in] and the biases of the 32-64-64-64-4096 MLP. */
RTC_API size_t rtcgbProposerParamCount(void);
RTC_API void rtcgbProposerGetParams(RTCGBProposer proposer, float* params);
RTC_API void rtcgbProposerSetParams(RTCGBProposer proposer, const float* params);

/* Mean softmax cross-entropy of B rays with the given treelet labels (-1:
   ignored, counted in the mean) and its gradient with respect to every
   parameter (rtcgbProposerParamCount() floats).  Returns the loss. */
RTC_API float rtcgbProposerGradients(RTCGBProposer proposer, const struct RTCRay* rays, unsigned int B,
                                     size_t byteStride, const int* labels, float* grads);

/* The cut: root node of each treelet (up to 4096 entries, 0xFFFFFFFF after
   the last) and the treelet of each triangle record of the BVH (max_records
   entries; 0xFFFFFFFF for triangles held above the cut).  Returns the number
   of treelets. */
RTC_API unsigned int rtcgbProposerGetTreelets(RTCGBProposer proposer, unsigned int* roots,
                                              unsigned int* record_treelet, unsigned int max_records);

/* rtcIntersect1M / rtcOccluded1M with the proposer's treelets searched first
   (records 16-byte aligned with a stride that is a multiple of 16; otherwise,
   and for robust scenes, the plain traversal runs). */
RTC_API void rtcgbIntersect1MLearned(RTCScene scene, RTCGBProposer proposer, struct RTCRayHit* rayhit,
                                     unsigned int M, size_t byteStride);
RTC_API void rtcgbOccluded1MLearned(RTCScene scene, RTCGBProposer proposer, struct RTCRay* ray, unsigned int M,
                                    size_t byteStride);

/* ---- Animated diffuse path tracing (no counterpart in the reference) --------

   A wavefront path tracer over a committed (non-robust) scene: per frame the
   camera rays, then per bounce a closest-hit traversal of the live rays, a
   cosine-weighted diffuse bounce (albedo 0.75, sky light on a miss) and the
   compaction of the surviving paths.  Each frame runs as one CUDA graph
   (captured on first use, one graph per mode) whose launches read their ray
   counts from device memory.  With rtcgbPathTracerAnimateSoup each frame first
   moves the soup's triangles by amplitude * sin(2 pi (frame / 60 + x)) along a
   random per-triangle normal (x: the triangle centroid's rest x coordinate)
   and refits the BVH inside the same graph.  Learned frames search the
   attached proposer's treelets first (same hits).  The scene must not be
   committed while a path tracer renders; after a full rebuild make a new one. */
typedef struct RTCGBPathTracerTy* RTCGBPathTracer;

typedef struct RTCGBFrameStats {
  double frame_ms;                  /* device time of the frame's graph */
  unsigned long long rays;          /* rays traced over all bounces */
  unsigned long long proposal_hits; /* learned frames: rays answered inside a proposed treelet */
  unsigned int rays_per_bounce[8];
  unsigned int learned;             /* 1 when the frame ran the learned graph */
  unsigned int errors;              /* traversal error bits; 0x100: a refit met an invalid vertex */
} RTCGBFrameStats;

/* camera: eye xyz, look-at xyz, up xyz, vertical field of view in degrees; bounces 1..8 */
RTC_API RTCGBPathTracer rtcgbNewPathTracer(RTCScene scene, unsigned int width, unsigned int height,
                                           unsigned int bounces, const float* camera);
RTC_API void rtcgbRetainPathTracer(RTCGBPathTracer tracer);
RTC_API void rtcgbReleasePathTracer(RTCGBPathTracer tracer);
/* The geometry must be a triangle soup whose shared vertex buffer is device memory. */
RTC_API void rtcgbPathTracerAnimateSoup(RTCGBPathTracer tracer, unsigned int geomID, float amplitude,
                                        unsigned int seed);
RTC_API void rtcgbPathTracerSetProposer(RTCGBPathTracer tracer, RTCGBProposer proposer);
/* Renders frame `frame` (learned != 0: with the proposer when it is current). */
RTC_API void rtcgbPathTracerRenderFrame(RTCGBPathTracer tracer, unsigned int frame, int learned,
                                        RTCGBFrameStats* stats);
/* Trains the attached proposer on the last frame's first diffuse bounce (closest-hit records). */
RTC_API void rtcgbPathTracerTrainProposer(RTCGBPathTracer tracer, unsigned int epochs, unsigned int batch,
                                          float learning_rate);
/* Radiance of the last frame, width * height * 3 floats (row-major, rgb). */
RTC_API void rtcgbPathTracerGetImage(RTCGBPathTracer tracer, float* rgb);

/* ---- Batched scenes (no counterpart in the reference) ----------------------

   A batched scene holds many independent scenes, one per geometry: its commit
   builds all their BVHs in one pass (one sort with the geometry ID in the key's
   top bits, one agglomerative clustering whose merges stay inside a geometry,
   one collapse; the work does not grow with the number of scenes), and one
   persistent traversal launch answers the rays of all of them.  Rays
   [batch_start[b], batch_start[b+1]) query geometry ID b only; hits report
   geomID b.  batch_start has num_batches + 1 entries (host or device memory),
   batch_start[0] = 0 and batch_start[num_batches] = M.  rtcIntersect1M and the
   learned queries are not available on batched scenes. */
RTC_API void rtcgbSetSceneBatched(RTCScene scene, int enable);
RTC_API void rtcgbIntersect1MBatched(RTCScene scene, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride,
                                     const unsigned int* batch_start, unsigned int num_batches);
RTC_API void rtcgbOccluded1MBatched(RTCScene scene, struct RTCRay* ray, unsigned int M, size_t byteStride,
                                    const unsigned int* batch_start, unsigned int num_batches);

/* Batched frames: the rebuild of every BVH of a committed batched scene and a
   batched closest-hit query over device-resident rays, captured once into one
   CUDA graph and replayed with one launch (optionally preceded by a copy of
   `pristine` over `rayhit`, both device memory).  The captured build runs with
   no host reads: its PLOC rounds and its collapse levels are two cooperative
   launches that end them themselves, so the device runs exactly as many
   rounds and levels as the data needs; a
   replay whose build fails (more than 1024 PLOC rounds, more than 64 levels, a
   different number of valid triangles) reports RTC_ERROR_UNKNOWN.  The scene's
   geometry IDs must be 0..n-1; a new
   commit of the scene invalidates the frame.  Results are those of
   rtcCommitScene + rtcgbIntersect1MBatched on the same data. */
typedef struct RTCGBBatchedFrameTy* RTCGBBatchedFrame;
typedef struct RTCGBBatchedFrameStats {
  double frame_ms;           /* device time of the last replay (copy + build + query) */
  double build_sah;          /* SAH of the replayed build */
  unsigned int status;       /* 0: the replayed build completed and is consistent */
  unsigned int num_nodes;    /* wide nodes of the replayed build */
  unsigned int ploc_rounds;  /* PLOC rounds the replayed build ran (device loop) */
  unsigned int levels;       /* collapse levels the replayed build ran (device loop) */
  unsigned int graph_nodes;  /* nodes of the captured graph */
  unsigned int replays;
} RTCGBBatchedFrameStats;
RTC_API RTCGBBatchedFrame rtcgbNewBatchedFrame(RTCScene scene, struct RTCRayHit* rayhit,
                                               const struct RTCRayHit* pristine, unsigned int M, size_t byteStride,
                                               const unsigned int* batch_start, unsigned int num_batches);
RTC_API void rtcgbBatchedFrameReplay(RTCGBBatchedFrame frame);
RTC_API void rtcgbGetBatchedFrameStats(RTCGBBatchedFrame frame, RTCGBBatchedFrameStats* stats);
RTC_API void rtcgbReleaseBatchedFrame(RTCGBBatchedFrame frame);

#endif
