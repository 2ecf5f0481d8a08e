/*
 * oracle.h -- CPU restatement of the reference's triangle ray-query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against (and the CPU baseline a benchmark reports beside it); the product
 * never links or calls it.
 *
 * What it restates (paths relative to the Embree 3.12.1 source tree):
 *   - primref generation and triangle validity
 *       kernels/common/scene_triangle_mesh.h:127-147, 220-232
 *   - 32-bin binned-SAH builder for 8-wide BVHs with Triangle4 leaves
 *       kernels/builders/heuristic_binning.h:16-112, 211-399
 *       kernels/builders/heuristic_binning_array_aligned.h:36-127
 *       kernels/builders/bvh_builder_sah.h:155-319
 *       kernels/bvh/bvh_builder_sah.cpp:565 (sahBlockSize 4, costs 1/1,
 *       minLeaf 4, maxLeaf 7 blocks x 4), kernels/bvh/bvh.h:71-73 (depth 40)
 *   - Triangle4 leaf fill  kernels/geometry/triangle.h:40-41, 98-120
 *   - single-ray traversal kernels/bvh/bvh_intersector1.cpp:30-195,
 *       node test kernels/bvh/node_intersector1.h:30-60, 527-585
 *   - robust mode (Triangle4v + Pluecker, rounding-aware node test)
 *       kernels/geometry/triangle_intersector_pluecker.h:60-111,
 *       kernels/geometry/trianglev.h:93-115, node_intersector1.h:122-153,622-637
 *   - Moeller-Trumbore leaf test
 *       kernels/geometry/triangle_intersector_moeller.h:62-104,
 *       epilog kernels/geometry/intersector_epilog.h:215-296,
 *       FMA placement common/math/vec3.h:204-209, common/math/math.h:367-373,
 *       common/simd/vfloat4_sse2.h:440-445 (AVX2: madd/msub are fused)
 *   - stream entry semantics kernels/common/rtcore.cpp:595-624, 848-875,
 *       kernels/bvh/bvh_intersector_stream_filters.cpp:11-151,
 *       kernels/common/ray.h:550-611
 *   - SAH statistic kernels/bvh/bvh_statistics.cpp:10-160
 *
 * Deliberate deviations (documented, they only touch ulp-level values):
 *   - rcp(): the reference uses a hardware reciprocal estimate + one Newton
 *     step (common/simd/vfloat4_sse2.h:293-320), whose bits depend on the CPU's
 *     estimate table; the oracle uses the correctly rounded 1/x, as the GPU
 *     library does.  t/u/v may therefore differ from the reference by ~1 ulp.
 *   - partitioning is a stable two-way split instead of the reference's
 *     in-place swap loop; it only changes the order inside a subtree, which
 *     matters for the middle-split fallback used beyond depth 32.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleScene OracleScene;

OracleScene* orc_scene_new(void);
void orc_scene_free(OracleScene* s);

/* Adds one triangle mesh (copied).  verts: FLOAT3 records with byte stride
   vstride; idx: UINT3 records with byte stride istride. */
int orc_scene_add_mesh(OracleScene* s, unsigned geomID,
                       const void* verts, size_t vstride, unsigned nverts,
                       const void* idx, size_t istride, unsigned ntris);

/* RTC_SCENE_FLAG_ROBUST: Triangle4v leaves (raw vertices) and the Pluecker
   test (kernels/common/scene.cpp:119-125, triangle_intersector_pluecker.h)
   with the rounding-aware node test (node_intersector1.h:122-153,622-637).
   Takes effect at the next commit. */
void orc_scene_set_robust(OracleScene* s, int robust);

/* Filter callbacks, the oracle's form of rtcSetGeometryIntersectFilterFunction /
   rtcSetGeometryOccludedFilterFunction (kernels/geometry/filter.h:14-37, 72-89):
   called for every candidate hit the traversal meets with its geometry ID,
   primitive ID, u, v and distance; returns 0 to reject the hit.  ifilter is
   used by orc_intersect1M, ofilter by orc_occluded1M (NULL: no callback).  The
   callbacks apply to every geometry of the scene. */
typedef int (*orc_filter_fn)(void* user, unsigned geomID, unsigned primID, float u, float v, float t);
void orc_scene_set_filters(OracleScene* s, orc_filter_fn ifilter, orc_filter_fn ofilter, void* user);

/* Builds the BVH8 (binned SAH).  Returns the number of valid primitives. */
long orc_scene_commit(OracleScene* s);

/* Scene statistics after commit. */
typedef struct {
  double sah;            /* bvh_statistics.cpp semantics */
  double node_sah, leaf_sah;
  uint64_t num_nodes, num_leaves, num_blocks, num_prims;
  uint32_t depth;
  float bounds[6];       /* geometry bounds lo xyz, hi xyz */
} OrcStats;
void orc_scene_stats(const OracleScene* s, OrcStats* out);

/* Stream queries with the reference's entry semantics.  rays point at
   RTCRayHit (intersect) / RTCRay (occluded) records with byte stride
   `stride`.  nthreads <= 0 means "all cores". */
void orc_intersect1M(const OracleScene* s, void* rays, unsigned M, size_t stride, int nthreads);
void orc_occluded1M(const OracleScene* s, void* rays, unsigned M, size_t stride, int nthreads);

/* Brute force over all valid triangles in primref order (small scenes).  The
   only difference from the BVH query is the visiting order, which decides
   exact ties. */
void orc_brute_intersect1M(const OracleScene* s, void* rays, unsigned M, size_t stride);
void orc_brute_occluded1M(const OracleScene* s, void* rays, unsigned M, size_t stride);

/* Per-ray traversal work counters of the last orc_intersect1M/occluded1M call
   are accumulated into out[0]=nodes, out[1]=leaves, out[2]=triangle tests. */
void orc_counters(uint64_t out[3]);

/* FP64 adjudication of a ray whose closest hit differs between two
   implementations.  (gA,pA,tA) and (gB,pB,tB) are the two reported hits
   (geomID == 0xffffffff means "no hit").  Return codes:
     0  real mismatch
     1  near tie: both triangles are hit and their FP64 distances agree within
        `tie_ulps` FP32 ulps
     2  grazing: the contested hit lies within 1e-6 (barycentric) of an edge
        or the FP64 determinant is degenerate
     3  A is right: A's triangle is hit in FP64 and strictly closer than B's
     4  B is right: symmetric case */
int orc_adjudicate(const OracleScene* s, const void* rayhit_in,
                   unsigned gA, unsigned pA, float tA,
                   unsigned gB, unsigned pB, float tB, int tie_ulps);

/* FP64 ray/triangle distance of one primitive: returns 1 and writes t,u,v
   when the ray's line crosses the triangle (u,v >= 0, u+v <= 1) in front of
   the origin; 0 otherwise. */
int orc_fp64_hit(const OracleScene* s, const void* rayhit_in, unsigned geomID,
                 unsigned primID, double* t, double* u, double* v);

/* The reference's single-triangle FP32 test (Moeller, or Pluecker in robust
   scenes) of one primitive against the ray's own (tnear, tfar]: returns 1 and
   writes t (the epilog's T * rcp(absDen)) when the test accepts the hit.
   Two triangles that both pass with distances a few ulps apart form an
   order tie: the test accepts T <= absDen * tfar before dividing, so which
   one a traversal reports depends on the order it tests them in. */
int orc_fp32_hit(const OracleScene* s, const void* rayhit_in, unsigned geomID, unsigned primID, float* t);

/* Single-triangle Moeller test with the reference arithmetic; exposes the
   intermediate values for unit tests.  Returns 1 when valid. */
int orc_moeller1(const float v0[3], const float v1[3], const float v2[3],
                 const float org[3], const float dir[3], float tnear, float tfar,
                 float out_UVTden[4], float out_tuv[3], float out_Ng[3]);

/* Single-triangle Pluecker test (robust mode); out_tuv = t, u, v. */
int orc_pluecker1(const float v0[3], const float v1[3], const float v2[3], const float org[3], const float dir[3],
                  float tnear, float tfar, float out_tuv[3], float out_Ng[3]);

/* Scenes with instances: rays against the top scene's own triangles (top may
   be NULL) and `ninst` instances of committed scenes with local-to-world maps
   l2w (12 floats each, columns vx, vy, vz, p).  Closest hits of instances
   report instID = inst_geomIDs[k].  RTCRayHit / RTCRay records, byte stride. */
void orc_intersect_instanced(const OracleScene* top, unsigned ninst, const OracleScene* const* scenes,
                             const float* l2w, const unsigned* inst_geomIDs, void* rays, unsigned M, size_t stride);
void orc_occluded_instanced(const OracleScene* top, unsigned ninst, const OracleScene* const* scenes,
                            const float* l2w, void* rays, unsigned M, size_t stride);

#ifdef __cplusplus
}
#endif
#endif
