// gb_trace.h -- host entry point of the traversal kernels (gb_trace.cu).
#pragma once
#include "gb_common.h"

namespace gb {

// Launch shapes of the traversal kernel: threads per CTA, resident CTAs per SM
// (the register budget of the plain variants: 65536 / (threads x ctas)),
// traversal stack entries kept in shared memory, and the idle lanes at which a
// warp fetches new rays.  Shape 0 is the default; the others are compiled for
// the plain closest-hit and any-hit kernels on 16-byte aligned records and
// chosen per scene by the traversal tuner.
struct TraceShapeDesc {
  int threads, ctas, shared_stack, refill;
};
inline constexpr TraceShapeDesc kTraceShapes[] = {
    {128, 9, 8, 4},   // default
    {128, 8, 8, 4},   // 64 registers a thread
    {128, 9, 16, 4},  // deeper shared stack
    {128, 9, 4, 4},   // shallower shared stack
    {64, 18, 8, 4},   // two-warp CTAs
    {256, 4, 8, 4},   // eight-warp CTAs, 64 registers
    {128, 9, 8, 8},   // refill at 8 idle lanes
};
inline constexpr int kNumTraceShapes = (int)(sizeof(kTraceShapes) / sizeof(kTraceShapes[0]));

struct TraceParams {
  const WideNode* nodes;
  const TriRecord* tris;
  char* rays;                 // RTCRayHit (closest) or RTCRay (any hit) records, device memory
  uint64_t stride;            // byte stride between records (multiple of 4)
  uint32_t nrays;
  unsigned int* ray_counter;  // zeroed before launch; persistent warps fetch rays from it
  unsigned int* err;          // error flags (kErr*)
  TraceCounters* counters;    // counting variant; proposal_hits also in the seeded variant
  uint32_t max_iters;         // per-ray loop bound
  uint32_t num_nodes;         // bounds of the node and triangle arrays
  uint32_t num_tris;
  int robust;                 // Pluecker test on (v0, v1, v2) records
  const unsigned int* nrays_ptr;  // optional: the ray count is read from device memory
  const uint4* seeds;         // optional: per ray up to four subtree roots (node indices,
                              // kInvalidID = none) traversed before the root
  const uint32_t* order;      // optional: the i-th fetched ray is record order[i] (ray reordering)
  const InstDesc* insts;      // optional: instance table of a scene with instance leaves
  uint32_t ninsts;
  const uint32_t* batch_start;  // optional (segmented BVHs): rays [batch_start[b], batch_start[b+1])
  const uint32_t* batch_root;   //   start at node batch_root[b] (kInvalidID: the batch hits nothing)
  uint32_t nbatches;
  // optional (closest hit, 16-byte aligned records, no instances/proposals/batches):
  // ray i skips the triangles (primID, geomID) = excl[excl_off[i] .. excl_off[i+1]),
  // the hits a filter callback rejected
  const uint32_t* excl_off;
  const uint2* excl;
  int shape;                  // index into kTraceShapes (0: default)
};

// Launches the persistent closest-hit (anyhit = false) or any-hit kernel.
// P.shape selects the launch shape of the plain kernels on 16-byte aligned
// records; the other variants (counting, proposals, instances, exclusion lists,
// unaligned records) always run in the default shape.
cudaError_t launch_trace(const TraceParams& P, bool anyhit, bool count, cudaStream_t st);

// The plain kernels in a tuned shape (1 <= P.shape < kNumTraceShapes; records
// 16-byte aligned).  Compiled in gb_trace_shapes.cu.
cudaError_t launch_tuned_shape(const TraceParams& P, bool anyhit, cudaStream_t st);

// Ray reordering: writes, for M records, keys = direction octant (3 bits) over a
// 45-bit Morton code of the origin in the box lo..hi (15 bits per axis) and
// vals = record index, then sorts them (6 digit passes) so that vals becomes a
// fetch order in which neighbouring rays start close together and point into
// the same octant.  Scratch: kb/vb (M entries), hist (sort_hist_entries(M)).
cudaError_t order_rays(const char* rays, uint64_t stride, uint32_t M, const float lo[3], const float hi[3],
                       uint64_t* keys, uint32_t* vals, uint64_t* kb, uint32_t* vb, uint32_t* hist, cudaStream_t st);

// Size of the staging area for host-resident rays in the no-allocation query.
constexpr uint64_t kNoAllocStagingBytes = 32ull << 20;

// Loads the no-allocation query's static scratch and kernels on the current
// device (called once per device when the device is created).
cudaError_t noalloc_prepare();

// Closest-hit query whose scratch (fetch counter, error flags, staging for
// host rays) is a static device array: it allocates no memory.  `rays` is
// device-accessible memory when rays_on_device, else host memory whose span
// must fit in kNoAllocStagingBytes.  Synchronises `st`; *err_flags receives
// the kernel's kErr* bits.
cudaError_t noalloc_closest(const DeviceBVH& bvh, char* rays, bool rays_on_device, uint32_t M, uint64_t stride,
                            cudaStream_t st, uint32_t* err_flags);

}  // namespace gb
