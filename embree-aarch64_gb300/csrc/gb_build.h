// gb_build.h -- host entry points of the GPU BVH builder (gb_build.cu).
#pragma once
#include "gb_common.h"

namespace gb {

// Builds the BVH of the given geometries (device buffers) on stream `st`.
// Synchronises `st` before returning; `out` owns two device allocations that
// free_bvh releases.  An empty or all-invalid scene yields num_nodes == 0.
cudaError_t build_bvh(const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, const BuildOptions& opt, DeviceBVH* out,
                      BuildStats* stats);
void free_bvh(DeviceBVH* b);

// Refits `bvh` in place to the geometries' current vertex positions (same
// topology: the geometries, their triangles and indices are those of the
// build).  Sets *fallback when a refit is impossible (e.g. a vertex became
// invalid); the caller then rebuilds.  Synchronises `st`.
cudaError_t refit_bvh(const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, DeviceBVH* bvh, BuildStats* stats,
                      bool* fallback);

// Refit split for work captured in CUDA graphs: refit_prepare uploads the
// geometry table once (synchronous); refit_enqueue only launches the refit
// kernels on `st` (no allocation, no synchronisation; errors accumulate in
// d_err until the caller reads it).  The BVH's host-side bounds are not updated.
struct RefitScratch {
  GeomDesc* d_geoms = nullptr;
  uint32_t* d_slot = nullptr;
  uint32_t nslots = 0;
  uint32_t* d_err = nullptr;
  float* node_box = nullptr;
  float4* tri_box = nullptr;  // per-triangle boxes written by the triangle pass
  double* d_sah = nullptr;  // SAH sums on the decoded and on the exact boxes
};
cudaError_t refit_prepare(const GeomDesc* h_geoms, int ngeoms, const DeviceBVH& bvh, RefitScratch* out,
                          cudaStream_t st);
cudaError_t refit_enqueue(const DeviceBVH& bvh, const RefitScratch& s, cudaStream_t st);
void refit_release(RefitScratch* s);

// Stable LSD radix sort of 64-bit keys with 32-bit values (device buffers).
cudaError_t sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, cudaStream_t st);
// The low 8 * passes bits only (passes even), with caller scratch (kb, vb: n
// entries; hist: sort_hist_entries(n)); no allocation, no synchronisation.
cudaError_t sort_pairs_passes(uint64_t* keys, uint32_t* vals, uint64_t* kb, uint32_t* vb, uint32_t* hist, uint32_t n,
                              int passes, cudaStream_t st);
uint32_t sort_hist_entries(uint32_t n);

}  // namespace gb
