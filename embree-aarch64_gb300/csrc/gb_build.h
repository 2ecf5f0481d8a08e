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

// Stable LSD radix sort of 64-bit keys with 32-bit values (device buffers).
cudaError_t sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, cudaStream_t st);

}  // namespace gb
