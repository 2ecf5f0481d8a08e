// gb_build.h -- host entry points of the GPU BVH builder (gb_build.cu).
#pragma once
#include <vector>

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

// A build that runs without host reads, so that it can be captured into a
// CUDA graph and replayed: every buffer is allocated up front, and the loops
// whose trip counts depend on the data (PLOC rounds, collapse levels) are
// enqueued a fixed number of times -- rounds and levels past the last real one
// are no-ops.  The plan comes from an ordinary build of the same geometries:
// the number of valid triangles, of non-empty segments, of PLOC rounds and of
// levels (the replay checks that they still suffice and flags it otherwise).
// The BVH stays in the build's own node and triangle arrays (sized for the
// maximum), with the roots of the segments in seg_index.
struct GraphBuildPlan {
  uint32_t valid_tris = 0;   // valid triangles of the ordinary build
  uint32_t roots = 0;        // non-empty segments (1 without segments)
  uint32_t ploc_rounds = 0;  // PLOC rounds of the ordinary build (the captured build loops on the device)
  uint32_t levels = 0;       // collapse levels of the ordinary build
  int leaf_max = 2;          // resolved leaf size
};
struct GraphBuild {
  GraphBuildPlan plan;
  BuildOptions opt;
  int ngeoms = 0;
  uint32_t total = 0, nseg = 1, nbin = 0, maxw = 0, maxb = 0, rs_blocks = 0, radius = 1;
  std::vector<void*> allocs;  // every device allocation (released by graph_build_release)
  GeomDesc* d_geoms = nullptr;
  float4 *plo = nullptr, *phi = nullptr;
  void* acc = nullptr;
  uint64_t *keys_a = nullptr, *keys_b = nullptr;
  uint32_t *vals_a = nullptr, *vals_b = nullptr, *hist = nullptr;
  float4 *bnlo = nullptr, *bnhi = nullptr, *clo[2] = {nullptr, nullptr}, *chi[2] = {nullptr, nullptr};
  uint32_t *bncnt = nullptr, *cidx[2] = {nullptr, nullptr}, *nn = nullptr, *bsurv = nullptr, *bmerge = nullptr;
  uint32_t *scan_sums = nullptr, *d_tot = nullptr, *d_root = nullptr, *d_iters = nullptr, *ploc_state = nullptr;
  float4* cost = nullptr;
  uint2* choice = nullptr;
  WideNode* nodes = nullptr;
  TriRecord* tris = nullptr;
  uint32_t *items[2] = {nullptr, nullptr}, *kids = nullptr, *nint = nullptr, *ntri = nullptr, *leaf_root = nullptr;
  double* d_sah = nullptr;
  uint32_t *d_leaves = nullptr, *cstate = nullptr, *seg_index = nullptr, *status = nullptr;
  uint32_t col_grid = 0;                                // CTAs of the cooperative collapse
  uint32_t *col_sums = nullptr, *col_bar = nullptr;     // its per-CTA sums and grid barrier
  TriRecord* prec = nullptr;                            // leaf records in primitive order
  unsigned long long* stamps = nullptr;                 // phase timestamps (BuildOptions::phase_stamps)
  uint32_t ploc_grid = 0;                               // CTAs of the cooperative PLOC rounds
  uint32_t *ploc_sums = nullptr, *ploc_bar = nullptr;   // their per-CTA sums and grid barrier
};
struct GraphBuildResult {
  uint32_t status = 0;  // 0: the build is complete and consistent; else kGraphBuild* bits
  uint32_t num_nodes = 0, depth = 0, num_leaves = 0;
  uint32_t ploc_rounds = 0;  // PLOC rounds the device ran
  double sah = 0, sah_exact = 0;
  std::vector<uint32_t> level_start;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // geometry bounds of the replayed build
  std::vector<uint32_t> roots;  // segmented builds: root node of each geometry slot (kInvalidID: empty)
  uint32_t nphases = 0;         // phase times (gpu.build_phases=1)
  double phase_us[kBuildPhases] = {};
};
enum : uint32_t { kGraphBuildCount = 1, kGraphBuildRounds = 2, kGraphBuildLevels = 4, kGraphBuildError = 8 };
cudaError_t graph_build_prepare(const GeomDesc* h_geoms, int ngeoms, const BuildOptions& opt,
                                const GraphBuildPlan& plan, GraphBuild* gbuild);
cudaError_t graph_build_enqueue(const GraphBuild& gbuild, cudaStream_t st);  // capturable
cudaError_t graph_build_result(const GraphBuild& gbuild, const float scene_lo[3], const float scene_hi[3],
                               GraphBuildResult* out, cudaStream_t st);  // synchronises st
void graph_build_release(GraphBuild* gbuild);

// A scene's rebuild replayed from a captured build graph: rtcCommitScene of a scene
// whose layout (geometries, triangle counts, valid triangles, options) is that of
// its last host-driven build launches the graph and reads the results once, at the
// end (no host reads between the build's phases).
struct CachedBuild {
  GraphBuild g;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};
// Captures the build of `ngeoms` geometries with the plan of the last build (its
// valid triangles, non-empty roots, depth, PLOC rounds and resolved leaf size).
cudaError_t cached_build_create(const GeomDesc* h_geoms, int ngeoms, const BuildOptions& opt,
                                const GraphBuildPlan& plan, cudaStream_t st, CachedBuild** out);
// Replays it for the geometries `h_geoms` (same layout; buffers may have moved).
// cudaErrorNotReady: the replayed build does not match the plan (e.g. a different
// number of valid triangles); the caller builds the ordinary way.
cudaError_t cached_build_run(CachedBuild* c, const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, DeviceBVH* out,
                             BuildStats* stats);
void cached_build_release(CachedBuild* c);

// Device-to-device copy by a kernel when dst, src and bytes are 16-byte multiples
// (faster than the copy engine), else cudaMemcpyAsync.  Capturable.
cudaError_t copy_device(void* dst, const void* src, size_t bytes, cudaStream_t st);

// Stable LSD radix sort of 64-bit keys with 32-bit values (device buffers).
cudaError_t sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, cudaStream_t st);
// The low 8 * passes bits only (passes even), with caller scratch (kb, vb: n
// entries; hist: sort_hist_entries(n)); no allocation, no synchronisation.
cudaError_t sort_pairs_passes(uint64_t* keys, uint32_t* vals, uint64_t* kb, uint32_t* vb, uint32_t* hist, uint32_t n,
                              int passes, cudaStream_t st);
uint32_t sort_hist_entries(uint32_t n);

}  // namespace gb
