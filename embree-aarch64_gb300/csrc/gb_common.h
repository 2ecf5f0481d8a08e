// gb_common.h -- data layouts shared by the GPU builder, the traversal kernels
// and the C-ABI host layer of the GB300 triangle ray-query library.
//
// HBM layout of one committed scene (all arrays 16-byte aligned):
//   WideNode  nodes[num_nodes]   80 B each: 8-wide node, child boxes quantised
//                                to 8 bits per plane relative to a per-node
//                                origin and power-of-two scale (5 x 16-B loads)
//   TriRecord tris[num_tris]     48 B each: v0, e1 = v0-v1, e2 = v2-v0 (the
//                                reference's Triangle4 lane contents,
//                                kernels/geometry/triangle.h:40-41) + ids
// Children of a node are stored contiguously: internal children at
// child_base + rank among internal slots, leaf triangles at tri_base + offset.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include <vector>

namespace gb {

constexpr uint32_t kInvalidID = 0xFFFFFFFFu;
constexpr int kLeafMaxLimit = 4;     // largest leaf the node encoding allows
// Default triangles per leaf child: 0 = by scene (see build_bvh): 2 for flat
// scenes and for scenes built to be refitted, 1 otherwise (the fastest measured
// for each; 2 also keeps the heightfield SAH within 1.15x of the reference
// builder's)
constexpr int kLeafMaxDefault = 0;
constexpr int kStackSize = 64;       // traversal stack entries (node groups)

// 80-byte wide node.
//   meta[s]: 0 = empty slot; otherwise bit 7 is set and, for a leaf, bits
//            5..6 hold (triangle count - 1) and bits 0..4 the first
//            triangle's offset from tri_base (0..28).  An empty slot's box is
//            inverted (qlo = 255, qhi = 0 on every axis), so the traversal's
//            slab test misses it without reading meta.
//   imask:   bit s set when slot s holds an internal child.
//   ex/ey/ez: IEEE-754 biased exponent of the per-axis scale 2^(e-127).
//   decoded child box: lo = p + qlo * scale, hi = p + qhi * scale (the
//   quantisation rounds outward, so the decoded box contains the child).
struct alignas(16) WideNode {
  float px, py, pz;
  uint8_t ex, ey, ez, imask;
  uint32_t child_base;
  uint32_t tri_base;
  uint8_t meta[8];
  uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
  uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "WideNode must be 80 bytes");

// 48-byte triangle record: (v0.xyz, primID), (e1.xyz, geomID), (e2.xyz, pad);
// in robust scenes (v0.xyz, primID), (v1.xyz, geomID), (v2.xyz, pad), the
// reference's Triangle4v values (kernels/geometry/trianglev.h:93-115).
struct alignas(16) TriRecord {
  float4 a;
  float4 b;
  float4 c;
};
static_assert(sizeof(TriRecord) == 48, "TriRecord must be 48 bytes");

// One geometry as the builder sees it (device pointers, byte strides).
// kind 1 (instances): `verts` points to `ntris` InstBox records, one primitive each.
struct GeomDesc {
  const char* verts;
  const char* idx;
  uint64_t vstride;
  uint64_t istride;
  uint32_t nverts;
  uint32_t ntris;
  uint32_t geomID;     // user-visible geometry ID
  uint32_t prim_offset; // exclusive prefix of ntris over the scene's geometries
  uint32_t kind = 0;    // 0: triangle mesh, 1: instances
  uint32_t pad = 0;
};

// World-space box of one instance (builder input of kind-1 geometries).
struct InstBox {
  float lo[3];
  float hi[3];
  uint32_t inst;    // index into the scene's InstDesc table
  uint32_t geomID;  // the instance geometry's ID
};

// One instance as the traversal sees it: the instanced scene's BVH and the
// world-to-local transform (columns vx, vy, vz, p).
struct alignas(16) InstDesc {
  const WideNode* nodes;
  const TriRecord* tris;
  uint32_t num_nodes;
  uint32_t num_tris;
  uint32_t geomID;
  uint32_t pad;
  float w2l[12];
};
static_assert(sizeof(InstDesc) == 80, "InstDesc is 80 bytes");

// Instance leaf record: a triangle-record slot whose c.w holds kInstanceLeaf;
// a.w = index into the InstDesc table, b.w = the instance's geometry ID.
constexpr uint32_t kInstanceLeaf = 1u;

// A committed BVH in device memory.
struct DeviceBVH {
  WideNode* nodes = nullptr;
  TriRecord* tris = nullptr;
  uint32_t num_nodes = 0;
  uint32_t num_tris = 0;     // valid primitives in the BVH
  uint32_t depth = 0;        // wide levels
  int robust = 0;            // triangle records hold (v0, v1, v2) for the Pluecker test
  float lo[3] = {0, 0, 0};   // geometry bounds (empty scene: +inf / -inf)
  float hi[3] = {0, 0, 0};
  std::vector<uint32_t> level_start;  // first node of each breadth-first level + end (for refit)
  std::vector<uint32_t> roots;  // segmented builds: root node of each geometry slot (kInvalidID: empty)
};

// Builder options (device config keys gpu.leaf_max=1..4, gpu.morton=axis|cube).
struct BuildOptions {
  int leaf_max = kLeafMaxDefault;
  // Morton scaling: 0 per-axis scales (gpu.morton=axis), 1 one scale for all
  // axes (gpu.morton=cube), 2 cube when the centroid box is flat (its smallest
  // extent below half its largest), per-axis otherwise (gpu.morton=auto)
  int morton_cube = 2;
  int robust = 0;       // RTC_SCENE_FLAG_ROBUST: triangle records hold v0, v1, v2
  int segmented = 0;    // one tree per geometry slot (batched scenes), roots at the first level
  int collapse = 1;     // binary -> 8-wide: 1 SAH-optimal (gpu.collapse=sah), 0 greedy (gpu.collapse=greedy)
  int ploc_radius = 1;  // PLOC search radius: 1, 2, 4, 8 or 16 (gpu.ploc_radius)
  int refit_target = 0; // every geometry is RTC_BUILD_QUALITY_REFIT: the tree will be refitted
  // sort key: 30-bit Morton codes (10 bits per axis, the default) or 63-bit (21 per
  // axis, gpu.morton_bits=63).  On a GB300 the 30-bit key builds the 4M soup in
  // 3.13 ms against 3.51 (4 radix passes instead of 8) with the same SAH within
  // 0.02 % and the same trace time on the soup and the heightfields.
  int morton_bits = 30;
  // gpu.build_phases=1: the captured (replayed) build records a device timestamp
  // between its phases (kBuildPhases intervals, BuildStats::phase_us)
  int phase_stamps = 0;
};

// Build statistics reported through the extension API.
struct BuildStats {
  double sah = 0;            // bvh_statistics.cpp semantics on the decoded boxes
  double sah_exact = 0;      // the same on the exact (unquantised) child boxes
  uint32_t leaf_max = 0;     // triangles per leaf child the build used
  double build_ms = 0;       // device time of the whole build
  uint32_t num_nodes = 0, num_leaves = 0, num_prims = 0, depth = 0;
  uint32_t ploc_iterations = 0;
  uint32_t ploc_rounds = 0;  // PLOC rounds over all clusters (before the one-CTA finish) that merged
  uint32_t refit = 0;        // 1 when the last commit refitted instead of rebuilding
  uint32_t nphases = 0;      // phases timed (replayed builds with gpu.build_phases=1), else 0
  double phase_us[8] = {};   // primitives + keys, sort, PLOC set-up, PLOC rounds, PLOC finish,
                             // collapse set-up, collapse levels, leaf records
};
constexpr int kBuildPhases = 8;

// Traversal work counters (counting variant of the kernels).
struct TraceCounters {
  unsigned long long nodes;
  unsigned long long tris;
  unsigned long long rays;
  unsigned long long proposal_hits;  // seeded queries: rays answered inside a proposed subtree
};

// Device-side error flags (bit mask).
enum : uint32_t {
  kErrStackOverflow = 1u,
  kErrIterationLimit = 2u,
  kErrBuild = 4u,
};

}  // namespace gb
