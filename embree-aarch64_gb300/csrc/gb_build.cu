// gb_build.cu -- GPU BVH builder behind rtcCommitScene.
//
// Replaces the reference's CPU binned-SAH builder (kernels/bvh/bvh_builder_sah.cpp:111-189,
// kernels/builders/bvh_builder_sah.h:222-319) with a GPU pipeline:
//   1. primrefs: per-triangle validity + AABB, scene and centroid bounds
//      (validity rule of kernels/common/scene_triangle_mesh.h:127-147)
//   2. 63-bit Morton codes of the centroids (21 bits per axis)
//   3. stable LSD radix sort of (code, primref index), 8-bit digits; passes
//      whose digit is constant over all keys are skipped.  Stable sorting by
//      key with the index as value gives exactly std::stable_sort's order.
//   4. PLOC agglomerative clustering (nearest neighbour by merged-box surface
//      area within a window of +-16 clusters, mutual pairs merge) -> binary tree
//   5. top-down collapse into 8-wide nodes (largest-area child opened first),
//      child boxes quantised to 8 bits per plane, children placed in slots
//      so that the ray's direction octant gives a near-to-far visiting order,
//      leaves of <= 4 triangles written as v0/e1/e2 records.
// Everything is deterministic: the same input gives the same bytes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gb_build.h"
#include "gb_common.h"
#include "gb_launch.h"

namespace gb {

#define GB_CHECK(x)                                \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return e_;              \
  } while (0)

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
#else
  uint32_t b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}

struct BoundsAcc {
  uint32_t glo[3], ghi[3];  // ordered-uint min/max of geometry bounds
  uint32_t clo[3], chi[3];  // of centroids
  uint32_t nvalid;
  uint32_t pad;
  unsigned long long kand, kor;
};

__device__ __forceinline__ float half_area(float3 lo, float3 hi) {
  const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx * (dy + dz) + dy * dz;
}

__device__ __forceinline__ float3 f3min(float3 a, float3 b) {
  return make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
}
__device__ __forceinline__ float3 f3max(float3 a, float3 b) {
  return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
}

// ---------------------------------------------------------------------------
// 1. primrefs
// ---------------------------------------------------------------------------

constexpr float kFltLarge = 1.844E18f;  // common/math/constants.h:34

__device__ __forceinline__ bool vtx_ok(float x, float y, float z) {
  return x > -kFltLarge && x < kFltLarge && y > -kFltLarge && y < kFltLarge && z > -kFltLarge && z < kFltLarge;
}

__device__ __forceinline__ float3 load_vtx(const GeomDesc& g, uint32_t i) {
  const float* p = reinterpret_cast<const float*>(g.verts + (uint64_t)i * g.vstride);
  return make_float3(p[0], p[1], p[2]);
}

__device__ __forceinline__ uint3 load_tri(const GeomDesc& g, uint32_t j) {
  const uint32_t* p = reinterpret_cast<const uint32_t*>(g.idx + (uint64_t)j * g.istride);
  return make_uint3(p[0], p[1], p[2]);
}

__device__ __forceinline__ int find_geom(const GeomDesc* geoms, int ngeoms, uint32_t gi) {
  int lo = 0, hi = ngeoms - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (geoms[mid].prim_offset <= gi) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// plo[i] = (lo.xyz, geometry slot), phi[i] = (hi.xyz, primID); invalid
// triangles get an empty box (+inf,-inf).  prec[i] (when non-null) receives
// primitive i's leaf record -- Triangle4 values v0, e1 = v0 - v1, e2 = v2 - v0
// (triangle.h:40-41), or v0, v1, v2 in robust scenes (trianglev.h:93-115), or
// an instance leaf -- read here in primitive order, where the vertex reads
// coalesce, so that the leaf writer later gathers one 48-byte record per leaf.
// Grid-stride: the bounds and the valid count are reduced per thread, per warp
// and per CTA, so the global atomics are 13 per CTA (a grid of a few CTAs per SM).
__global__ void __launch_bounds__(256) k_primrefs(const GeomDesc* __restrict__ geoms, int ngeoms, uint32_t total,
                                                  float4* __restrict__ plo, float4* __restrict__ phi,
                                                  BoundsAcc* acc, TriRecord* __restrict__ prec, int robust) {
  __shared__ uint32_t s_b[12];
  __shared__ uint32_t s_cnt;
  if (threadIdx.x < 12) s_b[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  float v[12];
#pragma unroll
  for (int k = 0; k < 12; k++) v[k] = (k % 6) < 3 ? INFINITY : -INFINITY;
  unsigned nok = 0;
  for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < total; gi += gridDim.x * blockDim.x) {
    bool ok = false;
    float3 lo = make_float3(INFINITY, INFINITY, INFINITY), hi = make_float3(-INFINITY, -INFINITY, -INFINITY);
    {
      const int gs = find_geom(geoms, ngeoms, gi);
      const GeomDesc g = geoms[gs];
      const uint32_t j = gi - g.prim_offset;
      if (g.kind == 1) {
        const InstBox bx = reinterpret_cast<const InstBox*>(g.verts)[j];
        if (vtx_ok(bx.lo[0], bx.lo[1], bx.lo[2]) && vtx_ok(bx.hi[0], bx.hi[1], bx.hi[2]) && bx.lo[0] <= bx.hi[0] &&
            bx.lo[1] <= bx.hi[1] && bx.lo[2] <= bx.hi[2]) {
          ok = true;
          lo = make_float3(bx.lo[0], bx.lo[1], bx.lo[2]);
          hi = make_float3(bx.hi[0], bx.hi[1], bx.hi[2]);
        }
        if (prec)
          prec[gi] = TriRecord{make_float4(0.f, 0.f, 0.f, __uint_as_float(bx.inst)),
                               make_float4(0.f, 0.f, 0.f, __uint_as_float(bx.geomID)),
                               make_float4(0.f, 0.f, 0.f, __uint_as_float(kInstanceLeaf))};
      } else {
      const uint3 t = load_tri(g, j);
      if (t.x < g.nverts && t.y < g.nverts && t.z < g.nverts) {
        const float3 a = load_vtx(g, t.x), b = load_vtx(g, t.y), c = load_vtx(g, t.z);
        if (vtx_ok(a.x, a.y, a.z) && vtx_ok(b.x, b.y, b.z) && vtx_ok(c.x, c.y, c.z)) {
          ok = true;
          lo = f3min(f3min(a, b), c);
          hi = f3max(f3max(a, b), c);
          if (prec) {
            const float3 e1 = robust ? b : make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
            const float3 e2 = robust ? c : make_float3(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z));
            prec[gi] = TriRecord{make_float4(a.x, a.y, a.z, __uint_as_float(j)),
                                 make_float4(e1.x, e1.y, e1.z, __uint_as_float(g.geomID)),
                                 make_float4(e2.x, e2.y, e2.z, 0.f)};
          }
        }
      }
      }
      plo[gi] = make_float4(lo.x, lo.y, lo.z, __uint_as_float((uint32_t)gs));
      phi[gi] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(j));
    }
    v[0] = fminf(v[0], lo.x); v[1] = fminf(v[1], lo.y); v[2] = fminf(v[2], lo.z);
    v[3] = fmaxf(v[3], hi.x); v[4] = fmaxf(v[4], hi.y); v[5] = fmaxf(v[5], hi.z);
    if (ok) {
      const float3 c = make_float3((lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f);
      v[6] = fminf(v[6], c.x); v[7] = fminf(v[7], c.y); v[8] = fminf(v[8], c.z);
      v[9] = fmaxf(v[9], c.x); v[10] = fmaxf(v[10], c.y); v[11] = fmaxf(v[11], c.z);
      nok++;
    }
  }
  // warp-reduce bounds then shared atomics
#pragma unroll
  for (int k = 0; k < 12; k++) {
    float x = v[k];
    const bool isMin = (k % 6) < 3;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float y = __shfl_xor_sync(0xFFFFFFFFu, x, o);
      x = isMin ? fminf(x, y) : fmaxf(x, y);
    }
    v[k] = x;
  }
  nok = __reduce_add_sync(0xFFFFFFFFu, nok);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      if ((k % 6) < 3) atomicMin(&s_b[k], f2ord(v[k]));
      else atomicMax(&s_b[k], f2ord(v[k]));
    }
    atomicAdd(&s_cnt, nok);
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    uint32_t* dst = (k < 3) ? &acc->glo[k] : (k < 6) ? &acc->ghi[k - 3] : (k < 9) ? &acc->clo[k - 6] : &acc->chi[k - 9];
    if ((k % 6) < 3) atomicMin(dst, s_b[k]); else atomicMax(dst, s_b[k]);
  }
  if (threadIdx.x == 0) atomicAdd(&acc->nvalid, s_cnt);
}

// ---------------------------------------------------------------------------
// 2. Morton codes
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint64_t spread21(uint32_t x) {
  uint64_t v = x & 0x1FFFFFu;
  v = (v | (v << 32)) & 0x1F00000000FFFFull;
  v = (v | (v << 16)) & 0x1F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  uint32_t v = x & 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// Segmented builds put the geometry slot (< kMaxSegments) in the key's top 12
// bits, so the sort groups every geometry's primitives.
// bits30 (gpu.morton_bits=30): 10 bits per axis, the lattice of the reference's
// Morton builder (kernels/builders/bvh_builder_morton.h:62-86, LATTICE_BITS_PER_DIM
// 10), so valid keys fit in 30 bits (42 with the slot) and the sort needs 4 (6)
// digit passes instead of 8; invalid primitives get bit 30 (42) set, above every
// valid key, so they sort after all valid ones.  key32: the 30-bit keys of an
// unsegmented build are written as 32-bit words (the sort then moves 4-byte keys).
constexpr uint32_t kMaxSegments = 4096;

// Grid-stride; the AND / OR of all keys (constant digits are not sorted) is
// reduced per thread, per warp and per CTA: two global atomics per CTA.
__global__ void __launch_bounds__(256) k_morton(const float4* __restrict__ plo, const float4* __restrict__ phi,
                                                uint32_t n, BoundsAcc* acc, uint64_t* __restrict__ keys,
                                                uint32_t* __restrict__ vals, int cube, int segmented, int bits30,
                                                int key32) {
  __shared__ unsigned long long s_and, s_or;
  if (threadIdx.x == 0) {
    s_and = ~0ull;
    s_or = 0ull;
  }
  __syncthreads();
  unsigned long long ka = ~0ull, ko = 0ull;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint64_t key = bits30 ? (1ull << (segmented ? 42 : 30)) : ~0ull;
    {
      const float4 a = plo[i], b = phi[i];
      if (a.x <= b.x) {
        const float lo[3] = {ord2f(acc->clo[0]), ord2f(acc->clo[1]), ord2f(acc->clo[2])};
        const float hi[3] = {ord2f(acc->chi[0]), ord2f(acc->chi[1]), ord2f(acc->chi[2])};
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        // one scale for all axes (the centroid box's largest extent) keeps the
        // scene's aspect ratio, so flat scenes (heightfields) are ordered mostly
        // in-plane, which lowers their SAH; per-axis scales trace faster on
        // volumetric scenes.  cube: 0 per-axis, 1 one scale, 2 one scale when
        // the centroid box is flat
        const float emax = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
        const float emin = fminf(fminf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
        const bool one_scale = cube == 1 || (cube == 2 && emin < 0.5f * emax);
        uint64_t code = 0;
        if (bits30) {
          uint32_t c30 = 0;
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const float ext = one_scale ? emax : hi[d] - lo[d];
            float x = ext > 0.0f ? (c[d] - lo[d]) / ext : 0.0f;
            x = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
            c30 |= spread10((uint32_t)x) << (2 - d);
          }
          key = segmented ? ((uint64_t)(__float_as_uint(a.w) & (kMaxSegments - 1)) << 30) | c30 : c30;
        } else {
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const float ext = one_scale ? emax : hi[d] - lo[d];
            float x = ext > 0.0f ? (c[d] - lo[d]) / ext : 0.0f;
            x = fminf(fmaxf(x * 2097152.0f, 0.0f), 2097151.0f);
            code |= spread21((uint32_t)x) << (2 - d);
          }
          key = segmented ? ((uint64_t)(__float_as_uint(a.w) & (kMaxSegments - 1)) << 51) | (code >> 12) : code;
        }
      }
      if (key32) reinterpret_cast<uint32_t*>(keys)[i] = (uint32_t)key;
      else keys[i] = key;
      vals[i] = i;
    }
    ka &= key;
    ko |= key;
  }
  // AND / OR over all keys to find constant digits
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ka &= __shfl_xor_sync(0xFFFFFFFFu, ka, o);
    ko |= __shfl_xor_sync(0xFFFFFFFFu, ko, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAnd(&s_and, ka);
    atomicOr(&s_or, ko);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAnd(&acc->kand, s_and);
    atomicOr(&acc->kor, s_or);
  }
}

// ---------------------------------------------------------------------------
// Device-to-device copies on the SMs.  A cudaMemcpyAsync between device buffers
// runs on a copy engine: measured on a GB300, restoring 47.5 GB of ray records
// inside a CUDA graph took 29.8 ms that way against 13.7 ms for this kernel.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_copy16(uint4* __restrict__ dst, const uint4* __restrict__ src, size_t n16) {
  for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n16; i += (size_t)gridDim.x * 256) dst[i] = src[i];
}

static int num_sms_build();

cudaError_t copy_device(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return cudaSuccess;
  if (((uintptr_t)dst | (uintptr_t)src | bytes) % 16 != 0)
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
  const size_t n16 = bytes / 16;
  const size_t grid = std::min<size_t>((n16 + 255) / 256, (size_t)num_sms_build() * 8);
  k_copy16<<<(unsigned)grid, 256, 0, st>>>(static_cast<uint4*>(dst), static_cast<const uint4*>(src), n16);
  note_launches(1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 3. stable LSD radix sort (64-bit keys, 32-bit values), onesweep style
// ---------------------------------------------------------------------------
//
// One pass over the keys counts every digit (8 bits each) at once; its last CTA
// turns the counts into each digit's bucket bases.  Then one scatter kernel per
// digit pass: CTAs take 4096-key tiles in ticket order, publish their digit counts
// and find the counts of all tiles before them by decoupled look-back (Merrill &
// Garland, "Single-pass Parallel Prefix Scan with Decoupled Look-back", 2016), rank
// their keys stably and scatter them.  No scan kernels and no host reads.  The
// reference's CPU sort (common/algorithms/parallel_sort.h:256-449) is the same
// stable 8-bit LSD sort, one histogram + scatter round per digit over task blocks.

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

// look-back status words: flag bits over a 30-bit count
constexpr uint32_t kLbAggregate = 1u << 30;   // the tile's own count is published
constexpr uint32_t kLbPrefix = 2u << 30;      // the inclusive prefix through the tile is published
constexpr uint32_t kLbValue = (1u << 30) - 1u;
constexpr uint32_t kLbSpinLimit = 1u << 22;   // re-reads of an unpublished word before giving up
// onesweep scratch (uint32 words, zeroed before each sort): bucket bases of the 8
// digit passes, tile tickets per pass, the histogram kernel's done counter, an
// error word, then per pass ntiles x 256 look-back status words
constexpr uint32_t kOsBases = 0, kOsTickets = 8 * 256, kOsDone = kOsTickets + 8, kOsErr = kOsDone + 1;
constexpr uint32_t kOsStatus = 2112;  // 16-byte aligned start of the status tables

__device__ __forceinline__ void lb_store(uint32_t* p, uint32_t v) { *reinterpret_cast<volatile uint32_t*>(p) = v; }
__device__ __forceinline__ uint32_t lb_load(const uint32_t* p) { return *reinterpret_cast<const volatile uint32_t*>(p); }

// Sum of the counts of the tiles before `tile` (status words status[j * stride],
// j < tile), following the chain back to the nearest published inclusive prefix.
// A word that stays unpublished for kLbSpinLimit re-reads sets kErrBuild in *err
// and counts as zero (the sort's result is then invalid and the host reports it).
__device__ __forceinline__ uint32_t lb_exclusive(const uint32_t* status, uint32_t tile, uint32_t stride,
                                                 unsigned int* err) {
  uint32_t excl = 0;
  for (int64_t j = (int64_t)tile - 1; j >= 0; j--) {
    uint32_t w = lb_load(status + (size_t)j * stride);
    for (uint32_t it = 0; w == 0u && it < kLbSpinLimit; it++) {
      __nanosleep(32);
      w = lb_load(status + (size_t)j * stride);
    }
    if (w == 0u) {
      atomicOr(err, kErrBuild);
      break;
    }
    excl += w & kLbValue;
    if (w & kLbPrefix) break;
  }
  return excl;
}

// Counts of every active digit (digit_mask bit d: digit d, bits 8d..8d+7) over all
// keys (K: 32- or 64-bit); the last CTA writes each digit's exclusive bucket bases.
template <typename K>
__global__ void __launch_bounds__(256) k_os_hist(const K* __restrict__ keys, uint32_t n, uint32_t digit_mask,
                                                 uint32_t* __restrict__ scratch) {
  __shared__ uint32_t s_h[8][256];
  __shared__ bool s_last;
  const int tid = threadIdx.x;
#pragma unroll
  for (int d = 0; d < 8; d++) s_h[d][tid] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * 256u + tid; i < n; i += gridDim.x * 256u) {
    const K k = keys[i];
#pragma unroll
    for (int d = 0; d < (int)sizeof(K); d++)
      if (digit_mask >> d & 1u) atomicAdd(&s_h[d][(uint32_t)(k >> (8 * d)) & 0xFFu], 1u);
  }
  __syncthreads();
#pragma unroll
  for (int d = 0; d < 8; d++)
    if ((digit_mask >> d & 1u) && s_h[d][tid]) atomicAdd(scratch + kOsBases + d * 256 + tid, s_h[d][tid]);
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(scratch + kOsDone, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // exclusive scan of each digit's 256 counts (one bin per thread)
  __shared__ uint32_t s_w[8];
  const int lane = tid & 31, warp = tid >> 5;
  for (int d = 0; d < 8; d++) {
    if (!(digit_mask >> d & 1u)) continue;
    const uint32_t c = lb_load(scratch + kOsBases + d * 256 + tid);
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; w++) before += s_w[w];
    scratch[kOsBases + d * 256 + tid] = before + x - c;
    __syncthreads();
  }
}

// One digit pass: tile `ticket` of kin/vin is ranked by digit (bits shift..shift+7)
// and scattered stably to kout/vout.  status: this pass's ntiles x 256 table.
// Warp w ranks keys base + w*512 .. +511 (16 rows of 32) by match_any into
// per-warp digit counts; the tile's digit counts are published for the look-back;
// the keys are placed in shared memory in (digit, original order) order and written
// out in runs, consecutive threads to consecutive positions of a digit's bucket.
constexpr int RS_WARPS = RS_THREADS / 32;
template <typename K>
constexpr size_t os_scatter_smem() { return (size_t)RS_TILE * (sizeof(K) + sizeof(uint32_t)); }

template <typename K>
__global__ void __launch_bounds__(RS_THREADS) k_os_scatter(const K* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           K* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, uint32_t* __restrict__ scratch,
                                                           uint32_t pass_slot, uint32_t* __restrict__ status,
                                                           unsigned int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char s_stage[];               // RS_TILE keys, then RS_TILE values
  K* s_keys = reinterpret_cast<K*>(s_stage);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + RS_TILE);
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_wcnt[RS_WARPS][256];  // per-warp digit counts, then per-warp offsets
  __shared__ uint32_t s_lstart[256];          // tile-local start of each digit
  __shared__ uint32_t s_glob[256];            // global position of local index 0 of each digit
  __shared__ uint32_t s_w[RS_WARPS];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s_tile = atomicAdd(scratch + kOsTickets + pass_slot, 1u);
#pragma unroll
  for (int w = 0; w < RS_WARPS; w++) s_wcnt[w][tid] = 0;
  __syncthreads();
  const uint32_t tile = s_tile, base = tile * RS_TILE;
  if (base >= n) return;  // (the grid has exactly one CTA per tile)
  const uint32_t tile_n = min((uint32_t)RS_TILE, n - base);
  const uint32_t lt = (1u << lane) - 1u;
  // ---- per-warp ranking (warp-synchronous: each warp owns its row of s_wcnt)
  K k[RS_ITEMS];
  uint32_t pos[RS_ITEMS];
  const uint32_t wbase = base + (uint32_t)warp * (RS_ITEMS * 32);
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const uint32_t i = wbase + r * 32 + lane;
    const bool in = i < n;
    k[r] = in ? kin[i] : (K)0;
    const uint32_t d = in ? (uint32_t)(k[r] >> shift) & 0xFFu : 256u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t rank = __popc(peers & lt);
    pos[r] = (in ? s_wcnt[warp][d] : 0u) + rank;
    __syncwarp();
    if (in && rank == 0) s_wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // ---- digit `tid`: tile count, per-warp offsets, tile-local start
  uint32_t cnt = 0;
#pragma unroll
  for (int w = 0; w < RS_WARPS; w++) {
    const uint32_t c = s_wcnt[w][tid];
    s_wcnt[w][tid] = cnt;
    cnt += c;
  }
  {
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; w++) before += s_w[w];
    s_lstart[tid] = before + x - cnt;
  }
  // publish this tile's count of digit `tid`, then add up the tiles before it
  {
    uint32_t excl = 0;
    if (tile == 0) {
      lb_store(status + tid, kLbPrefix | cnt);
    } else {
      lb_store(status + (size_t)tile * 256 + tid, kLbAggregate | cnt);
      excl = lb_exclusive(status + tid, tile, 256, err);
      lb_store(status + (size_t)tile * 256 + tid, kLbPrefix | ((excl + cnt) & kLbValue));
    }
    s_glob[tid] = scratch[kOsBases + (shift >> 3) * 256 + tid] + excl - s_lstart[tid];
  }
  __syncthreads();
  // ---- keys to shared memory in (digit, original order) order
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const uint32_t i = wbase + r * 32 + lane;
    if (i < n) {
      const uint32_t d = (uint32_t)(k[r] >> shift) & 0xFFu;
      const uint32_t j = s_lstart[d] + s_wcnt[warp][d] + pos[r];
      s_keys[j] = k[r];
      s_vals[j] = vin[i];
    }
  }
  __syncthreads();
  // ---- runs out: local index j of digit d goes to s_glob[d] + j
  for (uint32_t j = tid; j < tile_n; j += RS_THREADS) {
    const K key = s_keys[j];
    const uint32_t out = s_glob[(uint32_t)(key >> shift) & 0xFFu] + j;
    if (out < n) {
      kout[out] = key;
      vout[out] = s_vals[j];
    } else {
      atomicOr(err, kErrBuild);
    }
  }
}

// Exclusive scans of uint32 arrays.  One tile is 1024 threads x 8 consecutive
// elements.  Small arrays are scanned by one CTA; larger ones by
// reduce-then-scan over many CTAs (tile sums, a one-CTA scan of the sums, then
// each tile scanned again from its offset), which reads the array twice and
// writes it once.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER = 8;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_PER;

// Scans a[base, base + SCAN_TILE) in place, offset by carry; every thread gets
// the tile's total.  All threads of the CTA must call it.
__device__ __forceinline__ uint32_t scan_tile(uint32_t* __restrict__ a, uint32_t n, uint32_t base, uint32_t carry,
                                              uint32_t* s_w) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t v[SCAN_PER];
  uint32_t sum = 0;
  const uint32_t i0 = base + threadIdx.x * SCAN_PER;
#pragma unroll
  for (int k = 0; k < SCAN_PER; k++) {
    v[k] = (i0 + k < n) ? a[i0 + k] : 0u;
    sum += v[k];
  }
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_w[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    s_w[lane] = w;
  }
  __syncthreads();
  uint32_t excl = carry + (warp ? s_w[warp - 1] : 0u) + (x - sum);
#pragma unroll
  for (int k = 0; k < SCAN_PER; k++) {
    if (i0 + k < n) a[i0 + k] = excl;
    excl += v[k];
  }
  const uint32_t tile_total = s_w[31];
  __syncthreads();  // s_w is reused by the next call
  return tile_total;
}

// Element counts of the scans: n itself, or -- when the count is produced on
// the device (builds that run without host reads) -- ceil(*d_n / div) capped
// at n.  Grids are then sized for the cap and the tile loops are grid-stride.
__device__ __forceinline__ uint32_t scan_count(uint32_t n, const uint32_t* d_n, uint32_t div) {
  return d_n ? min(n, (*d_n + div - 1) / div) : n;
}

// Two arrays scanned by one launch (the survivors and merges of a PLOC round,
// the internal children and triangles of a collapse level): blockIdx.y picks
// the array, its total and (look-back scan) its state.
struct ScanPair {
  uint32_t* a[2];
  uint32_t* total[2];
};

// One CTA of 1024 threads over the whole array; optionally writes the total.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_excl(ScanPair sp, uint32_t n,
                                                            const uint32_t* __restrict__ d_n, uint32_t div) {
  __shared__ uint32_t s_w[32];
  uint32_t* __restrict__ a = sp.a[blockIdx.y];
  uint32_t* total = sp.total[blockIdx.y];
  n = scan_count(n, d_n, div);
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += SCAN_TILE) carry += scan_tile(a, n, base, carry, s_w);
  if (total && threadIdx.x == 0) *total = carry;
}

// Single-pass exclusive scan of larger arrays: CTAs take SCAN_TILE tiles in ticket
// order, publish their tile sums and add up those of the tiles before them by
// decoupled look-back, then scan their tile from that offset.  state (per array,
// state_words apart): [0] ticket, [1] CTAs finished, [2 + t] status word of tile
// t; zero on entry, and the last CTA to finish zeroes it again for the next scan
// (graph replays included).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_lb(ScanPair sp, uint32_t n,
                                                          const uint32_t* __restrict__ d_n, uint32_t div,
                                                          uint32_t* __restrict__ state_base, uint32_t state_words,
                                                          unsigned int* __restrict__ err) {
  __shared__ uint32_t s_w[32];
  __shared__ uint32_t s_tile, s_excl;
  __shared__ bool s_last;
  uint32_t* __restrict__ a = sp.a[blockIdx.y];
  uint32_t* total = sp.total[blockIdx.y];
  uint32_t* __restrict__ state = state_base + (size_t)blockIdx.y * state_words;
  n = scan_count(n, d_n, div);
  const uint32_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (threadIdx.x == 0) s_tile = atomicAdd(state, 1u);
  __syncthreads();
  const uint32_t t = s_tile;
  uint32_t* status = state + 2;
  if (t < ntiles) {
    const uint32_t i0 = t * SCAN_TILE + threadIdx.x * SCAN_PER;
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; k++) sum += (i0 + k < n) ? a[i0 + k] : 0u;
    sum = __reduce_add_sync(0xFFFFFFFFu, sum);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x < 32) {
      const uint32_t tile_sum = __reduce_add_sync(0xFFFFFFFFu, s_w[threadIdx.x]);
      if (threadIdx.x == 0) {
        uint32_t excl = 0;
        if (t == 0) {
          lb_store(status, kLbPrefix | (tile_sum & kLbValue));
        } else {
          lb_store(status + t, kLbAggregate | (tile_sum & kLbValue));
          excl = lb_exclusive(status, t, 1, err);
          lb_store(status + t, kLbPrefix | ((excl + tile_sum) & kLbValue));
        }
        s_excl = excl;
        if (t == ntiles - 1 && total) *total = excl + tile_sum;
      }
    }
    __syncthreads();
    scan_tile(a, n, t * SCAN_TILE, s_excl, s_w);
  } else if (t == 0 && total && threadIdx.x == 0) {
    *total = 0;  // empty input
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(state + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    for (uint32_t j = threadIdx.x; j < gridDim.x; j += SCAN_THREADS) status[j] = 0;
    if (threadIdx.x == 0) {
      state[0] = 0;
      state[1] = 0;
    }
  }
}

// ---- SAH-optimal collapse (dynamic programming over the binary tree, after
// Ylitie, Karras and Laine, "Efficient incoherent ray traversal on GPUs
// through compressed wide BVHs", HPG 2017).  cost(n, i) is the least SAH cost
// of the subtree of binary node n when it may take up to i child slots of a
// wide node: i = 1 is n itself as one child (a leaf when it holds at most
// leaf_max triangles -- then its cost is area x Triangle4 blocks -- else a wide
// node of its own: area + D(n, 8)); i > 1 is min(cost(n, i - 1), D(n, i)) with
// D(n, i) = min over k of cost(left, k) + cost(right, i - k).  The costs are
// the SAH statistic's terms (bvh_statistics.cpp:10-160), so the tree minimises
// the reported SAH for the given binary tree and leaf size.
//
// choice[n] packs the decisions: byte 0 = argmin k of D(n, 8) (the split of a
// wide node made from n); byte i - 1 (i = 2..8) = the k of D(n, i) when it beat
// cost(n, i - 1), else 0.

__device__ __forceinline__ void dp_store(float4* cost, uint2* choice, uint32_t n, const float c[8], uint2 ch) {
  __stcg(cost + 2 * (size_t)n, make_float4(c[0], c[1], c[2], c[3]));
  __stcg(cost + 2 * (size_t)n + 1, make_float4(c[4], c[5], c[6], c[7]));
  __stcg(choice + n, ch);
}

// A child's cost(., 1..8): a primitive (one triangle) costs its box area
// whatever the number of slots (one leaf block), so primitives have no table
// entries and the caller passes their areas; internal children's costs are
// stored already.
__device__ __forceinline__ void dp_child_costs(const float4* cost, uint32_t c, uint32_t cnt_c, float Ac, float (&out)[8]) {
  if (cnt_c == 1) {
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = Ac;
    return;
  }
  const float4 a = __ldcg(cost + 2 * (size_t)c), b = __ldcg(cost + 2 * (size_t)c + 1);
  out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w; out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
}

// cost(n, 1..8) and the choices of binary node n with children l and r (cnt_l,
// cnt_r triangles; a child of one triangle is a primitive, whose area Al / Ar
// the caller passes); A is n's box area.  The PLOC kernels call it as they
// create each node, so the table is complete when the clustering ends
// (children are always created before their parent).
__device__ __forceinline__ void dp_node(float4* cost, uint2* choice, uint32_t n, uint32_t l, uint32_t r, float A,
                                        uint32_t cnt_l, uint32_t cnt_r, float Al, float Ar, uint32_t leaf_max) {
  const uint32_t cnt = cnt_l + cnt_r;
  float cl[8], cr[8];
  dp_child_costs(cost, l, cnt_l, Al, cl);
  dp_child_costs(cost, r, cnt_r, Ar, cr);
  float D[9];
  uint32_t K[9];
#pragma unroll
  for (int i = 2; i <= 8; i++) {
    D[i] = INFINITY;
    K[i] = 1;
#pragma unroll
    for (int k = 1; k < i; k++) {
      const float v = cl[k - 1] + cr[i - k - 1];
      if (v < D[i]) {
        D[i] = v;
        K[i] = (uint32_t)k;
      }
    }
  }
  const float c_int = A + D[8];
  const float c_leaf = cnt <= leaf_max ? A * (float)((cnt + 3) / 4) : INFINITY;
  float c[8];
  c[0] = fminf(c_leaf, c_int);
  uint32_t b[8];
  b[0] = K[8];
#pragma unroll
  for (int i = 2; i <= 8; i++) {
    const bool split = D[i] < c[i - 2];
    c[i - 1] = split ? D[i] : c[i - 2];
    b[i - 1] = split ? K[i] : 0u;
  }
  dp_store(cost, choice, n, c,
           make_uint2(b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24), b[4] | (b[5] << 8) | (b[6] << 16) | (b[7] << 24)));
}


// Grid barrier of the cooperative build kernels (all CTAs resident).
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
};

// Barrier over all CTAs of a cooperative launch; every thread calls it.  A CTA
// that waits for more than kLbSpinLimit re-reads (a CTA missing) sets kErrBuild
// in *err; a CTA that finds *err set does not wait.  Returns false once *err
// is set, so the grid leaves its loop.
__device__ __forceinline__ bool grid_sync(GridBarrier* b, unsigned int* err) {
  __shared__ bool s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = lb_load(err) == 0u;
    if (ok) {
      const unsigned int g = lb_load(&b->gen);
      __threadfence();
      if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
        lb_store(&b->count, 0u);
        __threadfence();
        atomicAdd(&b->gen, 1u);
      } else {
        uint32_t it = 0;
        while (lb_load(&b->gen) == g && it < kLbSpinLimit) {
          __nanosleep(64);
          it++;
        }
        if (it == kLbSpinLimit) {
          atomicOr(err, kErrBuild);
          ok = false;
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok;
}

// ---------------------------------------------------------------------------
// 4. PLOC
// ---------------------------------------------------------------------------

// PLOC's search radius (clusters on each side in Morton order) is a template
// parameter of the nearest-neighbour kernel; gpu.ploc_radius picks 1, 2, 4, 8
// or 16.  Measured on a GB300, radius 1 gave the lowest SAH on heightfields,
// the fastest traversal and the fastest build (a wider window made the
// clusters' merges less local: the 4M soup went from 1033 to 889 Mrays/s
// closest between radius 1 and 16).
constexpr int PLOC_R_MAX = 16;
constexpr int PLOC_BLOCK = 256;
constexpr uint32_t PLOC_SMALL = 4096;   // finish on one CTA below this many clusters
constexpr int PLOC_SMALL_THREADS = 1024;
// k_ploc_small's shared memory: boxes, node ids, nearest neighbours, segments, counts
constexpr size_t kPlocSmallSmem = (size_t)PLOC_SMALL * (2 * sizeof(float3) + 4 * sizeof(uint32_t));

// binary nodes: bnlo[k] = (lo.xyz, left), bnhi[k] = (hi.xyz, right);
// leaves k < N: left = -1, right = primref index
// Cluster boxes carry their segment in clo.w (0 unless the build is segmented)
// and their triangle count in chi.w (so a merge has both children's counts
// with their boxes, without a dependent read of bncnt).
__global__ void __launch_bounds__(256) k_ploc_init(const float4* __restrict__ plo, const float4* __restrict__ phi,
                                                   const uint32_t* __restrict__ sorted, uint32_t n,
                                                   const uint32_t* __restrict__ d_n,
                                                   float4* __restrict__ bnlo, float4* __restrict__ bnhi,
                                                   uint32_t* __restrict__ bncnt, uint32_t* __restrict__ cidx,
                                                   float4* __restrict__ clo, float4* __restrict__ chi, int segmented) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || i >= *d_n) return;  // n bounds the grid, *d_n is the count of valid primitives
  const uint32_t p = sorted[i];
  const float4 a = plo[p], b = phi[p];
  bnlo[i] = make_float4(a.x, a.y, a.z, __int_as_float(-1));
  bnhi[i] = make_float4(b.x, b.y, b.z, __uint_as_float(p));
  bncnt[i] = 1;
  cidx[i] = i;
  clo[i] = make_float4(a.x, a.y, a.z, segmented ? a.w : __uint_as_float(0u));
  chi[i] = make_float4(b.x, b.y, b.z, __uint_as_float(1u));
}

// PLOC rounds run back to back without the host.  ploc_state (device memory):
// [0] cluster count n, [1] next binary node index, [2] rounds that merged,
// [3] 256-cluster tiles of n, [4] done -- set once n <= PLOC_SMALL (the one-CTA
// kernel finishes) or a round merged nothing; every kernel of a later round is
// then a no-op, so a fixed number of rounds can be enqueued (or captured) and
// the tree is the same whatever the number of extra rounds.  The kernels loop
// over the tiles grid-stride, so the grid is any size.
enum : int { kPlocN = 0, kPlocNext = 1, kPlocRounds = 2, kPlocTiles = 3, kPlocDone = 4, kPlocParity = 5,
             kPlocIters = 6, kPlocStateWords = 8 };
// device-decided PLOC loops (the cooperative rounds of captured builds) stop
// after this many rounds
constexpr uint32_t kPlocMaxIters = 1024;

// The two cluster buffers of the PLOC rounds; a round reads set ploc_state[kPlocParity]
// and writes the other one, so every round runs the same kernels with the same
// arguments (a loop body captured once serves every iteration).
struct PlocBufs {
  float4* clo[2];
  float4* chi[2];
  uint32_t* cidx[2];
};


// The clusters alternate between two buffers, one round reading A and writing
// B, the next the reverse; kPlocParity counts (mod 2) the rounds that ran, so
// the current clusters are in B when it is 1 whatever no-op rounds followed.
__global__ void k_ploc_state_init(const BoundsAcc* __restrict__ acc, uint32_t* __restrict__ ploc_state) {
  if (threadIdx.x == 0) {
    const uint32_t n = acc->nvalid;
    ploc_state[kPlocN] = n;
    ploc_state[kPlocNext] = n;  // binary leaves are the primitives 0..n-1
    ploc_state[kPlocRounds] = 0;
    ploc_state[kPlocTiles] = (n + PLOC_BLOCK - 1) / PLOC_BLOCK;
    ploc_state[kPlocDone] = n <= PLOC_SMALL ? 1u : 0u;
    ploc_state[kPlocParity] = 0;
    ploc_state[kPlocIters] = 0;
  }
}

// Nearest neighbour (least merged-box area within PLOC_R clusters on either
// side, same segment) of every cluster of one PLOC_BLOCK tile; the window with
// its halo is staged in shared memory.
template <int PLOC_R>
__device__ __forceinline__ void ploc_nn_tile(const float4* __restrict__ clo, const float4* __restrict__ chi, uint32_t n,
                                             uint32_t tile, uint32_t* __restrict__ nn, float3* s_lo, float3* s_hi,
                                             uint32_t* s_seg) {
  const int base = (int)(tile * PLOC_BLOCK);
  for (int k = threadIdx.x; k < PLOC_BLOCK + 2 * PLOC_R; k += PLOC_BLOCK) {
    const int j = base - PLOC_R + k;
    if (j >= 0 && j < (int)n) {
      const float4 a = clo[j], b = chi[j];
      s_lo[k] = make_float3(a.x, a.y, a.z);
      s_hi[k] = make_float3(b.x, b.y, b.z);
      s_seg[k] = __float_as_uint(a.w);
    }
  }
  __syncthreads();
  const int i = base + threadIdx.x;
  if (i < (int)n) {
    const float3 lo = s_lo[threadIdx.x + PLOC_R], hi = s_hi[threadIdx.x + PLOC_R];
    const uint32_t seg = s_seg[threadIdx.x + PLOC_R];
    unsigned long long best = ~0ull;
#pragma unroll 4
    for (int o = -PLOC_R; o <= PLOC_R; o++) {
      const int j = i + o;
      if (o == 0 || j < 0 || j >= (int)n || s_seg[threadIdx.x + PLOC_R + o] != seg) continue;
      const float a = half_area(f3min(lo, s_lo[threadIdx.x + PLOC_R + o]), f3max(hi, s_hi[threadIdx.x + PLOC_R + o]));
      const unsigned long long key = ((unsigned long long)__float_as_uint(a) << 32) | (uint32_t)j;
      best = key < best ? key : best;
    }
    nn[i] = best != ~0ull ? (uint32_t)best : (uint32_t)i;  // no neighbour in the segment: stays alone
  }
  __syncthreads();  // the window is reloaded for the next tile
}

// The same nearest neighbour for one cluster h, read from global memory (the
// halo clusters just outside a CTA's run of tiles; bit-identical to the tile
// form: same boxes, same area arithmetic, the least (area, index) key).
template <int PLOC_R>
__device__ __forceinline__ uint32_t ploc_nn_one(const float4* __restrict__ clo, const float4* __restrict__ chi,
                                                uint32_t n, int h) {
  const float4 a = clo[h], b = chi[h];
  const float3 lo = make_float3(a.x, a.y, a.z), hi = make_float3(b.x, b.y, b.z);
  const uint32_t seg = __float_as_uint(a.w);
  unsigned long long best = ~0ull;
  for (int o = -PLOC_R; o <= PLOC_R; o++) {
    const int j = h + o;
    if (o == 0 || j < 0 || j >= (int)n) continue;
    const float4 c = clo[j], d = chi[j];
    if (__float_as_uint(c.w) != seg) continue;
    const float ar = half_area(f3min(lo, make_float3(c.x, c.y, c.z)), f3max(hi, make_float3(d.x, d.y, d.z)));
    const unsigned long long key = ((unsigned long long)__float_as_uint(ar) << 32) | (uint32_t)j;
    best = key < best ? key : best;
  }
  return best != ~0ull ? (uint32_t)best : (uint32_t)h;
}

template <int PLOC_R>
__global__ void __launch_bounds__(PLOC_BLOCK) k_ploc_nn(const PlocBufs bufs, const uint32_t* __restrict__ ploc_state,
                                                        uint32_t* __restrict__ nn) {
  __shared__ float3 s_lo[PLOC_BLOCK + 2 * PLOC_R], s_hi[PLOC_BLOCK + 2 * PLOC_R];
  __shared__ uint32_t s_seg[PLOC_BLOCK + 2 * PLOC_R];
  if (ploc_state[kPlocDone]) return;
  const uint32_t n = ploc_state[kPlocN];
  const uint32_t par = ploc_state[kPlocParity] & 1u;
  for (uint32_t tile = blockIdx.x; tile * PLOC_BLOCK < n; tile += gridDim.x)
    ploc_nn_tile<PLOC_R>(bufs.clo[par], bufs.chi[par], n, tile, nn, s_lo, s_hi, s_seg);
}

// Survivor and merge counts of every tile of the round.
__global__ void __launch_bounds__(PLOC_BLOCK) k_ploc_count(const uint32_t* __restrict__ nn,
                                                           const uint32_t* __restrict__ ploc_state,
                                                           uint32_t* __restrict__ bsurv, uint32_t* __restrict__ bmerge) {
  if (ploc_state[kPlocDone]) return;
  const uint32_t n = ploc_state[kPlocN];
  for (uint32_t tile = blockIdx.x; tile * PLOC_BLOCK < n; tile += gridDim.x) {
    const uint32_t i = tile * PLOC_BLOCK + threadIdx.x;
    int surv = 0, merge = 0;
    if (i < n) {
      const uint32_t j = nn[i];
      const bool mutual = (j != i) && nn[j] == i;
      merge = mutual && i < j;
      surv = !(mutual && j < i);
    }
    const int cs = __syncthreads_count(surv);
    const int cm = __syncthreads_count(merge);
    if (threadIdx.x == 0) {
      bsurv[tile] = cs;
      bmerge[tile] = cm;
    }
  }
}

__device__ __forceinline__ uint32_t block_excl_scan_flag(int flag, uint32_t* s_warp) {
  // exclusive rank of this thread among flagged threads of the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t bal = __ballot_sync(0xFFFFFFFFu, flag);
  if (lane == 0) s_warp[warp] = __popc(bal);
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < warp; w++) pre += s_warp[w];
  __syncthreads();
  return pre + __popc(bal & ((1u << lane) - 1u));
}

// Survivors and merges of one tile: a cluster whose nearest neighbour is
// mutual merges with it (the lower index creates the node, the higher one is
// dropped), the others survive as they are; outputs go to position
// surv_off + rank among the tile's survivors, new nodes to node_next + merge_off
// + rank among its merges.  Each new node's collapse costs are computed here.
__device__ __forceinline__ void ploc_emit_tile(const PlocBufs& bufs, uint32_t par, const uint32_t* __restrict__ nn,
                                               uint32_t n, uint32_t node_next, uint32_t tile, uint32_t surv_off,
                                               uint32_t merge_off, float4* __restrict__ bnlo,
                                               float4* __restrict__ bnhi, uint32_t* __restrict__ bncnt,
                                               uint32_t node_cap, uint32_t* err, float4* __restrict__ dp_cost,
                                               uint2* __restrict__ dp_choice, uint32_t leaf_max, uint32_t* s_w) {
  const float4* __restrict__ clo = bufs.clo[par];
  const float4* __restrict__ chi = bufs.chi[par];
  const uint32_t* __restrict__ cidx = bufs.cidx[par];
  float4* __restrict__ olo = bufs.clo[par ^ 1u];
  float4* __restrict__ ohi = bufs.chi[par ^ 1u];
  uint32_t* __restrict__ oidx = bufs.cidx[par ^ 1u];
  const uint32_t i = tile * PLOC_BLOCK + threadIdx.x;
  int surv = 0, merge = 0;
  uint32_t j = 0;
  if (i < n) {
    j = nn[i];
    const bool mutual = (j != i) && nn[j] == i;
    merge = mutual && i < j;
    surv = !(mutual && j < i);
  }
  const uint32_t rs = block_excl_scan_flag(surv, s_w);
  const uint32_t rm = block_excl_scan_flag(merge, s_w);
  if (i >= n || !surv) return;
  const uint32_t pos = surv_off + rs;
  const float4 a = clo[i], b = chi[i];
  if (pos >= n) {
    atomicOr(err, kErrBuild);
    return;
  }
  if (merge) {
    const float4 c = clo[j], d = chi[j];
    const uint32_t id = node_next + merge_off + rm;
    if (id >= node_cap) {
      atomicOr(err, kErrBuild);
      return;
    }
    const uint32_t l = cidx[i], r = cidx[j];
    const float4 lo = make_float4(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z), a.w);
    const uint32_t cnt_l = __float_as_uint(b.w), cnt_r = __float_as_uint(d.w);
    const float4 hi = make_float4(fmaxf(b.x, d.x), fmaxf(b.y, d.y), fmaxf(b.z, d.z), __uint_as_float(cnt_l + cnt_r));
    bnlo[id] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(l));
    bnhi[id] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(r));
    bncnt[id] = cnt_l + cnt_r;
    if (dp_cost)
      dp_node(dp_cost, dp_choice, id, l, r, half_area(make_float3(lo.x, lo.y, lo.z), make_float3(hi.x, hi.y, hi.z)),
              cnt_l, cnt_r, cnt_l == 1 ? half_area(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)) : 0.f,
              cnt_r == 1 ? half_area(make_float3(c.x, c.y, c.z), make_float3(d.x, d.y, d.z)) : 0.f, leaf_max);
    olo[pos] = lo;
    ohi[pos] = hi;
    oidx[pos] = id;
  } else {
    olo[pos] = a;
    ohi[pos] = b;
    oidx[pos] = cidx[i];
  }
}

__global__ void __launch_bounds__(PLOC_BLOCK) k_ploc_emit(const PlocBufs bufs, const uint32_t* __restrict__ nn,
                                                          const uint32_t* __restrict__ ploc_state,
                                                          const uint32_t* __restrict__ bsurv_off,
                                                          const uint32_t* __restrict__ bmerge_off,
                                                          float4* __restrict__ bnlo, float4* __restrict__ bnhi,
                                                          uint32_t* __restrict__ bncnt, uint32_t node_cap, uint32_t* err,
                                                          float4* __restrict__ dp_cost, uint2* __restrict__ dp_choice,
                                                          uint32_t leaf_max) {
  __shared__ uint32_t s_w[PLOC_BLOCK / 32];
  if (ploc_state[kPlocDone]) return;
  const uint32_t n = ploc_state[kPlocN], node_next = ploc_state[kPlocNext];
  const uint32_t par = ploc_state[kPlocParity] & 1u;
  for (uint32_t tile = blockIdx.x; tile * PLOC_BLOCK < n; tile += gridDim.x)
    ploc_emit_tile(bufs, par, nn, n, node_next, tile, bsurv_off[tile], bmerge_off[tile], bnlo, bnhi, bncnt, node_cap,
                   err, dp_cost, dp_choice, leaf_max, s_w);
}

// After a round: the survivors are the new clusters, the merges took the next
// binary node indices; rounds end once n <= PLOC_SMALL or nothing merged.
__global__ void k_ploc_advance(const uint32_t* __restrict__ tot, uint32_t* __restrict__ ploc_state) {
  if (threadIdx.x != 0) return;
  if (!ploc_state[kPlocDone]) {
    const uint32_t n = tot[0], merged = tot[1];
    ploc_state[kPlocN] = n;
    ploc_state[kPlocNext] += merged;
    ploc_state[kPlocRounds] += merged > 0 ? 1u : 0u;
    ploc_state[kPlocTiles] = (n + PLOC_BLOCK - 1) / PLOC_BLOCK;
    ploc_state[kPlocParity] ^= 1u;
    if (n <= PLOC_SMALL || merged == 0) ploc_state[kPlocDone] = 1u;
  }
  ++ploc_state[kPlocIters];
}

// All PLOC rounds above PLOC_SMALL clusters in one cooperative launch (captured
// builds): per round (A) nearest neighbours of the CTA's contiguous run of
// tiles and of the PLOC_R clusters either side of it, (B) survivors and merges
// of each tile (mutual pairs decided from A alone), per-CTA sums, [barrier],
// (C) this CTA's offsets from the sums and its tiles' outputs, [barrier]: two
// grid barriers per round (with a third between A and B the 4M soup rebuilt
// in 2.50 ms, without it 2.46).  Each CTA keeps the round state (the k_ploc_advance
// rules) in registers; CTA 0 writes it back to ploc_state.  cta_sums holds
// 2 * gridDim.x words; *bar is zero on entry.
template <int PLOC_R>
__global__ void __launch_bounds__(PLOC_BLOCK) k_ploc_all(const PlocBufs bufs, uint32_t* __restrict__ ploc_state,
                                                         uint32_t* __restrict__ nn, uint32_t* __restrict__ tile_s,
                                                         uint32_t* __restrict__ tile_m, uint32_t* __restrict__ cta_sums,
                                                         float4* __restrict__ bnlo, float4* __restrict__ bnhi,
                                                         uint32_t* __restrict__ bncnt, uint32_t node_cap,
                                                         float4* __restrict__ dp_cost, uint2* __restrict__ dp_choice,
                                                         uint32_t leaf_max, GridBarrier* bar, unsigned int* err) {
  __shared__ float3 s_lo[PLOC_BLOCK + 2 * PLOC_R], s_hi[PLOC_BLOCK + 2 * PLOC_R];
  __shared__ uint32_t s_seg[PLOC_BLOCK + 2 * PLOC_R];
  __shared__ uint32_t s_w[PLOC_BLOCK / 32];
  __shared__ uint32_t s_red[4][PLOC_BLOCK / 32];
  __shared__ uint32_t s_halo_nn[2 * PLOC_R];  // nearest neighbours of the R clusters either side of the run
  uint32_t n = __ldcg(ploc_state + kPlocN), node_next = __ldcg(ploc_state + kPlocNext);
  uint32_t par = __ldcg(ploc_state + kPlocParity) & 1u, rounds = __ldcg(ploc_state + kPlocRounds);
  uint32_t iters = __ldcg(ploc_state + kPlocIters);
  bool done = __ldcg(ploc_state + kPlocDone) != 0u;
  while (!done && iters < kPlocMaxIters) {
    const uint32_t ntiles = (n + PLOC_BLOCK - 1) / PLOC_BLOCK;
    const uint32_t per = (ntiles + gridDim.x - 1) / gridDim.x;
    const uint32_t t0 = min(blockIdx.x * per, ntiles), t1 = min(t0 + per, ntiles);
    // (A) nearest neighbours of this CTA's run of tiles [r0, r1), and of the R
    // clusters either side of it (computed here as their own CTAs compute
    // them), so that (B) needs no grid barrier before it
    const int r0 = (int)(t0 * PLOC_BLOCK), r1 = (int)min(t1 * PLOC_BLOCK, n);
    for (uint32_t tile = t0; tile < t1; tile++)
      ploc_nn_tile<PLOC_R>(bufs.clo[par], bufs.chi[par], n, tile, nn, s_lo, s_hi, s_seg);
    if (threadIdx.x < 2 * PLOC_R && t0 < t1) {
      const int h = threadIdx.x < PLOC_R ? r0 - PLOC_R + (int)threadIdx.x : r1 + (int)threadIdx.x - PLOC_R;
      if (h >= 0 && h < (int)n) s_halo_nn[threadIdx.x] = ploc_nn_one<PLOC_R>(bufs.clo[par], bufs.chi[par], n, h);
    }
    __syncthreads();
    // (B) survivors and merges per tile (the run's nn written above by this CTA)
    auto nn_of = [&](uint32_t j) -> uint32_t {
      if ((int)j < r0) return s_halo_nn[(int)j - (r0 - PLOC_R)];
      if ((int)j >= r1) return s_halo_nn[PLOC_R + (int)j - r1];
      return nn[j];
    };
    uint32_t cs_sum = 0, cm_sum = 0;
    for (uint32_t tile = t0; tile < t1; tile++) {
      const uint32_t i = tile * PLOC_BLOCK + threadIdx.x;
      int surv = 0, merge = 0;
      if (i < n) {
        const uint32_t j = nn[i];
        const bool mutual = (j != i) && nn_of(j) == i;
        merge = mutual && i < j;
        surv = !(mutual && j < i);
      }
      const uint32_t cs = (uint32_t)__syncthreads_count(surv);
      const uint32_t cm = (uint32_t)__syncthreads_count(merge);
      if (threadIdx.x == 0) {
        tile_s[tile] = cs;
        tile_m[tile] = cm;
      }
      cs_sum += cs;
      cm_sum += cm;
    }
    if (threadIdx.x == 0) {
      __stcg(cta_sums + blockIdx.x, cs_sum);
      __stcg(cta_sums + gridDim.x + blockIdx.x, cm_sum);
    }
    if (!grid_sync(bar, err)) break;
    // (C) this CTA's offsets and the round's totals, then its tiles' outputs
    uint32_t v[4] = {0u, 0u, 0u, 0u};  // prefix survivors, prefix merges, total survivors, total merges
    for (uint32_t c = threadIdx.x; c < gridDim.x; c += blockDim.x) {
      const uint32_t a = __ldcg(cta_sums + c), b = __ldcg(cta_sums + gridDim.x + c);
      v[2] += a;
      v[3] += b;
      if (c < blockIdx.x) {
        v[0] += a;
        v[1] += b;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      v[q] = __reduce_add_sync(0xFFFFFFFFu, v[q]);
      if ((threadIdx.x & 31) == 0) s_red[q][threadIdx.x >> 5] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint32_t t = 0;
      for (int w = 0; w < PLOC_BLOCK / 32; w++) t += s_red[q][w];
      v[q] = t;
    }
    __syncthreads();  // s_red is reused next round
    uint32_t ps = v[0], pm = v[1];
    for (uint32_t tile = t0; tile < t1; tile++) {
      ploc_emit_tile(bufs, par, nn, n, node_next, tile, ps, pm, bnlo, bnhi, bncnt, node_cap, err, dp_cost, dp_choice,
                     leaf_max, s_w);
      ps += tile_s[tile];
      pm += tile_m[tile];
    }
    // next round (the k_ploc_advance rules, alike in every CTA)
    const uint32_t merged = v[3];
    n = v[2];
    node_next += merged;
    rounds += merged > 0 ? 1u : 0u;
    par ^= 1u;
    iters++;
    if (n <= PLOC_SMALL || merged == 0) done = true;
    if (!grid_sync(bar, err)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ploc_state[kPlocN] = n;
    ploc_state[kPlocNext] = node_next;
    ploc_state[kPlocRounds] = rounds;
    ploc_state[kPlocTiles] = (n + PLOC_BLOCK - 1) / PLOC_BLOCK;
    ploc_state[kPlocParity] = par;
    ploc_state[kPlocDone] = done ? 1u : 0u;
    ploc_state[kPlocIters] = iters;
  }
}

// Finishes clustering of the n <= PLOC_SMALL clusters left by the rounds
// inside one CTA (n and the next node index from ploc_state, where the final
// node count is written back).
__global__ void __launch_bounds__(PLOC_SMALL_THREADS) k_ploc_small(const float4* __restrict__ clo_a,
                                                                  const float4* __restrict__ chi_a,
                                                                  const uint32_t* __restrict__ cidx_a,
                                                                  const float4* __restrict__ clo_b,
                                                                  const float4* __restrict__ chi_b,
                                                                  const uint32_t* __restrict__ cidx_b,
                                                                  uint32_t* __restrict__ ploc_state,
                                                                  float4* __restrict__ bnlo,
                                                                  float4* __restrict__ bnhi,
                                                                  uint32_t* __restrict__ bncnt, uint32_t* root_out,
                                                                  uint32_t* iters_out, uint32_t node_cap,
                                                                  uint32_t* err, uint32_t nseg, int radius,
                                                                  float4* __restrict__ dp_cost,
                                                                  uint2* __restrict__ dp_choice, uint32_t leaf_max) {
  extern __shared__ unsigned char smem[];
  float3* s_lo = reinterpret_cast<float3*>(smem);
  float3* s_hi = s_lo + PLOC_SMALL;
  uint32_t* s_idx = reinterpret_cast<uint32_t*>(s_hi + PLOC_SMALL);
  uint32_t* s_nn = s_idx + PLOC_SMALL;
  uint32_t* s_seg = s_nn + PLOC_SMALL;
  uint32_t* s_cnt = s_seg + PLOC_SMALL;
  __shared__ uint32_t s_w[32];
  __shared__ uint32_t s_tot[2];
  constexpr int EPT = PLOC_SMALL / PLOC_SMALL_THREADS;  // elements per thread (contiguous)
  const uint32_t n0 = ploc_state[kPlocN], node_next0 = ploc_state[kPlocNext];
  const bool in_b = ploc_state[kPlocParity] != 0;
  const float4* __restrict__ clo = in_b ? clo_b : clo_a;
  const float4* __restrict__ chi = in_b ? chi_b : chi_a;
  const uint32_t* __restrict__ cidx = in_b ? cidx_b : cidx_a;
  if (n0 > PLOC_SMALL) {  // the rounds did not get below the threshold (too few enqueued)
    if (threadIdx.x == 0) atomicOr(err, kErrBuild);
    return;
  }
  for (uint32_t k = threadIdx.x; k < n0; k += blockDim.x) {
    const float4 a = clo[k], b = chi[k];
    s_lo[k] = make_float3(a.x, a.y, a.z);
    s_hi[k] = make_float3(b.x, b.y, b.z);
    s_idx[k] = cidx[k];
    s_seg[k] = __float_as_uint(a.w);
    s_cnt[k] = __float_as_uint(b.w);
  }
  uint32_t n = n0, node_next = node_next0, iters = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // every round merges at least the closest pair of each segment that still
  // has two clusters, so n0 - 1 rounds always suffice; the bound only guards
  // against a logic error.  A round without merges ends the clustering.
  while (n > 1) {
    if (iters >= PLOC_SMALL) {
      if (threadIdx.x == 0) atomicOr(err, kErrBuild);
      break;
    }
    iters++;
    // nearest neighbours
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const float3 lo = s_lo[i], hi = s_hi[i];
      const uint32_t seg = s_seg[i];
      unsigned long long best = ~0ull;
      for (int o = -radius; o <= radius; o++) {
        const int j = (int)i + o;
        if (o == 0 || j < 0 || j >= (int)n || s_seg[j] != seg) continue;
        const float a = half_area(f3min(lo, s_lo[j]), f3max(hi, s_hi[j]));
        const unsigned long long key = ((unsigned long long)__float_as_uint(a) << 32) | (uint32_t)j;
        best = key < best ? key : best;
      }
      s_nn[i] = best != ~0ull ? (uint32_t)best : i;
    }
    __syncthreads();
    // flags for this thread's contiguous chunk
    uint32_t cs = 0, cm = 0;
    int fs[EPT], fm[EPT];
    const uint32_t i0 = threadIdx.x * EPT;
#pragma unroll
    for (int e = 0; e < EPT; e++) {
      const uint32_t i = i0 + e;
      fs[e] = fm[e] = 0;
      if (i < n) {
        const uint32_t j = s_nn[i];
        const bool mutual = j != i && s_nn[j] == i;
        fm[e] = mutual && i < j;
        fs[e] = !(mutual && j < i);
      }
      cs += fs[e];
      cm += fm[e];
    }
    // block exclusive scan of (cs, cm) packed into one 32-bit word (both < 2^16)
    uint32_t x = cs | (cm << 16);
    const uint32_t mine = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = s_w[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      s_w[lane] = w;
      if (lane == 31) { s_tot[0] = w & 0xFFFFu; s_tot[1] = w >> 16; }
    }
    __syncthreads();
    const uint32_t excl = (warp ? s_w[warp - 1] : 0u) + (x - mine);
    uint32_t ps = excl & 0xFFFFu, pm = excl >> 16;
    // gather outputs into registers
    float3 olo[EPT], ohi[EPT];
    uint32_t oidx[EPT], opos[EPT], oseg[EPT], ocnt[EPT];
#pragma unroll
    for (int e = 0; e < EPT; e++) {
      const uint32_t i = i0 + e;
      opos[e] = 0xFFFFFFFFu;
      if (i < n && fs[e]) {
        float3 lo = s_lo[i], hi = s_hi[i];
        uint32_t id = s_idx[i], cnt = s_cnt[i];
        if (fm[e]) {
          const uint32_t j = s_nn[i];
          const uint32_t nid = node_next + pm;
          const uint32_t l = id, r = s_idx[j];
          if (nid >= node_cap) {
            atomicOr(err, kErrBuild);
            break;
          }
          const uint32_t cnt_l = cnt, cnt_r = s_cnt[j];
          const float Al = cnt_l == 1 ? half_area(lo, hi) : 0.f;
          const float Ar = cnt_r == 1 ? half_area(s_lo[j], s_hi[j]) : 0.f;
          lo = f3min(lo, s_lo[j]);
          hi = f3max(hi, s_hi[j]);
          bnlo[nid] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(l));
          bnhi[nid] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(r));
          cnt = cnt_l + cnt_r;
          bncnt[nid] = cnt;
          // children come from earlier rounds: their costs were stored before
          // this round's barriers
          if (dp_cost) dp_node(dp_cost, dp_choice, nid, l, r, half_area(lo, hi), cnt_l, cnt_r, Al, Ar, leaf_max);
          id = nid;
          pm++;
        }
        olo[e] = lo;
        ohi[e] = hi;
        oidx[e] = id;
        oseg[e] = s_seg[i];
        ocnt[e] = cnt;
        opos[e] = ps++;
      }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < EPT; e++) {
      if (opos[e] != 0xFFFFFFFFu) {
        s_lo[opos[e]] = olo[e];
        s_hi[opos[e]] = ohi[e];
        s_idx[opos[e]] = oidx[e];
        s_seg[opos[e]] = oseg[e];
        s_cnt[opos[e]] = ocnt[e];
      }
    }
    const uint32_t merged = s_tot[1];
    node_next += merged;
    n = s_tot[0];
    __syncthreads();
    if (merged == 0) break;
  }
  // one root per segment (nseg == 1: the single tree's root)
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
    const uint32_t seg = nseg > 1 ? s_seg[k] : 0u;
    if (seg < nseg) root_out[seg] = s_idx[k];
  }
  if (threadIdx.x == 0) {
    *iters_out += iters;
    ploc_state[kPlocNext] = node_next;  // binary nodes in use: [0, node_next)
  }
}

// ---------------------------------------------------------------------------
// 5. collapse to 8-wide quantised nodes
// ---------------------------------------------------------------------------

// Adds the per-thread values a, b to acc[0], acc[1] with one atomic each per
// CTA; every thread of the CTA calls it (blockDim.x a multiple of 32).
__device__ __forceinline__ void block_add2(double a, double b, double* acc) {
  __shared__ double s_a[32], s_b[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xFFFFFFFFu, a, o);
    b += __shfl_down_sync(0xFFFFFFFFu, b, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s_a[warp] = a;
    s_b[warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < nw; w++) {
      ta += s_a[w];
      tb += s_b[w];
    }
    if (ta != 0.0) atomicAdd(acc + 0, ta);
    if (tb != 0.0) atomicAdd(acc + 1, tb);
  }
}

struct BinTree {
  const float4* lo;
  const float4* hi;
  const uint32_t* cnt;
  uint32_t nleaves;
  uint32_t leaf_max;  // subtrees of at most this many triangles may become leaves
  uint32_t robust;    // write raw vertices into triangle records
  const uint2* choice;  // SAH-optimal collapse decisions (k_collapse_dp); null: greedy collapse
};

__device__ __forceinline__ bool bt_leaf(const BinTree& t, uint32_t k) { return k < t.nleaves; }
// Triangles of binary node k as the collapse needs them: with one-triangle
// leaves only "one (a primitive) or more" matters, so no count is read (2
// stands for any internal node).
__device__ __forceinline__ uint32_t bt_cnt(const BinTree& t, uint32_t k) {
  if (t.leaf_max == 1) return bt_leaf(t, k) ? 1u : 2u;
  return t.cnt[k];
}
__device__ __forceinline__ uint32_t bt_left(const BinTree& t, uint32_t k) { return __float_as_uint(t.lo[k].w); }
__device__ __forceinline__ uint32_t bt_right(const BinTree& t, uint32_t k) { return __float_as_uint(t.hi[k].w); }
__device__ __forceinline__ float3 bt_lo(const BinTree& t, uint32_t k) {
  const float4 a = t.lo[k];
  return make_float3(a.x, a.y, a.z);
}
__device__ __forceinline__ float3 bt_hi(const BinTree& t, uint32_t k) {
  const float4 a = t.hi[k];
  return make_float3(a.x, a.y, a.z);
}


__device__ __forceinline__ uint32_t dp_choice(const BinTree& t, uint32_t n, int i) {
  const uint2 c = t.choice[n];
  const uint32_t w = i - 1 < 4 ? c.x : c.y;
  return (w >> (8 * ((i - 1) & 3))) & 0xFFu;
}

// Children of the wide node made from binary node b by the recorded DP splits.
__device__ int gather_children_dp(const BinTree& t, uint32_t b, uint32_t kids[8]) {
  uint32_t sn[8];
  int si[8];
  int sp = 0, nk = 0;
  const uint32_t k8 = dp_choice(t, b, 1);  // byte 0: split of D(b, 8)
  sn[sp] = bt_left(t, b);
  si[sp++] = (int)k8;
  sn[sp] = bt_right(t, b);
  si[sp++] = 8 - (int)k8;
  while (sp > 0) {
    const uint32_t n = sn[--sp];
    int i = si[sp];
    while (i > 1 && (bt_leaf(t, n) || dp_choice(t, n, i) == 0)) i--;
    // the slots of the pending entries and the emitted children sum to at most
    // 8, so a split always fits; the capacity test only guards the stack
    if (i <= 1 || nk + sp + 2 > 8) {
      if (nk < 8) kids[nk++] = n;
      continue;
    }
    const int k = (int)dp_choice(t, n, i);
    sn[sp] = bt_left(t, n);
    si[sp++] = k;
    sn[sp] = bt_right(t, n);
    si[sp++] = i - k;
  }
  return nk;
}

// Chooses up to 8 children for the wide node that replaces binary node b.
__device__ int gather_children(const BinTree& t, uint32_t b, uint32_t kids[8]) {
  if (bt_leaf(t, b)) {
    kids[0] = b;
    return 1;
  }
  if (t.choice) return gather_children_dp(t, b, kids);
  kids[0] = bt_left(t, b);
  kids[1] = bt_right(t, b);
  int nk = 2;
  while (nk < 8) {
    int best = -1;
    bool bestMand = false;
    float bestA = -1.0f;
    for (int i = 0; i < nk; i++) {
      const uint32_t c = kids[i];
      if (bt_leaf(t, c)) continue;
      const bool mand = t.cnt[c] > t.leaf_max;
      const float A = half_area(bt_lo(t, c), bt_hi(t, c));
      if (!mand) {
        // opening a small subtree pays off only if its children's boxes
        // cover less area than its own box
        const uint32_t l = bt_left(t, c), r = bt_right(t, c);
        const float Al = half_area(bt_lo(t, l), bt_hi(t, l)), Ar = half_area(bt_lo(t, r), bt_hi(t, r));
        if (!(Al + Ar < A)) continue;
      }
      if ((mand && !bestMand) || (mand == bestMand && A > bestA)) {
        best = i;
        bestMand = mand;
        bestA = A;
      }
    }
    if (best < 0) break;
    const uint32_t c = kids[best];
    kids[best] = bt_left(t, c);
    kids[nk++] = bt_right(t, c);
  }
  return nk;
}

// The collapse runs level by level from a state in device memory, so levels
// can be enqueued (or captured) before their sizes are known: [kColN] items of
// the current level, [kColBase] its first wide node, [kColTri] its first
// triangle record, [kColDepth] levels done, [kColErr] overflow, and from
// [kColLevels] the first node of every level (plus the end).  Kernels loop
// grid-stride over the level's items; a level with no items is a no-op.
enum : int { kColN = 0, kColBase = 1, kColTri = 2, kColDepth = 3, kColErr = 4, kColLevels = 8, kColMaxLevels = 64,
             kColStateWords = kColLevels + kColMaxLevels + 1 };

// Exclusive scan of one value per thread over a CTA of 1024 threads.
__device__ __forceinline__ uint32_t cta_excl_scan_1024(uint32_t v, uint32_t* s_w, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_w[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    s_w[lane] = w;
  }
  __syncthreads();
  const uint32_t excl = (warp ? s_w[warp - 1] : 0u) + x - v;
  total = s_w[31];
  __syncthreads();
  return excl;
}

// First level: the roots of the non-empty segments in segment order (one CTA
// of 1024 threads, nseg <= 4 x 1024); seg_index[s] = position of segment s's
// root (kInvalidID for an empty segment).
__global__ void __launch_bounds__(1024) k_collapse_roots(const uint32_t* __restrict__ d_root, uint32_t nseg,
                                                         uint32_t nbin, uint32_t* __restrict__ items,
                                                         uint32_t* __restrict__ seg_index,
                                                         uint32_t* __restrict__ cstate) {
  __shared__ uint32_t s_w[32];
  uint32_t r[4], cnt = 0;
  const uint32_t s0 = threadIdx.x * 4;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    r[q] = s0 + q < nseg ? d_root[s0 + q] : kInvalidID;
    if (r[q] != kInvalidID && r[q] >= nbin) r[q] = kInvalidID, cstate[kColErr] = 1u;
    cnt += r[q] != kInvalidID;
  }
  uint32_t total = 0;
  uint32_t pos = cta_excl_scan_1024(cnt, s_w, total);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (s0 + q >= nseg) break;
    if (r[q] != kInvalidID) items[pos] = r[q];
    seg_index[s0 + q] = r[q] != kInvalidID ? pos++ : kInvalidID;
  }
  if (threadIdx.x == 0) {
    cstate[kColN] = total;
    cstate[kColBase] = 0;
    cstate[kColTri] = 0;
    cstate[kColDepth] = 0;
  }
}

// leaf_root entry of a one-triangle leaf: the primitive index with this bit set
// (primitive indices and binary node ids are below 2^31)
constexpr uint32_t kLeafPrim = 0x80000000u;

// The two item buffers of the collapse levels: level d reads items[d & 1] and writes
// items[(d & 1) ^ 1] (d = cstate[kColDepth]), so every level runs the same kernels
// with the same arguments.
struct ColItems {
  uint32_t* items[2];
};

__global__ void __launch_bounds__(128) k_collapse_count(BinTree t, const ColItems ci,
                                                        const uint32_t* __restrict__ cstate,
                                                        uint32_t* __restrict__ kids_out, uint32_t* __restrict__ nint,
                                                        uint32_t* __restrict__ ntri) {
  const uint32_t nitems = cstate[kColN];
  const uint32_t* __restrict__ items = ci.items[cstate[kColDepth] & 1u];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nitems; k += gridDim.x * blockDim.x) {
    uint32_t kids[8];
    const int nk = gather_children(t, items[k], kids);
    uint32_t ni = 0, nt = 0;
    for (int i = 0; i < 8; i++) {
      if (i < nk) {
        const uint32_t c = kids[i];
        const uint32_t cnt = bt_cnt(t, c);
        if (cnt > t.leaf_max) ni++; else nt += cnt;
        kids_out[8 * (size_t)k + i] = c;
      } else {
        kids_out[8 * (size_t)k + i] = 0xFFFFFFFFu;
      }
    }
    nint[k] = ni;
    ntri[k] = nt;
  }
}

// After a level: its wide nodes are written; the next level's items are its
// internal children (tot[0]), their triangles follow (tot[1]).  Level starts
// are kept for the first kColMaxLevels levels; max_levels bounds the depth of
// builds that need them all on the device (the host-driven build records
// them itself and has no bound: a chain-like binary tree, e.g. thousands of
// identical triangles, collapses into thousands of levels).
__global__ void k_collapse_advance(const uint32_t* __restrict__ tot, uint32_t* __restrict__ cstate, uint32_t node_cap,
                                   uint32_t max_levels) {
  if (threadIdx.x != 0) return;
  const uint32_t n = cstate[kColN];
  if (n == 0) {
    return;
  }
  const uint32_t d = cstate[kColDepth];
  if (d < (uint32_t)kColMaxLevels) cstate[kColLevels + d] = cstate[kColBase];
  const uint32_t base = cstate[kColBase] + n;
  cstate[kColBase] = base;
  cstate[kColTri] += tot[1];
  cstate[kColDepth] = d + 1;
  uint32_t next = tot[0];
  if ((next > 0 && d + 1 >= max_levels) || base + next > node_cap) {
    cstate[kColErr] = 1u;
    next = 0;
  }
  cstate[kColN] = next;
  if (next == 0 && d + 1 <= (uint32_t)kColMaxLevels) cstate[kColLevels + d + 1] = base;  // end of the last level
}

__device__ __forceinline__ uint32_t exp_for(float ext) {
  // smallest power of two 2^(E-127) with 255 * 2^(E-127) >= ext
  const float x = __fdiv_ru(ext, 255.0f);
  const uint32_t bits = __float_as_uint(x);
  uint32_t E = (bits >> 23) & 0xFFu;
  if (bits & 0x7FFFFFu) E += 1;
  if (E < 1) E = 1;
  if (E > 253) E = 253;
  return E;
}

__device__ __forceinline__ void write_tri(const GeomDesc* __restrict__ geoms, const float4* __restrict__ plo,
                                          const float4* __restrict__ phi, uint32_t prim, TriRecord* dst, bool robust) {
  const uint32_t gs = __float_as_uint(plo[prim].w);
  const uint32_t j = __float_as_uint(phi[prim].w);
  const GeomDesc g = geoms[gs];
  if (g.kind == 1) {  // instance leaf
    const InstBox bx = reinterpret_cast<const InstBox*>(g.verts)[j];
    dst->a = make_float4(0.f, 0.f, 0.f, __uint_as_float(bx.inst));
    dst->b = make_float4(0.f, 0.f, 0.f, __uint_as_float(bx.geomID));
    dst->c = make_float4(0.f, 0.f, 0.f, __uint_as_float(kInstanceLeaf));
    return;
  }
  const uint3 t = load_tri(g, j);
  const float3 p0 = load_vtx(g, t.x), p1 = load_vtx(g, t.y), p2 = load_vtx(g, t.z);
  // Triangle4: e1 = v0 - v1, e2 = v2 - v0 (triangle.h:40-41); Triangle4v of
  // robust scenes keeps v1 and v2 themselves (trianglev.h:93-115)
  const float3 e1 = robust ? p1 : make_float3(__fsub_rn(p0.x, p1.x), __fsub_rn(p0.y, p1.y), __fsub_rn(p0.z, p1.z));
  const float3 e2 = robust ? p2 : make_float3(__fsub_rn(p2.x, p0.x), __fsub_rn(p2.y, p0.y), __fsub_rn(p2.z, p0.z));
  dst->a = make_float4(p0.x, p0.y, p0.z, __uint_as_float(j));
  dst->b = make_float4(e1.x, e1.y, e1.z, __uint_as_float(g.geomID));
  dst->c = make_float4(e2.x, e2.y, e2.z, 0.f);
}

// Writes wide node k of the level and the triangle records of its leaves;
// adds the node's SAH terms and leaf count to sah_out / nleaf_out.

// The wide node of item k by one thread: wide levels (more items than there
// are lane groups to share them) are throughput-bound, and this form does the
// least work per node; collapse_emit_group gives the same node.
__device__ __forceinline__ void collapse_emit_node(
    const BinTree& t, const uint32_t* __restrict__ kids_in, uint32_t k, const uint32_t* __restrict__ off_int,
    const uint32_t* __restrict__ off_tri, uint32_t level_base, uint32_t next_base, uint32_t tri_next,
    WideNode* __restrict__ nodes, uint32_t* __restrict__ leaf_root, uint32_t* __restrict__ next_items,
    uint32_t node_cap, uint32_t tri_cap, uint32_t* err, double& sah_out, double& sahx_out, uint32_t& nleaf_out) {
  // all loops over the 8 children are unrolled, so the per-child values stay
  // in registers (no local-memory arrays)
  uint32_t kids[8];
  int nk = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    kids[i] = kids_in[8 * (size_t)k + i];
    if (kids[i] != 0xFFFFFFFFu) nk = i + 1;
  }
  // union box and quantisation frame
  float3 klo[8], khi[8];
  float3 ulo = make_float3(INFINITY, INFINITY, INFINITY), uhi = make_float3(-INFINITY, -INFINITY, -INFINITY);
#pragma unroll
  for (int i = 0; i < 8; i++) {
    klo[i] = khi[i] = make_float3(0.f, 0.f, 0.f);
    if (i < nk) {
      klo[i] = bt_lo(t, kids[i]);
      khi[i] = bt_hi(t, kids[i]);
      ulo = f3min(ulo, klo[i]);
      uhi = f3max(uhi, khi[i]);
    }
  }
  const uint32_t Ex = exp_for(__fsub_ru(uhi.x, ulo.x));
  const uint32_t Ey = exp_for(__fsub_ru(uhi.y, ulo.y));
  const uint32_t Ez = exp_for(__fsub_ru(uhi.z, ulo.z));
  const float sx = __uint_as_float(Ex << 23), sy = __uint_as_float(Ey << 23), sz = __uint_as_float(Ez << 23);
  const float ix = __uint_as_float((254u - Ex) << 23), iy = __uint_as_float((254u - Ey) << 23),
              iz = __uint_as_float((254u - Ez) << 23);
  // slot assignment: slot s prefers children far along the octant direction
  // with sign bits s (bit set = negative axis), so that visiting slots in
  // ascending order of (slot ^ ray octant) is roughly near-to-far.
  const float3 pc = make_float3((ulo.x + uhi.x) * 0.5f, (ulo.y + uhi.y) * 0.5f, (ulo.z + uhi.z) * 0.5f);
  float dx[8], dy[8], dz[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    dx[i] = (klo[i].x + khi[i].x) * 0.5f - pc.x;
    dy[i] = (klo[i].y + khi[i].y) * 0.5f - pc.y;
    dz[i] = (klo[i].z + khi[i].z) * 0.5f - pc.z;
  }
  // greedy: repeatedly the cheapest (child, free slot) pair, cost = the child's
  // offset from the node centre along the slot's octant direction
  uint32_t used = 0, assigned = 0;
  uint32_t kid_at = 0xFFFFFFFFu;  // 4 bits per slot: child index, 0xF = empty
  for (int it = 0; it < nk; it++) {
    float bc = INFINITY;
    int bi = -1, bs = -1;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      if (i >= nk || (assigned >> i & 1)) continue;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        if (used >> s & 1) continue;
        const float c = ((s & 1) ? -dx[i] : dx[i]) + ((s & 2) ? -dy[i] : dy[i]) + ((s & 4) ? -dz[i] : dz[i]);
        if (bi < 0 || c < bc) { bc = c; bi = i; bs = s; }
      }
    }
    assigned |= 1u << bi;
    used |= 1u << bs;
    kid_at = (kid_at & ~(0xFu << (4 * bs))) | ((uint32_t)bi << (4 * bs));
  }

  WideNode node;
  node.px = ulo.x;
  node.py = ulo.y;
  node.pz = ulo.z;
  node.ex = (uint8_t)Ex;
  node.ey = (uint8_t)Ey;
  node.ez = (uint8_t)Ez;
  node.imask = 0;
  node.child_base = next_base + off_int[k];
  node.tri_base = tri_next + off_tri[k];
  uint32_t int_rank = 0, tri_off = 0;
  double sah = 0.0, sahx = 0.0;  // on the decoded (quantised) and on the exact boxes
  uint32_t nleaf = 0;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const uint32_t i = (kid_at >> (4 * s)) & 0xFu;
    if (i == 0xFu) {
      node.meta[s] = 0;
      node.qlo_x[s] = node.qlo_y[s] = node.qlo_z[s] = 255;
      node.qhi_x[s] = node.qhi_y[s] = node.qhi_z[s] = 0;
      continue;
    }
    uint32_t c = 0;
    float3 a = make_float3(0.f, 0.f, 0.f), b = a;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if ((uint32_t)j == i) {
        c = kids[j];
        a = klo[j];
        b = khi[j];
      }
    }
    const float qlx = fminf(fmaxf(floorf(__fsub_rd(a.x, ulo.x) * ix), 0.f), 255.f);
    const float qly = fminf(fmaxf(floorf(__fsub_rd(a.y, ulo.y) * iy), 0.f), 255.f);
    const float qlz = fminf(fmaxf(floorf(__fsub_rd(a.z, ulo.z) * iz), 0.f), 255.f);
    const float qhx = fminf(fmaxf(ceilf(__fsub_ru(b.x, ulo.x) * ix), 0.f), 255.f);
    const float qhy = fminf(fmaxf(ceilf(__fsub_ru(b.y, ulo.y) * iy), 0.f), 255.f);
    const float qhz = fminf(fmaxf(ceilf(__fsub_ru(b.z, ulo.z) * iz), 0.f), 255.f);
    node.qlo_x[s] = (uint8_t)qlx; node.qlo_y[s] = (uint8_t)qly; node.qlo_z[s] = (uint8_t)qlz;
    node.qhi_x[s] = (uint8_t)qhx; node.qhi_y[s] = (uint8_t)qhy; node.qhi_z[s] = (uint8_t)qhz;
    // decoded (outward-rounded) box, as traversal sees it
    const float3 dlo = make_float3(__fmaf_rd(qlx, sx, ulo.x), __fmaf_rd(qly, sy, ulo.y), __fmaf_rd(qlz, sz, ulo.z));
    const float3 dhi = make_float3(__fmaf_ru(qhx, sx, ulo.x), __fmaf_ru(qhy, sy, ulo.y), __fmaf_ru(qhz, sz, ulo.z));
    const double A = (double)fmaxf(0.f, half_area(dlo, dhi));
    const double Ax = (double)fmaxf(0.f, half_area(a, b));
    const uint32_t cnt = bt_cnt(t, c);
    if (cnt > t.leaf_max) {
      node.meta[s] = (uint8_t)(0x80u | (uint32_t)s);
      node.imask |= (uint8_t)(1u << s);
      if (off_int[k] + int_rank >= node_cap || node.child_base + int_rank >= node_cap) {
        atomicOr(err, kErrBuild);
        return;
      }
      next_items[off_int[k] + int_rank] = c;
      int_rank++;
      sah += A;  // inner node term
      sahx += Ax;
    } else {
      node.meta[s] = (uint8_t)(0x80u | ((cnt - 1u) << 5) | tri_off);
      // the leaf's triangle records are written after the last level by
      // k_write_leaves, one thread per leaf: here only its binary subtree is
      // recorded at the slot of its first triangle
      if (node.tri_base + tri_off + cnt > tri_cap) {
        atomicOr(err, kErrBuild);
        return;
      }
      leaf_root[node.tri_base + tri_off] = cnt == 1 ? bt_right(t, c) | kLeafPrim : c;
      tri_off += cnt;
      sah += A * (double)((cnt + 3) / 4);  // leaf term: area x Triangle4 blocks
      sahx += Ax * (double)((cnt + 3) / 4);
      nleaf++;
    }
  }
  if (level_base + k >= node_cap) {
    atomicOr(err, kErrBuild);
    return;
  }
  nodes[level_base + k] = node;
  sah_out = sah;
  sahx_out = sahx;
  nleaf_out = nleaf;
}

// The wide node of item k, built by the 8 lanes of a lane group (lane & 7 is
// the child index; all 8 lanes call it with the same k; gmask names them).
// Children are placed in slots greedily, the cheapest (child, free slot) pair
// first with ties to the lower child and then the lower slot, the cost being
// the child's offset from the node centre along the slot's octant direction
// (slot s prefers children far along the direction with sign bits s), so that
// visiting slots in ascending order of (slot ^ ray octant) is roughly
// near-to-far.  Planes are quantised outward, internal children are numbered
// and leaf triangles laid out in slot order.
__device__ __forceinline__ void collapse_emit_group(
    const BinTree& t, const uint32_t* __restrict__ kids_in, uint32_t k, const uint32_t* __restrict__ off_int,
    const uint32_t* __restrict__ off_tri, uint32_t level_base, uint32_t next_base, uint32_t tri_next,
    WideNode* __restrict__ nodes, uint32_t* __restrict__ leaf_root, uint32_t* __restrict__ next_items,
    uint32_t node_cap, uint32_t tri_cap, uint32_t* err, uint32_t gmask, double& sah_out, double& sahx_out,
    uint32_t& nleaf_out) {
  const uint32_t i = threadIdx.x & 7u;
  const uint32_t kid = kids_in[8 * (size_t)k + i];
  const bool valid = kid != 0xFFFFFFFFu;
  const uint32_t vmask = __ballot_sync(gmask, valid) >> (threadIdx.x & 24u) & 0xFFu;
  const int nk = __popc(vmask);
  float3 lo = make_float3(0.f, 0.f, 0.f), hi = lo;
  if (valid) {
    lo = bt_lo(t, kid);
    hi = bt_hi(t, kid);
  }
  // union box and quantisation frame
  float3 ulo = valid ? lo : make_float3(INFINITY, INFINITY, INFINITY);
  float3 uhi = valid ? hi : make_float3(-INFINITY, -INFINITY, -INFINITY);
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    ulo.x = fminf(ulo.x, __shfl_xor_sync(gmask, ulo.x, o, 8));
    ulo.y = fminf(ulo.y, __shfl_xor_sync(gmask, ulo.y, o, 8));
    ulo.z = fminf(ulo.z, __shfl_xor_sync(gmask, ulo.z, o, 8));
    uhi.x = fmaxf(uhi.x, __shfl_xor_sync(gmask, uhi.x, o, 8));
    uhi.y = fmaxf(uhi.y, __shfl_xor_sync(gmask, uhi.y, o, 8));
    uhi.z = fmaxf(uhi.z, __shfl_xor_sync(gmask, uhi.z, o, 8));
  }
  const uint32_t Ex = exp_for(__fsub_ru(uhi.x, ulo.x));
  const uint32_t Ey = exp_for(__fsub_ru(uhi.y, ulo.y));
  const uint32_t Ez = exp_for(__fsub_ru(uhi.z, ulo.z));
  const float sx = __uint_as_float(Ex << 23), sy = __uint_as_float(Ey << 23), sz = __uint_as_float(Ez << 23);
  const float ix = __uint_as_float((254u - Ex) << 23), iy = __uint_as_float((254u - Ey) << 23),
              iz = __uint_as_float((254u - Ez) << 23);
  // slot costs of this lane's child
  const float3 pc = make_float3((ulo.x + uhi.x) * 0.5f, (ulo.y + uhi.y) * 0.5f, (ulo.z + uhi.z) * 0.5f);
  const float dx = (lo.x + hi.x) * 0.5f - pc.x, dy = (lo.y + hi.y) * 0.5f - pc.y, dz = (lo.z + hi.z) * 0.5f - pc.z;
  float cs[8];
#pragma unroll
  for (int s = 0; s < 8; s++) cs[s] = ((s & 1) ? -dx : dx) + ((s & 2) ? -dy : dy) + ((s & 4) ? -dz : dz);
  // greedy assignment: per round every unplaced child offers its cheapest free
  // slot; the group takes the least (cost, child, slot)
  uint32_t used = 0;
  int my_slot = -1;
  for (int it = 0; it < nk; it++) {
    unsigned long long key = ~0ull;
    if (valid && my_slot < 0) {
      float bc = INFINITY;
      int bs = -1;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        if (used >> s & 1u) continue;
        if (bs < 0 || cs[s] < bc) {
          bc = cs[s];
          bs = s;
        }
      }
      key = ((unsigned long long)f2ord(bc + 0.0f) << 32) | (i << 3) | (uint32_t)bs;  // + 0: -0 ties with +0
    }
    const uint32_t khi = __reduce_min_sync(gmask, (uint32_t)(key >> 32));
    const uint32_t klo = __reduce_min_sync(gmask, (uint32_t)(key >> 32) == khi ? (uint32_t)key : 0xFFFFFFFFu);
    const uint32_t win = klo >> 3, ws = klo & 7u;
    used |= 1u << ws;
    if (win == i) my_slot = (int)ws;
  }
  // this child's planes, its part of the SAH, its place among the slots
  uint32_t qlx = 0, qly = 0, qlz = 0, qhx = 0, qhy = 0, qhz = 0, cnt = 0;
  bool internal = false;
  double A = 0.0, Ax = 0.0;
  if (valid) {
    const float flx = fminf(fmaxf(floorf(__fsub_rd(lo.x, ulo.x) * ix), 0.f), 255.f);
    const float fly = fminf(fmaxf(floorf(__fsub_rd(lo.y, ulo.y) * iy), 0.f), 255.f);
    const float flz = fminf(fmaxf(floorf(__fsub_rd(lo.z, ulo.z) * iz), 0.f), 255.f);
    const float fhx = fminf(fmaxf(ceilf(__fsub_ru(hi.x, ulo.x) * ix), 0.f), 255.f);
    const float fhy = fminf(fmaxf(ceilf(__fsub_ru(hi.y, ulo.y) * iy), 0.f), 255.f);
    const float fhz = fminf(fmaxf(ceilf(__fsub_ru(hi.z, ulo.z) * iz), 0.f), 255.f);
    qlx = (uint32_t)flx; qly = (uint32_t)fly; qlz = (uint32_t)flz;
    qhx = (uint32_t)fhx; qhy = (uint32_t)fhy; qhz = (uint32_t)fhz;
    // decoded (outward-rounded) box, as traversal sees it
    const float3 dlo = make_float3(__fmaf_rd(flx, sx, ulo.x), __fmaf_rd(fly, sy, ulo.y), __fmaf_rd(flz, sz, ulo.z));
    const float3 dhi = make_float3(__fmaf_ru(fhx, sx, ulo.x), __fmaf_ru(fhy, sy, ulo.y), __fmaf_ru(fhz, sz, ulo.z));
    A = (double)fmaxf(0.f, half_area(dlo, dhi));
    Ax = (double)fmaxf(0.f, half_area(lo, hi));
    cnt = bt_cnt(t, kid);
    internal = cnt > t.leaf_max;
  }
  const uint32_t slot = valid ? (uint32_t)my_slot : 8u;
  const uint32_t int_slots = __reduce_or_sync(gmask, internal ? 1u << slot : 0u);
  uint32_t tri_off = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint32_t sj = __shfl_sync(gmask, slot, j, 8);
    const uint32_t cj = __shfl_sync(gmask, (valid && !internal) ? cnt : 0u, j, 8);
    if (sj < slot) tri_off += cj;
  }
  const uint32_t oi = off_int[k], ot = off_tri[k];
  const uint32_t child_base = next_base + oi, tri_base = tri_next + ot;
  uint32_t meta = 0;
  if (valid && internal) {
    const uint32_t rank = __popc(int_slots & ((1u << slot) - 1u));
    meta = 0x80u | slot;
    if (oi + rank >= node_cap || child_base + rank >= node_cap) atomicOr(err, kErrBuild);
    else next_items[oi + rank] = kid;
    sah_out += A;  // inner node term
    sahx_out += Ax;
  } else if (valid) {
    meta = 0x80u | ((cnt - 1u) << 5) | tri_off;
    // the leaf's triangle records are written after the last level by
    // k_write_leaves, one thread per leaf: here only its binary subtree is
    // recorded at the slot of its first triangle
    if (tri_base + tri_off + cnt > tri_cap) atomicOr(err, kErrBuild);
    else leaf_root[tri_base + tri_off] = cnt == 1 ? bt_right(t, kid) | kLeafPrim : kid;
    sah_out += A * (double)((cnt + 3) / 4);  // leaf term: area x Triangle4 blocks
    sahx_out += Ax * (double)((cnt + 3) / 4);
    nleaf_out++;
  }
  // the node's words: byte `slot` of each per-slot array (empty slots: meta 0,
  // lower planes 255, upper planes 0)
  const uint32_t sh = 8u * (slot & 3u);
  const bool hi4 = slot >= 4u && slot < 8u, lo4 = slot < 4u;
  auto word = [&](uint32_t v, bool part) { return part ? v << sh : 0u; };
  const uint32_t empty = (~used) & 0xFFu;
  auto fill = [&](uint32_t m4) {  // 0xFF in the bytes of the empty slots m4 (4 bits)
    return ((m4 & 1u) ? 0xFFu : 0u) | ((m4 & 2u) ? 0xFF00u : 0u) | ((m4 & 4u) ? 0xFF0000u : 0u) |
           ((m4 & 8u) ? 0xFF000000u : 0u);
  };
  const uint32_t m0 = __reduce_or_sync(gmask, word(meta, lo4)), m1 = __reduce_or_sync(gmask, word(meta, hi4));
  const uint32_t lx0 = __reduce_or_sync(gmask, word(qlx, lo4)) | fill(empty & 15u);
  const uint32_t lx1 = __reduce_or_sync(gmask, word(qlx, hi4)) | fill(empty >> 4);
  const uint32_t ly0 = __reduce_or_sync(gmask, word(qly, lo4)) | fill(empty & 15u);
  const uint32_t ly1 = __reduce_or_sync(gmask, word(qly, hi4)) | fill(empty >> 4);
  const uint32_t lz0 = __reduce_or_sync(gmask, word(qlz, lo4)) | fill(empty & 15u);
  const uint32_t lz1 = __reduce_or_sync(gmask, word(qlz, hi4)) | fill(empty >> 4);
  const uint32_t hx0 = __reduce_or_sync(gmask, word(qhx, lo4)), hx1 = __reduce_or_sync(gmask, word(qhx, hi4));
  const uint32_t hy0 = __reduce_or_sync(gmask, word(qhy, lo4)), hy1 = __reduce_or_sync(gmask, word(qhy, hi4));
  const uint32_t hz0 = __reduce_or_sync(gmask, word(qhz, lo4)), hz1 = __reduce_or_sync(gmask, word(qhz, hi4));
  if (level_base + k >= node_cap) {
    if (i == 0) atomicOr(err, kErrBuild);
    return;
  }
  // WideNode as five 16-byte words (gb_common.h layout)
  uint4* dst = reinterpret_cast<uint4*>(nodes + level_base + k);
  if (i == 0) {
    dst[0] = make_uint4(__float_as_uint(ulo.x), __float_as_uint(ulo.y), __float_as_uint(ulo.z),
                        Ex | (Ey << 8) | (Ez << 16) | ((int_slots & 0xFFu) << 24));
  } else if (i == 1) {
    dst[1] = make_uint4(child_base, tri_base, m0, m1);
  } else if (i == 2) {
    dst[2] = make_uint4(lx0, lx1, ly0, ly1);
  } else if (i == 3) {
    dst[3] = make_uint4(lz0, lz1, hx0, hx1);
  } else if (i == 4) {
    dst[4] = make_uint4(hy0, hy1, hz0, hz1);
  }
}

constexpr int COLLAPSE_THREADS = 128;
// Levels of at most this many items are emitted by lane groups (latency-bound:
// one node's greedy slot choice and reductions spread over 8 lanes), wider ones
// one node per thread.
constexpr uint32_t kGroupEmitMax = 16384;

// One wide node per 8-lane group; the SAH sums and the leaf count are reduced
// per CTA first (one atomic per CTA instead of one per node).
__global__ void __launch_bounds__(COLLAPSE_THREADS) k_collapse_emit(
    BinTree t, const uint32_t* __restrict__ kids_in, const uint32_t* __restrict__ cstate,
    const uint32_t* __restrict__ off_int, const uint32_t* __restrict__ off_tri, WideNode* __restrict__ nodes,
    uint32_t* __restrict__ leaf_root, const ColItems ci, double* sah_acc, uint32_t* leaf_count,
    uint32_t node_cap, uint32_t tri_cap, uint32_t* err) {
  const uint32_t nitems = cstate[kColN], level_base = cstate[kColBase], tri_next = cstate[kColTri];
  uint32_t* __restrict__ next_items = ci.items[(cstate[kColDepth] & 1u) ^ 1u];
  const uint32_t next_base = level_base + nitems;
  double sah = 0.0, sahx = 0.0;
  uint32_t nleaf = 0;
  if (nitems <= kGroupEmitMax) {
    const uint32_t gmask = 0xFFu << (threadIdx.x & 24u);
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 3; k < nitems; k += (gridDim.x * blockDim.x) >> 3)
      collapse_emit_group(t, kids_in, k, off_int, off_tri, level_base, next_base, tri_next, nodes, leaf_root,
                          next_items, node_cap, tri_cap, err, gmask, sah, sahx, nleaf);
  } else {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nitems; k += gridDim.x * blockDim.x) {
      double a = 0.0, b = 0.0;
      uint32_t l = 0;
      collapse_emit_node(t, kids_in, k, off_int, off_tri, level_base, next_base, tri_next, nodes, leaf_root,
                         next_items, node_cap, tri_cap, err, a, b, l);
      sah += a;
      sahx += b;
      nleaf += l;
    }
  }
  nleaf = __reduce_add_sync(0xFFFFFFFFu, nleaf);
  if ((threadIdx.x & 31) == 0 && nleaf) atomicAdd(leaf_count, nleaf);
  block_add2(sah, sahx, sah_acc);
}

// ---- all collapse levels in one cooperative launch (captured builds)
//
// A grid barrier between the phases of a level replaces the kernel boundaries
// of the level-by-level form (count, scan, emit, advance: four launches per
// level).  Every CTA keeps the level state in registers and advances it alike;
// CTA 0 writes it back to cstate at the end.


constexpr int COLLAPSE_ALL_THREADS = 256;

// Exclusive block scan of two values (a, b); returns (prefix a, prefix b) and
// the block totals in *ta, *tb.  All threads call it.
__device__ __forceinline__ uint2 block_excl_scan2(uint32_t a, uint32_t b, uint32_t* ta, uint32_t* tb) {
  __shared__ uint32_t s_a[COLLAPSE_ALL_THREADS / 32], s_b[COLLAPSE_ALL_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t xa = a, xb = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ya = __shfl_up_sync(0xFFFFFFFFu, xa, o), yb = __shfl_up_sync(0xFFFFFFFFu, xb, o);
    if (lane >= o) {
      xa += ya;
      xb += yb;
    }
  }
  if (lane == 31) {
    s_a[warp] = xa;
    s_b[warp] = xb;
  }
  __syncthreads();
  uint32_t oa = 0, ob = 0, sa = 0, sb = 0;
#pragma unroll
  for (int w = 0; w < COLLAPSE_ALL_THREADS / 32; w++) {
    if (w < warp) {
      oa += s_a[w];
      ob += s_b[w];
    }
    sa += s_a[w];
    sb += s_b[w];
  }
  __syncthreads();  // s_a, s_b are reused by the next call
  *ta = sa;
  *tb = sb;
  return make_uint2(oa + xa - a, ob + xb - b);
}

// Every level of the collapse, from the roots in cstate: each CTA takes a
// contiguous chunk of the level's items, (1) gathers their children and counts
// internal children and leaf triangles, publishes its sums, [barrier], (2)
// turns its counts into the level's exclusive offsets from the CTA sums, (3)
// writes its wide nodes and the next level's items, [barrier].  cta_sums holds
// 2 * gridDim.x words; *bar is zero on entry.
__global__ void __launch_bounds__(COLLAPSE_ALL_THREADS, 2) k_collapse_all(
    BinTree t, const ColItems ci, uint32_t* __restrict__ cstate, uint32_t* __restrict__ kids,
    uint32_t* __restrict__ nint, uint32_t* __restrict__ ntri, uint32_t* __restrict__ cta_sums,
    WideNode* __restrict__ nodes, uint32_t* __restrict__ leaf_root, double* sah_acc, uint32_t* leaf_count,
    uint32_t node_cap, uint32_t tri_cap, uint32_t max_levels, GridBarrier* bar, unsigned int* err) {
  uint32_t nitems = __ldcg(cstate + kColN), base = __ldcg(cstate + kColBase), tri_next = __ldcg(cstate + kColTri),
           depth = __ldcg(cstate + kColDepth);
  bool failed = __ldcg(cstate + kColErr) != 0u;
  double sah = 0.0, sahx = 0.0;
  uint32_t nleaf = 0;
  while (nitems > 0 && !failed) {
    const uint32_t* __restrict__ items = ci.items[depth & 1u];
    uint32_t* __restrict__ next_items = ci.items[(depth & 1u) ^ 1u];
    const uint32_t per = (nitems + gridDim.x - 1) / gridDim.x;
    const uint32_t first = min(blockIdx.x * per, nitems), last = min(first + per, nitems);
    // (1) children and counts
    uint32_t ci_sum = 0, ct_sum = 0;
    for (uint32_t k = first + threadIdx.x; k < last; k += blockDim.x) {
      uint32_t kk[8];
      const int nk = gather_children(t, items[k], kk);
      uint32_t ni = 0, nt = 0;
      for (int i = 0; i < 8; i++) {
        if (i < nk) {
          const uint32_t c = kk[i];
          const uint32_t cnt = bt_cnt(t, c);
          if (cnt > t.leaf_max) ni++; else nt += cnt;
          kids[8 * (size_t)k + i] = c;
        } else {
          kids[8 * (size_t)k + i] = 0xFFFFFFFFu;
        }
      }
      nint[k] = ni;
      ntri[k] = nt;
      ci_sum += ni;
      ct_sum += nt;
    }
    {
      uint32_t ta, tb;
      block_excl_scan2(ci_sum, ct_sum, &ta, &tb);
      if (threadIdx.x == 0) {
        __stcg(cta_sums + blockIdx.x, ta);
        __stcg(cta_sums + gridDim.x + blockIdx.x, tb);
      }
    }
    if (!grid_sync(bar, err)) break;
    // (2) offsets: this CTA's prefix and the level's totals from the CTA sums
    uint32_t pi = 0, pt = 0, ti = 0, tt = 0;
    for (uint32_t c = threadIdx.x; c < gridDim.x; c += blockDim.x) {
      const uint32_t a = __ldcg(cta_sums + c), b = __ldcg(cta_sums + gridDim.x + c);
      ti += a;
      tt += b;
      if (c < blockIdx.x) {
        pi += a;
        pt += b;
      }
    }
    {
      uint32_t s0, s1, s2, s3;
      block_excl_scan2(pi, pt, &s0, &s1);
      block_excl_scan2(ti, tt, &s2, &s3);
      pi = s0;
      pt = s1;
      ti = s2;
      tt = s3;
    }
    for (uint32_t k0 = first; k0 < last; k0 += blockDim.x) {
      const uint32_t k = k0 + threadIdx.x;
      const uint32_t a = k < last ? nint[k] : 0u, b = k < last ? ntri[k] : 0u;
      uint32_t ta, tb;
      const uint2 e = block_excl_scan2(a, b, &ta, &tb);
      if (k < last) {
        nint[k] = pi + e.x;
        ntri[k] = pt + e.y;
      }
      pi += ta;
      pt += tb;
    }
    __syncthreads();
    // (3) the wide nodes of this CTA's items: one per 8-lane group on narrow
    // levels, one per thread on wide ones
    if (nitems <= kGroupEmitMax) {
      const uint32_t gmask = 0xFFu << (threadIdx.x & 24u);
      for (uint32_t k = first + (threadIdx.x >> 3); k < last; k += blockDim.x >> 3)
        collapse_emit_group(t, kids, k, nint, ntri, base, base + nitems, tri_next, nodes, leaf_root, next_items,
                            node_cap, tri_cap, err, gmask, sah, sahx, nleaf);
    } else {
      for (uint32_t k = first + threadIdx.x; k < last; k += blockDim.x) {
        double a = 0.0, b = 0.0;
        uint32_t l = 0;
        collapse_emit_node(t, kids, k, nint, ntri, base, base + nitems, tri_next, nodes, leaf_root, next_items,
                           node_cap, tri_cap, err, a, b, l);
        sah += a;
        sahx += b;
        nleaf += l;
      }
    }
    // (4) the next level, alike in every CTA
    if (blockIdx.x == 0 && threadIdx.x == 0 && depth < (uint32_t)kColMaxLevels) cstate[kColLevels + depth] = base;
    base += nitems;
    tri_next += tt;
    depth++;
    uint32_t next = ti;
    if ((next > 0 && depth >= max_levels) || base + next > node_cap) {
      failed = true;
      next = 0;
      if (blockIdx.x == 0 && threadIdx.x == 0) cstate[kColErr] = 1u;
    }
    nitems = next;
    if (!grid_sync(bar, err)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cstate[kColN] = 0;
    cstate[kColBase] = base;
    cstate[kColTri] = tri_next;
    cstate[kColDepth] = depth;
    if (depth <= (uint32_t)kColMaxLevels) cstate[kColLevels + depth] = base;  // end of the last level
    if (lb_load(err) != 0u) cstate[kColErr] = 1u;
  }
  nleaf = __reduce_add_sync(0xFFFFFFFFu, nleaf);
  if ((threadIdx.x & 31) == 0 && nleaf) atomicAdd(leaf_count, nleaf);
  block_add2(sah, sahx, sah_acc);
}

// Writes the triangle records of every leaf: slot t holds the binary subtree of
// the leaf whose first triangle goes to t, or for a one-triangle leaf its
// primitive with kLeafPrim set (kInvalidID elsewhere); a subtree's primitives
// (at most 4) are written in depth-first order, left first.
__global__ void __launch_bounds__(256) k_write_leaves(BinTree t, const GeomDesc* __restrict__ geoms,
                                                      const float4* __restrict__ plo, const float4* __restrict__ phi,
                                                      const uint32_t* __restrict__ leaf_root, uint32_t ntris,
                                                      TriRecord* __restrict__ tris, uint32_t* err,
                                                      const TriRecord* __restrict__ prec) {
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  if (first >= ntris) return;
  const uint32_t c = leaf_root[first];
  if (c == kInvalidID) return;
  if (c & kLeafPrim) {  // one triangle: its primitive, no subtree to walk
    const uint32_t prim = c & ~kLeafPrim;
    if (prec) tris[first] = prec[prim];
    else write_tri(geoms, plo, phi, prim, &tris[first], t.robust != 0);
    return;
  }
  uint32_t st[8];
  int sp = 0;
  st[sp++] = c;
  uint32_t w = 0;
  while (sp > 0) {
    const uint32_t x = st[--sp];
    if (bt_leaf(t, x)) {
      if (first + w >= ntris || w >= (uint32_t)kLeafMaxLimit) {
        atomicOr(err, kErrBuild);
        return;
      }
      if (prec) tris[first + w] = prec[bt_right(t, x)];
      else write_tri(geoms, plo, phi, bt_right(t, x), &tris[first + w], t.robust != 0);
      w++;
    } else {
      if (sp + 2 > 8) {
        atomicOr(err, kErrBuild);
        return;
      }
      st[sp++] = bt_right(t, x);
      st[sp++] = bt_left(t, x);
    }
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------

template <typename T>
static cudaError_t dalloc(T** p, size_t count, cudaStream_t st) {
  return cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(T), st);
}

static inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

static int num_sms_build() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

// Blocks of 256 threads for a grid-stride kernel over n items: up to 8 per SM.
static unsigned grid_stride_blocks(uint64_t n) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)num_sms_build() * 8));
}

// Words of look-back state that scan_excl needs for n elements (ticket, done
// counter, one status word per tile); zero when allocated, and every scan leaves
// it zero again.
static inline uint32_t scan_scratch(uint32_t n) { return cdiv(n, SCAN_TILE) + 2; }

// Exclusive scans of a[0, n) and b[0, n) in place, by one launch (totals to
// *ta / *tb); sums holds 2 * scan_scratch(n) zeroed words.  With d_n the count
// is *d_n (at most n), read on the device, so the scans can be enqueued before
// the count is known.  One CTA per array for short arrays, else the look-back
// scan.
static void scan_excl2(uint32_t* a, uint32_t* b, uint32_t n, uint32_t* ta, uint32_t* tb, uint32_t* sums,
                       cudaStream_t st, unsigned int* err, const uint32_t* d_n = nullptr) {
  const ScanPair sp{{a, b}, {ta, tb}};
  if (n <= 2 * SCAN_TILE) {
    k_scan_excl<<<dim3(1, 2), SCAN_THREADS, 0, st>>>(sp, n, d_n, 1);
  } else {
    k_scan_lb<<<dim3(cdiv(n, SCAN_TILE), 2), SCAN_THREADS, 0, st>>>(sp, n, d_n, 1, sums, scan_scratch(n), err);
  }
  note_launches(1);
}

// Scratch words of onesweep_sort for n keys and `passes` digit passes.
static inline size_t onesweep_scratch_words(uint32_t n, int passes) {
  return kOsStatus + (size_t)passes * cdiv(n, RS_TILE) * 256u;
}

// Stable LSD sort of (ka, va) by the digits set in digit_mask (bit d: key bits
// 8d..8d+7), least significant first, ping-ponging with (kb, vb): on return
// (ka, va) name the buffers that hold the result.  scratch: at least
// onesweep_scratch_words(n, passes) words, zeroed here.  A look-back that gives up
// sets kErrBuild in *err (or in the scratch's error word when err is null).
template <typename K>
static cudaError_t onesweep_sort(K*& ka, uint32_t*& va, K*& kb, uint32_t*& vb, uint32_t n, uint32_t digit_mask,
                                 uint32_t* scratch, unsigned int* err, cudaStream_t st) {
  digit_mask &= (1u << sizeof(K)) - 1u;
  const int passes = __builtin_popcount(digit_mask);
  if (n == 0 || passes == 0) return cudaSuccess;
  if (n >= kLbValue) return cudaErrorInvalidValue;  // look-back counts are 30-bit
  const uint32_t ntiles = cdiv(n, RS_TILE);
  GB_CHECK(cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * onesweep_scratch_words(n, passes), st));
  const uint32_t hgrid = std::min<uint32_t>(ntiles, 4u * (uint32_t)num_sms_build());
  // 32 or 48 KB of staged keys and values beyond the static shared memory (per
  // device; a captured build sets it in graph_build_prepare)
  constexpr size_t smem = os_scatter_smem<K>();
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GB_CHECK(cudaStreamIsCapturing(st, &cap));
  if (cap == cudaStreamCaptureStatusNone)
    GB_CHECK(cudaFuncSetAttribute(k_os_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_os_hist<K><<<hgrid, 256, 0, st>>>(ka, n, digit_mask & ((1u << sizeof(K)) - 1u), scratch);
  uint32_t slot = 0;
  for (int d = 0; d < (int)sizeof(K); d++) {
    if (!(digit_mask >> d & 1u)) continue;
    k_os_scatter<K><<<ntiles, RS_THREADS, smem, st>>>(ka, va, kb, vb, n, 8 * d, scratch, slot,
                                                      scratch + kOsStatus + (size_t)slot * ntiles * 256u,
                                                      err ? err : scratch + kOsErr);
    std::swap(ka, kb);
    std::swap(va, vb);
    slot++;
  }
  note_launches(1 + passes);
  return cudaGetLastError();
}

// Stream-ordered scratch of one build: device allocations, pinned host
// buffers and events are released when the arena goes out of scope, on every
// return path (free() releases a buffer early to lower the peak).
struct BuildArena {
  cudaStream_t st;
  std::vector<void*> dev, pinned;
  std::vector<cudaEvent_t> events;
  explicit BuildArena(cudaStream_t s) : st(s) {}
  BuildArena(const BuildArena&) = delete;
  BuildArena& operator=(const BuildArena&) = delete;
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    const cudaError_t e = cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(T), st);
    if (e == cudaSuccess) dev.push_back(*p);
    return e;
  }
  template <typename T>
  cudaError_t host(T** p, size_t count) {
    const cudaError_t e = cudaMallocHost((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) pinned.push_back(*p);
    return e;
  }
  cudaError_t event(cudaEvent_t* e) {
    const cudaError_t r = cudaEventCreate(e);
    if (r == cudaSuccess) events.push_back(*e);
    return r;
  }
  void free(void* p) {
    for (size_t i = 0; i < dev.size(); i++)
      if (dev[i] == p) {
        cudaFreeAsync(p, st);
        dev.erase(dev.begin() + (long)i);
        return;
      }
  }
  ~BuildArena() {
    for (void* p : dev) cudaFreeAsync(p, st);
    if (!pinned.empty()) cudaStreamSynchronize(st);  // copies into them may still be in flight
    for (void* p : pinned) cudaFreeHost(p);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
};

cudaError_t build_bvh(const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, const BuildOptions& opt, DeviceBVH* out,
                      BuildStats* stats) {
  *out = DeviceBVH();
  *stats = BuildStats();
  for (int d = 0; d < 3; d++) { out->lo[d] = INFINITY; out->hi[d] = -INFINITY; }
  uint64_t total64 = 0;
  for (int g = 0; g < ngeoms; g++) total64 += h_geoms[g].ntris;
  if (total64 == 0) return cudaSuccess;
  if (total64 >= 0x7FFFFFFFull) return cudaErrorInvalidValue;
  const uint32_t total = (uint32_t)total64;

  BuildArena arena(st);  // scratch and events of this build, released on every return
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  GB_CHECK(arena.event(&ev0));
  GB_CHECK(arena.event(&ev1));
  GB_CHECK(cudaEventRecord(ev0, st));

  GeomDesc* d_geoms = nullptr;
  GB_CHECK(arena.alloc(&d_geoms, ngeoms));
  GB_CHECK(cudaMemcpyAsync(d_geoms, h_geoms, sizeof(GeomDesc) * ngeoms, cudaMemcpyHostToDevice, st));

  float4 *plo = nullptr, *phi = nullptr;
  BoundsAcc* acc = nullptr;
  GB_CHECK(arena.alloc(&plo, total));
  GB_CHECK(arena.alloc(&phi, total));
  GB_CHECK(arena.alloc(&acc, 1));
  BoundsAcc h_acc;
  for (int d = 0; d < 3; d++) { h_acc.glo[d] = h_acc.clo[d] = 0xFFFFFFFFu; h_acc.ghi[d] = h_acc.chi[d] = 0u; }
  h_acc.nvalid = 0;
  h_acc.pad = 0;
  h_acc.kand = ~0ull;
  h_acc.kor = 0ull;
  GB_CHECK(cudaMemcpyAsync(acc, &h_acc, sizeof(BoundsAcc), cudaMemcpyHostToDevice, st));
  // leaf records in primitive order (read back by k_write_leaves)
  TriRecord* prec = nullptr;
  GB_CHECK(arena.alloc(&prec, total));
  k_primrefs<<<grid_stride_blocks(total), 256, 0, st>>>(d_geoms, ngeoms, total, plo, phi, acc, prec,
                                                        opt.robust ? 1 : 0);
  note_launches(1);

  uint64_t *keys_a = nullptr, *keys_b = nullptr;
  uint32_t *vals_a = nullptr, *vals_b = nullptr;
  GB_CHECK(arena.alloc(&keys_a, total));
  GB_CHECK(arena.alloc(&keys_b, total));
  GB_CHECK(arena.alloc(&vals_a, total));
  GB_CHECK(arena.alloc(&vals_b, total));
  const bool segmented = opt.segmented != 0;
  const uint32_t nseg = segmented ? (uint32_t)ngeoms : 1u;
  if (segmented && (uint32_t)ngeoms > kMaxSegments) return cudaErrorInvalidValue;
  const bool key32 = opt.morton_bits == 30 && !segmented;  // 30-bit keys sorted as 32-bit words
  k_morton<<<grid_stride_blocks(total), 256, 0, st>>>(plo, phi, total, acc, keys_a, vals_a, opt.morton_cube,
                                                      segmented ? 1 : 0, opt.morton_bits == 30 ? 1 : 0,
                                                      key32 ? 1 : 0);
  note_launches(1);
  GB_CHECK(cudaGetLastError());
  GB_CHECK(cudaMemcpyAsync(&h_acc, acc, sizeof(BoundsAcc), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaStreamSynchronize(st));
  const uint32_t N = h_acc.nvalid;
  for (int d = 0; d < 3; d++) { out->lo[d] = ord2f(h_acc.glo[d]); out->hi[d] = ord2f(h_acc.ghi[d]); }
  if (N == 0) {
    for (int d = 0; d < 3; d++) { out->lo[d] = INFINITY; out->hi[d] = -INFINITY; }
    arena.free(d_geoms); arena.free(plo); arena.free(phi); arena.free(acc); arena.free(prec);
    arena.free(keys_a); arena.free(keys_b); arena.free(vals_a); arena.free(vals_b);
    return cudaStreamSynchronize(st);
  }

  // ---- radix sort (all `total` keys; invalid ones carry a key above every valid
  // one and sort last), the digits that are constant over all keys skipped
  {
    uint32_t digit_mask = 0;
    for (int d = 0; d < 8; d++)
      if (((h_acc.kand >> (8 * d)) & 0xFF) != ((h_acc.kor >> (8 * d)) & 0xFF)) digit_mask |= 1u << d;
    uint32_t* hist = nullptr;
    GB_CHECK(arena.alloc(&hist, onesweep_scratch_words(total, __builtin_popcount(digit_mask))));
    if (key32) {
      uint32_t *ka32 = reinterpret_cast<uint32_t*>(keys_a), *kb32 = reinterpret_cast<uint32_t*>(keys_b);
      GB_CHECK(onesweep_sort(ka32, vals_a, kb32, vals_b, total, digit_mask, hist, &acc->pad, st));
    } else {
      GB_CHECK(onesweep_sort(keys_a, vals_a, keys_b, vals_b, total, digit_mask, hist, &acc->pad, st));
    }
    arena.free(hist);
  }

  // ---- PLOC over the N valid primitives (sorted positions 0..N-1)
  float4 *bnlo = nullptr, *bnhi = nullptr;
  uint32_t* bncnt = nullptr;
  // leaf size: explicit, or by the scene -- flat scenes (centroid box's
  // smallest extent below half the largest: heightfields, terrain) and scenes
  // that will be refitted every frame take 2 triangles per leaf, the rest 1
  // (measured on a GB300: the 4M soup traces 5 % faster with 1; a 724^2
  // heightfield 8 % faster with 2, and its SAH is 1.12x the reference
  // builder's with 2, 1.31x with 1; the animated 4M soup, refitted per frame,
  // renders 4 % faster with 2, whose tree has 40 % fewer nodes to refit)
  int leaf_max = opt.leaf_max;
  if (leaf_max <= 0) {
    float emin = INFINITY, emax = 0.f;
    for (int d = 0; d < 3; d++) {
      const float e = ord2f(h_acc.chi[d]) - ord2f(h_acc.clo[d]);
      emin = std::min(emin, e);
      emax = std::max(emax, e);
    }
    leaf_max = (emin < 0.5f * emax || opt.refit_target) ? 2 : 1;
  }
  stats->leaf_max = (uint32_t)std::min(leaf_max, kLeafMaxLimit);
  const uint32_t nnodes_bin = 2 * N - 1;
  // SAH-optimal collapse: the cost table is filled as PLOC creates the nodes
  float4* dp_cost = nullptr;
  uint2* d_choice = nullptr;
  if (opt.collapse == 1) {
    GB_CHECK(arena.alloc(&dp_cost, 2 * (size_t)nnodes_bin));
    GB_CHECK(arena.alloc(&d_choice, nnodes_bin));
  }
  GB_CHECK(arena.alloc(&bnlo, nnodes_bin));
  GB_CHECK(arena.alloc(&bnhi, nnodes_bin));
  GB_CHECK(arena.alloc(&bncnt, nnodes_bin));
  float4 *clo_a, *chi_a, *clo_b, *chi_b;
  uint32_t *cidx_a, *cidx_b, *nn;
  GB_CHECK(arena.alloc(&clo_a, N));
  GB_CHECK(arena.alloc(&chi_a, N));
  GB_CHECK(arena.alloc(&clo_b, N));
  GB_CHECK(arena.alloc(&chi_b, N));
  GB_CHECK(arena.alloc(&cidx_a, N));
  GB_CHECK(arena.alloc(&cidx_b, N));
  GB_CHECK(arena.alloc(&nn, N));
  const uint32_t leaf_max_used = (uint32_t)std::min(std::max(leaf_max, 1), kLeafMaxLimit);
  k_ploc_init<<<cdiv(N, 256), 256, 0, st>>>(plo, phi, vals_a, N, &acc->nvalid, bnlo, bnhi, bncnt, cidx_a, clo_a,
                                            chi_a, segmented ? 1 : 0);
  note_launches(1);
  uint32_t *bsurv, *bmerge, *d_tot, *d_root, *d_iters;
  const uint32_t maxb = cdiv(N, PLOC_BLOCK);
  GB_CHECK(arena.alloc(&bsurv, maxb));
  GB_CHECK(arena.alloc(&bmerge, maxb));
  uint32_t* scan_sums = nullptr;  // look-back state of the PLOC and collapse scans (zero between scans)
  GB_CHECK(arena.alloc(&scan_sums, 2 * (size_t)scan_scratch(std::max(maxb, N))));
  GB_CHECK(cudaMemsetAsync(scan_sums, 0, sizeof(uint32_t) * 2 * scan_scratch(std::max(maxb, N)), st));
  GB_CHECK(arena.alloc(&d_tot, 4));
  GB_CHECK(arena.alloc(&d_root, nseg));
  GB_CHECK(cudaMemsetAsync(d_root, 0xFF, sizeof(uint32_t) * nseg, st));
  GB_CHECK(arena.alloc(&d_iters, 1));
  GB_CHECK(cudaMemsetAsync(d_iters, 0, sizeof(uint32_t), st));
  // PLOC rounds in batches of kPlocBatch between host reads of the state; the
  // count only shrinks, so the count read last bounds the grids of a batch,
  // and rounds after the last real one are no-ops (the done flag)
  constexpr int kPlocBatch = 4;
  uint32_t* ploc_state = nullptr;
  GB_CHECK(arena.alloc(&ploc_state, kPlocStateWords));
  uint32_t* h_tot = nullptr;
  GB_CHECK(arena.host(&h_tot, kPlocStateWords));
  k_ploc_state_init<<<1, 32, 0, st>>>(acc, ploc_state);
  note_launches(1);
  const int radius = opt.ploc_radius == 1 || opt.ploc_radius == 2 || opt.ploc_radius == 4 || opt.ploc_radius == 8
                         ? opt.ploc_radius
                         : PLOC_R_MAX;
  const PlocBufs pb{{clo_a, clo_b}, {chi_a, chi_b}, {cidx_a, cidx_b}};
  uint32_t round = 0;
  auto enqueue_round = [&](uint32_t grid) {
    switch (radius) {
      case 1: k_ploc_nn<1><<<grid, PLOC_BLOCK, 0, st>>>(pb, ploc_state, nn); break;
      case 2: k_ploc_nn<2><<<grid, PLOC_BLOCK, 0, st>>>(pb, ploc_state, nn); break;
      case 4: k_ploc_nn<4><<<grid, PLOC_BLOCK, 0, st>>>(pb, ploc_state, nn); break;
      case 8: k_ploc_nn<8><<<grid, PLOC_BLOCK, 0, st>>>(pb, ploc_state, nn); break;
      default: k_ploc_nn<PLOC_R_MAX><<<grid, PLOC_BLOCK, 0, st>>>(pb, ploc_state, nn); break;
    }
    k_ploc_count<<<grid, PLOC_BLOCK, 0, st>>>(nn, ploc_state, bsurv, bmerge);
    note_launches(2);
    scan_excl2(bsurv, bmerge, maxb, d_tot + 0, d_tot + 1, scan_sums, st, &acc->pad, ploc_state + kPlocTiles);
    k_ploc_emit<<<grid, PLOC_BLOCK, 0, st>>>(pb, nn, ploc_state, bsurv, bmerge, bnlo, bnhi, bncnt, nnodes_bin,
                                             &acc->pad, dp_cost, d_choice, leaf_max_used);
    k_ploc_advance<<<1, 32, 0, st>>>(d_tot, ploc_state);
    note_launches(2);
    round++;
  };
  uint32_t n = N;
  while (n > PLOC_SMALL) {
    const uint32_t nb = cdiv(n, PLOC_BLOCK);
    for (int b = 0; b < kPlocBatch; b++) enqueue_round(nb);
    GB_CHECK(cudaGetLastError());
    GB_CHECK(cudaMemcpyAsync(h_tot, ploc_state, kPlocStateWords * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaStreamSynchronize(st));
    n = h_tot[kPlocN];
    if (h_tot[kPlocDone]) break;
  }
  // a round without merges while more than PLOC_SMALL clusters remain cannot
  // happen without segments (the globally closest pair is mutual); with
  // segments it means every segment is down to one cluster (<= kMaxSegments)
  const uint32_t iters = round > 0 ? h_tot[kPlocRounds] : 0u;
  {
    const size_t smem = kPlocSmallSmem;
    GB_CHECK(cudaFuncSetAttribute(k_ploc_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_ploc_small<<<1, PLOC_SMALL_THREADS, smem, st>>>(clo_a, chi_a, cidx_a, clo_b, chi_b, cidx_b, ploc_state, bnlo,
                                                      bnhi, bncnt, d_root, d_iters, nnodes_bin, &acc->pad, nseg,
                                                      radius, dp_cost, d_choice, leaf_max_used);
    note_launches(1);
    GB_CHECK(cudaGetLastError());
  }
  uint32_t small_iters = 0, berr = 0;
  std::vector<uint32_t> seg_root(nseg, kInvalidID);
  GB_CHECK(cudaMemcpyAsync(seg_root.data(), d_root, sizeof(uint32_t) * nseg, cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(&small_iters, d_iters, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(&berr, &acc->pad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaStreamSynchronize(st));
  // the first collapse level holds one wide root per non-empty segment, in segment order
  std::vector<uint32_t> root_items;
  if (segmented) out->roots.assign(nseg, kInvalidID);
  for (uint32_t s = 0; s < nseg; s++) {
    if (seg_root[s] == kInvalidID) continue;
    if (seg_root[s] >= nnodes_bin) berr = 1;
    if (segmented) out->roots[s] = (uint32_t)root_items.size();
    root_items.push_back(seg_root[s]);
  }
  if (berr || root_items.empty() || (!segmented && root_items.size() != 1)) {
    return cudaErrorUnknown;
  }
  stats->ploc_iterations = iters + small_iters;
  stats->ploc_rounds = iters;
  arena.free(clo_b); arena.free(chi_b); arena.free(cidx_b);
  arena.free(clo_a); arena.free(chi_a); arena.free(cidx_a);
  arena.free(nn); arena.free(bsurv); arena.free(bmerge); arena.free(ploc_state);

  // ---- collapse, level by level (breadth-first node order)
  BinTree bt{bnlo, bnhi, bncnt, N, leaf_max_used, (uint32_t)(opt.robust != 0), d_choice};
  if (dp_cost) arena.free(dp_cost);
  WideNode* wnodes = nullptr;
  TriRecord* wtris = nullptr;
  const uint32_t maxw = N;  // wide internal nodes <= binary internal nodes + 1
  GB_CHECK(arena.alloc(&wnodes, maxw));
  GB_CHECK(arena.alloc(&wtris, N));
  uint32_t *items_a, *items_b, *kids, *nint, *ntri;
  GB_CHECK(arena.alloc(&items_a, maxw));
  GB_CHECK(arena.alloc(&items_b, maxw));
  GB_CHECK(arena.alloc(&kids, (size_t)8 * maxw));
  GB_CHECK(arena.alloc(&nint, maxw));
  GB_CHECK(arena.alloc(&ntri, maxw));
  uint32_t* leaf_root = nullptr;  // binary subtree of each leaf, at its first triangle's slot
  GB_CHECK(arena.alloc(&leaf_root, N));
  GB_CHECK(cudaMemsetAsync(leaf_root, 0xFF, sizeof(uint32_t) * N, st));
  double* d_sah = nullptr;
  uint32_t* d_leaves = nullptr;
  GB_CHECK(arena.alloc(&d_sah, 2));  // quantised, exact
  GB_CHECK(arena.alloc(&d_leaves, 1));
  GB_CHECK(cudaMemsetAsync(d_sah, 0, 2 * sizeof(double), st));
  GB_CHECK(cudaMemsetAsync(d_leaves, 0, sizeof(uint32_t), st));
  uint32_t *cstate = nullptr, *seg_index = nullptr, *h_col = nullptr;
  GB_CHECK(arena.alloc(&cstate, kColStateWords));
  GB_CHECK(arena.alloc(&seg_index, nseg));
  GB_CHECK(arena.host(&h_col, kColStateWords));
  GB_CHECK(cudaMemsetAsync(cstate, 0, sizeof(uint32_t) * kColStateWords, st));
  k_collapse_roots<<<1, 1024, 0, st>>>(d_root, nseg, nnodes_bin, items_a, seg_index, cstate);
  note_launches(1);
  const ColItems citems{{items_a, items_b}};
  uint32_t level = 0;
  const uint32_t max_levels = 0xFFFFFFFFu;  // host-driven: level starts recorded here, no bound
  auto enqueue_level = [&](uint32_t nitems_known) {  // the level's size, read by the host
    const uint32_t grid = cdiv(nitems_known, 128);
    k_collapse_count<<<grid, 128, 0, st>>>(bt, citems, cstate, kids, nint, ntri);
    note_launches(1);
    scan_excl2(nint, ntri, nitems_known, d_tot + 0, d_tot + 1, scan_sums, st, &acc->pad);
    k_collapse_emit<<<cdiv((uint64_t)nitems_known * (nitems_known <= kGroupEmitMax ? 8 : 1), COLLAPSE_THREADS),
                      COLLAPSE_THREADS, 0, st>>>(
        bt, kids, cstate, nint, ntri, wnodes, leaf_root, citems, d_sah, d_leaves, maxw, N, &acc->pad);
    k_collapse_advance<<<1, 32, 0, st>>>(d_tot, cstate, maxw, max_levels);
    note_launches(2);
    level++;
  };
  // one level per host read of the state: the grid fits the level
  uint32_t nitems = (uint32_t)root_items.size();
  std::vector<uint32_t> level_start;
  uint32_t level_base = 0;
  while (nitems > 0) {
    level_start.push_back(level_base);
    enqueue_level(nitems);
    GB_CHECK(cudaGetLastError());
    GB_CHECK(cudaMemcpyAsync(h_col, cstate, sizeof(uint32_t) * kColLevels, cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaStreamSynchronize(st));
    if (h_col[kColErr]) return cudaErrorUnknown;
    nitems = h_col[kColN];
    level_base = h_col[kColBase];
  }
  const uint32_t num_nodes = level_base, depth = (uint32_t)level_start.size();
  const uint32_t tri_next = level < 1 ? 0u : h_col[kColTri];
  k_write_leaves<<<cdiv(N, 256), 256, 0, st>>>(bt, d_geoms, plo, phi, leaf_root, N, wtris, &acc->pad, prec);
  note_launches(1);
  GB_CHECK(cudaGetLastError());
  arena.free(leaf_root);
  GB_CHECK(cudaMemcpyAsync(&berr, &acc->pad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaStreamSynchronize(st));
  if (berr || tri_next != N) {
    return cudaErrorUnknown;
  }
  double sah_sum[2] = {0.0, 0.0};
  uint32_t nleaves = 0;
  GB_CHECK(cudaMemcpyAsync(sah_sum, d_sah, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(&nleaves, d_leaves, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));

  // exact-size outputs
  GB_CHECK(cudaMalloc((void**)&out->nodes, (size_t)num_nodes * sizeof(WideNode)));
  GB_CHECK(cudaMalloc((void**)&out->tris, (size_t)N * sizeof(TriRecord)));
  GB_CHECK(copy_device(out->nodes, wnodes, (size_t)num_nodes * sizeof(WideNode), st));
  GB_CHECK(copy_device(out->tris, wtris, (size_t)N * sizeof(TriRecord), st));
  out->num_nodes = num_nodes;
  out->num_tris = N;
  out->depth = depth;
  out->robust = opt.robust != 0;
  level_start.push_back(num_nodes);
  out->level_start = level_start;

  arena.free(wnodes); arena.free(wtris);
  arena.free(items_a); arena.free(items_b); arena.free(kids);
  arena.free(nint); arena.free(ntri); arena.free(d_sah); arena.free(d_leaves);
  if (d_choice) arena.free(d_choice);
  arena.free(d_tot); arena.free(d_root); arena.free(d_iters); arena.free(scan_sums);
  arena.free(bnlo); arena.free(bnhi); arena.free(bncnt);
  arena.free(plo); arena.free(phi); arena.free(acc); arena.free(d_geoms); arena.free(prec);
  arena.free(keys_a); arena.free(keys_b); arena.free(vals_a); arena.free(vals_b);
  GB_CHECK(cudaEventRecord(ev1, st));
  GB_CHECK(cudaStreamSynchronize(st));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);

  // SAH relative to the root box (bvh_statistics.cpp: root node counts once)
  const float gx = out->hi[0] - out->lo[0], gy = out->hi[1] - out->lo[1], gz = out->hi[2] - out->lo[2];
  const double Aroot = std::max(0.0, (double)(gx * (gy + gz) + gy * gz));
  stats->sah = Aroot > 0 ? (Aroot + sah_sum[0]) / Aroot : 0.0;
  stats->sah_exact = Aroot > 0 ? (Aroot + sah_sum[1]) / Aroot : 0.0;
  stats->build_ms = ms;
  stats->num_nodes = num_nodes;
  stats->num_leaves = nleaves;
  stats->num_prims = N;
  stats->depth = depth;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// builds without host reads (captured into CUDA graphs)
// ---------------------------------------------------------------------------

__global__ void k_acc_init(BoundsAcc* __restrict__ acc) {
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; d++) {
      acc->glo[d] = acc->clo[d] = 0xFFFFFFFFu;
      acc->ghi[d] = acc->chi[d] = 0u;
    }
    acc->nvalid = 0;
    acc->pad = 0;
    acc->kand = ~0ull;
    acc->kor = 0ull;
  }
}

// Status of a replayed build: the plan's counts still hold, the rounds and
// levels sufficed, and no kernel flagged an error.
__global__ void k_graph_build_check(const BoundsAcc* __restrict__ acc, const uint32_t* __restrict__ ploc_state,
                                    const uint32_t* __restrict__ cstate, uint32_t valid_tris,
                                    uint32_t* __restrict__ status) {
  if (threadIdx.x != 0) return;
  uint32_t s = 0;
  if (acc->nvalid != valid_tris) s |= kGraphBuildCount;
  if (!ploc_state[kPlocDone] || ploc_state[kPlocN] > PLOC_SMALL) s |= kGraphBuildRounds;
  if (cstate[kColN] != 0 || cstate[kColTri] != valid_tris) s |= kGraphBuildLevels;
  if (acc->pad || cstate[kColErr]) s |= kGraphBuildError;
  *status = s;
}

// Device time (globaltimer, ns) into stamps[k]: one thread, enqueued between the
// phases of a captured build when BuildOptions::phase_stamps is set.
__global__ void k_phase_stamp(unsigned long long* stamps, int k) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  stamps[k] = t;
}

cudaError_t graph_build_prepare(const GeomDesc* h_geoms, int ngeoms, const BuildOptions& opt,
                                const GraphBuildPlan& plan, GraphBuild* g) {
  *g = GraphBuild{};
  g->plan = plan;
  g->opt = opt;
  g->ngeoms = ngeoms;
  uint64_t total64 = 0;
  for (int k = 0; k < ngeoms; k++) total64 += h_geoms[k].ntris;
  const uint32_t N = plan.valid_tris;
  if (total64 == 0 || total64 >= 0x7FFFFFFFull || N == 0 || N > total64 || plan.roots == 0 || plan.roots > N ||
      plan.levels == 0 || plan.levels > (uint32_t)kColMaxLevels)
    return cudaErrorInvalidValue;
  if (opt.segmented && (uint32_t)ngeoms > kMaxSegments) return cudaErrorInvalidValue;
  g->total = (uint32_t)total64;
  g->nseg = opt.segmented ? (uint32_t)ngeoms : 1u;
  g->nbin = 2 * N - plan.roots;
  g->maxw = N;
  g->maxb = cdiv(N, PLOC_BLOCK);
  g->rs_blocks = cdiv(g->total, RS_TILE);
  g->radius = (opt.ploc_radius == 1 || opt.ploc_radius == 2 || opt.ploc_radius == 4 || opt.ploc_radius == 8)
                  ? (uint32_t)opt.ploc_radius
                  : (uint32_t)PLOC_R_MAX;
  auto alloc = [&](auto** p, size_t count) -> cudaError_t {
    using T = std::remove_pointer_t<std::remove_reference_t<decltype(*p)>>;
    const cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) g->allocs.push_back((void*)*p);
    return e;
  };
  const uint32_t T = g->total, maxw = g->maxw;
  BoundsAcc* acc = nullptr;
  cudaError_t e = cudaSuccess;
  // the cooperative collapse: as many CTAs as can be resident at once
  {
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collapse_all, COLLAPSE_ALL_THREADS, 0)) !=
        cudaSuccess)
      return e;
    g->col_grid = (uint32_t)std::max(1, std::min(per_sm, 4)) * (uint32_t)num_sms_build();
    // and the cooperative PLOC rounds (of the chosen search radius)
    const void* pk = g->radius == 1   ? (const void*)k_ploc_all<1>
                     : g->radius == 2 ? (const void*)k_ploc_all<2>
                     : g->radius == 4 ? (const void*)k_ploc_all<4>
                     : g->radius == 8 ? (const void*)k_ploc_all<8>
                                      : (const void*)k_ploc_all<PLOC_R_MAX>;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pk, PLOC_BLOCK, 0)) != cudaSuccess) return e;
    g->ploc_grid = (uint32_t)std::max(1, std::min(per_sm, 8)) * (uint32_t)num_sms_build();
  }
  if ((e = alloc(&g->d_geoms, ngeoms)) || (e = alloc(&g->plo, T)) || (e = alloc(&g->phi, T)) ||
      (e = alloc(&acc, 1)) || (e = alloc(&g->keys_a, T)) || (e = alloc(&g->keys_b, T)) ||
      (e = alloc(&g->vals_a, T)) || (e = alloc(&g->vals_b, T)) || (e = alloc(&g->hist, sort_hist_entries(T))) ||
      (e = alloc(&g->bnlo, 2 * (size_t)N)) || (e = alloc(&g->bnhi, 2 * (size_t)N)) ||
      (e = alloc(&g->bncnt, 2 * (size_t)N)) || (e = alloc(&g->clo[0], N)) || (e = alloc(&g->clo[1], N)) ||
      (e = alloc(&g->chi[0], N)) || (e = alloc(&g->chi[1], N)) || (e = alloc(&g->cidx[0], N)) ||
      (e = alloc(&g->cidx[1], N)) || (e = alloc(&g->nn, N)) || (e = alloc(&g->bsurv, g->maxb)) ||
      (e = alloc(&g->bmerge, g->maxb)) ||
      (e = alloc(&g->scan_sums, 2 * (size_t)scan_scratch(std::max(g->maxb, maxw)))) ||
      (e = alloc(&g->d_tot, 4)) || (e = alloc(&g->d_root, g->nseg)) || (e = alloc(&g->d_iters, 1)) ||
      (e = alloc(&g->ploc_state, kPlocStateWords)) || (e = alloc(&g->cost, 2 * (size_t)(2 * N))) ||
      (e = alloc(&g->choice, 2 * N)) || (e = alloc(&g->nodes, maxw)) || (e = alloc(&g->tris, N)) ||
      (e = alloc(&g->items[0], maxw)) || (e = alloc(&g->items[1], maxw)) || (e = alloc(&g->kids, 8 * (size_t)maxw)) ||
      (e = alloc(&g->nint, maxw)) || (e = alloc(&g->ntri, maxw)) || (e = alloc(&g->leaf_root, N)) ||
      (e = alloc(&g->d_sah, 2)) || (e = alloc(&g->d_leaves, 1)) || (e = alloc(&g->cstate, kColStateWords)) ||
      (e = alloc(&g->seg_index, g->nseg)) || (e = alloc(&g->status, 1)) ||
      (e = alloc(&g->col_sums, 2 * (size_t)g->col_grid)) || (e = alloc(&g->col_bar, 2)) ||
      (e = alloc(&g->prec, T)) || (e = alloc(&g->ploc_sums, 2 * (size_t)g->ploc_grid)) ||
      (e = alloc(&g->ploc_bar, 2)) || (opt.phase_stamps && (e = alloc(&g->stamps, kBuildPhases + 1)))) {
    graph_build_release(g);
    return e;
  }
  g->acc = acc;
  e = cudaMemcpy(g->d_geoms, h_geoms, sizeof(GeomDesc) * ngeoms, cudaMemcpyHostToDevice);
  // the scans' look-back state starts at zero and every scan leaves it so
  if (e == cudaSuccess)
    e = cudaMemset(g->scan_sums, 0, sizeof(uint32_t) * 2 * scan_scratch(std::max(g->maxb, maxw)));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_os_scatter<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)os_scatter_smem<uint64_t>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_os_scatter<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)os_scatter_smem<uint32_t>());
  if (e != cudaSuccess) graph_build_release(g);
  const size_t smem = kPlocSmallSmem;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ploc_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e;
}


cudaError_t graph_build_enqueue(const GraphBuild& g, cudaStream_t st) {
  const uint32_t T = g.total, N = g.plan.valid_tris, maxw = g.maxw;
  BoundsAcc* acc = reinterpret_cast<BoundsAcc*>(g.acc);
  auto stamp = [&](int k) {
    if (g.stamps) k_phase_stamp<<<1, 1, 0, st>>>(g.stamps, k);
  };
  stamp(0);
  k_acc_init<<<1, 32, 0, st>>>(acc);
  k_primrefs<<<grid_stride_blocks(T), 256, 0, st>>>(g.d_geoms, g.ngeoms, T, g.plo, g.phi, acc, g.prec,
                                                    g.opt.robust ? 1 : 0);
  const bool key32 = g.opt.morton_bits == 30 && !g.opt.segmented;  // 30-bit keys sorted as 32-bit words
  k_morton<<<grid_stride_blocks(T), 256, 0, st>>>(g.plo, g.phi, T, acc, g.keys_a, g.vals_a, g.opt.morton_cube,
                                                  g.opt.segmented ? 1 : 0, g.opt.morton_bits == 30 ? 1 : 0,
                                                  key32 ? 1 : 0);
  note_launches(3);
  stamp(1);
  // all digits of the key width (the ordinary build skips constant ones: the same order)
  uint64_t *ka = g.keys_a, *kb = g.keys_b;
  uint32_t *va = g.vals_a, *vb = g.vals_b;
  // the digits the key width can use: 63-bit keys 8, 30-bit keys 4 (6 with the slot)
  const uint32_t digits = g.opt.morton_bits == 30 ? (g.opt.segmented ? 0x3Fu : 0x0Fu) : 0xFFu;
  if (key32) {
    uint32_t *ka32 = reinterpret_cast<uint32_t*>(ka), *kb32 = reinterpret_cast<uint32_t*>(kb);
    GB_CHECK(onesweep_sort(ka32, va, kb32, vb, T, digits, g.hist, &acc->pad, st));
  } else {
    GB_CHECK(onesweep_sort(ka, va, kb, vb, T, digits, g.hist, &acc->pad, st));
  }
  stamp(2);
  // PLOC: the rounds in one cooperative launch that ends them itself, then the
  // one-CTA finish
  GB_CHECK(cudaMemsetAsync(g.d_root, 0xFF, sizeof(uint32_t) * g.nseg, st));
  GB_CHECK(cudaMemsetAsync(g.d_iters, 0, sizeof(uint32_t), st));
  const uint32_t leaf_max = (uint32_t)std::min(std::max(g.plan.leaf_max, 1), kLeafMaxLimit);
  float4* dp_cost = g.opt.collapse == 1 ? g.cost : nullptr;
  uint2* dp_choice = g.opt.collapse == 1 ? g.choice : nullptr;
  k_ploc_init<<<cdiv(N, 256), 256, 0, st>>>(g.plo, g.phi, va, N, &acc->nvalid, g.bnlo, g.bnhi, g.bncnt, g.cidx[0],
                                            g.clo[0], g.chi[0], g.opt.segmented ? 1 : 0);
  stamp(3);
  k_ploc_state_init<<<1, 32, 0, st>>>(acc, g.ploc_state);
  note_launches(2);
  const uint32_t nbin_cap = 2 * N;
  const PlocBufs pb{{g.clo[0], g.clo[1]}, {g.chi[0], g.chi[1]}, {g.cidx[0], g.cidx[1]}};
  // the rounds above PLOC_SMALL clusters in one cooperative launch, then the one-CTA finish
  GB_CHECK(cudaMemsetAsync(g.ploc_bar, 0, sizeof(GridBarrier), st));
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.ploc_grid);
    cfg.blockDim = dim3(PLOC_BLOCK);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(g.ploc_bar);
    switch (g.radius) {
      case 1: GB_CHECK(cudaLaunchKernelEx(&cfg, k_ploc_all<1>, pb, g.ploc_state, g.nn, g.bsurv, g.bmerge, g.ploc_sums,
                                          g.bnlo, g.bnhi, g.bncnt, nbin_cap, dp_cost, dp_choice, leaf_max, bar,
                                          &acc->pad)); break;
      case 2: GB_CHECK(cudaLaunchKernelEx(&cfg, k_ploc_all<2>, pb, g.ploc_state, g.nn, g.bsurv, g.bmerge, g.ploc_sums,
                                          g.bnlo, g.bnhi, g.bncnt, nbin_cap, dp_cost, dp_choice, leaf_max, bar,
                                          &acc->pad)); break;
      case 4: GB_CHECK(cudaLaunchKernelEx(&cfg, k_ploc_all<4>, pb, g.ploc_state, g.nn, g.bsurv, g.bmerge, g.ploc_sums,
                                          g.bnlo, g.bnhi, g.bncnt, nbin_cap, dp_cost, dp_choice, leaf_max, bar,
                                          &acc->pad)); break;
      case 8: GB_CHECK(cudaLaunchKernelEx(&cfg, k_ploc_all<8>, pb, g.ploc_state, g.nn, g.bsurv, g.bmerge, g.ploc_sums,
                                          g.bnlo, g.bnhi, g.bncnt, nbin_cap, dp_cost, dp_choice, leaf_max, bar,
                                          &acc->pad)); break;
      default: GB_CHECK(cudaLaunchKernelEx(&cfg, k_ploc_all<PLOC_R_MAX>, pb, g.ploc_state, g.nn, g.bsurv, g.bmerge,
                                           g.ploc_sums, g.bnlo, g.bnhi, g.bncnt, nbin_cap, dp_cost, dp_choice,
                                           leaf_max, bar, &acc->pad)); break;
    }
    note_launches(2);
  }
  stamp(4);
  {
    const size_t smem = kPlocSmallSmem;
    k_ploc_small<<<1, PLOC_SMALL_THREADS, smem, st>>>(g.clo[0], g.chi[0], g.cidx[0], g.clo[1], g.chi[1], g.cidx[1],
                                                      g.ploc_state, g.bnlo, g.bnhi, g.bncnt, g.d_root, g.d_iters,
                                                      nbin_cap, &acc->pad, g.nseg, (int)g.radius, dp_cost, dp_choice,
                                                      leaf_max);
    note_launches(1);
  }
  stamp(5);
  // collapse decisions and levels
  BinTree bt{g.bnlo, g.bnhi, g.bncnt, N, leaf_max, (uint32_t)(g.opt.robust != 0), dp_choice};
  GB_CHECK(cudaMemsetAsync(g.leaf_root, 0xFF, sizeof(uint32_t) * N, st));
  GB_CHECK(cudaMemsetAsync(g.d_sah, 0, 2 * sizeof(double), st));
  GB_CHECK(cudaMemsetAsync(g.d_leaves, 0, sizeof(uint32_t), st));
  GB_CHECK(cudaMemsetAsync(g.cstate, 0, sizeof(uint32_t) * kColStateWords, st));
  // collapse levels in a loop the device ends
  stamp(6);
  // all collapse levels in one cooperative launch
  k_collapse_roots<<<1, 1024, 0, st>>>(g.d_root, g.nseg, g.nbin, g.items[0], g.seg_index, g.cstate);
  GB_CHECK(cudaMemsetAsync(g.col_bar, 0, sizeof(GridBarrier), st));
  {
    const ColItems ci{{g.items[0], g.items[1]}};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.col_grid);
    cfg.blockDim = dim3(COLLAPSE_ALL_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CHECK(cudaLaunchKernelEx(&cfg, k_collapse_all, bt, ci, g.cstate, g.kids, g.nint, g.ntri, g.col_sums, g.nodes,
                                g.leaf_root, g.d_sah, g.d_leaves, maxw, N, (uint32_t)kColMaxLevels,
                                reinterpret_cast<GridBarrier*>(g.col_bar), &acc->pad));
  }
  note_launches(2);
  stamp(7);
  k_write_leaves<<<cdiv(N, 256), 256, 0, st>>>(bt, g.d_geoms, g.plo, g.phi, g.leaf_root, N, g.tris, &acc->pad,
                                                g.prec);
  stamp(8);
  k_graph_build_check<<<1, 32, 0, st>>>(acc, g.ploc_state, g.cstate, N, g.status);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t graph_build_result(const GraphBuild& g, const float scene_lo[3], const float scene_hi[3],
                               GraphBuildResult* out, cudaStream_t st) {
  *out = GraphBuildResult{};
  std::vector<uint32_t> col(kColStateWords);
  double sah[2] = {0.0, 0.0};
  GB_CHECK(cudaMemcpyAsync(&out->status, g.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(col.data(), g.cstate, sizeof(uint32_t) * kColStateWords, cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(sah, g.d_sah, sizeof(sah), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(&out->num_leaves, g.d_leaves, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(&out->ploc_rounds, g.ploc_state + kPlocIters, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  BoundsAcc h_acc{};
  GB_CHECK(cudaMemcpyAsync(&h_acc, g.acc, sizeof(BoundsAcc), cudaMemcpyDeviceToHost, st));
  out->roots.assign(g.nseg, kInvalidID);
  if (g.opt.segmented)
    GB_CHECK(cudaMemcpyAsync(out->roots.data(), g.seg_index, sizeof(uint32_t) * g.nseg, cudaMemcpyDeviceToHost, st));
  unsigned long long ts[kBuildPhases + 1] = {};
  if (g.stamps) GB_CHECK(cudaMemcpyAsync(ts, g.stamps, sizeof(ts), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaStreamSynchronize(st));
  if (g.stamps) {
    out->nphases = kBuildPhases;
    for (int k = 0; k < kBuildPhases; k++) out->phase_us[k] = (double)(ts[k + 1] - ts[k]) * 1e-3;
  }
  out->num_nodes = col[kColBase];
  out->depth = std::min<uint32_t>(col[kColDepth], (uint32_t)kColMaxLevels);
  out->level_start.assign(col.begin() + kColLevels, col.begin() + kColLevels + out->depth + 1);
  // the replayed build's own geometry bounds, unless the caller passes the scene's
  for (int d = 0; d < 3; d++) {
    out->lo[d] = scene_lo ? scene_lo[d] : ord2f(h_acc.glo[d]);
    out->hi[d] = scene_hi ? scene_hi[d] : ord2f(h_acc.ghi[d]);
  }
  if (!g.opt.segmented) out->roots.assign(1, 0u);
  const float gx = out->hi[0] - out->lo[0], gy = out->hi[1] - out->lo[1], gz = out->hi[2] - out->lo[2];
  const double Aroot = std::max(0.0, (double)(gx * (gy + gz) + gy * gz));
  out->sah = Aroot > 0 ? (Aroot + sah[0]) / Aroot : 0.0;
  out->sah_exact = Aroot > 0 ? (Aroot + sah[1]) / Aroot : 0.0;
  return cudaSuccess;
}

void graph_build_release(GraphBuild* g) {
  for (void* p : g->allocs) cudaFree(p);
  *g = GraphBuild{};
}

void cached_build_release(CachedBuild* c) {
  if (!c) return;
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  graph_build_release(&c->g);
  delete c;
}

cudaError_t cached_build_create(const GeomDesc* h_geoms, int ngeoms, const BuildOptions& opt,
                                const GraphBuildPlan& plan, cudaStream_t st, CachedBuild** out) {
  *out = nullptr;
  CachedBuild* c = new CachedBuild;
  cudaError_t e = graph_build_prepare(h_geoms, ngeoms, opt, plan, &c->g);
  if (e == cudaSuccess) e = cudaEventCreate(&c->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->e1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const cudaError_t e1 = graph_build_enqueue(c->g, st);
    const cudaError_t e2 = cudaStreamEndCapture(st, &c->graph);
    e = e1 != cudaSuccess ? e1 : e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->exec, c->graph, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cached_build_release(c);
    return e;
  }
  *out = c;
  return cudaSuccess;
}

cudaError_t cached_build_run(CachedBuild* c, const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, DeviceBVH* out,
                             BuildStats* stats) {
  if (!c || ngeoms != c->g.ngeoms) return cudaErrorNotReady;
  // the geometry table is read by the graph's kernels: buffers may have moved
  GB_CHECK(cudaMemcpyAsync(c->g.d_geoms, h_geoms, sizeof(GeomDesc) * ngeoms, cudaMemcpyHostToDevice, st));
  GB_CHECK(cudaEventRecord(c->e0, st));
  GB_CHECK(cudaGraphLaunch(c->exec, st));
  GB_CHECK(cudaEventRecord(c->e1, st));
  GraphBuildResult r;
  GB_CHECK(graph_build_result(c->g, nullptr, nullptr, &r, st));
  if (r.status != 0) return cudaErrorNotReady;
  const uint32_t N = c->g.plan.valid_tris;
  GB_CHECK(cudaMalloc((void**)&out->nodes, (size_t)r.num_nodes * sizeof(WideNode)));
  GB_CHECK(cudaMalloc((void**)&out->tris, (size_t)N * sizeof(TriRecord)));
  GB_CHECK(copy_device(out->nodes, c->g.nodes, (size_t)r.num_nodes * sizeof(WideNode), st));
  GB_CHECK(copy_device(out->tris, c->g.tris, (size_t)N * sizeof(TriRecord), st));
  GB_CHECK(cudaStreamSynchronize(st));
  out->num_nodes = r.num_nodes;
  out->num_tris = N;
  out->depth = r.depth;
  out->robust = c->g.opt.robust != 0;
  for (int d = 0; d < 3; d++) { out->lo[d] = r.lo[d]; out->hi[d] = r.hi[d]; }
  out->level_start = r.level_start;
  out->roots = r.roots;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->e0, c->e1);
  *stats = BuildStats{};
  stats->sah = r.sah;
  stats->sah_exact = r.sah_exact;
  stats->leaf_max = (uint32_t)c->g.plan.leaf_max;
  stats->build_ms = ms;
  stats->num_nodes = r.num_nodes;
  stats->num_leaves = r.num_leaves;
  stats->num_prims = N;
  stats->depth = r.depth;
  stats->ploc_iterations = r.ploc_rounds;
  stats->nphases = r.nphases;
  for (int k = 0; k < kBuildPhases; k++) stats->phase_us[k] = r.phase_us[k];
  return cudaSuccess;
}

// Sorts (key, value) pairs by their low `passes` digits with the builder's
// radix sort.  Device pointers; results in keys/vals (even pass counts).
cudaError_t sort_pairs_passes(uint64_t* keys, uint32_t* vals, uint64_t* kb, uint32_t* vb, uint32_t* hist, uint32_t n,
                              int passes, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (passes < 0 || passes > 8 || (passes & 1)) return cudaErrorInvalidValue;
  uint64_t* ka = keys;
  uint32_t* va = vals;
  return onesweep_sort(ka, va, kb, vb, n, (1u << passes) - 1u, hist, nullptr, st);
}

// onesweep scratch for all 8 digits of n keys
uint32_t sort_hist_entries(uint32_t n) { return (uint32_t)onesweep_scratch_words(n, 8); }

cudaError_t sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint64_t* kb = nullptr;
  uint32_t* vb = nullptr;
  uint32_t* hist = nullptr;
  GB_CHECK(dalloc(&kb, n, st));
  GB_CHECK(dalloc(&vb, n, st));
  GB_CHECK(dalloc(&hist, (size_t)sort_hist_entries(n), st));
  uint64_t* ka = keys;
  uint32_t* va = vals;
  cudaError_t e = onesweep_sort(ka, va, kb, vb, n, 0xFFu, hist, nullptr, st);  // 8 passes: back in keys/vals
  uint32_t serr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&serr, hist + kOsErr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(kb, st);
  cudaFreeAsync(vb, st);
  cudaFreeAsync(hist, st);
  const cudaError_t s2 = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (s2 != cudaSuccess) return s2;
  return serr ? cudaErrorUnknown : cudaSuccess;
}


// ---------------------------------------------------------------------------
// 6. refit: same topology, new vertex positions
//
// Replaces the reference's BVH refitter (kernels/bvh/bvh_refit.cpp:30-247),
// which recomputes node bounds bottom-up for meshes whose topology did not
// change.  Triangle records are re-gathered from the updated vertex buffers,
// then every breadth-first level, deepest first, recomputes its children's
// boxes (leaves from their triangles' vertices, inner children from the box
// the deeper level stored) and requantises them in the node's new frame.
// Slot order and leaf grouping stay as built.
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool refit_tri_vertices(const GeomDesc* __restrict__ geoms,
                                                   const uint32_t* __restrict__ slot_of, uint32_t nslots,
                                                   const TriRecord& rec, float3& p0, float3& p1, float3& p2) {
  const uint32_t primID = __float_as_uint(rec.a.w), geomID = __float_as_uint(rec.b.w);
  if (geomID >= nslots) return false;
  const uint32_t slot = slot_of[geomID];
  if (slot == kInvalidID) return false;
  const GeomDesc g = geoms[slot];
  if (primID >= g.ntris) return false;
  const uint3 t = load_tri(g, primID);
  if (t.x >= g.nverts || t.y >= g.nverts || t.z >= g.nverts) return false;
  p0 = load_vtx(g, t.x);
  p1 = load_vtx(g, t.y);
  p2 = load_vtx(g, t.z);
  return vtx_ok(p0.x, p0.y, p0.z) && vtx_ok(p1.x, p1.y, p1.z) && vtx_ok(p2.x, p2.y, p2.z);
}

// Rewrites every triangle record from the current vertices and stores the
// triangle's box (tri_box[2i] = lo, [2i + 1] = hi) for the node levels.
__global__ void __launch_bounds__(256) k_refit_tris(const GeomDesc* __restrict__ geoms,
                                                    const uint32_t* __restrict__ slot_of, uint32_t nslots,
                                                    TriRecord* __restrict__ tris, uint32_t n, int robust,
                                                    float4* __restrict__ tri_box, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  TriRecord rec = tris[i];
  float3 p0, p1, p2;
  if (!refit_tri_vertices(geoms, slot_of, nslots, rec, p0, p1, p2)) {
    atomicOr(err, kErrBuild);  // the host falls back to a full build
    return;
  }
  const float3 e1 = robust ? p1 : make_float3(__fsub_rn(p0.x, p1.x), __fsub_rn(p0.y, p1.y), __fsub_rn(p0.z, p1.z));
  const float3 e2 = robust ? p2 : make_float3(__fsub_rn(p2.x, p0.x), __fsub_rn(p2.y, p0.y), __fsub_rn(p2.z, p0.z));
  rec.a = make_float4(p0.x, p0.y, p0.z, rec.a.w);
  rec.b = make_float4(e1.x, e1.y, e1.z, rec.b.w);
  rec.c = make_float4(e2.x, e2.y, e2.z, 0.f);
  tris[i] = rec;
  const float3 lo = f3min(f3min(p0, p1), p2), hi = f3max(f3max(p0, p1), p2);
  tri_box[2 * (size_t)i] = make_float4(lo.x, lo.y, lo.z, 0.f);
  tri_box[2 * (size_t)i + 1] = make_float4(hi.x, hi.y, hi.z, 0.f);
}

// Refits wide node k from its children's boxes (inner children: node_box of the
// level below; leaf children: the boxes k_refit_tris stored for their
// triangles, independent loads); returns the node's SAH terms on the decoded
// and on the exact boxes.
__device__ __forceinline__ void refit_node(const float4* __restrict__ tri_box, uint32_t num_tris,
                                           WideNode* __restrict__ nodes, uint32_t num_nodes,
                                           float* __restrict__ node_box, uint32_t k, uint32_t* err, double& sah_out,
                                           double& sahx_out) {
  WideNode node = nodes[k];
  float3 clo[8], chi[8];
  float3 ulo = make_float3(INFINITY, INFINITY, INFINITY), uhi = make_float3(-INFINITY, -INFINITY, -INFINITY);
  uint32_t rank = 0;
  for (int s = 0; s < 8; s++) {
    clo[s] = make_float3(INFINITY, INFINITY, INFINITY);
    chi[s] = make_float3(-INFINITY, -INFINITY, -INFINITY);
    const uint32_t m = node.meta[s];
    if (m == 0) continue;
    if (node.imask >> s & 1u) {
      const uint32_t c = node.child_base + rank++;
      if (c >= num_nodes || c <= k) {
        atomicOr(err, kErrBuild);
        return;
      }
      clo[s] = make_float3(node_box[6 * (size_t)c + 0], node_box[6 * (size_t)c + 1], node_box[6 * (size_t)c + 2]);
      chi[s] = make_float3(node_box[6 * (size_t)c + 3], node_box[6 * (size_t)c + 4], node_box[6 * (size_t)c + 5]);
    } else {
      const uint32_t cnt = ((m >> 5) & 3u) + 1u, first = node.tri_base + (m & 31u);
      if (first + cnt > num_tris) {
        atomicOr(err, kErrBuild);
        return;
      }
#pragma unroll
      for (uint32_t q = 0; q < 4; q++) {
        if (q < cnt) {
          const float4 a = tri_box[2 * (size_t)(first + q)], b = tri_box[2 * (size_t)(first + q) + 1];
          clo[s] = f3min(clo[s], make_float3(a.x, a.y, a.z));
          chi[s] = f3max(chi[s], make_float3(b.x, b.y, b.z));
        }
      }
    }
    ulo = f3min(ulo, clo[s]);
    uhi = f3max(uhi, chi[s]);
  }
  const uint32_t Ex = exp_for(__fsub_ru(uhi.x, ulo.x));
  const uint32_t Ey = exp_for(__fsub_ru(uhi.y, ulo.y));
  const uint32_t Ez = exp_for(__fsub_ru(uhi.z, ulo.z));
  const float sx = __uint_as_float(Ex << 23), sy = __uint_as_float(Ey << 23), sz = __uint_as_float(Ez << 23);
  const float ix = __uint_as_float((254u - Ex) << 23), iy = __uint_as_float((254u - Ey) << 23),
              iz = __uint_as_float((254u - Ez) << 23);
  node.px = ulo.x;
  node.py = ulo.y;
  node.pz = ulo.z;
  node.ex = (uint8_t)Ex;
  node.ey = (uint8_t)Ey;
  node.ez = (uint8_t)Ez;
  double sah = 0.0, sahx = 0.0;
  for (int s = 0; s < 8; s++) {
    if (node.meta[s] == 0) continue;
    const float3 a = clo[s], b = chi[s];
    sahx += (double)fmaxf(0.f, half_area(a, b));
    const float qlx = fminf(fmaxf(floorf(__fsub_rd(a.x, ulo.x) * ix), 0.f), 255.f);
    const float qly = fminf(fmaxf(floorf(__fsub_rd(a.y, ulo.y) * iy), 0.f), 255.f);
    const float qlz = fminf(fmaxf(floorf(__fsub_rd(a.z, ulo.z) * iz), 0.f), 255.f);
    const float qhx = fminf(fmaxf(ceilf(__fsub_ru(b.x, ulo.x) * ix), 0.f), 255.f);
    const float qhy = fminf(fmaxf(ceilf(__fsub_ru(b.y, ulo.y) * iy), 0.f), 255.f);
    const float qhz = fminf(fmaxf(ceilf(__fsub_ru(b.z, ulo.z) * iz), 0.f), 255.f);
    node.qlo_x[s] = (uint8_t)qlx; node.qlo_y[s] = (uint8_t)qly; node.qlo_z[s] = (uint8_t)qlz;
    node.qhi_x[s] = (uint8_t)qhx; node.qhi_y[s] = (uint8_t)qhy; node.qhi_z[s] = (uint8_t)qhz;
    const float3 dlo = make_float3(__fmaf_rd(qlx, sx, ulo.x), __fmaf_rd(qly, sy, ulo.y), __fmaf_rd(qlz, sz, ulo.z));
    const float3 dhi = make_float3(__fmaf_ru(qhx, sx, ulo.x), __fmaf_ru(qhy, sy, ulo.y), __fmaf_ru(qhz, sz, ulo.z));
    sah += (double)fmaxf(0.f, half_area(dlo, dhi));  // leaves of <= 4 triangles: one block each
  }
  nodes[k] = node;
  node_box[6 * (size_t)k + 0] = ulo.x; node_box[6 * (size_t)k + 1] = ulo.y; node_box[6 * (size_t)k + 2] = ulo.z;
  node_box[6 * (size_t)k + 3] = uhi.x; node_box[6 * (size_t)k + 4] = uhi.y; node_box[6 * (size_t)k + 5] = uhi.z;
  sah_out = sah;
  sahx_out = sahx;
}

// One node of the level [begin, end) per thread; SAH sums reduced per CTA.
__global__ void __launch_bounds__(128) k_refit_level(const float4* __restrict__ tri_box, uint32_t num_tris,
                                                     WideNode* __restrict__ nodes, uint32_t num_nodes,
                                                     float* __restrict__ node_box, uint32_t begin, uint32_t end,
                                                     double* sah_acc, uint32_t* err) {
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  double sah = 0.0, sahx = 0.0;
  if (k < end && k < num_nodes) refit_node(tri_box, num_tris, nodes, num_nodes, node_box, k, err, sah, sahx);
  block_add2(sah, sahx, sah_acc);
}

cudaError_t refit_bvh(const GeomDesc* h_geoms, int ngeoms, cudaStream_t st, DeviceBVH* bvh, BuildStats* stats,
                      bool* fallback) {
  *fallback = false;
  if (bvh->num_nodes == 0 || bvh->level_start.size() < 2) {
    *fallback = true;
    return cudaSuccess;
  }
  cudaEvent_t ev0, ev1;
  GB_CHECK(cudaEventCreate(&ev0));
  GB_CHECK(cudaEventCreate(&ev1));
  GB_CHECK(cudaEventRecord(ev0, st));
  uint32_t nslots = 0;
  for (int g = 0; g < ngeoms; g++) nslots = std::max(nslots, h_geoms[g].geomID + 1);
  std::vector<uint32_t> slot_of(std::max(nslots, 1u), kInvalidID);
  for (int g = 0; g < ngeoms; g++) slot_of[h_geoms[g].geomID] = (uint32_t)g;
  GeomDesc* d_geoms = nullptr;
  uint32_t *d_slot = nullptr, *d_err = nullptr;
  float* node_box = nullptr;
  float4* tri_box = nullptr;
  double* d_sah = nullptr;
  GB_CHECK(dalloc(&d_geoms, ngeoms, st));
  GB_CHECK(dalloc(&tri_box, 2 * (size_t)bvh->num_tris, st));
  GB_CHECK(dalloc(&d_slot, slot_of.size(), st));
  GB_CHECK(dalloc(&d_err, 1, st));
  GB_CHECK(dalloc(&node_box, (size_t)6 * bvh->num_nodes, st));
  GB_CHECK(dalloc(&d_sah, 2, st));
  GB_CHECK(cudaMemcpyAsync(d_geoms, h_geoms, sizeof(GeomDesc) * ngeoms, cudaMemcpyHostToDevice, st));
  GB_CHECK(cudaMemcpyAsync(d_slot, slot_of.data(), sizeof(uint32_t) * slot_of.size(), cudaMemcpyHostToDevice, st));
  GB_CHECK(cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st));
  GB_CHECK(cudaMemsetAsync(d_sah, 0, 2 * sizeof(double), st));
  k_refit_tris<<<cdiv(bvh->num_tris, 256), 256, 0, st>>>(d_geoms, d_slot, (uint32_t)slot_of.size(), bvh->tris,
                                                         bvh->num_tris, bvh->robust, tri_box, d_err);
  note_launches(1);
  for (size_t l = bvh->level_start.size() - 1; l-- > 0;) {
    const uint32_t b = bvh->level_start[l], e = bvh->level_start[l + 1];
    if (e <= b) continue;
    k_refit_level<<<cdiv(e - b, 128), 128, 0, st>>>(tri_box, bvh->num_tris, bvh->nodes, bvh->num_nodes, node_box, b,
                                                   e, d_sah, d_err);
    note_launches(1);
  }
  GB_CHECK(cudaGetLastError());
  uint32_t err = 0;
  float root[6];
  double sah_sum[2] = {0.0, 0.0};
  GB_CHECK(cudaMemcpyAsync(&err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(root, node_box, sizeof(root), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaMemcpyAsync(sah_sum, d_sah, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CHECK(cudaEventRecord(ev1, st));
  cudaFreeAsync(d_geoms, st);
  cudaFreeAsync(d_slot, st);
  cudaFreeAsync(d_err, st);
  cudaFreeAsync(node_box, st);
  cudaFreeAsync(tri_box, st);
  cudaFreeAsync(d_sah, st);
  GB_CHECK(cudaStreamSynchronize(st));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (err) {  // a vertex became invalid or the records are inconsistent: rebuild
    *fallback = true;
    return cudaSuccess;
  }
  for (int d = 0; d < 3; d++) {
    bvh->lo[d] = root[d];
    bvh->hi[d] = root[3 + d];
  }
  const float gx = bvh->hi[0] - bvh->lo[0], gy = bvh->hi[1] - bvh->lo[1], gz = bvh->hi[2] - bvh->lo[2];
  const double Aroot = std::max(0.0, (double)(gx * (gy + gz) + gy * gz));
  stats->sah = Aroot > 0 ? (Aroot + sah_sum[0]) / Aroot : 0.0;
  stats->sah_exact = Aroot > 0 ? (Aroot + sah_sum[1]) / Aroot : 0.0;
  stats->build_ms = ms;
  stats->num_nodes = bvh->num_nodes;
  stats->num_prims = bvh->num_tris;
  stats->depth = bvh->depth;
  stats->refit = 1;
  return cudaSuccess;
}

cudaError_t refit_prepare(const GeomDesc* h_geoms, int ngeoms, const DeviceBVH& bvh, RefitScratch* out,
                          cudaStream_t st) {
  *out = RefitScratch{};
  if (bvh.num_nodes == 0 || bvh.level_start.size() < 2) return cudaErrorInvalidValue;
  uint32_t nslots = 0;
  for (int g = 0; g < ngeoms; g++) nslots = std::max(nslots, h_geoms[g].geomID + 1);
  std::vector<uint32_t> slot_of(std::max(nslots, 1u), kInvalidID);
  for (int g = 0; g < ngeoms; g++) slot_of[h_geoms[g].geomID] = (uint32_t)g;
  out->nslots = (uint32_t)slot_of.size();
  GB_CHECK(cudaMalloc(&out->d_geoms, sizeof(GeomDesc) * std::max(ngeoms, 1)));
  GB_CHECK(cudaMalloc(&out->d_slot, sizeof(uint32_t) * slot_of.size()));
  GB_CHECK(cudaMalloc(&out->d_err, sizeof(uint32_t)));
  GB_CHECK(cudaMalloc(&out->node_box, sizeof(float) * 6 * bvh.num_nodes));
  GB_CHECK(cudaMalloc(&out->tri_box, sizeof(float4) * 2 * std::max<size_t>(bvh.num_tris, 1)));
  GB_CHECK(cudaMalloc(&out->d_sah, 2 * sizeof(double)));
  GB_CHECK(cudaMemcpyAsync(out->d_geoms, h_geoms, sizeof(GeomDesc) * ngeoms, cudaMemcpyHostToDevice, st));
  GB_CHECK(cudaMemcpyAsync(out->d_slot, slot_of.data(), sizeof(uint32_t) * slot_of.size(), cudaMemcpyHostToDevice, st));
  GB_CHECK(cudaMemsetAsync(out->d_err, 0, sizeof(uint32_t), st));
  return cudaStreamSynchronize(st);
}

cudaError_t refit_enqueue(const DeviceBVH& bvh, const RefitScratch& s, cudaStream_t st) {
  GB_CHECK(cudaMemsetAsync(s.d_sah, 0, 2 * sizeof(double), st));
  k_refit_tris<<<cdiv(bvh.num_tris, 256), 256, 0, st>>>(s.d_geoms, s.d_slot, s.nslots, bvh.tris, bvh.num_tris,
                                                        bvh.robust, s.tri_box, s.d_err);
  note_launches(1);
  for (size_t l = bvh.level_start.size() - 1; l-- > 0;) {
    const uint32_t b = bvh.level_start[l], e = bvh.level_start[l + 1];
    if (e <= b) continue;
    k_refit_level<<<cdiv(e - b, 128), 128, 0, st>>>(s.tri_box, bvh.num_tris, bvh.nodes, bvh.num_nodes, s.node_box, b,
                                                   e, s.d_sah, s.d_err);
    note_launches(1);
  }
  return cudaGetLastError();
}

void refit_release(RefitScratch* s) {
  void* ptrs[] = {s->d_geoms, s->d_slot, s->d_err, s->node_box, s->tri_box, s->d_sah};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  *s = RefitScratch{};
}

void free_bvh(DeviceBVH* b) {
  if (b->nodes) cudaFree(b->nodes);
  if (b->tris) cudaFree(b->tris);
  b->nodes = nullptr;
  b->tris = nullptr;
  b->num_nodes = b->num_tris = 0;
}

}  // namespace gb
