// gb_trace.cu -- closest-hit and any-hit stream traversal behind
// rtcIntersect1M / rtcOccluded1M.
//
// Replaces the reference's single-ray / hybrid traversal
// (kernels/bvh/bvh_intersector1.cpp:30-195, bvh_intersector_hybrid.cpp:36-375)
// with persistent CTAs: each warp fetches 32 rays with one atomic, every lane
// walks the 8-wide quantised BVH with a short stack of node groups
// (child base + hit bits), visiting children in the order given by the ray's
// direction octant.
//
// Arithmetic that decides hits is the reference's, bit for bit:
//   Moeller-Trumbore  kernels/geometry/triangle_intersector_moeller.h:62-104
//   dot / cross FMA placement  common/math/vec3.h:204-209, math.h:367-373
//   epilog t = T * rcp(absDen)  triangle_intersector_moeller.h:29-35
// with rcp the correctly rounded reciprocal.  This file is compiled with
// --fmad=false and every rounding step is spelled out with intrinsics.
//
// The node test only prunes: it decodes each child box rounded outward and
// widens the slab interval by (1 + 2*gamma_3) (Ize, "Robust BVH Ray
// Traversal", JCGT 2013), so a box that contains an accepted intersection
// is never culled.
#include <cuda_runtime.h>

#include "gb_common.h"
#include "gb_trace.h"

namespace gb {

constexpr int TRACE_THREADS = 128;
// 1 + 2*gamma_3 rounded up to float: gamma_3 = 3u/(1-3u), u = 2^-24
constexpr float kSlabGrow = 1.00000036f;
constexpr float kMinRcpInput = 1E-18f;  // common/math/constants.h:31

__device__ __forceinline__ float dot3(const float3 a, const float3 b) {
  return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, __fmul_rn(a.z, b.z)));
}
__device__ __forceinline__ float3 cross3(const float3 a, const float3 b) {
  return make_float3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
                     __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}

// Returns true when the triangle is hit inside (absDen*tnear, absDen*tfar].
__device__ __forceinline__ bool moeller(const float3 v0, const float3 e1, const float3 e2, const float3 O,
                                        const float3 D, const float tnear, const float tfar, float& U, float& V,
                                        float& T, float& absDen) {
  const float3 C = make_float3(__fsub_rn(v0.x, O.x), __fsub_rn(v0.y, O.y), __fsub_rn(v0.z, O.z));
  const float3 R = cross3(C, D);
  const float3 Ng = cross3(e2, e1);
  const float den = dot3(Ng, D);
  absDen = fabsf(den);
  const uint32_t sgn = __float_as_uint(den) & 0x80000000u;
  U = __uint_as_float(__float_as_uint(dot3(R, e2)) ^ sgn);
  V = __uint_as_float(__float_as_uint(dot3(R, e1)) ^ sgn);
  if (!((den != 0.0f) & (U >= 0.0f) & (V >= 0.0f) & (__fadd_rn(U, V) <= absDen))) return false;
  T = __uint_as_float(__float_as_uint(dot3(Ng, C)) ^ sgn);
  return (__fmul_rn(absDen, tnear) < T) & (T <= __fmul_rn(absDen, tfar));
}

struct TRay {
  float3 org, dir, rdir;
  float tnear;     // raw ray tnear (triangle test)
  float tnear_c;   // max(tnear, 0) (node test)
  uint32_t oct;    // bit a set when rdir_a < 0
};

__device__ __forceinline__ float rcp_safe(float d) {
  // zero_fix: |d| < 1e-18 -> +1e-18  (common/math/vec3fa.h:172-177)
  if (fabsf(d) < kMinRcpInput) d = kMinRcpInput;
  return __frcp_rn(d);
}

__device__ __forceinline__ void init_ray(TRay& r) {
  r.rdir = make_float3(rcp_safe(r.dir.x), rcp_safe(r.dir.y), rcp_safe(r.dir.z));
  r.oct = (r.rdir.x < 0.0f ? 1u : 0u) | (r.rdir.y < 0.0f ? 2u : 0u) | (r.rdir.z < 0.0f ? 4u : 0u);
  r.tnear_c = fmaxf(r.tnear, 0.0f);
}

__device__ __forceinline__ uint32_t byte_of(uint2 v, int s) {
  return ((s < 4 ? v.x : v.y) >> (8 * (s & 3))) & 0xFFu;
}

// Intersects the 8 children of `np`.  Returns the node group of hit internal
// children (hit bits 24..31 keyed by slot ^ oct, imask in bits 0..7) and the
// triangle group of hit leaves (24 triangle bits).
__device__ __forceinline__ void intersect_node(const WideNode* __restrict__ np, const TRay& r, const float tfar,
                                               uint32_t& g_base, uint32_t& g_bits, uint32_t& t_base,
                                               uint32_t& t_bits) {
  const uint4* q = reinterpret_cast<const uint4*>(np);
  const uint4 n0 = __ldg(q + 0);
  const uint4 n1 = __ldg(q + 1);
  const uint4 n2 = __ldg(q + 2);
  const uint4 n3 = __ldg(q + 3);
  const uint4 n4 = __ldg(q + 4);
  const float px = __uint_as_float(n0.x), py = __uint_as_float(n0.y), pz = __uint_as_float(n0.z);
  const uint32_t ex = n0.w & 0xFFu, ey = (n0.w >> 8) & 0xFFu, ez = (n0.w >> 16) & 0xFFu, imask = n0.w >> 24;
  const float sx = __uint_as_float(ex << 23), sy = __uint_as_float(ey << 23), sz = __uint_as_float(ez << 23);
  const uint2 meta = make_uint2(n1.z, n1.w);
  const uint2 qlx = make_uint2(n2.x, n2.y), qly = make_uint2(n2.z, n2.w);
  const uint2 qlz = make_uint2(n3.x, n3.y), qhx = make_uint2(n3.z, n3.w);
  const uint2 qhy = make_uint2(n4.x, n4.y), qhz = make_uint2(n4.z, n4.w);
  const float tfar_c = fmaxf(tfar, 0.0f);
  uint32_t hits = 0, tb = 0;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const uint32_t m = byte_of(meta, s);
    // outward-rounded decode of the child box
    const float lx = __fmaf_rd((float)byte_of(qlx, s), sx, px), hx = __fmaf_ru((float)byte_of(qhx, s), sx, px);
    const float ly = __fmaf_rd((float)byte_of(qly, s), sy, py), hy = __fmaf_ru((float)byte_of(qhy, s), sy, py);
    const float lz = __fmaf_rd((float)byte_of(qlz, s), sz, pz), hz = __fmaf_ru((float)byte_of(qhz, s), sz, pz);
    const float t0x = __fmul_rn(__fsub_rn(lx, r.org.x), r.rdir.x), t1x = __fmul_rn(__fsub_rn(hx, r.org.x), r.rdir.x);
    const float t0y = __fmul_rn(__fsub_rn(ly, r.org.y), r.rdir.y), t1y = __fmul_rn(__fsub_rn(hy, r.org.y), r.rdir.y);
    const float t0z = __fmul_rn(__fsub_rn(lz, r.org.z), r.rdir.z), t1z = __fmul_rn(__fsub_rn(hz, r.org.z), r.rdir.z);
    const float tmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), r.tnear_c));
    const float tmax = __fmul_ru(fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tfar_c)),
                                 kSlabGrow);
    if (m != 0 && tmin <= tmax) {
      if (imask >> s & 1u) hits |= 1u << (24 + (s ^ r.oct));
      else tb |= (m >> 5) << (m & 31u);
    }
  }
  g_base = n1.x;
  g_bits = hits | imask;
  t_base = n1.y;
  t_bits = tb;
}

struct Ctx {
  const WideNode* __restrict__ nodes;
  const TriRecord* __restrict__ tris;
  unsigned int* err;
  uint32_t max_iters;
  uint32_t num_nodes;
  uint32_t num_tris;
};

template <bool ANYHIT, bool COUNT>
__device__ __forceinline__ bool traverse(const Ctx& c, const TRay& r, float& t_best, uint32_t& hit_tri, float& hit_u,
                                         float& hit_v, unsigned long long& n_nodes, unsigned long long& n_tris) {
  uint2 stack[kStackSize];
  int sp = 0;
  // virtual group holding the root as internal slot 0
  uint32_t g_base = 0, g_bits = (1u << (24 + r.oct)) | 1u;
  uint32_t t_base = 0, t_bits = 0;
  uint32_t iters = 0;
  for (;;) {
    if (++iters > c.max_iters) {
      atomicOr(c.err, kErrIterationLimit);
      return false;
    }
    if (g_bits & 0xFF000000u) {
      const uint32_t k = __ffs(g_bits >> 24) - 1;
      g_bits &= ~(1u << (24 + k));
      const uint32_t slot = k ^ r.oct;
      const uint32_t child = g_base + __popc(g_bits & ((1u << slot) - 1u) & 0xFFu);
      if (g_bits & 0xFF000000u) {
        if (sp >= kStackSize) {
          atomicOr(c.err, kErrStackOverflow);
          return false;
        }
        stack[sp++] = make_uint2(g_base, g_bits);
      }
      if (child >= c.num_nodes) {  // corrupt BVH: report, never read out of bounds
        atomicOr(c.err, kErrBuild);
        return false;
      }
      if (COUNT) n_nodes++;
      intersect_node(c.nodes + child, r, t_best, g_base, g_bits, t_base, t_bits);
    }
    while (t_bits) {
      const uint32_t idx = __ffs(t_bits) - 1;
      t_bits &= t_bits - 1;
      const uint32_t ti = t_base + idx;
      if (ti >= c.num_tris) {
        atomicOr(c.err, kErrBuild);
        return false;
      }
      const float4* tp = reinterpret_cast<const float4*>(c.tris + ti);
      const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), d = __ldg(tp + 2);
      if (COUNT) n_tris++;
      float U, V, T, absDen;
      if (moeller(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(d.x, d.y, d.z), r.org, r.dir,
                  r.tnear, t_best, U, V, T, absDen)) {
        if (ANYHIT) {
          hit_tri = ti;
          return true;
        }
        const float rcp = __frcp_rn(absDen);
        t_best = __fmul_rn(T, rcp);
        hit_u = __fmul_rn(U, rcp);
        hit_v = __fmul_rn(V, rcp);
        hit_tri = ti;
      }
    }
    if (!(g_bits & 0xFF000000u)) {
      if (sp == 0) break;
      const uint2 e = stack[--sp];
      g_base = e.x;
      g_bits = e.y;
    }
  }
  return hit_tri != kInvalidID;
}

template <bool ALIGNED>
__device__ __forceinline__ void load_ray(const char* p, TRay& r, float& tfar) {
  if (ALIGNED) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    const float4 b = *reinterpret_cast<const float4*>(p + 16);
    tfar = *reinterpret_cast<const float*>(p + 32);
    r.org = make_float3(a.x, a.y, a.z);
    r.tnear = a.w;
    r.dir = make_float3(b.x, b.y, b.z);
  } else {
    const float* f = reinterpret_cast<const float*>(p);
    r.org = make_float3(f[0], f[1], f[2]);
    r.tnear = f[3];
    r.dir = make_float3(f[4], f[5], f[6]);
    tfar = f[8];
  }
}

template <bool ANYHIT, bool COUNT, bool ALIGNED>
__global__ void __launch_bounds__(TRACE_THREADS) k_trace(TraceParams P) {
  Ctx c{P.nodes, P.tris, P.err, P.max_iters, P.num_nodes, P.num_tris};
  const int lane = threadIdx.x & 31;
  unsigned long long n_nodes = 0, n_tris = 0, n_rays = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(P.ray_counter, 32u);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base >= P.nrays) break;
    const uint32_t rid = base + lane;
    if (rid >= P.nrays) continue;
    char* rec = P.rays + (uint64_t)rid * P.stride;
    TRay r;
    float tfar;
    load_ray<ALIGNED>(rec, r, tfar);
    if (ANYHIT) {
      // bvh_intersector_stream_filters.cpp:75: skip invalid and already occluded rays
      if (!(r.tnear <= tfar) || tfar < 0.0f) continue;
    } else {
      if (!(r.tnear <= tfar)) continue;
    }
    if (COUNT) n_rays++;
    init_ray(r);
    float t_best = tfar, u = 0.f, v = 0.f;
    uint32_t hit_tri = kInvalidID;
    const bool hit = traverse<ANYHIT, COUNT>(c, r, t_best, hit_tri, u, v, n_nodes, n_tris);
    if (!hit) continue;
    if (ANYHIT) {
      *reinterpret_cast<float*>(rec + 32) = -INFINITY;
      continue;
    }
    const float4* tp = reinterpret_cast<const float4*>(c.tris + hit_tri);
    const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), d = __ldg(tp + 2);
    const float3 Ng = cross3(make_float3(d.x, d.y, d.z), make_float3(b.x, b.y, b.z));
    *reinterpret_cast<float*>(rec + 32) = t_best;
    if (ALIGNED) {
      *reinterpret_cast<float4*>(rec + 48) = make_float4(Ng.x, Ng.y, Ng.z, u);
      *reinterpret_cast<uint4*>(rec + 64) =
          make_uint4(__float_as_uint(v), __float_as_uint(a.w), __float_as_uint(b.w), kInvalidID);
    } else {
      float* f = reinterpret_cast<float*>(rec + 48);
      f[0] = Ng.x; f[1] = Ng.y; f[2] = Ng.z; f[3] = u; f[4] = v;
      uint32_t* w = reinterpret_cast<uint32_t*>(rec + 68);
      w[0] = __float_as_uint(a.w); w[1] = __float_as_uint(b.w); w[2] = kInvalidID;
    }
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      n_nodes += __shfl_xor_sync(0xFFFFFFFFu, n_nodes, o);
      n_tris += __shfl_xor_sync(0xFFFFFFFFu, n_tris, o);
      n_rays += __shfl_xor_sync(0xFFFFFFFFu, n_rays, o);
    }
    if (lane == 0) {
      atomicAdd(&P.counters->nodes, n_nodes);
      atomicAdd(&P.counters->tris, n_tris);
      atomicAdd(&P.counters->rays, n_rays);
    }
  }
}

template <bool ANYHIT, bool COUNT, bool ALIGNED>
static cudaError_t launch_one(const TraceParams& P, cudaStream_t st) {
  static int blocks_per_sm = -1, num_sms = 0;
  if (blocks_per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<ANYHIT, COUNT, ALIGNED>, TRACE_THREADS, 0);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  uint64_t want = ((uint64_t)P.nrays + TRACE_THREADS - 1) / TRACE_THREADS;
  uint64_t grid = (uint64_t)num_sms * blocks_per_sm;
  if (want < grid) grid = want;
  if (grid < 1) grid = 1;
  k_trace<ANYHIT, COUNT, ALIGNED><<<(unsigned)grid, TRACE_THREADS, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_trace(const TraceParams& P, bool anyhit, bool count, cudaStream_t st) {
  const bool aligned = ((uintptr_t)P.rays % 16 == 0) && (P.stride % 16 == 0);
  if (anyhit) {
    if (count) return aligned ? launch_one<true, true, true>(P, st) : launch_one<true, true, false>(P, st);
    return aligned ? launch_one<true, false, true>(P, st) : launch_one<true, false, false>(P, st);
  }
  if (count) return aligned ? launch_one<false, true, true>(P, st) : launch_one<false, true, false>(P, st);
  return aligned ? launch_one<false, false, true>(P, st) : launch_one<false, false, false>(P, st);
}

}  // namespace gb
