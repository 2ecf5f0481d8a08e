// gb_trace_kernel.cuh -- the persistent traversal kernel k_trace and the
// device arithmetic it uses, shared by the translation unit of the default
// launch shape (gb_trace.cu) and the one of the tuned shapes (gb_trace_shapes.cu).
//
// Replaces the reference's single-ray / hybrid traversal
// (kernels/bvh/bvh_intersector1.cpp:30-195, bvh_intersector_hybrid.cpp:36-375)
// with persistent CTAs: warps refill idle lanes with rays fetched by one
// atomic, every lane walks the 8-wide quantised BVH with a short stack of node
// groups (child base + hit bits) and postponed triangle groups, visiting
// children in the order given by the ray's direction octant.
//
// Arithmetic that decides hits is the reference's, bit for bit:
//   Moeller-Trumbore  kernels/geometry/triangle_intersector_moeller.h:62-104
//   dot / cross FMA placement  common/math/vec3.h:204-209, math.h:367-373
//   epilog t = T * rcp(absDen)  triangle_intersector_moeller.h:29-35
// with rcp the correctly rounded reciprocal.  Files including this one are
// compiled with --fmad=false and every rounding step is spelled out with
// intrinsics.
//
// The node test only prunes: its slab distances are widened by a bound on
// their rounding error, so a box that contains an accepted intersection is
// never culled.
#pragma once
#include <cuda_runtime.h>

#include "gb_build.h"
#include "gb_common.h"
#include "gb_trace.h"

namespace gb {

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

// stable_triangle_normal (common/math/vec3.h:210-222): per component the
// cross product of (a,b) or (b,c) whose cancelling product is smaller.
__device__ __forceinline__ float3 stable_normal(const float3 a, const float3 b, const float3 c) {
  const float ab_x = __fmul_rn(a.z, b.y), ab_y = __fmul_rn(a.x, b.z), ab_z = __fmul_rn(a.y, b.x);
  const float bc_x = __fmul_rn(b.z, c.y), bc_y = __fmul_rn(b.x, c.z), bc_z = __fmul_rn(b.y, c.x);
  const float3 cab = make_float3(__fmaf_rn(a.y, b.z, -ab_x), __fmaf_rn(a.z, b.x, -ab_y), __fmaf_rn(a.x, b.y, -ab_z));
  const float3 cbc = make_float3(__fmaf_rn(b.y, c.z, -bc_x), __fmaf_rn(b.z, c.x, -bc_y), __fmaf_rn(b.x, c.y, -bc_z));
  return make_float3(fabsf(ab_x) < fabsf(bc_x) ? cab.x : cbc.x, fabsf(ab_y) < fabsf(bc_y) ? cab.y : cbc.y,
                     fabsf(ab_z) < fabsf(bc_z) ? cab.z : cbc.z);
}

__device__ __forceinline__ float3 f3sub(const float3 a, const float3 b) {
  return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float3 f3add(const float3 a, const float3 b) {
  return make_float3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}

// Pluecker test of robust scenes (triangle_intersector_pluecker.h:60-111):
// vertices relative to the origin, edge functions U,V,W accepted within
// ulp*|U+V+W| of zero, t = rcp(2 Ng.D) * 2 v0.Ng inside [tnear, tfar].
__device__ __forceinline__ bool pluecker(const float3 tv0, const float3 tv1, const float3 tv2, const float3 O,
                                         const float3 D, const float tnear, const float tfar, float& U, float& V,
                                         float& UVW, float& t) {
  const float3 v0 = f3sub(tv0, O), v1 = f3sub(tv1, O), v2 = f3sub(tv2, O);
  const float3 e0 = f3sub(v2, v0), e1 = f3sub(v0, v1), e2 = f3sub(v1, v2);
  U = dot3(cross3(e0, f3add(v2, v0)), D);
  V = dot3(cross3(e1, f3add(v0, v1)), D);
  const float W = dot3(cross3(e2, f3add(v1, v2)), D);
  UVW = __fadd_rn(__fadd_rn(U, V), W);
  const float eps = __fmul_rn(1.1920928955078125e-07f, fabsf(UVW));
  if (!((fminf(fminf(U, V), W) >= -eps) | (fmaxf(fmaxf(U, V), W) <= eps))) return false;
  const float3 Ng = stable_normal(e0, e1, e2);
  const float dd = dot3(Ng, D), den = __fadd_rn(dd, dd);
  const float tt = dot3(v0, Ng), T = __fadd_rn(tt, tt);
  t = __fmul_rn(__frcp_rn(den), T);
  return (tnear <= t) & (t <= tfar) & (den != 0.0f);
}

// Geometric normal of a robust-scene hit, as the test computed it.
__device__ __forceinline__ float3 pluecker_normal(const float3 tv0, const float3 tv1, const float3 tv2, const float3 O) {
  const float3 v0 = f3sub(tv0, O), v1 = f3sub(tv1, O), v2 = f3sub(tv2, O);
  return stable_normal(f3sub(v2, v0), f3sub(v0, v1), f3sub(v1, v2));
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

// Three-input minimum / maximum (PTX ISA 8.8, sm_100 and later).
__device__ __forceinline__ float fmax3(const float a, const float b, const float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmin3(const float a, const float b, const float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Byte k of w as the float 1 + bb * 2^-15 (exact): one byte permute puts bb
// in mantissa bits 8..15 under the exponent of 1.0 (0x3F80bb00).
__device__ __forceinline__ float ubyte_f(uint32_t w, uint32_t k) {
  return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | (k << 4)));
}

// Rounding slack of the slab test, relative to (|p - o| + 2^15 s) |1/d|: the
// computed slab distances carry at most ~6 unit roundoffs of that magnitude
// (one each from p - o, the product with 1/d, 1/d itself, the offset a - 2^15 b,
// the FMA and the subtraction of the slack); 8u = 2^-21 covers them with
// margin.  The 2^15 s term widens a box by 2^15 * 8u = 1.6 % of one
// quantisation step.  It is formed from the products the test needs anyway:
// |a| + |B| with a = fl((p - o) / d) >= |p - o| |1/d| (1 - u) and B = 2^15 s / d
// exact, so (|a| + |B|) * 2^-21 (1 + 2^-21), all rounded up, is at least
// (|p - o| + 2^15 s) |1/d| 8u; the floor 2^-144 (32 ulps of the smallest
// subnormal) covers the absolute rounding errors where the products underflow.
constexpr float kSlabEps = 0x1.000008p-21f;  // 2^-21 (1 + 2^-21)
constexpr float kSlabFloor = 0x1p-144f;      // 2^-144

// Intersects the 8 children of `np`.  Child box planes are p + q * 2^e; with
// B = 2^15 * 2^e / d and A = (p - o) / d - B precomputed per node and axis, a
// plane distance is one FMA (1 + q * 2^-15) * B + A = (p - o) / d + q * 2^e / d,
// whose first factor is the plane byte placed in a float's mantissa (no
// integer-to-float conversion or subtraction per plane), widened by the
// rounding slack (near planes down, far planes up) so a box that contains an
// accepted intersection is never culled.  Where B overflows (a 2^55 scale and
// |1/d| near 1e18) the products are NaN and fminf/fmaxf drop that plane, so
// the box only grows.  Returns the node group of hit internal children (bit
// 31 - j set when slot j ^ oct was hit, so the next child to visit is the
// leading one; imask in bits 0..7) and the triangle group of hit leaves (up to
// 32 triangle bits).  perm: the row of the ray's octant in the slot
// permutation table (perm[m] has bit 7 - j set when m has bit j ^ oct).
__device__ __forceinline__ void intersect_node(const WideNode* __restrict__ np, const TRay& r, const float tfar,
                                               uint32_t& g_base, uint32_t& g_bits, uint32_t& t_base,
                                               uint32_t& t_bits, const uint8_t* __restrict__ perm) {
  const uint4* q = reinterpret_cast<const uint4*>(np);
  const uint4 n0 = __ldg(q + 0);
  const uint4 n1 = __ldg(q + 1);
  const uint4 n2 = __ldg(q + 2);
  const uint4 n3 = __ldg(q + 3);
  const uint4 n4 = __ldg(q + 4);
  const uint32_t imask = n0.w >> 24;
  float bx, by, bz, anx, afx, any_, afy, anz, afz;
  {
    const float sx = __uint_as_float((n0.w & 0xFFu) << 23);
    const float sy = __uint_as_float(((n0.w >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((n0.w >> 16) & 0xFFu) << 23);
    const float xo = __fsub_rn(__uint_as_float(n0.x), r.org.x);
    const float yo = __fsub_rn(__uint_as_float(n0.y), r.org.y);
    const float zo = __fsub_rn(__uint_as_float(n0.z), r.org.z);
    const float ax = __fmul_rn(xo, r.rdir.x), ay = __fmul_rn(yo, r.rdir.y), az = __fmul_rn(zo, r.rdir.z);
    // B = 2^15 s / d (exact scaling of s / d by a power of two), A = a - B
    bx = __fmul_rn(sx * 32768.0f, r.rdir.x);
    by = __fmul_rn(sy * 32768.0f, r.rdir.y);
    bz = __fmul_rn(sz * 32768.0f, r.rdir.z);
    const float ax2 = __fsub_rn(ax, bx), ay2 = __fsub_rn(ay, by), az2 = __fsub_rn(az, bz);
    const float ex = __fmaf_ru(__fadd_ru(fabsf(ax), fabsf(bx)), kSlabEps, kSlabFloor);
    const float ey = __fmaf_ru(__fadd_ru(fabsf(ay), fabsf(by)), kSlabEps, kSlabFloor);
    const float ez = __fmaf_ru(__fadd_ru(fabsf(az), fabsf(bz)), kSlabEps, kSlabFloor);
    anx = __fsub_rd(ax2, ex); afx = __fadd_ru(ax2, ex);
    any_ = __fsub_rd(ay2, ey); afy = __fadd_ru(ay2, ey);
    anz = __fsub_rd(az2, ez); afz = __fadd_ru(az2, ez);
  }
  // near / far quantised planes by the ray direction's sign per axis
  const bool px = r.rdir.x >= 0.0f, py = r.rdir.y >= 0.0f, pz = r.rdir.z >= 0.0f;
  const uint32_t nx0 = px ? n2.x : n3.z, nx1 = px ? n2.y : n3.w, fx0 = px ? n3.z : n2.x, fx1 = px ? n3.w : n2.y;
  const uint32_t ny0 = py ? n2.z : n4.x, ny1 = py ? n2.w : n4.y, fy0 = py ? n4.x : n2.z, fy1 = py ? n4.y : n2.w;
  const uint32_t nz0 = pz ? n3.x : n4.z, nz1 = pz ? n3.y : n4.w, fz0 = pz ? n4.z : n3.x, fz1 = pz ? n4.w : n3.y;
  // + 0.0f turns a -0 into +0: the sign test below reads tmax - tmin, which
  // must not be -0 for the equal interval [+0, +0]
  const float tfar_c = fmaxf(tfar, 0.0f) + 0.0f;
  // the per-child work is only the slab test; the masks are built once per
  // node (ALU is the kernel's busiest pipe: this form measured 6-8 % faster
  // than testing validity and expanding leaves per child).  A child is missed
  // when tmax - tmin is negative: its sign bit is shifted into miss8 by one
  // funnel shift (children 7..0, so child s lands in bit s); an overflowed
  // plane pair (inf - inf = NaN, positive) counts as a hit, as tmin <= tmax did.
  // The six plane FMAs of a child run as three packed f32x2 FMAs (x and y near
  // planes, x and y far planes, z near and far), each half rounded exactly as
  // the scalar FMA (1.2 % faster than six scalar FMAs).
  const float2 b_xy = make_float2(bx, by), an_xy = make_float2(anx, any_), af_xy = make_float2(afx, afy);
  const float2 b_zz = make_float2(bz, bz), a_z = make_float2(anz, afz);
  uint32_t miss8 = 0;
#pragma unroll
  for (int s = 7; s >= 0; s--) {
    const uint32_t k = s & 3;
    const float2 tn = __ffma2_rn(make_float2(ubyte_f(s < 4 ? nx0 : nx1, k), ubyte_f(s < 4 ? ny0 : ny1, k)), b_xy, an_xy);
    const float2 tf = __ffma2_rn(make_float2(ubyte_f(s < 4 ? fx0 : fx1, k), ubyte_f(s < 4 ? fy0 : fy1, k)), b_xy, af_xy);
    const float2 tz = __ffma2_rn(make_float2(ubyte_f(s < 4 ? nz0 : nz1, k), ubyte_f(s < 4 ? fz0 : fz1, k)), b_zz, a_z);
    const float tmin = fmax3(tn.x, tn.y, fmaxf(tz.x, r.tnear_c));
    const float tmax = fmin3(tf.x, tf.y, fminf(tz.y, tfar_c));
    miss8 = __funnelshift_l(__float_as_uint(__fsub_rn(tmax, tmin)), miss8, 1);
  }
  // Empty slots hold inverted boxes (lower planes 255, upper planes 0), so they
  // miss without a validity mask (dropping the per-node gather of the meta
  // bytes' valid bits measured 1.6 % faster on the 4M soup, 2 % on the
  // heightfield).  Where overflowed planes make an empty slot count as hit, it
  // is a leaf slot (its imask bit is clear) whose meta byte lacks bit 7, and
  // it adds no triangles.
  const uint32_t hit8 = ~miss8 & 0xFFu;
  // internal children: bit 31 - j of the group is slot j ^ oct (near to far),
  // one lookup in the octant's row of the permutation table
  const uint32_t inner = perm[hit8 & imask];
  // leaves that were hit: their triangle bits (count, offset in the meta byte)
  uint32_t leaf = hit8 & ~imask & 0xFFu, tb = 0;
  const uint64_t meta = (uint64_t)n1.z | ((uint64_t)n1.w << 32);
  while (leaf) {
    const int s = __ffs(leaf) - 1;
    leaf &= leaf - 1u;
    const uint32_t m = (uint32_t)(meta >> (8 * s)) & 0xFFu;
    if (m & 0x80u) tb |= ((2u << ((m >> 5) & 3u)) - 1u) << (m & 31u);
  }
  g_base = n1.x;
  g_bits = (inner << 24) | imask;
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

// Triangle work waits (its group is pushed) while fewer than this percentage of
// the warp's active lanes have some.  0 disables postponing: with the default
// leaves (1 triangle for volumetric scenes, 2 for flat ones) it measured 1-2 %
// faster than 10 % (the best with 2-triangle leaves everywhere), and 20 % was
// slower still.
constexpr int kPostponePct = 0;
constexpr uint32_t kTriGroup = 0x80000000u;  // stack entry flag: triangle group

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

// Persistent traversal.  Every lane owns one ray at a time; a warp refills
// its idle lanes with one atomic once SH::kRefillIdle of them are idle.  Each
// loop iteration an active lane (1) visits one node of its current group,
// (2) tests its pending triangles -- unless few lanes of the warp have
// triangle work, in which case the group is pushed and tested later -- and
// (3) pops the stack when its group is exhausted.
//
// SEEDED: the ray's stack starts as [root, seed3, seed2, seed1] with seed0 as
// the current group, so the proposed subtrees are searched first and the whole
// tree afterwards.  The answer is the plain traversal's: an any-hit ray that
// hits inside a proposed subtree is occluded in the whole tree, and a closest
// hit found there only lowers tfar before the full search, which still tests
// every triangle whose distance can be the minimum.  `seeding` stays set until
// the root group is popped; a ray whose final hit was found while it was set
// counts as a proposal hit.
//
// INST: the scene holds instance leaves (kInstanceLeaf records).  Reaching one,
// the lane pushes the rest of its triangle group and a marker, switches to the
// instanced scene's BVH and transforms its ray into the instance's space the
// way the reference does (kernels/geometry/instance_intersector.cpp:56-69,
// xfmPoint / xfmVector of common/math/affinespace.h:102-103).  The ray
// parameter t is the same in both spaces (affine map, direction not
// renormalised), so tfar carries over.  Popping the marker reloads the world
// ray from its record.  Instances inside instances are skipped (one instance
// level, RTC_MAX_INSTANCE_LEVEL_COUNT = 1).
constexpr uint32_t kInstMarker = 0xFFFFFFFFu;  // stack entry (kInstMarker, 0)

__device__ __forceinline__ void to_instance(const float* __restrict__ m, TRay& r) {
  const float3 o = r.org, d = r.dir;
  r.org = make_float3(__fmaf_rn(o.x, m[0], __fmaf_rn(o.y, m[3], __fmaf_rn(o.z, m[6], m[9]))),
                      __fmaf_rn(o.x, m[1], __fmaf_rn(o.y, m[4], __fmaf_rn(o.z, m[7], m[10]))),
                      __fmaf_rn(o.x, m[2], __fmaf_rn(o.y, m[5], __fmaf_rn(o.z, m[8], m[11]))));
  r.dir = make_float3(__fmaf_rn(d.x, m[0], __fmaf_rn(d.y, m[3], __fmul_rn(d.z, m[6]))),
                      __fmaf_rn(d.x, m[1], __fmaf_rn(d.y, m[4], __fmul_rn(d.z, m[7]))),
                      __fmaf_rn(d.x, m[2], __fmaf_rn(d.y, m[5], __fmul_rn(d.z, m[8]))));
}

// Launch shape (SH, one of kTraceShapes): threads per CTA, the resident CTAs
// per SM whose register budget the plain variants are compiled for (9 x 128
// threads: at most 56 registers a thread; 4 % faster than the 8 that 64
// registers allow on the 4M soup), traversal stack entries kept in shared
// memory, and the number of idle lanes at which a warp fetches new rays.  The
// counting, seeded and instance variants keep their registers (under the same
// bound they would spill 32-150 bytes), and so does the variant with per-ray
// exclusion lists (EXCL: filter callbacks).
template <int THREADS, int CTAS, int SHARED_STACK, int REFILL>
struct Shape {
  static constexpr int kThreads = THREADS, kCtas = CTAS, kSharedStack = SHARED_STACK, kRefillIdle = REFILL;
  static_assert(SHARED_STACK >= 1 && SHARED_STACK <= kStackSize, "shared stack entries");
  static_assert(THREADS % 32 == 0 && REFILL >= 1 && REFILL <= 32, "launch shape");
};
using DefaultShape = Shape<kTraceShapes[0].threads, kTraceShapes[0].ctas, kTraceShapes[0].shared_stack,
                           kTraceShapes[0].refill>;

template <bool ANYHIT, bool COUNT, bool ALIGNED, bool ROBUST, bool SEEDED, bool INST = false, bool EXCL = false,
          class SH = DefaultShape>
__global__ void __launch_bounds__(SH::kThreads, (COUNT || SEEDED || INST || EXCL) ? 1 : SH::kCtas)
    k_trace(TraceParams P) {
  constexpr int kSharedStack = SH::kSharedStack;
  Ctx c{P.nodes, P.tris, P.err, P.max_iters, P.num_nodes, P.num_tris};
  uint32_t cur_inst = kInvalidID, hit_inst = kInvalidID;  // INST: instance being traversed / of the hit
  const int lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t nrays = P.nrays_ptr ? *P.nrays_ptr : P.nrays;
  // stack of node / triangle groups: the first kSharedStack entries live in
  // shared memory ([entry][thread]: a warp's accesses are conflict-free), the
  // deeper ones in local memory.  8 entries measured 2.6 % faster than an
  // all-local stack (4: 2 % slower, 16: as 8 minus 0.5 %).
  uint2 stack[kStackSize];
  int sp = 0;
  __shared__ uint2 s_stack[kSharedStack][SH::kThreads];
  // slot permutation by octant: s_perm[o][m] has bit 7 - j set when m has bit
  // j ^ o (one shared-memory byte load per node instead of a three-stage swap
  // network: 1.4 % faster; the reversed order lets one count of leading zeros
  // find the next child: 0.5 %)
  __shared__ uint8_t s_perm[8][256];
  for (int i = threadIdx.x; i < 8 * 256; i += SH::kThreads) {
    const uint32_t o = i >> 8, m = i & 255;
    uint32_t v = 0;
    for (int j = 0; j < 8; j++) v |= ((m >> (j ^ o)) & 1u) << (7 - j);
    s_perm[o][m] = (uint8_t)v;
  }
  __syncthreads();
  const int stk_tid = threadIdx.x;
  auto push = [&](uint2 e) {
    if (sp < kSharedStack) s_stack[sp][stk_tid] = e; else stack[sp] = e;
    sp++;
  };
  auto pop = [&]() -> uint2 {
    --sp;
    return sp < kSharedStack ? s_stack[sp][stk_tid] : stack[sp];
  };
  bool active = false, exhausted = false, seeding = false;
  char* rec = nullptr;
  TRay r;
  float t_best = 0.f, hu = 0.f, hv = 0.f;
  uint32_t hit_tri = kInvalidID, seed_tri = kInvalidID, g_base = 0, g_bits = 0, t_base = 0, t_bits = 0, iters = 0;
  uint32_t ex_lo = 0, ex_hi = 0;  // EXCL: this ray's range of excluded triangles
  unsigned long long n_nodes = 0, n_tris = 0, n_rays = 0, n_prop = 0;
  for (;;) {
    // ---- refill idle lanes
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
    if (!exhausted && __popc(idle) >= SH::kRefillIdle) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(P.ray_counter, (unsigned)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (base + __popc(idle) >= nrays) exhausted = true;
      if (!active) {
        uint32_t rid = base + __popc(idle & lt_mask);
        if (rid < nrays) {
          if (P.order) rid = __ldg(P.order + rid);  // the record this fetch slot traces
          if (EXCL) {
            ex_lo = __ldg(P.excl_off + rid);
            ex_hi = __ldg(P.excl_off + rid + 1);
          }
          rec = P.rays + (uint64_t)rid * P.stride;
          float tfar;
          load_ray<ALIGNED>(rec, r, tfar);
          // stream semantics: only tnear <= tfar rays are traced; any-hit also
          // skips already occluded rays (bvh_intersector_stream_filters.cpp:75)
          const bool valid = ANYHIT ? ((r.tnear <= tfar) && !(tfar < 0.0f)) : (r.tnear <= tfar);
          // batched queries: the ray's batch (binary search) gives its tree's root
          uint32_t root = 0;
          if (P.batch_root) {
            uint32_t lo = 0, hi = P.nbatches;
            while (hi - lo > 1) {
              const uint32_t mid = (lo + hi) >> 1;
              if (__ldg(P.batch_start + mid) <= rid) lo = mid; else hi = mid;
            }
            root = __ldg(P.batch_root + lo);
          }
          if (INST) {  // a ray that ended inside an instance left the lane in its space
            c.nodes = P.nodes;
            c.tris = P.tris;
            c.num_nodes = P.num_nodes;
            c.num_tris = P.num_tris;
            cur_inst = kInvalidID;
            hit_inst = kInvalidID;
          }
          if (valid && root < c.num_nodes) {
            init_ray(r);
            t_best = tfar;
            hit_tri = kInvalidID;
            g_base = root;
            g_bits = (0x80000000u >> r.oct) | 1u;  // virtual group: the root as internal slot 0
            t_bits = 0;
            sp = 0;
            iters = 0;
            active = true;
            if (SEEDED) {
              // a virtual group (n, root bits) visits node n alone
              const uint4 s4 = P.seeds[rid];
              const uint32_t sd[4] = {s4.x, s4.y, s4.z, s4.w};
              push(make_uint2(g_base, g_bits));
              seed_tri = kInvalidID;
              seeding = false;
              for (int q = 3; q >= 0; q--) {
                if (sd[q] == 0u || sd[q] >= c.num_nodes) continue;
                if (seeding) push(make_uint2(g_base, g_bits));
                g_base = sd[q];
                seeding = true;
              }
              if (!seeding) sp = 0;  // no proposal: plain traversal from the root
            }
            if (COUNT) n_rays++;
          }
        }
      }
    }
    if (!__any_sync(0xFFFFFFFFu, active)) {
      if (exhausted) break;
      continue;
    }
    bool done = false, visited = false;
    if (active && ++iters > c.max_iters) {
      atomicOr(c.err, kErrIterationLimit);
      active = false;
    }
    // ---- (1) one node of the current group
    if (active && t_bits == 0 && (g_bits & 0xFF000000u)) {
      const uint32_t k = __clz(g_bits);  // visiting position of the next child (bit 31 - k)
      g_bits &= ~(0x80000000u >> k);
      const uint32_t slot = k ^ r.oct;
      const uint32_t child = g_base + __popc(g_bits & ((1u << slot) - 1u) & 0xFFu);
      if (g_bits & 0xFF000000u) {
        if (sp < kStackSize) push(make_uint2(g_base, g_bits));
        else { atomicOr(c.err, kErrStackOverflow); active = false; }
      }
      if (active && child >= c.num_nodes) { atomicOr(c.err, kErrBuild); active = false; }
      if (active) {
        if (COUNT) n_nodes++;
        intersect_node(c.nodes + child, r, t_best, g_base, g_bits, t_base, t_bits, s_perm[r.oct]);
        visited = true;
      }
    }
    // ---- (2) triangles, postponed while few lanes have any
    if constexpr (kPostponePct > 0) {
      const uint32_t want = __ballot_sync(0xFFFFFFFFu, active && t_bits != 0);
      const uint32_t act = __ballot_sync(0xFFFFFFFFu, active);
      if (visited && t_bits != 0 && __popc(want) * 100 < __popc(act) * kPostponePct) {
        if (sp < kStackSize) {
          push(make_uint2(t_base | kTriGroup, t_bits));
          t_bits = 0;
        }
      }
    }
    while (active && t_bits) {
      const uint32_t idx = __ffs(t_bits) - 1;
      t_bits &= t_bits - 1;
      const uint32_t ti = t_base + idx;
      if (ti >= c.num_tris) { atomicOr(c.err, kErrBuild); active = false; break; }
      const float4* tp = reinterpret_cast<const float4*>(c.tris + ti);
      const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), d = __ldg(tp + 2);
      if (EXCL) {  // a triangle whose hit a filter callback rejected
        bool skip = false;
        for (uint32_t e = ex_lo; e < ex_hi && !skip; e++) {
          const uint2 x = __ldg(P.excl + e);
          skip = x.x == __float_as_uint(a.w) && x.y == __float_as_uint(b.w);
        }
        if (skip) continue;
      }
      if (INST && __float_as_uint(d.w) == kInstanceLeaf) {
        const uint32_t ii = __float_as_uint(a.w);
        if (cur_inst != kInvalidID) continue;  // nested instance: not traversed
        if (ii >= P.ninsts) { atomicOr(c.err, kErrBuild); active = false; break; }
        const InstDesc* in = P.insts + ii;
        const uint32_t bn = in->num_nodes;
        if (bn == 0) continue;  // empty instanced scene
        if (sp + 3 > kStackSize) { atomicOr(c.err, kErrStackOverflow); active = false; break; }
        // the node group of this visit (its hit internal children) and the rest of this
        // leaf group resume after the instance
        if (g_bits & 0xFF000000u) push(make_uint2(g_base, g_bits));
        if (t_bits) push(make_uint2(t_base | kTriGroup, t_bits));
        push(make_uint2(kInstMarker, 0u));
        t_bits = 0;
        cur_inst = ii;
        c.nodes = in->nodes;
        c.tris = in->tris;
        c.num_nodes = bn;
        c.num_tris = in->num_tris;
        to_instance(in->w2l, r);
        init_ray(r);
        g_base = 0;
        g_bits = (0x80000000u >> r.oct) | 1u;
        break;
      }
      if (COUNT) n_tris++;
      if (ROBUST) {
        float U, V, UVW, t;
        if (pluecker(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(d.x, d.y, d.z), r.org,
                     r.dir, r.tnear, t_best, U, V, UVW, t)) {
          hit_tri = ti;
          if (INST) hit_inst = cur_inst;
          if (SEEDED && seeding) seed_tri = ti;
          if (ANYHIT) { done = true; t_bits = 0; break; }
          // PlueckerHitM::finalize: u,v = U,V * rcp(UVW), 0 when |UVW| < 1e-18
          const float rcp = fabsf(UVW) < kMinRcpInput ? 0.0f : __frcp_rn(UVW);
          t_best = t;
          hu = __fmul_rn(U, rcp);
          hv = __fmul_rn(V, rcp);
        }
      } else {
        float U, V, T, absDen;
        if (moeller(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(d.x, d.y, d.z), r.org, r.dir,
                    r.tnear, t_best, U, V, T, absDen)) {
          hit_tri = ti;
          if (INST) hit_inst = cur_inst;
          if (SEEDED && seeding) seed_tri = ti;
          if (ANYHIT) { done = true; t_bits = 0; break; }
          const float rcp = __frcp_rn(absDen);
          t_best = __fmul_rn(T, rcp);
          hu = __fmul_rn(U, rcp);
          hv = __fmul_rn(V, rcp);
        }
      }
    }
    // ---- (3) next group from the stack, or finish
    if (active && !done && t_bits == 0 && !(g_bits & 0xFF000000u)) {
      if (sp > 0) {
        const uint2 e = pop();
        if (INST && e.x == kInstMarker && e.y == 0u) {
          // leaving the instance: world ray and top-level BVH again
          float unused_tfar;
          load_ray<ALIGNED>(rec, r, unused_tfar);
          init_ray(r);
          c.nodes = P.nodes;
          c.tris = P.tris;
          c.num_nodes = P.num_nodes;
          c.num_tris = P.num_tris;
          cur_inst = kInvalidID;
          g_bits = 0;
          t_bits = 0;
        } else if ((INST || kPostponePct > 0) && (e.x & kTriGroup)) {
          // triangle groups are pushed only by instance entries and by postponing
          t_base = e.x & ~kTriGroup;
          t_bits = e.y;
          g_bits = 0;
        }
        else { g_base = e.x; g_bits = e.y; }
        if (SEEDED && sp == 0) seeding = false;  // the root group: proposals are done
      } else {
        done = true;
      }
    }
    if (active && done) {
      active = false;
      if (SEEDED && hit_tri != kInvalidID && hit_tri == seed_tri) n_prop++;
      if (hit_tri != kInvalidID) {
        if (ANYHIT) {
          *reinterpret_cast<float*>(rec + 32) = -INFINITY;
        } else {
          const TriRecord* htris = (INST && hit_inst != kInvalidID) ? P.insts[hit_inst].tris : P.tris;
          const uint32_t inst_id = (INST && hit_inst != kInvalidID) ? P.insts[hit_inst].geomID : kInvalidID;
          const float4* tp = reinterpret_cast<const float4*>(htris + hit_tri);
          const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), d = __ldg(tp + 2);
          const float3 Ng = ROBUST ? pluecker_normal(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                                                     make_float3(d.x, d.y, d.z), r.org)
                                   : cross3(make_float3(d.x, d.y, d.z), make_float3(b.x, b.y, b.z));
          *reinterpret_cast<float*>(rec + 32) = t_best;
          if (ALIGNED) {
            *reinterpret_cast<float4*>(rec + 48) = make_float4(Ng.x, Ng.y, Ng.z, hu);
            *reinterpret_cast<uint4*>(rec + 64) =
                make_uint4(__float_as_uint(hv), __float_as_uint(a.w), __float_as_uint(b.w), inst_id);
          } else {
            float* f = reinterpret_cast<float*>(rec + 48);
            f[0] = Ng.x; f[1] = Ng.y; f[2] = Ng.z; f[3] = hu; f[4] = hv;
            uint32_t* w = reinterpret_cast<uint32_t*>(rec + 68);
            w[0] = __float_as_uint(a.w); w[1] = __float_as_uint(b.w); w[2] = inst_id;
          }
        }
      }
    }
  }
  if (SEEDED) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n_prop += __shfl_xor_sync(0xFFFFFFFFu, n_prop, o);
    if (lane == 0 && n_prop) atomicAdd(&P.counters->proposal_hits, n_prop);
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


// One launch of k_trace in shape SH: a persistent grid of (SMs x resident CTAs)
// blocks, or fewer when the rays do not fill it.  The occupancy is looked up
// once per instantiation.
template <bool ANYHIT, bool COUNT, bool ALIGNED, bool ROBUST, bool SEEDED, bool INST, bool EXCL, class SH>
static cudaError_t launch_shaped(const TraceParams& P, cudaStream_t st) {
  static int blocks_per_sm = -1, num_sms = 0;
  if (blocks_per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<ANYHIT, COUNT, ALIGNED, ROBUST, SEEDED, INST, EXCL, SH>,
                                                  SH::kThreads, 0);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  uint64_t want = ((uint64_t)P.nrays + SH::kThreads - 1) / SH::kThreads;
  uint64_t grid = (uint64_t)num_sms * blocks_per_sm;
  if (want < grid) grid = want;
  if (grid < 1) grid = 1;
  k_trace<ANYHIT, COUNT, ALIGNED, ROBUST, SEEDED, INST, EXCL, SH><<<(unsigned)grid, SH::kThreads, 0, st>>>(P);
  return cudaGetLastError();
}

}  // namespace gb
