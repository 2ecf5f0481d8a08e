// gb_learned.cu -- the learned hit proposer: hash-grid encoding, MLP training
// (forward, backward, Adam) and fused top-4 inference.  See gb_learned.h for
// the network and the parameter layout.
//
// Tensor-core products use mma.sync m16n8k16 with BF16 operands and FP32
// accumulators.  Rounding points (the only places values become BF16): the
// encoded features, each hidden activation after bias + ReLU, the softmax
// gradient and each back-propagated hidden gradient.  Every other value is
// FP32; this file is compiled with --fmad=false so the encoder's arithmetic is
// exactly the one a CPU restatement computes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>

#include "gb_build.h"
#include "gb_launch.h"
#include "gb_learned.h"

namespace gb {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint16_t f2bf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }
__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
  return (uint32_t)f2bf(lo) | ((uint32_t)f2bf(hi) << 16);
}
__device__ __forceinline__ uint32_t lds32(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// ---------------------------------------------------------------------------
// Hash-grid encoding
// ---------------------------------------------------------------------------

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// Point of level l in [0,1]^3: the normalised origin (levels 0-7) or the unit
// direction mapped from [-1,1]^3 (levels 8-15).
__device__ __forceinline__ void level_point(const char* rec, const GridSpec& g, int l, float q[3]) {
  const float* f = reinterpret_cast<const float*>(rec);
  if (l < kOriginLevels) {
#pragma unroll
    for (int a = 0; a < 3; a++) q[a] = clamp01(__fmul_rn(__fsub_rn(f[a], g.lo[a]), g.scale[a]));
  } else {
    const float dx = f[4], dy = f[5], dz = f[6];
    const float n2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    const float inv = n2 > 0.0f ? __fdiv_rn(1.0f, __fsqrt_rn(n2)) : 0.0f;
    const float d[3] = {dx, dy, dz};
#pragma unroll
    for (int a = 0; a < 3; a++) q[a] = clamp01(__fmul_rn(__fadd_rn(__fmul_rn(d[a], inv), 1.0f), 0.5f));
  }
}

__device__ __forceinline__ uint32_t level_res(int l) {
  return l < kOriginLevels ? (16u << l) : (4u << (l - kOriginLevels));
}

// Dense index while the level's (R+1)^3 vertices fit the table, else the
// spatial hash of Teschner et al. (2003) with the primes instant-NGP uses.
__device__ __forceinline__ uint32_t grid_index(uint32_t R, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t n = R + 1;
  if ((uint64_t)n * n * n <= kTableSize) return x + n * (y + n * z);
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (kTableSize - 1u);
}

struct Cell {
  uint32_t i[3];
  float f[3];
};

__device__ __forceinline__ Cell level_cell(const float q[3], uint32_t R) {
  Cell c;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float p = __fmul_rn(q[a], (float)R);
    uint32_t ii = (uint32_t)floorf(p);
    if (ii > R - 1) ii = R - 1;
    c.i[a] = ii;
    c.f[a] = __fsub_rn(p, (float)ii);
  }
  return c;
}

// Corner k (bit 0: x, bit 1: y, bit 2: z) of a cell: table entry and weight.
__device__ __forceinline__ void corner(const Cell& c, uint32_t R, int k, uint32_t& e, float& w) {
  const uint32_t x = c.i[0] + (k & 1), y = c.i[1] + ((k >> 1) & 1), z = c.i[2] + ((k >> 2) & 1);
  const float wx = (k & 1) ? c.f[0] : __fsub_rn(1.0f, c.f[0]);
  const float wy = (k & 2) ? c.f[1] : __fsub_rn(1.0f, c.f[1]);
  const float wz = (k & 4) ? c.f[2] : __fsub_rn(1.0f, c.f[2]);
  w = __fmul_rn(__fmul_rn(wx, wy), wz);
  e = grid_index(R, x, y, z);
}

// Two features of level l (trilinear interpolation of the BF16 table, FP32 sums
// in corner order), packed as BF16.
__device__ __forceinline__ uint32_t encode_level(const uint16_t* __restrict__ Pb, const char* rec, const GridSpec& g,
                                                 int l) {
  float q[3];
  level_point(rec, g, l, q);
  const uint32_t R = level_res(l);
  const Cell c = level_cell(q, R);
  const uint32_t* tab = reinterpret_cast<const uint32_t*>(Pb + kOffTable) + (size_t)l * kTableSize;
  float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t e;
    float w;
    corner(c, R, k, e, w);
    const uint32_t pr = __ldg(tab + e);
    s0 = __fadd_rn(s0, __fmul_rn(w, bf2f((uint16_t)(pr & 0xFFFFu))));
    s1 = __fadd_rn(s1, __fmul_rn(w, bf2f((uint16_t)(pr >> 16))));
  }
  return pack_bf2(s0, s1);
}

__global__ void k_encode_fwd(const char* rays, uint64_t stride, const uint32_t* idx, uint32_t B, GridSpec g,
                             const uint16_t* __restrict__ Pb, uint16_t* X0) {
  const uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= (uint64_t)B * kLevels) return;
  const uint32_t b = (uint32_t)(it / kLevels), l = (uint32_t)(it % kLevels);
  const uint32_t r = idx ? idx[b] : b;
  reinterpret_cast<uint32_t*>(X0)[(size_t)b * (kIn / 2) + l] = encode_level(Pb, rays + (uint64_t)r * stride, g, l);
}

__global__ void k_encode_bwd(const char* rays, uint64_t stride, const uint32_t* idx, uint32_t B, GridSpec g,
                             const float* __restrict__ dX0, float* G) {
  const uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= (uint64_t)B * kLevels) return;
  const uint32_t b = (uint32_t)(it / kLevels), l = (uint32_t)(it % kLevels);
  const uint32_t r = idx ? idx[b] : b;
  const float g0 = dX0[(size_t)b * kIn + 2 * l], g1 = dX0[(size_t)b * kIn + 2 * l + 1];
  float q[3];
  level_point(rays + (uint64_t)r * stride, g, l, q);
  const uint32_t R = level_res(l);
  const Cell c = level_cell(q, R);
  float* tab = G + kOffTable + (size_t)l * kTableSize * kFeat;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t e;
    float w;
    corner(c, R, k, e, w);
    atomicAdd(tab + 2 * (size_t)e, __fmul_rn(w, g0));
    atomicAdd(tab + 2 * (size_t)e + 1, __fmul_rn(w, g1));
  }
}

// ---------------------------------------------------------------------------
// Training: generic BF16 GEMM (FP32 out) and element-wise kernels
// ---------------------------------------------------------------------------

// C[m][n] (+)= sum_k A(m,k) B(k,n) with A(m,k) = A[m*sam + k*sak] and
// B(k,n) = B[k*sbk + n*sbn]; 64x64 tiles, 4 warps of 32x32, K in steps of 32,
// blockIdx.z splits K (atomic accumulation into a zeroed C).
constexpr int kGT = 64, kGK = 32, kGLd = kGK + 8;

__global__ void __launch_bounds__(128) k_gemm(int M, int N, int K, const uint16_t* __restrict__ A, long sam,
                                              long sak, const uint16_t* __restrict__ B, long sbk, long sbn,
                                              float* C, long ldc, int kps, int atomic) {
  __shared__ __align__(16) uint16_t As[kGT * kGLd];
  __shared__ __align__(16) uint16_t Bs[kGT * kGLd];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.x * kGT, n0 = blockIdx.y * kGT;
  const int kb = blockIdx.z * kps, ke = min(K, kb + kps);
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += kGK) {
#pragma unroll 4
    for (int e = tid; e < kGT * kGK; e += 128) {
      int m, k;
      if (sak == 1) { m = e >> 5; k = e & 31; } else { m = e & 63; k = e >> 6; }
      const int gm = m0 + m, gk = k0 + k;
      As[m * kGLd + k] = (gm < M && gk < ke) ? A[(long)gm * sam + (long)gk * sak] : (uint16_t)0;
      int n, kk;
      if (sbk == 1) { n = e >> 5; kk = e & 31; } else { n = e & 63; kk = e >> 6; }
      const int gn = n0 + n, gk2 = k0 + kk;
      Bs[n * kGLd + kk] = (gn < N && gk2 < ke) ? B[(long)gk2 * sbk + (long)gn * sbn] : (uint16_t)0;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kGK; ks += 16) {
      uint32_t a[2][4];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const uint16_t* ap = As + (wm + i * 16) * kGLd + ks + 2 * t;
        a[i][0] = lds32(ap + g * kGLd);
        a[i][1] = lds32(ap + (g + 8) * kGLd);
        a[i][2] = lds32(ap + g * kGLd + 8);
        a[i][3] = lds32(ap + (g + 8) * kGLd + 8);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint16_t* bp = Bs + (wn + j * 8 + g) * kGLd + ks + 2 * t;
        const uint32_t b0 = lds32(bp), b1 = lds32(bp + 8);
        mma_bf16(acc[0][j], a[0], b0, b1);
        mma_bf16(acc[1][j], a[1], b0, b1);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int m = m0 + wm + i * 16 + g + ((q & 2) ? 8 : 0);
        const int n = n0 + wn + j * 8 + 2 * t + (q & 1);
        if (m < M && n < N) {
          if (atomic) atomicAdd(C + (long)m * ldc + n, acc[i][j][q]);
          else C[(long)m * ldc + n] = acc[i][j][q];
        }
      }
}

void gemm(int M, int N, int K, const uint16_t* A, long sam, long sak, const uint16_t* B, long sbk, long sbn, float* C,
          long ldc, bool atomic, int splits, cudaStream_t st) {
  int kps = (K + splits - 1) / splits;
  kps = (kps + kGK - 1) / kGK * kGK;
  splits = (K + kps - 1) / kps;
  dim3 grid((M + kGT - 1) / kGT, (N + kGT - 1) / kGT, splits);
  k_gemm<<<grid, 128, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, kps, atomic ? 1 : 0);
}

__global__ void k_bias_relu(const float* __restrict__ Z, const float* __restrict__ bias, uint16_t* H, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  H[i] = f2bf(fmaxf(__fadd_rn(Z[i], bias[i % kHidden]), 0.0f));
}

__global__ void k_relu_bwd(const float* __restrict__ dH, const uint16_t* __restrict__ H, uint16_t* dZ, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dZ[i] = bf2f(H[i]) > 0.0f ? f2bf(dH[i]) : (uint16_t)0;
}

// db[c] += sum over rows of dZ[row][c] (BF16 values, FP32 sums).
__global__ void k_colsum(const uint16_t* __restrict__ dZ, int N, uint32_t B, float* db) {
  __shared__ float part[8][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.0f;
  if (c < N)
    for (uint32_t r = blockIdx.y * 8 + threadIdx.y; r < B; r += gridDim.y * 8) s += bf2f(dZ[(size_t)r * N + c]);
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < N) {
    float tsum = 0.0f;
    for (int y = 0; y < 8; y++) tsum += part[y][threadIdx.x];
    atomicAdd(db + c, tsum);
  }
}

void colsum(const uint16_t* dZ, int N, uint32_t B, float* db, cudaStream_t st) {
  dim3 grid((N + 31) / 32, std::max(1u, std::min(256u, B / 256)));
  k_colsum<<<grid, dim3(32, 8), 0, st>>>(dZ, N, B, db);
}

// Softmax cross-entropy over the 4096 logits of a row (one warp per row):
// dZ4 = (softmax(z) - onehot(y)) / B in BF16; rows with y < 0 get zero.
// acc: [0] loss sum, [1] rows whose label ranks first, [2] ... in the top 4,
// [3] labelled rows.
__global__ void k_softmax_xent(const float* __restrict__ Z4, const float* __restrict__ b4,
                               const int32_t* __restrict__ labels, const uint32_t* __restrict__ idx, uint32_t B,
                               float inv_B, uint16_t* dZ4, float* acc) {
  const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= B) return;
  const float* z = Z4 + (size_t)row * kTreelets;
  uint16_t* d = dZ4 + (size_t)row * kTreelets;
  const int32_t y = labels[idx ? idx[row] : row];
  float mx = -INFINITY;
  for (int j = lane * 4; j < kTreelets; j += 128) {
    const float4 v = *reinterpret_cast<const float4*>(z + j);
    mx = fmaxf(mx, fmaxf(fmaxf(v.x + b4[j], v.y + b4[j + 1]), fmaxf(v.z + b4[j + 2], v.w + b4[j + 3])));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
  float s = 0.0f;
  for (int j = lane * 4; j < kTreelets; j += 128) {
    const float4 v = *reinterpret_cast<const float4*>(z + j);
    s += expf(v.x + b4[j] - mx) + expf(v.y + b4[j + 1] - mx) + expf(v.z + b4[j + 2] - mx) + expf(v.w + b4[j + 3] - mx);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
  const float lse = mx + logf(s);
  if (y < 0 || y >= kTreelets) {
    for (int j = lane; j < kTreelets; j += 32) d[j] = 0;
    return;
  }
  const float zy = z[y] + b4[y];
  int above = 0;
  for (int j = lane; j < kTreelets; j += 32) {
    const float zj = z[j] + b4[j];
    above += (zj > zy) || (zj == zy && j < y);
    const float p = expf(zj - lse);
    d[j] = f2bf((p - (j == y ? 1.0f : 0.0f)) * inv_B);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) above += __shfl_xor_sync(kFull, above, o);
  if (lane == 0) {
    atomicAdd(acc + 0, lse - zy);
    atomicAdd(acc + 1, above == 0 ? 1.0f : 0.0f);
    atomicAdd(acc + 2, above < kTopK ? 1.0f : 0.0f);
    atomicAdd(acc + 3, 1.0f);
  }
}

__global__ void k_adam(float* P, const float* __restrict__ G, float* m, float* v, uint16_t* Pb, uint64_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float gi = G[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float p = P[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    P[i] = p;
    Pb[i] = f2bf(p);
  }
}

__global__ void k_to_bf16(const float* __restrict__ P, uint16_t* Pb, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    Pb[i] = f2bf(P[i]);
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}

// Uniform initialisation: table entries in +-1e-4, weights in +-sqrt(6 / fan_in)
// (He et al. 2015 for ReLU layers), biases zero.
__global__ void k_init_params(float* P, uint32_t seed) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float u = (float)(hash32((uint32_t)i * 0x9E3779B9u ^ hash32(seed + (uint32_t)(i >> 32))) >> 8) *
                        (1.0f / 16777216.0f) * 2.0f - 1.0f;
    float scale;
    if (i < kOffW1) scale = 1e-4f;
    else if (i < kOffB1) scale = sqrtf(6.0f / kIn);
    else if (i < kOffW2) scale = 0.0f;
    else if (i < kOffB2) scale = sqrtf(6.0f / kHidden);
    else if (i < kOffW3) scale = 0.0f;
    else if (i < kOffB3) scale = sqrtf(6.0f / kHidden);
    else if (i < kOffW4) scale = 0.0f;
    else if (i < kOffB4) scale = sqrtf(6.0f / kHidden);
    else scale = 0.0f;
    P[i] = u * scale;
  }
}

// Treelet label of each logged closest-hit record; -1 for misses and for
// triangles outside every treelet.  count[0] += labelled records.
__global__ void k_label(const char* recs, uint64_t stride, uint32_t M, const uint32_t* __restrict__ prim_treelet,
                        uint32_t nprims, const uint32_t* __restrict__ geom_prefix, uint32_t ngeom, int32_t* labels,
                        unsigned int* count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const uint32_t* w = reinterpret_cast<const uint32_t*>(recs + (uint64_t)i * stride);
  const uint32_t prim = w[17], geom = w[18];
  int32_t lab = -1;
  if (geom < ngeom) {
    const uint32_t base = geom_prefix[geom];
    if (base != kInvalidID && (uint64_t)base + prim < nprims) {
      const uint32_t tl = prim_treelet[base + prim];
      if (tl != kInvalidID) lab = (int32_t)tl;
    }
  }
  labels[i] = lab;
  const unsigned n = __popc(__ballot_sync(__activemask(), lab >= 0));
  if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && n) atomicAdd(count, n);
}

__global__ void k_sort_keys(const int32_t* __restrict__ labels, uint32_t M, uint64_t* keys, uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  keys[i] = labels[i] < 0 ? 1ull : 0ull;
  vals[i] = i;
}

__global__ void k_shuffle_keys(uint32_t n, uint32_t seed, uint64_t* keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = ((uint64_t)hash32(i ^ hash32(seed)) << 32) | hash32(i * 0x85EBCA6Bu + seed);
}

// ---------------------------------------------------------------------------
// Inference: one CTA of 8 warps proposes for tiles of 128 rays.  The hidden
// layers run from shared memory; the 4096x64 output weights stream through a
// double-buffered shared-memory stage (128 rows per stage, cp.async), and each
// thread keeps the running top 4 of the columns it owns for its two rows.
// ---------------------------------------------------------------------------

constexpr int kPW = 8;
constexpr int kPRays = kPW * 16;
constexpr int kCN = 128;
constexpr int kLdX = kIn + 8;
constexpr int kLdH = kHidden + 8;

struct PropSmem {
  uint16_t x[kPRays * kLdX];
  uint16_t h[kPRays * kLdH];
  uint16_t w1[kHidden * kLdX];
  uint16_t w2[kHidden * kLdH];
  uint16_t w3[kHidden * kLdH];
  uint16_t w4[2][kCN * kLdH];
  float b[3][kHidden];
};
static_assert(offsetof(PropSmem, w4) % 16 == 0, "cp.async destination alignment");
static_assert((kLdH * 2) % 16 == 0, "row pitch of the streamed stage");

template <int K, int LDA>
__device__ __forceinline__ void hidden_layer(const uint16_t* A, const uint16_t* W, int ldw, const float* bias,
                                             uint16_t* out, int g, int t) {
  uint32_t a[K / 16][4];
#pragma unroll
  for (int ks = 0; ks < K / 16; ks++) {
    const uint16_t* ap = A + ks * 16 + 2 * t;
    a[ks][0] = lds32(ap + g * LDA);
    a[ks][1] = lds32(ap + (g + 8) * LDA);
    a[ks][2] = lds32(ap + g * LDA + 8);
    a[ks][3] = lds32(ap + (g + 8) * LDA + 8);
  }
  __syncwarp();  // `out` may alias A
#pragma unroll
  for (int nt = 0; nt < kHidden / 8; nt++) {
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++) {
      const uint16_t* wr = W + (nt * 8 + g) * ldw + ks * 16 + 2 * t;
      mma_bf16(c, a[ks], lds32(wr), lds32(wr + 8));
    }
    const int col = nt * 8 + 2 * t;
    const float b0 = bias[col], b1 = bias[col + 1];
    *reinterpret_cast<uint32_t*>(out + g * kLdH + col) =
        pack_bf2(fmaxf(__fadd_rn(c[0], b0), 0.0f), fmaxf(__fadd_rn(c[1], b1), 0.0f));
    *reinterpret_cast<uint32_t*>(out + (g + 8) * kLdH + col) =
        pack_bf2(fmaxf(__fadd_rn(c[2], b0), 0.0f), fmaxf(__fadd_rn(c[3], b1), 0.0f));
  }
}

// Sorted (descending) running top 4; columns arrive in increasing order, so a
// tie keeps the lower column.
__device__ __forceinline__ void top4_insert(float (&v)[4], int (&ix)[4], float x, int i) {
  if (!(x > v[3])) return;
  if (x > v[2]) {
    v[3] = v[2]; ix[3] = ix[2];
    if (x > v[1]) {
      v[2] = v[1]; ix[2] = ix[1];
      if (x > v[0]) { v[1] = v[0]; ix[1] = ix[0]; v[0] = x; ix[0] = i; }
      else { v[1] = x; ix[1] = i; }
    } else { v[2] = x; ix[2] = i; }
  } else { v[3] = x; ix[3] = i; }
}

// Top 4 of the four lanes (t = 0..3) that share a row; ties to the lower column.
__device__ __forceinline__ void merge4(float (&v)[4], int (&ix)[4], int (&out)[4]) {
#pragma unroll
  for (int r = 0; r < 4; r++) {
    float bv = v[0];
    int bi = ix[0];
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      const float ov = __shfl_xor_sync(kFull, bv, o);
      const int oi = __shfl_xor_sync(kFull, bi, o);
      if (ov > bv || (ov == bv && (unsigned)oi < (unsigned)bi)) { bv = ov; bi = oi; }
    }
    out[r] = bi;
    if (bi >= 0 && bi == ix[0]) {
      v[0] = v[1]; ix[0] = ix[1]; v[1] = v[2]; ix[1] = ix[2]; v[2] = v[3]; ix[2] = ix[3];
      v[3] = -INFINITY; ix[3] = -1;
    }
  }
}

__device__ __forceinline__ void stage_w4(uint16_t* dst, const uint16_t* W4, int ch, int tid) {
#pragma unroll
  for (int i = tid; i < kCN * 8; i += kPW * 32) {
    const int row = i >> 3, part = i & 7;
    cp_async16(dst + row * kLdH + part * 8, W4 + ((size_t)ch * kCN + row) * kHidden + part * 8);
  }
}

__global__ void __launch_bounds__(kPW * 32, 2)
    k_propose(const char* rays, uint64_t stride, uint32_t M, const uint32_t* d_count, GridSpec grid,
              const uint16_t* __restrict__ Pb, const float* __restrict__ P,
              const uint32_t* __restrict__ node_of_treelet, int ntl, uint4* seeds, uint32_t* treelets) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PropSmem& S = *reinterpret_cast<PropSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  for (int i = tid; i < kHidden * kIn / 2; i += kPW * 32) {
    const int o = (2 * i) / kIn, k = (2 * i) % kIn;
    *reinterpret_cast<uint32_t*>(S.w1 + o * kLdX + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW1)[i];
  }
  for (int i = tid; i < kHidden * kHidden / 2; i += kPW * 32) {
    const int o = (2 * i) / kHidden, k = (2 * i) % kHidden;
    *reinterpret_cast<uint32_t*>(S.w2 + o * kLdH + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW2)[i];
    *reinterpret_cast<uint32_t*>(S.w3 + o * kLdH + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW3)[i];
  }
  for (int i = tid; i < 3 * kHidden; i += kPW * 32) {
    const size_t off = i < kHidden ? kOffB1 : (i < 2 * kHidden ? kOffB2 : kOffB3);
    S.b[i / kHidden][i % kHidden] = P[off + i % kHidden];
  }
  __syncthreads();
  const uint16_t* W4 = Pb + kOffW4;
  const float* b4 = P + kOffB4;
  if (d_count) M = min(M, *d_count);
  const uint32_t ntiles = (M + kPRays - 1) / kPRays;
  constexpr int kChunks = kTreelets / kCN;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t r0 = tile * kPRays;
    stage_w4(S.w4[0], W4, 0, tid);
    cp_async_commit();
    for (int it = tid; it < kPRays * kLevels; it += kPW * 32) {
      const int rr = it / kLevels, l = it % kLevels;
      const uint32_t rid = r0 + rr;
      const uint32_t pk = rid < M ? encode_level(Pb, rays + (uint64_t)rid * stride, grid, l) : 0u;
      *reinterpret_cast<uint32_t*>(S.x + rr * kLdX + 2 * l) = pk;
    }
    __syncthreads();
    uint16_t* hrow = S.h + warp * 16 * kLdH;
    hidden_layer<kIn, kLdX>(S.x + warp * 16 * kLdX, S.w1, kLdX, S.b[0], hrow, g, t);
    __syncwarp();
    hidden_layer<kHidden, kLdH>(hrow, S.w2, kLdH, S.b[1], hrow, g, t);
    __syncwarp();
    hidden_layer<kHidden, kLdH>(hrow, S.w3, kLdH, S.b[2], hrow, g, t);
    __syncwarp();
    uint32_t a[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
      const uint16_t* ap = hrow + ks * 16 + 2 * t;
      a[ks][0] = lds32(ap + g * kLdH);
      a[ks][1] = lds32(ap + (g + 8) * kLdH);
      a[ks][2] = lds32(ap + g * kLdH + 8);
      a[ks][3] = lds32(ap + (g + 8) * kLdH + 8);
    }
    float va[4], vb[4];
    int ia[4], ib[4];
#pragma unroll
    for (int q = 0; q < 4; q++) { va[q] = vb[q] = -INFINITY; ia[q] = ib[q] = -1; }
    for (int ch = 0; ch < kChunks; ch++) {
      if (ch + 1 < kChunks) {
        stage_w4(S.w4[(ch + 1) & 1], W4, ch + 1, tid);
        cp_async_commit();
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      const uint16_t* w = S.w4[ch & 1];
#pragma unroll 4
      for (int nt = 0; nt < kCN / 8; nt++) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
          const uint16_t* wr = w + (nt * 8 + g) * kLdH + ks * 16 + 2 * t;
          mma_bf16(c, a[ks], lds32(wr), lds32(wr + 8));
        }
        const int col = ch * kCN + nt * 8 + 2 * t;
        if (col < ntl) {
          const float bb = __ldg(b4 + col);
          top4_insert(va, ia, __fadd_rn(c[0], bb), col);
          top4_insert(vb, ib, __fadd_rn(c[2], bb), col);
        }
        if (col + 1 < ntl) {
          const float bb = __ldg(b4 + col + 1);
          top4_insert(va, ia, __fadd_rn(c[1], bb), col + 1);
          top4_insert(vb, ib, __fadd_rn(c[3], bb), col + 1);
        }
      }
      __syncthreads();
    }
    int oa[4], ob[4];
    merge4(va, ia, oa);
    merge4(vb, ib, ob);
    if (t == 0) {
      const uint32_t ra = r0 + warp * 16 + g, rb = ra + 8;
      auto node = [&](int tl) { return tl >= 0 ? __ldg(node_of_treelet + tl) : kInvalidID; };
      if (ra < M) {
        if (seeds) seeds[ra] = make_uint4(node(oa[0]), node(oa[1]), node(oa[2]), node(oa[3]));
        if (treelets)
          reinterpret_cast<uint4*>(treelets)[ra] = make_uint4((uint32_t)oa[0], (uint32_t)oa[1], (uint32_t)oa[2], (uint32_t)oa[3]);
      }
      if (rb < M) {
        if (seeds) seeds[rb] = make_uint4(node(ob[0]), node(ob[1]), node(ob[2]), node(ob[3]));
        if (treelets)
          reinterpret_cast<uint4*>(treelets)[rb] = make_uint4((uint32_t)ob[0], (uint32_t)ob[1], (uint32_t)ob[2], (uint32_t)ob[3]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05).  One CTA per SM
// holds all 512 TMEM columns: two 128x256 FP32 accumulators.  Warps 0-15
// encode the rays, run the hidden layers and scan the accumulators; warp 16
// (the producer) streams the output weights and issues the MMAs.  Hand-offs
// are mbarriers, never CTA-wide barriers:
//   tma_bar[s]  stage s holds a weight chunk (bulk copy complete)
//   mma_bar[b]  accumulator b holds a chunk's logits (tcgen05.commit)
//   epi_bar[b]  accumulator b has been read by all 16 scanning warps
//   a_bar       the tile's last hidden layer is in the A operand
// The output weights live in global memory in the UMMA canonical K-major
// layout with K = 80: the 64 weights, then the bias split into two BF16 parts
// (hi, lo) that the A operand multiplies by ones, so the MMA adds the bias;
// unused treelets carry a -inf bias.  Each 256-treelet chunk (40 KB) is one
// contiguous block for one bulk copy.  In the scan, warp w reads TMEM lanes
// 32 (w % 4) .. +31 (its rows) and the column quarter w / 4 of each chunk; the
// four partial top-4 lists of a row are merged through shared memory at the
// end of the tile.  Every mbarrier wait is bounded; on a timeout the kernel
// sets kErrIterationLimit and stops.
// ---------------------------------------------------------------------------

constexpr int kTcScanWarps = 16;
constexpr int kTcScanThreads = kTcScanWarps * 32;
constexpr int kTcThreads = kTcScanThreads + 32;     // + the producer warp
constexpr int kTcRays = 128;                        // UMMA M
constexpr int kTcN = 256;                           // UMMA N: treelets per chunk
constexpr int kTcK = kHidden + 16;                  // 64 weights + bias (hi, lo) + zero padding
constexpr int kTcChunks = kTreelets / kTcN;         // 16
constexpr uint32_t kTcChunkBytes = kTcN * kTcK * 2; // 40 KB
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kTcStages = 2;                   // weight chunks in flight
// kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A and
// B (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcRays >> 4) << 24);

struct TcSmem {
  uint16_t w4[kTcStages][kTcN * kTcK];  // streamed output weights + bias (UMMA layout)
  uint16_t a[2][kTcRays * kTcK];    // last hidden layers of two tiles + ones (UMMA layout)
  float mv[kTcRays][4][4];          // partial top-4 per row and column quarter
  int mi[kTcRays][4][4];
  unsigned long long tma_bar[kTcStages];
  unsigned long long a_bar[2];
  unsigned long long mma_bar[2];
  unsigned long long epi_bar[2];
  uint32_t tmem_base;
  uint32_t fail;
};
static_assert(offsetof(TcSmem, a) % 1024 == 0, "operand tiles start on 1 KB boundaries");
constexpr uint32_t kTcTileBytes = kTcRays * kTcK * 2;  // one A tile, 20 KB
static_assert(offsetof(TcSmem, tma_bar) % 8 == 0, "mbarrier alignment");

// element offset of (row, k) in the UMMA K-major core-matrix layout (K = 80:
// ten 8x8 core matrices per 8-row group, 128 B apart along K, 1280 B along rows)
__device__ __forceinline__ uint32_t umma_off(uint32_t row, uint32_t k) {
  return (row >> 3) * (kTcK * 8) + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t umma_desc(const void* smem) {
  constexpr uint64_t kLbo = 128, kSbo = kTcK * 16;
  return (uint64_t)((smem_u32(smem) >> 4) & 0x3FFFu) | (((kLbo >> 4) & 0x3FFFu) << 16) |
         (((kSbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Waits for the phase with the given parity; gives up after kWaitNs of wall
// time (a try_wait may itself suspend for a while, so the bound is on time,
// not on the number of tries).
constexpr uint64_t kWaitNs = 2000000000ull;
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, uint32_t parity) {
  const uint32_t a = smem_u32(b);
  uint64_t t0 = 0;
  for (uint32_t i = 0;; i++) {
    uint32_t ok = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i == 0) t0 = global_ns();
    else if ((i & 63) == 0 && global_ns() - t0 > kWaitNs) return false;
  }
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// two 32-column loads, one wait
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// barrier among the scanning warps only (the producer warp does not take part)
__device__ __forceinline__ void scan_sync() { asm volatile("bar.sync 1, %0;\n" ::"n"(kTcScanThreads) : "memory"); }

__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

// The streamed weights in the UMMA layout: chunk c (treelets 256c..256c+255)
// is a contiguous block; k 64 / 65 hold the bias as BF16 hi + lo parts, k 66-79
// are zero.  Refreshed whenever the BF16 mirror changes.
__global__ void k_permute_w4(const uint16_t* __restrict__ Pb, const float* __restrict__ P, int ntl,
                             uint16_t* __restrict__ w4p) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // one 16-byte row piece per thread
  if (i >= kTreelets * (kTcK / 8)) return;
  const uint32_t n = i / (kTcK / 8), kc = i % (kTcK / 8);
  const uint32_t c = n / kTcN, r = n % kTcN;
  uint4 v;
  if (kc < kHidden / 8) {
    v = *reinterpret_cast<const uint4*>(Pb + kOffW4 + (size_t)n * kHidden + kc * 8);
  } else if (kc == kHidden / 8) {
    const float b = P[kOffB4 + n];
    uint32_t hi = bf16_bits(-INFINITY), lo = 0;
    if ((int)n < ntl) {
      hi = bf16_bits(b);
      lo = bf16_bits(b - __uint_as_float(hi << 16));
    }
    v = make_uint4(hi | (lo << 16), 0u, 0u, 0u);
  } else {
    v = make_uint4(0u, 0u, 0u, 0u);
  }
  *reinterpret_cast<uint4*>(w4p + (size_t)c * kTcN * kTcK + umma_off(r, kc * 8)) = v;
}

// Encoder and hidden layers for tiles of 128 rays (8 warps, 16 rows each):
// each tile's last hidden layer is written, with the bias ones, in the UMMA
// layout k_propose_tc bulk-copies (tile t at H + t * kTcRays * kTcK).
struct HidSmem {
  uint16_t x[kTcRays * kLdX];
  uint16_t h[kTcRays * kLdH];
  uint16_t w1[kHidden * kLdX];
  uint16_t w2[kHidden * kLdH];
  uint16_t w3[kHidden * kLdH];
  float b[3][kHidden];
};

__global__ void __launch_bounds__(256) k_propose_hidden(const char* rays, uint64_t stride, uint32_t M,
                                                        const uint32_t* d_count, GridSpec grid,
                                                        const uint16_t* __restrict__ Pb, const float* __restrict__ P,
                                                        uint16_t* __restrict__ H) {
  extern __shared__ __align__(16) unsigned char hid_smem_raw[];
  HidSmem& S = *reinterpret_cast<HidSmem*>(hid_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  for (int i = tid; i < kHidden * kIn / 2; i += 256) {
    const int o = (2 * i) / kIn, k = (2 * i) % kIn;
    *reinterpret_cast<uint32_t*>(S.w1 + o * kLdX + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW1)[i];
  }
  for (int i = tid; i < kHidden * kHidden / 2; i += 256) {
    const int o = (2 * i) / kHidden, k = (2 * i) % kHidden;
    *reinterpret_cast<uint32_t*>(S.w2 + o * kLdH + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW2)[i];
    *reinterpret_cast<uint32_t*>(S.w3 + o * kLdH + k) = reinterpret_cast<const uint32_t*>(Pb + kOffW3)[i];
  }
  for (int i = tid; i < 3 * kHidden; i += 256) {
    const size_t off = i < kHidden ? kOffB1 : (i < 2 * kHidden ? kOffB2 : kOffB3);
    S.b[i / kHidden][i % kHidden] = P[off + i % kHidden];
  }
  __syncthreads();
  if (d_count) M = min(M, *d_count);
  const uint32_t ntiles = (M + kTcRays - 1) / kTcRays;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t r0 = tile * kTcRays;
    for (int it = tid; it < kTcRays * kLevels; it += 256) {
      const int rr = it / kLevels, l = it % kLevels;
      const uint32_t rid = r0 + rr;
      const uint32_t pk = rid < M ? encode_level(Pb, rays + (uint64_t)rid * stride, grid, l) : 0u;
      *reinterpret_cast<uint32_t*>(S.x + rr * kLdX + 2 * l) = pk;
    }
    __syncthreads();
    {
      const int row0 = warp * 16;
      uint16_t* hrow = S.h + row0 * kLdH;
      hidden_layer<kIn, kLdX>(S.x + row0 * kLdX, S.w1, kLdX, S.b[0], hrow, g, t);
      __syncwarp();
      hidden_layer<kHidden, kLdH>(hrow, S.w2, kLdH, S.b[1], hrow, g, t);
      __syncwarp();
      hidden_layer<kHidden, kLdH>(hrow, S.w3, kLdH, S.b[2], hrow, g, t);
    }
    __syncthreads();
    // 16-byte pieces in memory order: row group, K core matrix, row within the group
    uint4* dst = reinterpret_cast<uint4*>(H + (size_t)tile * kTcRays * kTcK);
    for (int pc = tid; pc < kTcRays * (kTcK / 8); pc += 256) {
      const int grp = pc / (kTcK), rem = pc % (kTcK), kc = rem >> 3, r = grp * 8 + (rem & 7);
      uint4 v;
      if (kc < kHidden / 8) v = *reinterpret_cast<const uint4*>(S.h + r * kLdH + kc * 8);
      else if (kc == kHidden / 8) v = make_uint4(0x3F803F80u, 0u, 0u, 0u);  // 1.0, 1.0 in BF16
      else v = make_uint4(0u, 0u, 0u, 0u);
      dst[pc] = v;
    }
  }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_propose_tc(uint32_t M, const uint32_t* d_count, const uint16_t* __restrict__ H,
                 const uint16_t* __restrict__ W4p, const uint32_t* __restrict__ node_of_treelet, uint4* seeds,
                 uint32_t* treelets, uint32_t* err) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(tc_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool producer = warp == kTcScanWarps;
  if (producer) {
    if (lane == 0) {
      for (uint32_t b = 0; b < kTcStages; b++) mbar_init(&S.tma_bar[b], 1);
      for (int b = 0; b < 2; b++) {
        mbar_init(&S.a_bar[b], 1);
        mbar_init(&S.mma_bar[b], 1);
        mbar_init(&S.epi_bar[b], kTcScanWarps);
      }
      S.fail = 0;
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem_base)),
                 "n"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;
  if (d_count) M = min(M, *d_count);
  const uint32_t ntiles = (M + kTcRays - 1) / kTcRays;
  const uint32_t my_tiles = blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
  const uint32_t total_chunks = my_tiles * kTcChunks;
  auto tile_src = [&](uint32_t k) { return H + (size_t)(blockIdx.x + k * gridDim.x) * kTcRays * kTcK; };

  // phases started on each barrier by the producer (bulk copies and MMA
  // commits): after a failure the producer waits for the last one of each, so
  // that no copy or MMA is in flight when the CTA frees its shared memory and TMEM
  uint32_t n_w[kTcStages], n_a[2] = {0u, 0u}, n_m[2] = {0u, 0u};
  for (uint32_t q = 0; q < kTcStages; q++) n_w[q] = 0u;
  if (producer) {
    if (lane == 0 && total_chunks > 0) {
      bool ok = true;
      bulk_load(S.a[0], tile_src(0), kTcTileBytes, &S.a_bar[0]);
      n_a[0]++;
      if (my_tiles > 1) bulk_load(S.a[1], tile_src(1), kTcTileBytes, &S.a_bar[1]), n_a[1]++;
      for (uint32_t q = 0; q < kTcStages && q < total_chunks; q++) {
        bulk_load(S.w4[q], W4p + (size_t)(q % kTcChunks) * kTcN * kTcK, kTcChunkBytes, &S.tma_bar[q]);
        n_w[q]++;
      }
      for (uint32_t gc = 0; gc < total_chunks && ok; gc++) {
        const uint32_t k = gc / kTcChunks, c = gc % kTcChunks, s = gc & 1u, ab = k & 1u;
        const uint32_t ws = gc % kTcStages;
        if (c == 0) ok = mbar_wait(&S.a_bar[ab], (k >> 1) & 1u);                       // A operand of tile k
        if (ok) ok = mbar_wait(&S.tma_bar[ws], (gc / kTcStages) & 1u);                 // weights of chunk gc
        if (ok && gc >= 2) ok = mbar_wait(&S.epi_bar[s], ((gc - 2) >> 1) & 1u);         // accumulator s read
        if (!ok) break;
        tc_fence_after();
        const uint64_t adesc0 = umma_desc(S.a[ab]), bdesc0 = umma_desc(S.w4[ws]);
#pragma unroll
        for (int ks = 0; ks < kTcK / 16; ks++)  // +256 B per K step: two core matrices
          umma_bf16(tmem + s * kTcN, adesc0 + (uint64_t)(ks * 16), bdesc0 + (uint64_t)(ks * 16), ks > 0);
        umma_commit(&S.mma_bar[s]);
        n_m[s]++;
        // stage (gc - 1) % kTcStages is free once chunk gc - 1's MMAs are done: it
        // takes chunk gc - 1 + kTcStages
        if (gc >= 1 && gc - 1 + kTcStages < total_chunks) {
          if (!(ok = mbar_wait(&S.mma_bar[(gc - 1) & 1u], ((gc - 1) >> 1) & 1u))) break;
          const uint32_t nc = gc - 1 + kTcStages;
          bulk_load(S.w4[nc % kTcStages], W4p + (size_t)(nc % kTcChunks) * kTcN * kTcK, kTcChunkBytes,
                    &S.tma_bar[nc % kTcStages]);
          n_w[nc % kTcStages]++;
        }
        // after the last MMA of tile k, its A buffer takes tile k + 2
        if (c == kTcChunks - 1 && k + 2 < my_tiles) {
          if (!(ok = mbar_wait(&S.mma_bar[s], (gc >> 1) & 1u))) break;
          bulk_load(S.a[ab], tile_src(k + 2), kTcTileBytes, &S.a_bar[ab]);
          n_a[ab]++;
        }
      }
      if (!ok) {
        *(volatile uint32_t*)&S.fail = 1u;
        atomicOr(err, kErrIterationLimit);
      }
    }
    __syncwarp();
  } else {
    uint32_t gc = 0;
    const int quarter = warp >> 2;
    for (uint32_t k = 0; k < my_tiles; k++) {
      const uint32_t tile = blockIdx.x + k * gridDim.x;
      float v[4];
      int ix[4];
#pragma unroll
      for (int q = 0; q < 4; q++) { v[q] = -INFINITY; ix[q] = -1; }
      bool ok = true;
      for (int c = 0; c < kTcChunks; c++, gc++) {
        const uint32_t s = gc & 1u;
        if (!mbar_wait(&S.mma_bar[s], (gc >> 1) & 1u)) { ok = false; break; }
        tc_fence_after();
        const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + s * kTcN + (uint32_t)quarter * 64;
        uint32_t acc0[32], acc1[32];
        tmem_ld32(taddr, acc0);
        tmem_ld32(taddr + 32, acc1);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.epi_bar[s]);  // this warp is done with accumulator s
        const int col0 = c * kTcN + quarter * 64;
        float m0 = __uint_as_float(acc0[0]), m1 = __uint_as_float(acc1[0]);
#pragma unroll
        for (int q = 1; q < 32; q++) {
          m0 = fmaxf(m0, __uint_as_float(acc0[q]));
          m1 = fmaxf(m1, __uint_as_float(acc1[q]));
        }
        if (m0 > v[3]) {
#pragma unroll
          for (int q = 0; q < 32; q++) top4_insert(v, ix, __uint_as_float(acc0[q]), col0 + q);
        }
        if (m1 > v[3]) {
#pragma unroll
          for (int q = 0; q < 32; q++) top4_insert(v, ix, __uint_as_float(acc1[q]), col0 + 32 + q);
        }
      }
      // the failure decision is taken by all scanning warps together, after a
      // barrier they all reach (a warp that timed out left its chunk loop early)
      volatile uint32_t* fail_flag = &S.fail;
      if (!ok) *fail_flag = 1u;
      {  // merge the four column quarters of each row (ties to the lower column)
        const int row = (warp & 3) * 32 + lane;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          S.mv[row][quarter][q] = v[q];
          S.mi[row][quarter][q] = ix[q];
        }
      }
      scan_sync();
      if (*fail_flag) {
        if (tid == 0) atomicOr(err, kErrIterationLimit);
        break;
      }
      if (tid < kTcRays) {
        float bv[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
        int bi[4] = {-1, -1, -1, -1};
        for (int qq = 0; qq < 4; qq++)
          for (int q = 0; q < 4; q++) {
            const float x = S.mv[tid][qq][q];
            const int i = S.mi[tid][qq][q];
            if (i < 0) continue;
            int pos = 4;
            while (pos > 0 && (x > bv[pos - 1] || (x == bv[pos - 1] && (unsigned)i < (unsigned)bi[pos - 1]))) pos--;
            if (pos < 4) {
              for (int m = 3; m > pos; m--) { bv[m] = bv[m - 1]; bi[m] = bi[m - 1]; }
              bv[pos] = x;
              bi[pos] = i;
            }
          }
        const uint32_t rid = tile * kTcRays + tid;
        if (rid < M) {
          auto node = [&](int tl) { return tl >= 0 ? __ldg(node_of_treelet + tl) : kInvalidID; };
          if (seeds) seeds[rid] = make_uint4(node(bi[0]), node(bi[1]), node(bi[2]), node(bi[3]));
          if (treelets)
            reinterpret_cast<uint4*>(treelets)[rid] =
                make_uint4((uint32_t)bi[0], (uint32_t)bi[1], (uint32_t)bi[2], (uint32_t)bi[3]);
        }
      }
      scan_sync();  // S.mv is written again by the next tile
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (producer) {
    // after a failure, copies and MMAs still in flight complete before the CTA
    // ends (each wait is bounded; phase n - 1 is the last one started)
    if (lane == 0 && *(volatile uint32_t*)&S.fail) {
      for (uint32_t q = 0; q < kTcStages; q++)
        if (n_w[q]) mbar_wait(&S.tma_bar[q], (n_w[q] - 1u) & 1u);
      for (int q = 0; q < 2; q++) {
        if (n_a[q]) mbar_wait(&S.a_bar[q], (n_a[q] - 1u) & 1u);
        if (n_m[q]) mbar_wait(&S.mma_bar[q], (n_m[q] - 1u) & 1u);
      }
    }
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(kTmemCols) : "memory");
  }
}

inline unsigned blocks_for(uint64_t n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

}  // namespace

// ---------------------------------------------------------------------------
// Proposer
// ---------------------------------------------------------------------------

#define GB_TRY(x)                               \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return e_;           \
  } while (0)

cudaError_t Proposer::init(const std::vector<uint32_t>& node_of_treelet, const std::vector<uint32_t>& prim_treelet,
                           const std::vector<uint32_t>& geom_prefix, const GridSpec& g, uint32_t seed,
                           cudaStream_t st) {
  release();
  // set once, outside any stream capture that later launches the kernel
  GB_TRY(cudaFuncSetAttribute(k_propose, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PropSmem)));
  num_treelets = (uint32_t)std::min<size_t>(node_of_treelet.size(), kTreelets);
  num_prims = (uint32_t)prim_treelet.size();
  num_geom_ids_ = (uint32_t)geom_prefix.size();
  grid = g;
  stats = TrainStats{};
  GB_TRY(cudaMalloc(&P_, kNumParams * sizeof(float)));
  GB_TRY(cudaMalloc(&Pb_, kNumParams * sizeof(uint16_t)));
  GB_TRY(cudaMalloc(&G_, kNumParams * sizeof(float)));
  GB_TRY(cudaMalloc(&m_, kNumParams * sizeof(float)));
  GB_TRY(cudaMalloc(&v_, kNumParams * sizeof(float)));
  GB_TRY(cudaMalloc(&node_of_treelet_, kTreelets * sizeof(uint32_t)));
  GB_TRY(cudaMalloc(&prim_treelet_, std::max<size_t>(1, num_prims) * sizeof(uint32_t)));
  GB_TRY(cudaMalloc(&geom_prefix_, std::max<size_t>(1, num_geom_ids_) * sizeof(uint32_t)));
  GB_TRY(cudaMalloc(&acc_, 16 * sizeof(float)));
  GB_TRY(cudaMalloc(&W4p_, (size_t)kTreelets * kTcK * sizeof(uint16_t)));
  GB_TRY(cudaMalloc(&err_, sizeof(uint32_t)));
  GB_TRY(cudaMemsetAsync(err_, 0, sizeof(uint32_t), st));
  GB_TRY(cudaFuncSetAttribute(k_propose_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem)));
  GB_TRY(cudaFuncSetAttribute(k_propose_hidden, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(HidSmem)));
  std::vector<uint32_t> nodes(kTreelets, kInvalidID);
  std::copy(node_of_treelet.begin(), node_of_treelet.begin() + num_treelets, nodes.begin());
  GB_TRY(cudaMemcpyAsync(node_of_treelet_, nodes.data(), kTreelets * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  if (num_prims)
    GB_TRY(cudaMemcpyAsync(prim_treelet_, prim_treelet.data(), num_prims * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  if (num_geom_ids_)
    GB_TRY(cudaMemcpyAsync(geom_prefix_, geom_prefix.data(), num_geom_ids_ * sizeof(uint32_t), cudaMemcpyHostToDevice,
                           st));
  GB_TRY(cudaMemsetAsync(m_, 0, kNumParams * sizeof(float), st));
  GB_TRY(cudaMemsetAsync(v_, 0, kNumParams * sizeof(float), st));
  const unsigned blocks = (unsigned)num_sms() * 8;
  k_init_params<<<blocks, 256, 0, st>>>(P_, seed);
  k_to_bf16<<<blocks, 256, 0, st>>>(P_, Pb_, kNumParams);
  note_launches(2);
  GB_TRY(refresh_w4(st));
  GB_TRY(cudaGetLastError());
  return cudaStreamSynchronize(st);
}

cudaError_t Proposer::refresh_w4(cudaStream_t st) {
  k_permute_w4<<<blocks_for((uint64_t)kTreelets * (kTcK / 8), 256), 256, 0, st>>>(Pb_, P_, (int)num_treelets, W4p_);
  note_launches(1);
  return cudaGetLastError();
}

void Proposer::release() {
  void* ptrs[] = {P_, Pb_, G_, m_, v_, node_of_treelet_, prim_treelet_, geom_prefix_, acc_, X0_, H1_, H2_, H3_,
                  dZ4_, dZ_, Z_, Z4_, dH_, dX0_, W4p_, err_, H_};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  P_ = G_ = m_ = v_ = acc_ = Z_ = Z4_ = dH_ = dX0_ = nullptr;
  Pb_ = X0_ = H1_ = H2_ = H3_ = dZ4_ = dZ_ = nullptr;
  node_of_treelet_ = prim_treelet_ = geom_prefix_ = err_ = nullptr;
  W4p_ = H_ = nullptr;
  hcap_ = 0;
  cap_ = 0;
}

cudaError_t Proposer::ensure_batch(uint32_t B) {
  if (B <= cap_) return cudaSuccess;
  void* ptrs[] = {X0_, H1_, H2_, H3_, dZ4_, dZ_, Z_, Z4_, dH_, dX0_};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  X0_ = H1_ = H2_ = H3_ = dZ4_ = dZ_ = nullptr;
  Z_ = Z4_ = dH_ = dX0_ = nullptr;
  cap_ = 0;
  const size_t b = B;
  GB_TRY(cudaMalloc(&X0_, b * kIn * 2));
  GB_TRY(cudaMalloc(&H1_, b * kHidden * 2));
  GB_TRY(cudaMalloc(&H2_, b * kHidden * 2));
  GB_TRY(cudaMalloc(&H3_, b * kHidden * 2));
  GB_TRY(cudaMalloc(&dZ_, b * kHidden * 2));
  GB_TRY(cudaMalloc(&dZ4_, b * kTreelets * 2));
  GB_TRY(cudaMalloc(&Z_, b * kHidden * 4));
  GB_TRY(cudaMalloc(&Z4_, b * kTreelets * 4));
  GB_TRY(cudaMalloc(&dH_, b * kHidden * 4));
  GB_TRY(cudaMalloc(&dX0_, b * kIn * 4));
  cap_ = B;
  return cudaSuccess;
}

// Forward and backward pass of one batch; gradients land in G_ (zeroed here),
// the loss statistics in acc_.
cudaError_t Proposer::step_forward_backward(const char* rays, uint64_t stride, const uint32_t* idx,
                                            const int32_t* labels, uint32_t B, cudaStream_t st) {
  GB_TRY(ensure_batch(B));
  GB_TRY(cudaMemsetAsync(G_, 0, kNumParams * sizeof(float), st));
  const uint64_t nl = (uint64_t)B * kLevels, nh = (uint64_t)B * kHidden;
  const int splits = (int)std::max(1u, std::min(128u, B / 256));
  k_encode_fwd<<<blocks_for(nl, 256), 256, 0, st>>>(rays, stride, idx, B, grid, Pb_, X0_);
  // forward: Z = X W^T (B(k=i, n=o) = W[o][i]), bias + ReLU
  gemm(B, kHidden, kIn, X0_, kIn, 1, Pb_ + kOffW1, 1, kIn, Z_, kHidden, false, 1, st);
  k_bias_relu<<<blocks_for(nh, 256), 256, 0, st>>>(Z_, P_ + kOffB1, H1_, nh);
  gemm(B, kHidden, kHidden, H1_, kHidden, 1, Pb_ + kOffW2, 1, kHidden, Z_, kHidden, false, 1, st);
  k_bias_relu<<<blocks_for(nh, 256), 256, 0, st>>>(Z_, P_ + kOffB2, H2_, nh);
  gemm(B, kHidden, kHidden, H2_, kHidden, 1, Pb_ + kOffW3, 1, kHidden, Z_, kHidden, false, 1, st);
  k_bias_relu<<<blocks_for(nh, 256), 256, 0, st>>>(Z_, P_ + kOffB3, H3_, nh);
  gemm(B, kTreelets, kHidden, H3_, kHidden, 1, Pb_ + kOffW4, 1, kHidden, Z4_, kTreelets, false, 1, st);
  k_softmax_xent<<<blocks_for((uint64_t)B * 32, 256), 256, 0, st>>>(Z4_, P_ + kOffB4, labels, idx, B, 1.0f / (float)B,
                                                                     dZ4_, acc_);
  // output layer: db4, dW4 = dZ4^T H3 (A(m=o,k=b) = dZ4[b][o]), dH3 = dZ4 W4 (B(k=o,n=i) = W4[o][i])
  colsum(dZ4_, kTreelets, B, G_ + kOffB4, st);
  gemm(kTreelets, kHidden, B, dZ4_, 1, kTreelets, H3_, kHidden, 1, G_ + kOffW4, kHidden, true, splits / 4 + 1, st);
  gemm(B, kHidden, kTreelets, dZ4_, kTreelets, 1, Pb_ + kOffW4, kHidden, 1, dH_, kHidden, false, 1, st);
  // hidden layers 3, 2, 1
  const uint16_t* Hs[3] = {H3_, H2_, H1_};
  const uint16_t* Xs[3] = {H2_, H1_, X0_};
  const size_t offW[3] = {kOffW3, kOffW2, kOffW1}, offB[3] = {kOffB3, kOffB2, kOffB1};
  const int fan_in[3] = {kHidden, kHidden, kIn};
  for (int L = 0; L < 3; L++) {
    k_relu_bwd<<<blocks_for(nh, 256), 256, 0, st>>>(dH_, Hs[L], dZ_, nh);
    colsum(dZ_, kHidden, B, G_ + offB[L], st);
    gemm(kHidden, fan_in[L], B, dZ_, 1, kHidden, Xs[L], fan_in[L], 1, G_ + offW[L], fan_in[L], true, splits, st);
    float* dX = L < 2 ? dH_ : dX0_;
    // dX = dZ W (B(k=o, n=i) = W[o][i]); dH_ is consumed by k_relu_bwd above before being overwritten
    gemm(B, fan_in[L], kHidden, dZ_, kHidden, 1, Pb_ + offW[L], fan_in[L], 1, dX, fan_in[L], false, 1, st);
  }
  k_encode_bwd<<<blocks_for(nl, 256), 256, 0, st>>>(rays, stride, idx, B, grid, dX0_, G_);
  note_launches(26);
  return cudaGetLastError();
}

cudaError_t Proposer::train(const char* records, uint64_t stride, uint32_t M, uint32_t epochs, uint32_t batch,
                            float lr, cudaStream_t st) {
  if (M == 0 || epochs == 0) return cudaSuccess;
  if (batch < 256) batch = 256;
  int32_t* labels = nullptr;
  uint64_t* keys = nullptr;
  uint32_t *vals = nullptr, *order = nullptr;
  unsigned int* count = nullptr;
  cudaError_t err = cudaSuccess;
  auto fail = [&](cudaError_t e) {
    if (labels) cudaFree(labels);
    if (keys) cudaFree(keys);
    if (vals) cudaFree(vals);
    if (order) cudaFree(order);
    if (count) cudaFree(count);
    return e;
  };
  if ((err = cudaMalloc(&labels, (size_t)M * 4)) != cudaSuccess) return fail(err);
  if ((err = cudaMalloc(&keys, (size_t)M * 8)) != cudaSuccess) return fail(err);
  if ((err = cudaMalloc(&vals, (size_t)M * 4)) != cudaSuccess) return fail(err);
  if ((err = cudaMalloc(&order, (size_t)M * 4)) != cudaSuccess) return fail(err);
  if ((err = cudaMalloc(&count, 4)) != cudaSuccess) return fail(err);
  cudaMemsetAsync(count, 0, 4, st);
  k_label<<<blocks_for(M, 256), 256, 0, st>>>(records, stride, M, prim_treelet_, num_prims, geom_prefix_,
                                              num_geom_ids_, labels, count);
  k_sort_keys<<<blocks_for(M, 256), 256, 0, st>>>(labels, M, keys, vals);
  note_launches(2);
  // stable partition: labelled records first, in record order
  if ((err = sort_pairs(keys, vals, M, st)) != cudaSuccess) return fail(err);
  unsigned int n_lab = 0;
  cudaMemcpyAsync(&n_lab, count, 4, cudaMemcpyDeviceToHost, st);
  if ((err = cudaStreamSynchronize(st)) != cudaSuccess) return fail(err);
  stats.samples = n_lab;
  if (n_lab == 0) return fail(cudaSuccess);
  const float b1 = 0.9f, b2 = 0.99f, eps = 1e-10f;
  for (uint32_t ep = 0; ep < epochs; ep++) {
    cudaMemcpyAsync(order, vals, (size_t)n_lab * 4, cudaMemcpyDeviceToDevice, st);
    k_shuffle_keys<<<blocks_for(n_lab, 256), 256, 0, st>>>(n_lab, 0x5EEDu + 7919u * (stats.steps + ep), keys);
    note_launches(1);
    if ((err = sort_pairs(keys, order, n_lab, st)) != cudaSuccess) return fail(err);
    cudaMemsetAsync(acc_, 0, 16 * sizeof(float), st);
    for (uint32_t b0 = 0; b0 < n_lab; b0 += batch) {
      const uint32_t B = std::min(batch, n_lab - b0);
      if ((err = step_forward_backward(records, stride, order + b0, labels, B, st)) != cudaSuccess) return fail(err);
      stats.steps++;
      const float c1 = 1.0f / (1.0f - std::pow(b1, (float)stats.steps));
      const float c2 = 1.0f / (1.0f - std::pow(b2, (float)stats.steps));
      k_adam<<<(unsigned)num_sms() * 8, 256, 0, st>>>(P_, G_, m_, v_, Pb_, kNumParams, lr, b1, b2, eps, c1, c2);
      note_launches(1);
    }
    float acc[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(acc, acc_, sizeof(acc), cudaMemcpyDeviceToHost, st);
    if ((err = cudaStreamSynchronize(st)) != cudaSuccess) return fail(err);
    if (acc[3] > 0) {
      stats.loss = acc[0] / acc[3];
      stats.top1 = acc[1] / acc[3];
      stats.top4 = acc[2] / acc[3];
    }
  }
  if ((err = refresh_w4(st)) != cudaSuccess) return fail(err);
  return fail(cudaGetLastError());
}

cudaError_t Proposer::predict(const char* rays, uint64_t stride, uint32_t M, uint4* seeds, uint32_t* treelets,
                              cudaStream_t st, const uint32_t* d_count, uint32_t* err) {
  if (M == 0) return cudaSuccess;
  if (!use_mma_sync) {
    const uint32_t ntiles = (M + kTcRays - 1) / kTcRays;
    if ((size_t)ntiles * kTcRays * kTcK > hcap_) {
      if (H_) cudaFree(H_);
      H_ = nullptr;
      hcap_ = 0;
      GB_TRY(cudaMalloc(&H_, (size_t)ntiles * kTcTileBytes));
      hcap_ = (size_t)ntiles * kTcRays * kTcK;
    }
    k_propose_hidden<<<std::min<uint32_t>(ntiles, (uint32_t)num_sms() * 4), 256, sizeof(HidSmem), st>>>(
        rays, stride, M, d_count, grid, Pb_, P_, H_);
    k_propose_tc<<<std::min<uint32_t>(ntiles, (uint32_t)num_sms()), kTcThreads, sizeof(TcSmem), st>>>(
        M, d_count, H_, W4p_, node_of_treelet_, seeds, treelets, err ? err : err_);
    note_launches(2);
    return cudaGetLastError();
  }
  const uint32_t ntiles = (M + kPRays - 1) / kPRays;
  const uint32_t grid_n = std::min<uint32_t>(ntiles, (uint32_t)num_sms() * 2);
  k_propose<<<grid_n, kPW * 32, sizeof(PropSmem), st>>>(rays, stride, M, d_count, grid, Pb_, P_, node_of_treelet_,
                                                        (int)num_treelets, seeds, treelets);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t Proposer::gradients(const char* rays, uint64_t stride, const int32_t* labels, uint32_t B, float* grads,
                                float* loss, cudaStream_t st) {
  GB_TRY(cudaMemsetAsync(acc_, 0, 16 * sizeof(float), st));
  GB_TRY(step_forward_backward(rays, stride, nullptr, labels, B, st));
  GB_TRY(cudaMemcpyAsync(grads, G_, kNumParams * sizeof(float), cudaMemcpyDeviceToDevice, st));
  float acc[4];
  GB_TRY(cudaMemcpyAsync(acc, acc_, sizeof(acc), cudaMemcpyDeviceToHost, st));
  GB_TRY(cudaStreamSynchronize(st));
  *loss = acc[0] / (float)B;
  return cudaSuccess;
}

cudaError_t Proposer::get_params(float* host, cudaStream_t st) const {
  GB_TRY(cudaMemcpyAsync(host, P_, kNumParams * sizeof(float), cudaMemcpyDefault, st));
  return cudaStreamSynchronize(st);
}

cudaError_t Proposer::set_params(const float* host, cudaStream_t st) {
  GB_TRY(cudaMemcpyAsync(P_, host, kNumParams * sizeof(float), cudaMemcpyDefault, st));
  k_to_bf16<<<(unsigned)num_sms() * 8, 256, 0, st>>>(P_, Pb_, kNumParams);
  note_launches(1);
  GB_TRY(refresh_w4(st));
  GB_TRY(cudaGetLastError());
  return cudaStreamSynchronize(st);
}

// ---------------------------------------------------------------------------
// Treelet cut
// ---------------------------------------------------------------------------

cudaError_t choose_treelets(const DeviceBVH& bvh, cudaStream_t st, std::vector<uint32_t>* roots,
                            std::vector<uint32_t>* record_treelet, std::vector<uint32_t>* record_prim,
                            std::vector<uint32_t>* record_geom, uint32_t max_treelets) {
  roots->clear();
  max_treelets = std::min<uint32_t>(std::max<uint32_t>(max_treelets, 1u), (uint32_t)kTreelets);
  const uint32_t nn = bvh.num_nodes, nt = bvh.num_tris;
  record_treelet->assign(nt, kInvalidID);
  record_prim->assign(nt, kInvalidID);
  record_geom->assign(nt, kInvalidID);
  if (nn == 0) return cudaSuccess;
  std::vector<WideNode> nodes(nn);
  std::vector<TriRecord> tris(nt);
  GB_TRY(cudaMemcpyAsync(nodes.data(), bvh.nodes, (size_t)nn * sizeof(WideNode), cudaMemcpyDeviceToHost, st));
  GB_TRY(cudaMemcpyAsync(tris.data(), bvh.tris, (size_t)nt * sizeof(TriRecord), cudaMemcpyDeviceToHost, st));
  GB_TRY(cudaStreamSynchronize(st));
  for (uint32_t r = 0; r < nt; r++) {
    uint32_t p, gid;
    std::memcpy(&p, &tris[r].a.w, 4);
    std::memcpy(&gid, &tris[r].b.w, 4);
    (*record_prim)[r] = p;
    (*record_geom)[r] = gid;
  }
  auto child_of = [&](const WideNode& n, int s) {
    return n.child_base + (uint32_t)__builtin_popcount(n.imask & ((1u << s) - 1u));
  };
  // triangles below each node (children follow their parents in breadth-first order)
  std::vector<uint64_t> count(nn, 0);
  for (int64_t i = (int64_t)nn - 1; i >= 0; i--) {
    const WideNode& n = nodes[i];
    uint64_t c = 0;
    for (int s = 0; s < 8; s++) {
      if (!n.meta[s]) continue;
      if (n.imask & (1u << s)) {
        const uint32_t ch = child_of(n, s);
        if (ch > (uint32_t)i && ch < nn) c += count[ch];
      } else {
        c += ((n.meta[s] >> 5) & 3u) + 1u;
      }
    }
    count[i] = c;
  }
  // greedy split of the largest subtree while the budget allows; triangles
  // held directly by a split node belong to no treelet, so a node is split
  // only while those are at most 1/8 of its subtree (the root always is)
  std::priority_queue<std::pair<uint64_t, uint32_t>> heap;
  heap.push({count[0], 0u});
  std::vector<uint32_t> cut;
  while (!heap.empty()) {
    const auto top = heap.top();
    heap.pop();
    const WideNode& n = nodes[top.second];
    int nint = 0;
    uint64_t direct = 0;
    for (int s = 0; s < 8; s++) {
      if (!n.meta[s]) continue;
      if (n.imask & (1u << s)) nint++;
      else direct += ((n.meta[s] >> 5) & 3u) + 1u;
    }
    const bool splittable = nint > 0 && (top.second == 0u || direct * 8 <= top.first);
    if (splittable && cut.size() + heap.size() + (size_t)nint <= (size_t)max_treelets) {
      for (int s = 0; s < 8; s++)
        if (n.meta[s] && (n.imask & (1u << s))) {
          const uint32_t ch = child_of(n, s);
          if (ch > top.second && ch < nn) heap.push({count[ch], ch});
        }
    } else if (top.second != 0u) {
      cut.push_back(top.second);
    }
  }
  std::sort(cut.begin(), cut.end());
  *roots = cut;
  // label every record below each root
  std::vector<uint32_t> stack;
  for (uint32_t t = 0; t < cut.size(); t++) {
    stack.assign(1, cut[t]);
    while (!stack.empty()) {
      const uint32_t id = stack.back();
      stack.pop_back();
      const WideNode& n = nodes[id];
      for (int s = 0; s < 8; s++) {
        if (!n.meta[s]) continue;
        if (n.imask & (1u << s)) {
          const uint32_t ch = child_of(n, s);
          if (ch > id && ch < nn) stack.push_back(ch);
        } else {
          const uint32_t first = n.tri_base + (n.meta[s] & 31u), cnt = ((n.meta[s] >> 5) & 3u) + 1u;
          for (uint32_t k = 0; k < cnt && first + k < nt; k++) (*record_treelet)[first + k] = t;
        }
      }
    }
  }
  return cudaSuccess;
}

}  // namespace gb
