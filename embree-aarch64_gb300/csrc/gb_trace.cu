// gb_trace.cu -- closest-hit and any-hit stream traversal behind
// rtcIntersect1M / rtcOccluded1M: launches of the persistent kernel k_trace
// (gb_trace_kernel.cuh) in the default launch shape, ray reordering, and the
// query without allocations.  The tuned launch shapes are compiled in
// gb_trace_shapes.cu.
#include <cuda_runtime.h>

#include <mutex>

#include "gb_launch.h"
#include "gb_trace_kernel.cuh"

namespace gb {

template <bool ANYHIT, bool COUNT, bool ALIGNED, bool ROBUST, bool SEEDED = false, bool INST = false,
          bool EXCL = false>
static cudaError_t launch_one(const TraceParams& P, cudaStream_t st) {
  return launch_shaped<ANYHIT, COUNT, ALIGNED, ROBUST, SEEDED, INST, EXCL, DefaultShape>(P, st);
}

template <bool ANYHIT, bool COUNT>
static cudaError_t launch_variant(const TraceParams& P, bool aligned, cudaStream_t st) {
  // scenes with instances (non-robust, no proposals or batches: checked by the caller)
  if (P.insts) {
    if (P.robust || P.seeds || P.batch_root) return cudaErrorInvalidValue;
    return aligned ? launch_one<ANYHIT, COUNT, true, false, false, true>(P, st)
                   : launch_one<ANYHIT, COUNT, false, false, false, true>(P, st);
  }
  // seeded queries: 16-byte aligned records of non-robust scenes (checked by the caller)
  if (P.seeds) {
    if (!aligned || P.robust) return cudaErrorInvalidValue;
    return launch_one<ANYHIT, COUNT, true, false, true>(P, st);
  }
  if (P.robust) return aligned ? launch_one<ANYHIT, COUNT, true, true>(P, st) : launch_one<ANYHIT, COUNT, false, true>(P, st);
  return aligned ? launch_one<ANYHIT, COUNT, true, false>(P, st) : launch_one<ANYHIT, COUNT, false, false>(P, st);
}

cudaError_t launch_trace(const TraceParams& P, bool anyhit, bool count, cudaStream_t st) {
  const bool aligned = ((uintptr_t)P.rays % 16 == 0) && (P.stride % 16 == 0);
  if (P.shape < 0 || P.shape >= kNumTraceShapes) return cudaErrorInvalidValue;
  // tuned shapes: the plain closest-hit and any-hit kernels on 16-byte aligned records
  if (P.shape != 0 && aligned && !count && !P.insts && !P.seeds && !P.excl_off && !P.excl)
    return launch_tuned_shape(P, anyhit, st);
  // exclusion lists: closest hit on aligned records of plain scenes (checked here)
  if (P.excl_off || P.excl) {
    if (anyhit || count || !aligned || !P.excl_off || P.insts || P.seeds || P.batch_root || P.order)
      return cudaErrorInvalidValue;
    return P.robust ? launch_one<false, false, true, true, false, false, true>(P, st)
                    : launch_one<false, false, true, false, false, false, true>(P, st);
  }
  if (anyhit) return count ? launch_variant<true, true>(P, aligned, st) : launch_variant<true, false>(P, aligned, st);
  return count ? launch_variant<false, true>(P, aligned, st) : launch_variant<false, false>(P, aligned, st);
}

// ---------------------------------------------------------------------------
// Ray reordering
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint64_t spread15(uint32_t x) {
  uint64_t v = x & 0x7FFFu;
  v = (v | (v << 16)) & 0x00FF0000FFull;
  v = (v | (v << 8)) & 0x0F00F00F00Full;
  v = (v | (v << 4)) & 0xC30C30C30C3ull;
  v = (v | (v << 2)) & 0x249249249249ull;
  return v;
}

__global__ void __launch_bounds__(256) k_ray_keys(const char* __restrict__ rays, uint64_t stride, uint32_t M,
                                                  float lx, float ly, float lz, float sx, float sy, float sz,
                                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const float* f = reinterpret_cast<const float*>(rays + (uint64_t)i * stride);
  const float o[3] = {(f[0] - lx) * sx, (f[1] - ly) * sy, (f[2] - lz) * sz};
  uint64_t code = 0;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float q = fminf(fmaxf(o[a] * 32768.0f, 0.0f), 32767.0f);  // NaN -> 0
    code |= spread15((uint32_t)q) << (2 - a);
  }
  const uint64_t oct = (f[4] < 0.0f ? 1u : 0u) | (f[5] < 0.0f ? 2u : 0u) | (f[6] < 0.0f ? 4u : 0u);
  keys[i] = (oct << 45) | code;
  vals[i] = i;
}

cudaError_t order_rays(const char* rays, uint64_t stride, uint32_t M, const float lo[3], const float hi[3],
                       uint64_t* keys, uint32_t* vals, uint64_t* kb, uint32_t* vb, uint32_t* hist, cudaStream_t st) {
  float s[3];
  for (int a = 0; a < 3; a++) {
    const float ext = hi[a] - lo[a];
    s[a] = (ext > 0.0f && ext < INFINITY) ? 1.0f / ext : 0.0f;
  }
  k_ray_keys<<<(M + 255) / 256, 256, 0, st>>>(rays, stride, M, lo[0], lo[1], lo[2], s[0], s[1], s[2], keys, vals);
  note_launches(1);
  return sort_pairs_passes(keys, vals, kb, vb, hist, M, 6, st);
}

// ---------------------------------------------------------------------------
// Query without allocations.
//
// For callers that must not allocate device memory during a query -- a
// process whose memory is fully reserved by its own allocator (so cudaMalloc
// would fail), a real-time loop that cannot take cudaMalloc's implicit device
// synchronisation, or a service held to a fixed memory budget -- the scratch
// of the closest-hit query lives in this file-scope array, which every GPU
// that loads the library holds until the process exits: 256 bytes of query
// state (fetch counter, error flags, counters) followed by kNoAllocStagingBytes
// (32 MiB) of staging for host-resident rays.  All calls share it and it keeps
// the last call's contents: each call clears the state words it relies on,
// and calls whose GPU work overlaps (concurrent streams or host threads) race
// on it, so callers serialise them.
// ---------------------------------------------------------------------------

constexpr uint64_t kNoAllocStateBytes = 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocStateBytes + kNoAllocStagingBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch array on the current device, looked up once
// per device (the symbol name is only a host-side stand-in for it).
static cudaError_t noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

// Resolves the scratch array's address and loads the four traversal kernels the
// no-allocation query can launch (plain / robust, 16-byte aligned or not) on the
// current device.  With CUDA's lazy loading, the module that holds the array and
// each kernel's code would otherwise be loaded -- taking device memory -- by the
// first query; the library calls this once per device when the device is created.
cudaError_t noalloc_prepare() {
  unsigned char* p = nullptr;
  cudaError_t e = noalloc_scratch(&p);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes a;
  if ((e = cudaFuncGetAttributes(&a, k_trace<false, false, true, false, false, false, false>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, k_trace<false, false, false, false, false, false, false>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&a, k_trace<false, false, true, true, false, false, false>)) != cudaSuccess) return e;
  return cudaFuncGetAttributes(&a, k_trace<false, false, false, true, false, false, false>);
}

cudaError_t noalloc_closest(const DeviceBVH& bvh, char* rays, bool rays_on_device, uint32_t M, uint64_t stride,
                            cudaStream_t st, uint32_t* err_flags) {
  *err_flags = 0;
  if (M == 0 || bvh.num_nodes == 0) return cudaSuccess;
  const uint64_t span = (uint64_t)(M - 1) * stride + sizeof(float) * 20;
  if (!rays_on_device && span > kNoAllocStagingBytes) return cudaErrorInvalidValue;
  unsigned char* scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) return e;
  unsigned int* state = reinterpret_cast<unsigned int*>(scratch);
  char* staging = reinterpret_cast<char*>(scratch + kNoAllocStateBytes);
  if ((e = cudaMemsetAsync(state, 0, kNoAllocStateBytes, st)) != cudaSuccess) return e;
  if (!rays_on_device && (e = cudaMemcpyAsync(staging, rays, span, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  TraceParams P{};
  P.nodes = bvh.nodes;
  P.tris = bvh.tris;
  P.rays = rays_on_device ? rays : staging;
  P.stride = stride;
  P.nrays = M;
  P.ray_counter = state;
  P.err = state + 1;
  P.counters = reinterpret_cast<TraceCounters*>(state + 2);
  P.max_iters = 4 * bvh.num_nodes + 64;
  P.num_nodes = bvh.num_nodes;
  P.num_tris = bvh.num_tris;
  P.robust = bvh.robust;
  if ((e = launch_trace(P, false, false, st)) != cudaSuccess) return e;
  if (!rays_on_device && (e = cudaMemcpyAsync(rays, staging, span, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  unsigned int flags = 0;
  if ((e = cudaMemcpyAsync(&flags, state + 1, sizeof(flags), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *err_flags = flags;
  return cudaSuccess;
}

}  // namespace gb
