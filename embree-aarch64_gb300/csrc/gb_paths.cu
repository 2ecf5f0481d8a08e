// gb_paths.cu -- wavefront diffuse path tracing with frames captured as CUDA
// graphs (see gb_paths.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "gb_launch.h"
#include "gb_paths.h"

namespace gb {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kAlbedo = 0.75f;
constexpr float kBounceEps = 1e-4f;  // tnear of secondary rays

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(mix32(x) >> 8) * (1.0f / 16777216.0f); }

// Moves every triangle of the soup along its random unit normal.
__global__ void k_displace(float* verts, uint64_t vstride, const char* idx, uint64_t istride, uint32_t ntris,
                           uint32_t nverts, const float* __restrict__ rest, const uint32_t* frame, float amplitude,
                           uint32_t seed) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntris) return;
  const uint32_t* tri = reinterpret_cast<const uint32_t*>(idx + (uint64_t)t * istride);
  const uint32_t v[3] = {tri[0], tri[1], tri[2]};
  if (v[0] >= nverts || v[1] >= nverts || v[2] >= nverts) return;
  const float x = (rest[3 * v[0]] + rest[3 * v[1]] + rest[3 * v[2]]) * (1.0f / 3.0f);
  const float z = 1.0f - 2.0f * u01(seed * 0x9E3779B9u ^ (2 * t));
  const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
  const float phi = kTwoPi * u01(seed * 0x85EBCA6Bu ^ (2 * t + 1));
  const float n[3] = {r * cosf(phi), r * sinf(phi), z};
  const float off = amplitude * sinf(kTwoPi * ((float)*frame * (1.0f / 60.0f) + x));
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float* p = reinterpret_cast<float*>(reinterpret_cast<char*>(verts) + (uint64_t)v[k] * vstride);
#pragma unroll
    for (int a = 0; a < 3; a++) p[a] = rest[3 * v[k] + a] + off * n[a];
  }
}

__device__ __forceinline__ void write_ray(char* rec, float ox, float oy, float oz, float tnear, float dx, float dy,
                                          float dz, uint32_t id) {
  float4* q = reinterpret_cast<float4*>(rec);
  q[0] = make_float4(ox, oy, oz, tnear);
  q[1] = make_float4(dx, dy, dz, 0.0f);
  q[2] = make_float4(INFINITY, __uint_as_float(kInvalidID), __uint_as_float(id), 0.0f);
  q[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  q[4] = make_float4(0.0f, __uint_as_float(kInvalidID), __uint_as_float(kInvalidID), __uint_as_float(kInvalidID));
}

// Pinhole camera rays through pixel centres, one per path (id = pixel).
__global__ void k_camera(char* rays, uint32_t width, uint32_t height, float4 eye, float4 cu, float4 cv, float4 cw,
                         uint32_t* count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = width * height;
  if (i == 0) *count = n;
  if (i >= n) return;
  const float sx = (2.0f * ((float)(i % width) + 0.5f) / (float)width - 1.0f);
  const float sy = (1.0f - 2.0f * ((float)(i / width) + 0.5f) / (float)height);
  write_ray(rays + (uint64_t)i * 80, eye.x, eye.y, eye.z, 0.0f, cw.x + sx * cu.x + sy * cv.x,
            cw.y + sx * cu.y + sy * cv.y, cw.z + sx * cu.z + sy * cv.z, i);
}

// Shades the closest hits of one bounce: a miss takes the sky's radiance, a hit
// continues (cosine-weighted diffuse bounce, albedo kAlbedo) unless it is the
// last bounce; survivors are compacted into `out` (warp-aggregated atomics).
__global__ void k_shade(const char* __restrict__ in, const uint32_t* __restrict__ count_in, char* out,
                        uint32_t* count_out, float* throughput, float* image, const uint32_t* frame, uint32_t bounce,
                        uint32_t last, uint32_t npaths) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const uint32_t n = min(*count_in, npaths);
  bool spawn = false;
  float o[3] = {0, 0, 0}, d[3] = {0, 0, 0};
  uint32_t path = 0;
  if (i < n) {
    const float* f = reinterpret_cast<const float*>(in + (uint64_t)i * 80);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(f);
    path = w[10];
    if (path < npaths) {
      float* thr = throughput + 3 * (size_t)path;
      if (bounce == 0) thr[0] = thr[1] = thr[2] = 1.0f;
      const float dx = f[4], dy = f[5], dz = f[6];
      if (w[18] == kInvalidID) {
        const float len = sqrtf(dx * dx + dy * dy + dz * dz);
        const float up = len > 0.0f ? 0.5f + 0.5f * dz / len : 0.5f;
        const float sky[3] = {0.55f + 0.35f * up, 0.65f + 0.3f * up, 0.8f + 0.2f * up};
        for (int a = 0; a < 3; a++) image[3 * (size_t)path + a] = thr[a] * sky[a];
      } else if (last) {
        for (int a = 0; a < 3; a++) image[3 * (size_t)path + a] = 0.0f;
      } else {
        const float t = f[8];
        float nx = f[12], ny = f[13], nz = f[14];
        const float nl = sqrtf(nx * nx + ny * ny + nz * nz);
        if (nl > 0.0f) { nx /= nl; ny /= nl; nz /= nl; } else { nx = 0.0f; ny = 0.0f; nz = 1.0f; }
        if (nx * dx + ny * dy + nz * dz > 0.0f) { nx = -nx; ny = -ny; nz = -nz; }
        // orthonormal basis (Duff et al. 2017)
        const float sgn = nz >= 0.0f ? 1.0f : -1.0f;
        const float a = -1.0f / (sgn + nz), b = nx * ny * a;
        const float t1[3] = {1.0f + sgn * nx * nx * a, sgn * b, -sgn * nx};
        const float t2[3] = {b, sgn + ny * ny * a, -ny};
        const uint32_t key = mix32(*frame * 0x27d4eb2dU ^ bounce * 0x165667b1U) ^ path;
        const float u1 = u01(key * 2u), u2 = u01(key * 2u + 1u);
        const float r = sqrtf(u1), phi = kTwoPi * u2;
        const float lx = r * cosf(phi), ly = r * sinf(phi), lz = sqrtf(fmaxf(0.0f, 1.0f - u1));
        const float nn[3] = {nx, ny, nz};
        for (int k = 0; k < 3; k++) {
          o[k] = f[k] + t * f[4 + k];
          d[k] = t1[k] * lx + t2[k] * ly + nn[k] * lz;
        }
        for (int k = 0; k < 3; k++) thr[k] *= kAlbedo;
        spawn = true;
      }
    }
  }
  const unsigned m = __ballot_sync(kFull, spawn);
  uint32_t base = 0;
  if (lane == 0 && m) base = atomicAdd(count_out, (unsigned)__popc(m));
  base = __shfl_sync(kFull, base, 0);
  if (spawn) {
    const uint32_t slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot < npaths) write_ray(out + (uint64_t)slot * 80, o[0], o[1], o[2], kBounceEps, d[0], d[1], d[2], path);
  }
}

inline unsigned cdiv(uint64_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

#define GB_TRY(x)                     \
  do {                                \
    cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

cudaError_t PathTracer::init(const DeviceBVH* bvh, uint32_t width, uint32_t height, uint32_t bounces,
                             const CameraSpec& cam, cudaStream_t st) {
  release();
  if (!bvh || width == 0 || height == 0 || bounces == 0 || bounces > kMaxBounces) return cudaErrorInvalidValue;
  if ((uint64_t)width * height >= (1ull << 31)) return cudaErrorInvalidValue;
  bvh_ = bvh;
  width_ = width;
  height_ = height;
  bounces_ = bounces;
  // camera basis: w toward the look-at point, u right, v up, scaled by the field of view
  double e[3], w[3], u[3], v[3];
  for (int a = 0; a < 3; a++) { e[a] = cam.eye[a]; w[a] = cam.look[a] - cam.eye[a]; }
  auto norm = [](double* x) {
    const double l = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    if (l > 0) for (int a = 0; a < 3; a++) x[a] /= l;
  };
  norm(w);
  u[0] = w[1] * cam.up[2] - w[2] * cam.up[1];
  u[1] = w[2] * cam.up[0] - w[0] * cam.up[2];
  u[2] = w[0] * cam.up[1] - w[1] * cam.up[0];
  norm(u);
  v[0] = u[1] * w[2] - u[2] * w[1];
  v[1] = u[2] * w[0] - u[0] * w[2];
  v[2] = u[0] * w[1] - u[1] * w[0];
  const double th = std::tan(cam.fov_deg * 3.14159265358979323846 / 360.0), aspect = (double)width / height;
  for (int a = 0; a < 3; a++) {
    cam_[a] = (float)e[a];
    cam_[3 + a] = (float)(u[a] * th * aspect);
    cam_[6 + a] = (float)(v[a] * th);
    cam_[9 + a] = (float)w[a];
  }
  const size_t n = (size_t)width * height;
  GB_TRY(cudaMalloc(&rays_[0], n * 80));
  GB_TRY(cudaMalloc(&rays_[1], n * 80));
  GB_TRY(cudaMalloc(&log_, n * 80));
  GB_TRY(cudaMalloc(&seeds_, n * sizeof(uint4)));
  GB_TRY(cudaMalloc(&throughput_, n * 3 * sizeof(float)));
  GB_TRY(cudaMalloc(&image_, n * 3 * sizeof(float)));
  GB_TRY(cudaMalloc(&counts_, (kMaxBounces + 1) * sizeof(uint32_t)));
  GB_TRY(cudaMalloc(&frame_, sizeof(uint32_t)));
  GB_TRY(cudaMalloc(&scratch_, 16 * sizeof(uint32_t)));
  GB_TRY(cudaMallocHost(&h_frame_, 256));
  GB_TRY(cudaEventCreate(&ev_[0]));
  GB_TRY(cudaEventCreate(&ev_[1]));
  GB_TRY(cudaMemsetAsync(image_, 0, n * 3 * sizeof(float), st));
  GB_TRY(cudaMemsetAsync(scratch_, 0, 16 * sizeof(uint32_t), st));
  GB_TRY(cudaMemsetAsync(frame_, 0, sizeof(uint32_t), st));
  return cudaStreamSynchronize(st);
}

cudaError_t PathTracer::animate(const SoupAnimation& anim, const RefitScratch* refit, cudaStream_t st) {
  if (!anim.verts || !anim.idx || !refit) return cudaErrorInvalidValue;
  if (rest_) cudaFree(rest_);
  rest_ = nullptr;
  GB_TRY(cudaMalloc(&rest_, (size_t)std::max(anim.nverts, 1u) * 3 * sizeof(float)));
  GB_TRY(cudaMemcpy2DAsync(rest_, 12, anim.verts, anim.vstride, 12, anim.nverts, cudaMemcpyDeviceToDevice, st));
  anim_ = anim;
  refit_ = refit;
  animated_ = true;
  invalidate();
  return cudaStreamSynchronize(st);
}

void PathTracer::invalidate() {
  for (int m = 0; m < 2; m++)
    if (exec_[m]) {
      cudaGraphExecDestroy(exec_[m]);
      exec_[m] = nullptr;
    }
}

namespace {
struct FrameBody {
  // Enqueues one frame on `st`; returns the number of kernels launched.
  static cudaError_t enqueue(const DeviceBVH* bvh, uint32_t W, uint32_t H, uint32_t bounces, const float* cam,
                             bool learned, Proposer* prop, bool animated, const SoupAnimation& anim,
                             const RefitScratch* refit, const float* rest, char* const rays[2], char* log,
                             uint4* seeds, float* thr, float* image, uint32_t* counts, uint32_t* frame,
                             uint32_t* scratch, cudaStream_t st, unsigned* kernels) {
    unsigned nk = 0;
    const uint32_t n = W * H;
    if (animated) {
      k_displace<<<cdiv(anim.ntris, 256), 256, 0, st>>>(anim.verts, anim.vstride, anim.idx, anim.istride, anim.ntris,
                                                        anim.nverts, rest, frame, anim.amplitude, anim.seed);
      nk++;
      GB_TRY(refit_enqueue(*bvh, *refit, st));
      nk += (unsigned)bvh->level_start.size();  // tris + one per level (upper bound)
    }
    GB_TRY(cudaMemsetAsync(counts, 0, (kMaxBounces + 1) * sizeof(uint32_t), st));
    GB_TRY(cudaMemsetAsync(scratch + 1, 0, 9 * sizeof(uint32_t), st));  // error flags and counters
    k_camera<<<cdiv(n, 256), 256, 0, st>>>(rays[0], W, H, make_float4(cam[0], cam[1], cam[2], 0),
                                           make_float4(cam[3], cam[4], cam[5], 0),
                                           make_float4(cam[6], cam[7], cam[8], 0),
                                           make_float4(cam[9], cam[10], cam[11], 0), counts);
    nk++;
    int cur = 0;
    for (uint32_t b = 0; b < bounces; b++) {
      TraceParams P{};
      P.nodes = bvh->nodes;
      P.tris = bvh->tris;
      P.rays = rays[cur];
      P.stride = 80;
      P.nrays = n;
      P.nrays_ptr = counts + b;
      P.ray_counter = scratch;
      P.err = scratch + 1;
      P.counters = reinterpret_cast<TraceCounters*>(scratch + 2);
      P.max_iters = 4 * bvh->num_nodes + 64;
      P.num_nodes = bvh->num_nodes;
      P.num_tris = bvh->num_tris;
      P.robust = bvh->robust;
      GB_TRY(cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st));
      if (learned && prop) {
        GB_TRY(prop->predict(rays[cur], 80, n, seeds, nullptr, st, counts + b, scratch + 1));
        nk++;
        P.seeds = seeds;
        P.max_iters = 8 * bvh->num_nodes + 64;
      }
      GB_TRY(launch_trace(P, false, false, st));
      nk++;
      if (b == (bounces > 1 ? 1u : 0u)) GB_TRY(copy_device(log, rays[cur], (size_t)n * 80, st));
      k_shade<<<cdiv(n, 256), 256, 0, st>>>(rays[cur], counts + b, rays[cur ^ 1], counts + b + 1, thr, image, frame, b,
                                            b + 1 == bounces ? 1u : 0u, n);
      nk++;
      cur ^= 1;
    }
    *kernels = nk;
    return cudaGetLastError();
  }
};
}  // namespace

cudaError_t PathTracer::capture(bool learned, cudaStream_t st) {
  unsigned nk = 0;
  auto body = [&](cudaStream_t s) {
    return FrameBody::enqueue(bvh_, width_, height_, bounces_, cam_, learned, proposer_, animated_, anim_, refit_,
                              rest_, rays_, log_, seeds_, throughput_, image_, counts_, frame_, scratch_, s, &nk);
  };
  // one eager frame first: it sets the launch configurations up outside the capture
  GB_TRY(body(st));
  GB_TRY(cudaStreamSynchronize(st));
  cudaGraph_t g = nullptr;
  GB_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const cudaError_t e1 = body(st);
  const cudaError_t e2 = cudaStreamEndCapture(st, &g);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return e1 != cudaSuccess ? e1 : e2;
  }
  const cudaError_t e3 = cudaGraphInstantiate(&exec_[learned ? 1 : 0], g, 0);
  cudaGraphDestroy(g);
  kernels_[learned ? 1 : 0] = nk;
  return e3;
}

cudaError_t PathTracer::render(uint32_t frame, bool learned, cudaStream_t st, FrameStats* out) {
  *out = FrameStats{};
  learned = learned && proposer_ != nullptr;
  const int m = learned ? 1 : 0;
  *h_frame_ = frame;
  if (!exec_[m]) {
    GB_TRY(cudaMemcpyAsync(frame_, h_frame_, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    GB_TRY(capture(learned, st));
  }
  GB_TRY(cudaMemcpyAsync(frame_, h_frame_, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  GB_TRY(cudaEventRecord(ev_[0], st));
  GB_TRY(cudaGraphLaunch(exec_[m], st));
  GB_TRY(cudaEventRecord(ev_[1], st));
  note_launches(kernels_[m]);
  uint32_t* h = h_frame_ + 1;  // pinned: [0..8] counts, [9..24] scratch, [25] refit errors
  GB_TRY(cudaMemcpyAsync(h, counts_, (kMaxBounces + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_TRY(cudaMemcpyAsync(h + 9, scratch_, 10 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  if (animated_) GB_TRY(cudaMemcpyAsync(h + 19, refit_->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GB_TRY(cudaStreamSynchronize(st));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
  out->frame_ms = ms;
  out->learned = learned ? 1u : 0u;
  for (uint32_t b = 0; b < bounces_; b++) {
    out->rays_per_bounce[b] = std::min(h[b], width_ * height_);
    out->rays += out->rays_per_bounce[b];
  }
  TraceCounters tc;
  std::memcpy(&tc, h + 11, sizeof(tc));
  out->proposal_hits = tc.proposal_hits;
  out->errors = h[10] | ((animated_ && h[19]) ? 0x100u : 0u);
  log_count_ = bounces_ > 1 ? out->rays_per_bounce[1] : out->rays_per_bounce[0];
  return cudaSuccess;
}

cudaError_t PathTracer::image(float* host_rgb, cudaStream_t st) const {
  GB_TRY(cudaMemcpyAsync(host_rgb, image_, (size_t)width_ * height_ * 3 * sizeof(float), cudaMemcpyDefault, st));
  return cudaStreamSynchronize(st);
}

void PathTracer::release() {
  invalidate();
  void* ptrs[] = {rays_[0], rays_[1], log_, seeds_, rest_, throughput_, image_, counts_, frame_, scratch_};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h_frame_) cudaFreeHost(h_frame_);
  for (cudaEvent_t& e : ev_)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  rays_[0] = rays_[1] = log_ = nullptr;
  seeds_ = nullptr;
  rest_ = throughput_ = image_ = nullptr;
  counts_ = frame_ = scratch_ = h_frame_ = nullptr;
  animated_ = false;
}

}  // namespace gb
