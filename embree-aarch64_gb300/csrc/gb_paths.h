// gb_paths.h -- wavefront diffuse path tracing over a committed scene, one
// CUDA graph per frame (gb_paths.cu).
//
// A frame: (optionally) moves the vertices of an animated triangle soup and
// refits the BVH, generates the camera rays, then per bounce traces the live
// rays (closest hit; with the learned proposer's treelets searched first in
// learned frames), shades them and compacts the surviving paths into the next
// bounce's ray buffer.  Every launch reads its ray count from device memory,
// so the whole frame is captured once per mode and replayed with
// cudaGraphLaunch.
#pragma once
#include <cstdint>

#include "gb_build.h"
#include "gb_common.h"
#include "gb_learned.h"
#include "gb_trace.h"

namespace gb {

constexpr int kMaxBounces = 8;

struct CameraSpec {
  float eye[3], look[3], up[3];
  float fov_deg;  // vertical field of view
};

struct FrameStats {
  double frame_ms = 0;
  uint64_t rays = 0;
  uint64_t proposal_hits = 0;
  uint32_t rays_per_bounce[kMaxBounces] = {};
  uint32_t learned = 0;
  uint32_t errors = 0;  // kErr* bits of the frame's traversals | 0x100 when a refit failed
};

// Per-frame displacement of a triangle soup: triangle t moves by
// amplitude * sin(2 pi (frame / 60 + x_t)) along its own random unit normal
// (x_t: the x coordinate of its centroid in the rest pose).
struct SoupAnimation {
  float* verts = nullptr;       // device vertex buffer the scene reads (FLOAT3 records)
  uint64_t vstride = 12;
  const char* idx = nullptr;    // device index buffer (UINT3 records)
  uint64_t istride = 12;
  uint32_t ntris = 0;
  uint32_t nverts = 0;
  float amplitude = 0.002f;
  uint32_t seed = 14;
};

class PathTracer {
 public:
  cudaError_t init(const DeviceBVH* bvh, uint32_t width, uint32_t height, uint32_t bounces, const CameraSpec& cam,
                   cudaStream_t st);
  // Frames move the soup and refit `bvh` (geometry table `refit`, owned by the caller).
  cudaError_t animate(const SoupAnimation& anim, const RefitScratch* refit, cudaStream_t st);
  void set_proposer(Proposer* p) { proposer_ = p; invalidate(); }
  cudaError_t render(uint32_t frame, bool learned, cudaStream_t st, FrameStats* out);
  // closest-hit records of the last frame's first diffuse bounce (device) and their count
  const char* log_records() const { return (const char*)log_; }
  uint32_t log_count() const { return log_count_; }
  cudaError_t image(float* host_rgb, cudaStream_t st) const;
  void release();
  ~PathTracer() { release(); }

 private:
  cudaError_t capture(bool learned, cudaStream_t st);
  void invalidate();

  const DeviceBVH* bvh_ = nullptr;
  uint32_t width_ = 0, height_ = 0, bounces_ = 0;
  float cam_[12] = {};
  Proposer* proposer_ = nullptr;
  SoupAnimation anim_{};
  const RefitScratch* refit_ = nullptr;
  bool animated_ = false;

  char* rays_[2] = {nullptr, nullptr};
  char* log_ = nullptr;
  uint32_t log_count_ = 0;
  uint4* seeds_ = nullptr;
  float* rest_ = nullptr;         // rest pose of the animated vertices
  float* throughput_ = nullptr;   // per path, rgb
  float* image_ = nullptr;        // per pixel, rgb
  uint32_t* counts_ = nullptr;    // [kMaxBounces + 1] live rays per bounce
  uint32_t* frame_ = nullptr;     // device copy of the frame index
  uint32_t* scratch_ = nullptr;   // [0] fetch counter, [1] error flags, [2..9] TraceCounters
  uint32_t* h_frame_ = nullptr;   // pinned
  cudaGraphExec_t exec_[2] = {nullptr, nullptr};
  unsigned kernels_[2] = {0, 0};  // kernels per replay of each graph
  cudaEvent_t ev_[2] = {nullptr, nullptr};
};

}  // namespace gb
