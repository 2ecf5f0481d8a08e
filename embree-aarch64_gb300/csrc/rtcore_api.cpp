// rtcore_api.cpp -- the C ABI (rtc* entry points) over the GPU builder and
// traversal kernels.
//
// Object model and error convention follow the reference's API layer
// (kernels/common/rtcore.cpp, kernels/common/device.cpp:258-318,
// kernels/common/rtcore.h:28-122): reference-counted handles, every entry
// point catches its own exceptions and turns them into an RTCError that is
// passed to the device's error callback and stored per (device, thread)
// until rtcGetDeviceError reads and clears it.  Errors without a device go
// to a per-thread slot read by rtcGetDeviceError(NULL).
//
// GPU residency: rtcCommitScene copies each enabled triangle geometry's
// buffers to HBM (device pointers are used in place) and runs the GPU
// builder on the calling thread's stream.  Queries copy host rays to a
// per-thread device buffer (or trace device rays in place), launch the
// persistent traversal kernel and return after the stream is synchronised.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "rtcore_gb300.h"
#include "rtcore_gb300_ext.h"
#include "gb_build.h"
#include "gb_common.h"
#include "gb_launch.h"
#include "gb_learned.h"
#include "gb_paths.h"
#include "gb_trace.h"

namespace {

struct rtc_error : public std::exception {
  RTCError code;
  std::string msg;
  rtc_error(RTCError c, std::string m) : code(c), msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

[[noreturn]] void fail(RTCError c, const char* m) { throw rtc_error(c, m); }

void cuda_ok(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return;
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) throw rtc_error(RTC_ERROR_OUT_OF_MEMORY, m);
  throw rtc_error(RTC_ERROR_UNKNOWN, m);
}

struct RefCounted {
  std::atomic<long> refs{1};
  virtual ~RefCounted() {}
  void inc() { refs.fetch_add(1); }
  void dec() {
    if (refs.fetch_sub(1) == 1) delete this;
  }
};

std::mutex g_mutex;  // device creation / properties (rtcore.cpp:20-25)

// ---------------------------------------------------------------------------
// device
// ---------------------------------------------------------------------------

struct Device : RefCounted {
  RTCErrorFunction error_fn = nullptr;
  void* error_user = nullptr;
  RTCMemoryMonitorFunction mem_fn = nullptr;
  void* mem_user = nullptr;
  int verbose = 0;
  int benchmark = 0;
  int cuda_device = -1;
  gb::BuildOptions build_opt;
  // host-resident rays: 0 copy all / trace / copy back, 1 chunked 3-stream
  // pipeline, 2 direct (the kernel reads and writes host memory itself where
  // the device can address it, else the pipeline).  Direct is the default: on
  // GB300 the kernel reaches host memory over NVLink-C2C at the pace it
  // consumes rays, so no copy phase is exposed.
  int host_mode = 2;
  bool proposer_mma = false;  // gpu.proposer=mma: proposer inference on mma.sync instead of tcgen05
  // gpu.graph_rebuild=0 turns off rebuilds replayed from a captured build graph
  // (scenes committed again with an unchanged layout; the graph keeps the build's
  // buffers allocated while the scene lives)
  int graph_rebuild = 1;
  int reorder = 0;            // gpu.reorder=1: streams of >= 65536 rays are traced in octant + origin-Morton order
  int trace_shape = 0;        // gpu.trace_shape=N: launch shape of the plain traversal (gb::kTraceShapes)
  int pageable_access = 0;     // cudaDevAttrPageableMemoryAccess
  int host_ptr_registered = 0; // cudaDevAttrCanUseHostPointerForRegisteredMem
  std::mutex mtx;

  explicit Device(const char* cfg) {
    if (cfg) parse(cfg);
    if (cuda_device < 0) cuda_ok(cudaGetDevice(&cuda_device), "cudaGetDevice");
    int n = 0;
    cuda_ok(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (cuda_device >= n) fail(RTC_ERROR_INVALID_ARGUMENT, "gpu.device out of range");
    cudaDeviceGetAttribute(&pageable_access, cudaDevAttrPageableMemoryAccess, cuda_device);
    cudaDeviceGetAttribute(&host_ptr_registered, cudaDevAttrCanUseHostPointerForRegisteredMem, cuda_device);
    cudaGetLastError();
    // rtcgbIntersect1MNoAlloc's static scratch (32 MiB + 256 B) and kernels are loaded
    // now, on this device, so that no call of it loads them (and takes memory) later
    int prev = 0;
    cuda_ok(cudaGetDevice(&prev), "cudaGetDevice");
    cuda_ok(cudaSetDevice(cuda_device), "cudaSetDevice");
    cudaError_t e = gb::noalloc_prepare();
    cudaSetDevice(prev);
    cuda_ok(e, "no-allocation query set-up");
  }

  // Config string: comma separated key=value tokens (kernels/common/state.cpp:217-450).
  // Honoured: verbose, benchmark, gpu.device, gpu.leaf_max, gpu.morton, gpu.morton_bits, gpu.collapse, gpu.ploc_radius,
  // gpu.host_rays, gpu.proposer, gpu.reorder, gpu.graph_rebuild, gpu.build_phases, gpu.trace_shape;
  // the CPU tasking and ISA keys
  // (threads, isa, max_isa, set_affinity, ...) are accepted and ignored.
  void parse(const char* cfg) {
    std::string s(cfg);
    size_t i = 0;
    while (i < s.size()) {
      size_t j = s.find(',', i);
      if (j == std::string::npos) j = s.size();
      std::string tok = s.substr(i, j - i);
      size_t eq = tok.find('=');
      auto trim = [](std::string x) {
        size_t a = x.find_first_not_of(" \t"), b = x.find_last_not_of(" \t");
        return a == std::string::npos ? std::string() : x.substr(a, b - a + 1);
      };
      if (eq != std::string::npos) {
        std::string k = trim(tok.substr(0, eq)), v = trim(tok.substr(eq + 1));
        if (k == "verbose") verbose = atoi(v.c_str());
        else if (k == "benchmark") benchmark = atoi(v.c_str());
        else if (k == "gpu.device") cuda_device = atoi(v.c_str());
        else if (k == "gpu.leaf_max") build_opt.leaf_max = atoi(v.c_str());
        else if (k == "gpu.morton") build_opt.morton_cube = v == "cube" ? 1 : v == "axis" ? 0 : 2;
        else if (k == "gpu.collapse") build_opt.collapse = v == "greedy" ? 0 : 1;
        else if (k == "gpu.ploc_radius") build_opt.ploc_radius = atoi(v.c_str());
        else if (k == "gpu.morton_bits") build_opt.morton_bits = atoi(v.c_str()) == 63 ? 63 : 30;
        else if (k == "gpu.graph_rebuild") graph_rebuild = atoi(v.c_str()) != 0;
        else if (k == "gpu.build_phases") build_opt.phase_stamps = atoi(v.c_str()) != 0;
        else if (k == "gpu.host_rays") host_mode = v == "copy" ? 0 : v == "direct" ? 2 : 1;
        else if (k == "gpu.proposer") proposer_mma = (v == "mma");
        else if (k == "gpu.reorder") reorder = atoi(v.c_str());
        else if (k == "gpu.trace_shape") {
          trace_shape = atoi(v.c_str());
          if (trace_shape < 0 || trace_shape >= gb::kNumTraceShapes)
            fail(RTC_ERROR_INVALID_ARGUMENT, "gpu.trace_shape: no such traversal launch shape");
        }
      }
      i = j + 1;
    }
  }

  void set_current() const { cuda_ok(cudaSetDevice(cuda_device), "cudaSetDevice"); }

  // memory monitor hook (device.cpp:318-328): a veto becomes OUT_OF_MEMORY
  void memory(ssize_t bytes, bool post) {
    if (mem_fn && bytes != 0 && !mem_fn(mem_user, bytes, post) && bytes > 0)
      fail(RTC_ERROR_OUT_OF_MEMORY, "memory monitor forced termination");
  }
};

thread_local RTCError t_thread_error = RTC_ERROR_NONE;
thread_local std::unordered_map<const Device*, RTCError> t_device_error;

void process_error(Device* d, RTCError e, const char* str) {
  if (!d) {
    if (t_thread_error == RTC_ERROR_NONE) t_thread_error = e;
    return;
  }
  if (d->verbose >= 1) fprintf(stderr, "rtcore-gb300: error %d (%s)\n", (int)e, str ? str : "");
  if (d->error_fn) d->error_fn(d->error_user, e, str);
  RTCError& slot = t_device_error[d];
  if (slot == RTC_ERROR_NONE) slot = e;
}

#define API_BEGIN try {
#define API_END(dev)                                                   \
  }                                                                    \
  catch (rtc_error & e) {                                              \
    process_error(dev, e.code, e.what());                              \
  }                                                                    \
  catch (std::bad_alloc&) {                                            \
    process_error(dev, RTC_ERROR_OUT_OF_MEMORY, "out of memory");      \
  }                                                                    \
  catch (std::exception & e) {                                         \
    process_error(dev, RTC_ERROR_UNKNOWN, e.what());                   \
  }                                                                    \
  catch (...) {                                                        \
    process_error(dev, RTC_ERROR_UNKNOWN, "unknown exception caught"); \
  }

#define VERIFY_HANDLE(h) \
  if ((h) == nullptr) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");

// ---------------------------------------------------------------------------
// buffers and geometry
// ---------------------------------------------------------------------------

struct Buffer : RefCounted {
  Device* device;
  char* ptr;
  size_t bytes;
  bool shared;
  Buffer(Device* d, size_t n, void* p) : device(d), ptr((char*)p), bytes(n), shared(p != nullptr) {
    device->inc();
    if (!shared) {
      ptr = (char*)malloc(std::max<size_t>(n, 16));
      if (!ptr) fail(RTC_ERROR_OUT_OF_MEMORY, "out of memory");
    }
  }
  ~Buffer() override {
    if (!shared) free(ptr);
    device->dec();
  }
};

struct View {
  Buffer* buf = nullptr;  // keeps a reference
  const char* ptr = nullptr;
  size_t stride = 0;
  size_t num = 0;
  RTCFormat format = RTC_FORMAT_UNDEFINED;
  void set(Buffer* b, size_t offset, size_t s, size_t n, RTCFormat f) {
    if (b) b->inc();
    if (buf) buf->dec();
    buf = b;
    ptr = b ? b->ptr + offset : nullptr;
    stride = s;
    num = n;
    format = f;
  }
  View() = default;
  View(const View&) = delete;
  View& operator=(const View&) = delete;
  ~View() {
    if (buf) buf->dec();
  }
};

cudaMemoryType pointer_type(const void* p) {
  if (!p) return cudaMemoryTypeUnregistered;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return cudaMemoryTypeUnregistered;
  }
  return a.type;
}

bool is_device_pointer(const void* p) {
  const cudaMemoryType t = pointer_type(p);
  return t == cudaMemoryTypeDevice || t == cudaMemoryTypeManaged;
}

struct Scene;
void release_scene_ref(Scene* s);

// Affine maps of instances, columns vx, vy, vz, p (the reference's
// AffineSpace3fa).  Fused multiply-adds where the reference's SSE/AVX2 code
// fuses them (madd chains of linearspace3.h / affinespace.h); this file is
// compiled with -ffp-contract=off so nothing else is fused.
namespace xf {
inline float dot3(const float* a, const float* b) { return std::fma(a[0], b[0], std::fma(a[1], b[1], a[2] * b[2])); }
inline void cross3(const float* a, const float* b, float* o) {
  o[0] = std::fma(a[1], b[2], -(a[2] * b[1]));
  o[1] = std::fma(a[2], b[0], -(a[0] * b[2]));
  o[2] = std::fma(a[0], b[1], -(a[1] * b[0]));
}
// world-to-local: rcp(AffineSpace3fa) = (adjoint / det, -(inverse * p))
// (common/math/affinespace.h:83, common/math/linearspace3.h:44-50), with the
// correctly rounded 1/det.  Returns false for a singular or non-finite map.
inline bool invert(const float* m, float* out) {
  const float *vx = m, *vy = m + 3, *vz = m + 6, *p = m + 9;
  float c0[3], c1[3], c2[3];
  cross3(vy, vz, c0);
  cross3(vz, vx, c1);
  cross3(vx, vy, c2);
  const float det = dot3(vx, c0);
  if (!(det != 0.0f) || !std::isfinite(det)) return false;
  const float r = 1.0f / det;
  for (int j = 0; j < 3; j++) {  // transposed adjoint: column j = (c0[j], c1[j], c2[j])
    out[3 * j + 0] = c0[j] * r;
    out[3 * j + 1] = c1[j] * r;
    out[3 * j + 2] = c2[j] * r;
  }
  for (int c = 0; c < 3; c++) out[9 + c] = -std::fma(p[0], out[c], std::fma(p[1], out[3 + c], p[2] * out[6 + c]));
  for (int k = 0; k < 12; k++)
    if (!std::isfinite(out[k])) return false;
  return true;
}
// xfmPoint (affinespace.h:102): madd chains ending in the translation
inline void xfm_point(const float* m, const float* q, float* o) {
  for (int c = 0; c < 3; c++) o[c] = std::fma(q[0], m[c], std::fma(q[1], m[3 + c], std::fma(q[2], m[6 + c], m[9 + c])));
}
}  // namespace xf

struct Geometry : RefCounted {
  Device* device;
  RTCGeometryType type;
  View vertices, indices;
  bool enabled = true;
  unsigned mask = 0xFFFFFFFFu;
  RTCBuildQuality quality = RTC_BUILD_QUALITY_MEDIUM;
  void* user = nullptr;
  RTCFilterFunctionN ifilter = nullptr;  // rtcSetGeometryIntersectFilterFunction
  RTCFilterFunctionN ofilter = nullptr;  // rtcSetGeometryOccludedFilterFunction
  unsigned time_steps = 1;
  uint64_t topo_version = 0;  // bumped when the index buffer is set or updated
  // device copies of host buffers
  char* d_verts = nullptr;
  char* d_idx = nullptr;
  size_t cap_verts = 0, cap_idx = 0;
  // instances: the instanced scene (retained) and the local-to-world map
  Scene* inst_scene = nullptr;
  float l2w[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};

  Geometry(Device* d, RTCGeometryType t) : device(d), type(t) { device->inc(); }
  ~Geometry() override {
    if (d_verts) cudaFree(d_verts);
    if (d_idx) cudaFree(d_idx);
    if (inst_scene) release_scene_ref(inst_scene);
    device->dec();
  }

  // TriangleMesh::setBuffer checks (kernels/common/scene_triangle_mesh.cpp:35-84)
  void set_buffer(RTCBufferType type, unsigned slot, RTCFormat format, Buffer* b, size_t offset, size_t stride,
                  size_t num) {
    if ((((size_t)(b ? b->ptr : nullptr) + offset) & 0x3) || (stride & 0x3))
      fail(RTC_ERROR_INVALID_OPERATION, "data must be 4 bytes aligned");
    if (type == RTC_BUFFER_TYPE_VERTEX) {
      if (format != RTC_FORMAT_FLOAT3) fail(RTC_ERROR_INVALID_OPERATION, "invalid vertex buffer format");
      if (stride * num > 16ull * 1024ull * 1024ull * 1024ull)
        fail(RTC_ERROR_INVALID_OPERATION, "vertex buffer can be at most 16GB large");
      if (slot >= time_steps) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid vertex buffer slot");
      vertices.set(b, offset, stride, num, format);
    } else if (type == RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE) {
      // no vertex attribute slots exist (rtcSetGeometryVertexAttributeCount is not provided)
      if (format < RTC_FORMAT_FLOAT || format > RTC_FORMAT_FLOAT16)
        fail(RTC_ERROR_INVALID_OPERATION, "invalid vertex attribute buffer format");
      fail(RTC_ERROR_INVALID_OPERATION, "invalid vertex attribute buffer slot");
    } else if (type == RTC_BUFFER_TYPE_INDEX) {
      if (slot != 0) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid buffer slot");
      if (format != RTC_FORMAT_UINT3) fail(RTC_ERROR_INVALID_OPERATION, "invalid index buffer format");
      indices.set(b, offset, stride, num, format);
      topo_version++;
    } else {
      fail(RTC_ERROR_INVALID_ARGUMENT, "unknown buffer type");
    }
  }

  View* view(RTCBufferType type, unsigned slot) {
    if (type == RTC_BUFFER_TYPE_INDEX) {
      if (slot != 0) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid buffer slot");
      return &indices;
    }
    if (type == RTC_BUFFER_TYPE_VERTEX) {
      if (slot >= time_steps) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid buffer slot");
      return &vertices;
    }
    fail(RTC_ERROR_INVALID_ARGUMENT, "unknown buffer type");
  }

  // Device view of one buffer: in place for device memory, else a copy.
  const char* upload(const View& v, char** dbuf, size_t* cap, cudaStream_t st) {
    if (!v.ptr || v.num == 0) return nullptr;
    if (is_device_pointer(v.ptr)) return v.ptr;
    const size_t bytes = (v.num - 1) * v.stride + (v.format == RTC_FORMAT_FLOAT3 || v.format == RTC_FORMAT_UINT3 ? 12 : v.stride);
    if (bytes > *cap) {
      if (*dbuf) cudaFree(*dbuf);
      *dbuf = nullptr;
      *cap = 0;
      device->memory((ssize_t)bytes, false);
      cuda_ok(cudaMalloc((void**)dbuf, bytes), "cudaMalloc geometry");
      *cap = bytes;
    }
    cuda_ok(cudaMemcpyAsync(*dbuf, v.ptr, bytes, cudaMemcpyHostToDevice, st), "upload geometry");
    return *dbuf;
  }
};

// ---------------------------------------------------------------------------
// per-thread query context
// ---------------------------------------------------------------------------

struct ThreadCtx {
  cudaStream_t own = nullptr;
  cudaStream_t user = nullptr;
  bool user_set = false;
  char* dbuf = nullptr;
  size_t cap = 0;
  unsigned int* dscratch = nullptr;     // [0] ray counter, [1] error flags, [2..] counters
  unsigned int* hscratch = nullptr;     // pinned mirror
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
  static constexpr int kMaxChunks = 32;
  cudaStream_t s_in = nullptr, s_out = nullptr;     // copy streams of the pipeline
  cudaEvent_t ev_in[kMaxChunks] = {}, ev_tr[kMaxChunks] = {};
  bool counting = false;
  RTCGBQueryStats last{};
  int device = -1;

  // The thread's own stream is a blocking stream: it is ordered after work the
  // caller issued on the legacy default stream (for example the copy that
  // filled a device ray buffer), as a synchronous query must be.
  cudaStream_t stream() {
    if (user_set) return user;
    if (!own) cuda_ok(cudaStreamCreateWithFlags(&own, cudaStreamDefault), "cudaStreamCreate");
    return own;
  }
  void ensure(int dev) {
    if (device == dev && dscratch) return;
    device = dev;
    cuda_ok(cudaMalloc((void**)&dscratch, 64), "cudaMalloc scratch");
    cuda_ok(cudaMallocHost((void**)&hscratch, 64), "cudaMallocHost");
    cuda_ok(cudaEventCreate(&e0), "event");
    cuda_ok(cudaEventCreate(&e1), "event");
    cuda_ok(cudaEventCreate(&e2), "event");
    cuda_ok(cudaEventCreate(&e3), "event");
  }
  void ensure_pipeline() {
    if (s_in) return;
    cuda_ok(cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_ok(cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int i = 0; i < kMaxChunks; i++) {
      cuda_ok(cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming), "event");
      cuda_ok(cudaEventCreateWithFlags(&ev_tr[i], cudaEventDisableTiming), "event");
    }
  }
  char* obuf = nullptr;     // ray reordering: keys, values and sort scratch
  size_t ocap = 0;
  char* order_buffer(size_t bytes) {
    if (bytes > ocap) {
      if (obuf) cudaFree(obuf);
      obuf = nullptr;
      ocap = 0;
      const size_t want = std::max(bytes, ocap * 2);
      cuda_ok(cudaMalloc((void**)&obuf, want), "cudaMalloc ray order");
      ocap = want;
    }
    return obuf;
  }
  uint4* seeds = nullptr;   // learned queries: per-ray proposals
  size_t seeds_cap = 0;
  uint4* seed_buffer(size_t n) {
    if (n > seeds_cap) {
      if (seeds) cudaFree(seeds);
      seeds = nullptr;
      seeds_cap = 0;
      const size_t want = std::max(n, seeds_cap * 2);
      cuda_ok(cudaMalloc((void**)&seeds, want * sizeof(uint4)), "cudaMalloc proposals");
      seeds_cap = want;
    }
    return seeds;
  }
  char* buffer(size_t bytes) {
    if (bytes > cap) {
      if (dbuf) cudaFree(dbuf);
      dbuf = nullptr;
      cap = 0;
      size_t want = std::max(bytes, cap * 2);
      cuda_ok(cudaMalloc((void**)&dbuf, want), "cudaMalloc rays");
      cap = want;
    }
    return dbuf;
  }
  ~ThreadCtx() {
    if (dbuf) cudaFree(dbuf);
    if (seeds) cudaFree(seeds);
    if (obuf) cudaFree(obuf);
    if (dscratch) cudaFree(dscratch);
    if (hscratch) cudaFreeHost(hscratch);
    if (own) cudaStreamDestroy(own);
    if (s_in) cudaStreamDestroy(s_in);
    if (s_out) cudaStreamDestroy(s_out);
    for (cudaEvent_t e : {e0, e1, e2, e3})
      if (e) cudaEventDestroy(e);
    for (int i = 0; i < kMaxChunks; i++) {
      if (ev_in[i]) cudaEventDestroy(ev_in[i]);
      if (ev_tr[i]) cudaEventDestroy(ev_tr[i]);
    }
  }
};

thread_local ThreadCtx t_ctx;

// ---------------------------------------------------------------------------
// scene
// ---------------------------------------------------------------------------

struct Scene : RefCounted {
  Device* device;
  std::mutex mtx;
  std::vector<Geometry*> geoms;  // index = geomID
  std::set<unsigned> free_ids;
  RTCSceneFlags flags = RTC_SCENE_FLAG_NONE;
  RTCBuildQuality quality = RTC_BUILD_QUALITY_MEDIUM;
  RTCProgressMonitorFunction progress = nullptr;
  void* progress_ptr = nullptr;
  bool committed = false;
  gb::DeviceBVH bvh;
  gb::BuildStats stats;
  // topology of the last full build: (geomID, geometry, index version, triangles, vertices)
  struct SigEntry {
    unsigned id;
    const Geometry* g;
    uint64_t topo;
    size_t ntris, nverts;
    bool operator==(const SigEntry& o) const {
      return id == o.id && g == o.g && topo == o.topo && ntris == o.ntris && nverts == o.nverts;
    }
  };
  std::vector<SigEntry> built_sig;
  bool built_robust = false;
  // rebuilds replayed from a captured build graph: the layout key of the last
  // host-driven build and, once the scene was built twice with that layout, the graph
  std::vector<uint64_t> layout_key;
  gb::CachedBuild* gcache = nullptr;
  uint64_t build_serial = 0;  // counts full builds (a refit keeps the BVH's structure)
  std::vector<gb::GeomDesc> descs;  // geometry table of the committed BVH (device buffers)
  bool batched = false;             // rtcgbSetSceneBatched: one tree per geometry
  uint32_t* d_roots = nullptr;      // batched BVH: root node per geometry ID (device)
  uint32_t nroots = 0;
  uint64_t commit_serial = 0;       // counts commits (builds and refits)
  // filter callbacks are called: some geometry had one, or the scene had
  // RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION, at the last commit (the reference picks its
  // filtering intersectors at commit, kernels/common/scene.cpp:679, 721)
  bool filters = false;
  // instances of the committed BVH: device table, and the instanced scenes it
  // reads (retained) with their commit serials at this scene's commit
  gb::InstDesc* d_insts = nullptr;
  uint32_t ninsts = 0;
  uint64_t inst_nodes = 0;          // nodes of all instanced BVHs (iteration bound)
  std::vector<std::pair<Scene*, uint64_t>> inst_refs;
  // launch shape of the plain traversal kernels for this scene's queries
  // (rtcgbSetSceneTraversalShape / rtcgbTuneSceneTraversal; from the device's
  // gpu.trace_shape until set)
  std::atomic<int> trace_shape{0};

  explicit Scene(Device* d) : device(d), trace_shape(d->trace_shape) { device->inc(); }
  void drop_instances();
  ~Scene() override {
    for (Geometry* g : geoms)
      if (g) g->dec();
    drop_instances();
    if (d_roots) cudaFree(d_roots);
    gb::free_bvh(&bvh);
    gb::cached_build_release(gcache);
    device->dec();
  }

  // Scene::bind (kernels/common/scene.cpp:595-623) with the ID pool's
  // smallest-free-ID policy.
  unsigned attach(Geometry* g, unsigned id) {
    std::lock_guard<std::mutex> lk(mtx);
    if (id == RTC_INVALID_GEOMETRY_ID) {
      if (!free_ids.empty()) {
        id = *free_ids.begin();
        free_ids.erase(free_ids.begin());
      } else {
        id = (unsigned)geoms.size();
        geoms.push_back(nullptr);
      }
    } else {
      if (id < geoms.size() && geoms[id]) fail(RTC_ERROR_INVALID_ARGUMENT, "geometry ID already assigned");
      while (geoms.size() <= id) {
        free_ids.insert((unsigned)geoms.size());
        geoms.push_back(nullptr);
      }
      free_ids.erase(id);
    }
    g->inc();
    geoms[id] = g;
    return id;
  }

  void detach(unsigned id) {
    std::lock_guard<std::mutex> lk(mtx);
    if (id >= geoms.size() || !geoms[id]) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid geometry ID");
    geoms[id]->dec();
    geoms[id] = nullptr;
    free_ids.insert(id);
  }

  void commit() {
    std::lock_guard<std::mutex> lk(mtx);
    device->set_current();
    t_ctx.ensure(device->cuda_device);
    cudaStream_t st = t_ctx.stream();
    if (progress && !progress(progress_ptr, 0.0)) fail(RTC_ERROR_CANCELLED, "progress monitor forced termination");
    std::vector<gb::GeomDesc> descs;
    uint64_t total = 0;
    // instances: world boxes for the builder, the traversal's table, the scenes they read
    std::vector<gb::InstBox> iboxes;
    std::vector<gb::InstDesc> idescs;
    std::vector<std::pair<Scene*, uint64_t>> irefs;
    uint64_t inodes = 0;
    const bool robust_now = (flags & RTC_SCENE_FLAG_ROBUST) != 0;
    bool filters_now = (flags & RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION) != 0;
    for (const Geometry* g : geoms)
      if (g && g->enabled && (g->ifilter || g->ofilter)) filters_now = true;
    for (unsigned id = 0; id < geoms.size(); id++) {
      Geometry* g = geoms[id];
      if (!g || !g->enabled || g->type != RTC_GEOMETRY_TYPE_INSTANCE || !g->inst_scene) continue;
      if (g->inst_scene->filters) filters_now = true;  // queries then refuse (instances)
      if (batched) fail(RTC_ERROR_INVALID_OPERATION, "batched scenes hold triangle meshes only");
      if (robust_now) fail(RTC_ERROR_INVALID_OPERATION, "instances in robust scenes are not supported");
      Scene* is = g->inst_scene;
      if (is == this) fail(RTC_ERROR_INVALID_OPERATION, "a scene cannot instance itself");
      if (!is->committed) fail(RTC_ERROR_INVALID_OPERATION, "instanced scene not committed");
      if (is->bvh.robust || is->batched) fail(RTC_ERROR_INVALID_OPERATION, "instanced scene must be a plain triangle scene");
      irefs.push_back({is, is->commit_serial});
      if (is->bvh.num_nodes == 0) continue;  // empty scene: nothing to hit
      gb::InstDesc in{};
      if (!xf::invert(g->l2w, in.w2l)) continue;  // singular transform: the instance is never hit
      in.nodes = is->bvh.nodes;
      in.tris = is->bvh.tris;
      in.num_nodes = is->bvh.num_nodes;
      in.num_tris = is->bvh.num_tris;
      in.geomID = id;
      // xfmBounds (affinespace.h:105-118) of the instanced scene's box, widened
      // by a few ulps of its magnitude so that rounding never culls a hit
      gb::InstBox b{};
      for (int a = 0; a < 3; a++) { b.lo[a] = INFINITY; b.hi[a] = -INFINITY; }
      for (int k = 0; k < 8; k++) {
        const float q[3] = {(k & 1) ? is->bvh.hi[0] : is->bvh.lo[0], (k & 2) ? is->bvh.hi[1] : is->bvh.lo[1],
                            (k & 4) ? is->bvh.hi[2] : is->bvh.lo[2]};
        float w[3];
        xf::xfm_point(g->l2w, q, w);
        for (int a = 0; a < 3; a++) { b.lo[a] = std::min(b.lo[a], w[a]); b.hi[a] = std::max(b.hi[a], w[a]); }
      }
      for (int a = 0; a < 3; a++) {
        const float mag = std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a])) + (b.hi[a] - b.lo[a]);
        b.lo[a] -= 4e-6f * mag;
        b.hi[a] += 4e-6f * mag;
      }
      b.inst = (uint32_t)idescs.size();
      b.geomID = id;
      iboxes.push_back(b);
      idescs.push_back(in);
      inodes += in.num_nodes;
    }
    for (unsigned id = 0; id < geoms.size(); id++) {
      Geometry* g = geoms[id];
      if (!g || !g->enabled || g->type != RTC_GEOMETRY_TYPE_TRIANGLE) continue;
      if (!g->vertices.ptr || !g->indices.ptr || g->indices.num == 0) continue;
      gb::GeomDesc d{};
      d.verts = g->upload(g->vertices, &g->d_verts, &g->cap_verts, st);
      d.idx = g->upload(g->indices, &g->d_idx, &g->cap_idx, st);
      d.vstride = g->vertices.stride;
      d.istride = g->indices.stride;
      d.nverts = (uint32_t)g->vertices.num;
      d.ntris = (uint32_t)g->indices.num;
      d.geomID = id;
      d.prim_offset = (uint32_t)total;
      total += d.ntris;
      descs.push_back(d);
    }
    // all instances as one kind-1 geometry of box primitives
    gb::InstBox* d_boxes = nullptr;
    std::unique_ptr<gb::InstBox, void (*)(gb::InstBox*)> boxes_guard(nullptr, [](gb::InstBox* q) { if (q) cudaFree(q); });
    if (!iboxes.empty()) {
      cuda_ok(cudaMalloc((void**)&d_boxes, iboxes.size() * sizeof(gb::InstBox)), "cudaMalloc instances");
      boxes_guard.reset(d_boxes);
      cuda_ok(cudaMemcpyAsync(d_boxes, iboxes.data(), iboxes.size() * sizeof(gb::InstBox), cudaMemcpyHostToDevice, st),
              "instances");
      gb::GeomDesc d{};
      d.verts = (const char*)d_boxes;
      d.ntris = (uint32_t)iboxes.size();
      d.geomID = gb::kInvalidID;
      d.prim_offset = (uint32_t)total;
      d.kind = 1;
      total += d.ntris;
      descs.push_back(d);
    }
    if (total >= 0x7FFFFFFFull) fail(RTC_ERROR_INVALID_OPERATION, "too many primitives");
    std::vector<SigEntry> sig;
    bool all_refit = !descs.empty();
    for (const gb::GeomDesc& d : descs) {
      if (d.kind != 0) {  // scenes with instances are always rebuilt
        all_refit = false;
        continue;
      }
      const Geometry* g = geoms[d.geomID];
      sig.push_back(SigEntry{d.geomID, g, g->topo_version, d.ntris, d.nverts});
      all_refit &= g->quality == RTC_BUILD_QUALITY_REFIT;
    }
    const bool robust = (flags & RTC_SCENE_FLAG_ROBUST) != 0;  // scene.cpp:119-125: Triangle4v + Pluecker
    // geometries marked RTC_BUILD_QUALITY_REFIT whose topology is unchanged
    // since the last build are refitted (kernels/bvh/bvh_refit.cpp:30-247)
    if (committed && all_refit && bvh.num_nodes > 0 && sig == built_sig && robust == built_robust) {
      gb::BuildStats bs = stats;
      bool fallback = false;
      cuda_ok(gb::refit_bvh(descs.data(), (int)descs.size(), st, &bvh, &bs, &fallback), "rtcCommitScene (refit)");
      if (!fallback) {
        stats = bs;
        this->descs = descs;
        filters = filters_now;
        commit_serial++;
        if (progress) progress(progress_ptr, 1.0);
        return;
      }
    }
    // estimated device bytes of the build (scratch + result)
    device->memory((ssize_t)(total * 256 + 4096), false);
    gb::free_bvh(&bvh);
    committed = false;
    gb::BuildStats bs;
    gb::BuildOptions opt = device->build_opt;
    opt.robust = robust;
    opt.segmented = batched ? 1 : 0;
    opt.refit_target = all_refit ? 1 : 0;
    // the layout of this build: geometry slots and counts, options (buffer addresses
    // and strides are read from the geometry table at run time)
    std::vector<uint64_t> key = {(uint64_t)opt.robust, (uint64_t)opt.segmented, (uint64_t)opt.refit_target,
                                 (uint64_t)opt.leaf_max, (uint64_t)opt.morton_cube, (uint64_t)opt.morton_bits,
                                 (uint64_t)opt.collapse, (uint64_t)opt.ploc_radius, (uint64_t)opt.phase_stamps};
    for (const gb::GeomDesc& d : descs)
      key.insert(key.end(), {(uint64_t)d.geomID, (uint64_t)d.ntris, (uint64_t)d.nverts, (uint64_t)d.kind});
    const bool cacheable = device->graph_rebuild && iboxes.empty() && !descs.empty();
    bool replayed = false;
    if (cacheable && gcache && key == layout_key) {
      const cudaError_t e = gb::cached_build_run(gcache, descs.data(), (int)descs.size(), st, &bvh, &bs);
      if (e == cudaSuccess) {
        replayed = true;
      } else {
        cudaGetLastError();
        gb::free_bvh(&bvh);
        gb::cached_build_release(gcache);
        gcache = nullptr;
        if (e != cudaErrorNotReady) cuda_ok(e, "rtcCommitScene (replayed build)");
      }
    } else if (gcache && key != layout_key) {
      gb::cached_build_release(gcache);
      gcache = nullptr;
    }
    if (!replayed) {
      cuda_ok(gb::build_bvh(descs.data(), (int)descs.size(), st, opt, &bvh, &bs), "rtcCommitScene");
      // built twice with this layout: capture the build for the next commits
      if (cacheable && !gcache && key == layout_key && bs.num_prims > 0 && bs.depth >= 1 && bs.depth <= 64) {
        gb::GraphBuildPlan plan;
        plan.valid_tris = bs.num_prims;
        plan.roots = 0;
        for (uint32_t r : bvh.roots) plan.roots += r != gb::kInvalidID ? 1u : 0u;
        if (!opt.segmented || plan.roots == 0) plan.roots = 1;
        plan.ploc_rounds = bs.ploc_iterations;
        plan.levels = bs.depth;
        plan.leaf_max = (int)bs.leaf_max;
        gb::BuildOptions gopt = opt;
        gopt.leaf_max = plan.leaf_max;
        if (gb::cached_build_create(descs.data(), (int)descs.size(), gopt, plan, st, &gcache) != cudaSuccess) {
          cudaGetLastError();
          gcache = nullptr;  // keep building the ordinary way
        }
      }
      layout_key = key;
    }
    if (d_roots) cudaFree(d_roots);
    d_roots = nullptr;
    nroots = 0;
    if (batched) {
      // root of every geometry ID (descs are in slot order; bvh.roots is per slot)
      std::vector<uint32_t> by_id(geoms.size(), gb::kInvalidID);
      for (size_t k = 0; k < descs.size() && k < bvh.roots.size(); k++) by_id[descs[k].geomID] = bvh.roots[k];
      nroots = (uint32_t)by_id.size();
      cuda_ok(cudaMalloc((void**)&d_roots, std::max<size_t>(1, by_id.size()) * sizeof(uint32_t)), "cudaMalloc roots");
      cuda_ok(cudaMemcpyAsync(d_roots, by_id.data(), by_id.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st),
              "roots");
      cuda_ok(cudaStreamSynchronize(st), "roots");
    }
    stats = bs;
    committed = true;
    filters = filters_now;
    build_serial++;
    commit_serial++;
    this->descs = descs;
    drop_instances();
    if (!idescs.empty()) {
      cuda_ok(cudaMalloc((void**)&d_insts, idescs.size() * sizeof(gb::InstDesc)), "cudaMalloc instance table");
      cuda_ok(cudaMemcpyAsync(d_insts, idescs.data(), idescs.size() * sizeof(gb::InstDesc), cudaMemcpyHostToDevice, st),
              "instance table");
      cuda_ok(cudaStreamSynchronize(st), "instance table");
      ninsts = (uint32_t)idescs.size();
      inst_nodes = inodes;
    }
    for (auto& r : irefs) r.first->inc();
    inst_refs = irefs;
    built_sig = sig;
    built_robust = robust;
    if (progress) progress(progress_ptr, 1.0);
    if (device->benchmark)
      printf("BENCHMARK_BUILD %f %f %f %u\n", bs.build_ms * 1e-3, bs.build_ms > 0 ? bs.num_prims / (bs.build_ms * 1e-3) : 0.0,
             bs.sah, (unsigned)(bvh.num_nodes * sizeof(gb::WideNode) + bvh.num_tris * sizeof(gb::TriRecord)));
    if (device->verbose >= 2)
      fprintf(stderr, "rtcore-gb300: built %u prims, %u nodes, depth %u, SAH %.3f, %.3f ms\n", bs.num_prims,
              bs.num_nodes, bs.depth, bs.sah, bs.build_ms);
  }
};

void Scene::drop_instances() {
  if (d_insts) cudaFree(d_insts);
  d_insts = nullptr;
  ninsts = 0;
  inst_nodes = 0;
  for (auto& r : inst_refs) r.first->dec();
  inst_refs.clear();
}

void release_scene_ref(Scene* s) { s->dec(); }

// ---------------------------------------------------------------------------
// learned proposer
// ---------------------------------------------------------------------------

struct ProposerObj : RefCounted {
  Scene* scene;
  uint64_t build_serial;
  gb::Proposer net;
  std::vector<uint32_t> roots, record_treelet;
  std::mutex mtx;
  explicit ProposerObj(Scene* s) : scene(s), build_serial(s->build_serial) { scene->inc(); }
  ~ProposerObj() override {
    scene->device->set_current();
    net.release();
    scene->dec();
  }
  // usable for queries on the scene as currently built
  bool current() const { return scene->committed && build_serial == scene->build_serial && !scene->bvh.robust; }
};

// ---------------------------------------------------------------------------
// queries
// ---------------------------------------------------------------------------

// Batched queries on a segmented BVH: rays [start[b], start[b+1]) query geometry b.
struct BatchArgs {
  const uint32_t* start = nullptr;  // caller's array (host or device), nbatches + 1 entries
  uint32_t nbatches = 0;
};

// Filter callbacks (rtcSetGeometryIntersectFilterFunction, rtcSetGeometryOccludedFilterFunction,
// RTCIntersectContext::filter).  The reference calls them for every candidate hit inside its
// traversal (kernels/geometry/intersector_epilog.h:237-276, 397-435;
// kernels/geometry/filter.h:14-37, 72-89): the geometry's callback, then the context's; a
// hit is rejected when either clears valid[0]; a closest-hit query keeps the nearest
// accepted hit, an occlusion query stops at the first accepted one.  Here the traversal
// stays on the GPU and the callbacks run on the calling thread between launches.  Each round
// traces the pending rays for their nearest hit among the triangles no callback has rejected
// for them (the kernel skips each ray's rejected (primID, geomID) list), calls the callbacks
// for those hits with N = 1, the ray's tfar set to the hit distance and the hit in an
// RTCHit, and traces again only the rays whose hit was rejected.  For callbacks that decide
// from their arguments, the result is the reference's: the nearest accepted hit, occlusion
// iff some hit in range is accepted.  The callbacks see the hits in distance order (the
// reference: traversal order), and what they write to the ray or hit is kept for accepted
// hits only (the reference restores tfar only).
void run_filtered(Scene* scene, const RTCIntersectContext* uctx, void* rays, unsigned M, size_t stride, bool anyhit,
                  size_t recsize) {
  ThreadCtx& c = t_ctx;
  const gb::DeviceBVH& bvh = scene->bvh;
  Device* dev = scene->device;
  dev->set_current();
  c.ensure(dev->cuda_device);
  cudaStream_t st = c.stream();
  const size_t span = (size_t)(M - 1) * stride + recsize;
  // the caller's records, on the host
  const bool on_device = is_device_pointer(rays);
  std::vector<char> staged;
  char* host = (char*)rays;
  if (on_device) {
    staged.resize(span);
    cuda_ok(cudaMemcpyAsync(staged.data(), rays, span, cudaMemcpyDeviceToHost, st), "D2H rays");
    cuda_ok(cudaStreamSynchronize(st), "D2H rays");
    host = staged.data();
  }
  // stream validity (kernels/bvh/bvh_intersector_stream_filters.cpp:75, 145)
  std::vector<uint32_t> pend;
  for (unsigned i = 0; i < M; i++) {
    RTCRay r;
    std::memcpy(&r, host + (size_t)i * stride, sizeof(RTCRay));
    if (!(r.tnear <= r.tfar) || (anyhit && r.tfar < 0.0f)) continue;
    pend.push_back(i);
  }
  // rejected (primID, geomID) lists of the pending rays, CSR: ray j's list is
  // items[off[j] .. off[j+1]); rebuilt for the rays kept after each round
  std::vector<uint32_t> off(pend.size() + 1, 0u), next_off;
  std::vector<uint2> items, next_items;
  std::vector<RTCRayHit> work;
  float k_ms_total = 0.0f;
  unsigned launches = 0;
  const unsigned inst0 = uctx ? uctx->instID[0] : RTC_INVALID_GEOMETRY_ID;
  while (!pend.empty()) {
    const size_t n = pend.size();
    work.assign(n, RTCRayHit{});
    for (size_t j = 0; j < n; j++) {
      std::memcpy(&work[j].ray, host + (size_t)pend[j] * stride, sizeof(RTCRay));
      work[j].hit.geomID = work[j].hit.primID = work[j].hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
    }
    // device layout: records (80 B each), list offsets, lists
    const size_t b_work = n * sizeof(RTCRayHit), b_off = ((n + 1) * 4 + 15) & ~size_t(15);
    char* d = c.buffer(b_work + b_off + items.size() * sizeof(uint2) + 16);
    cuda_ok(cudaMemcpyAsync(d, work.data(), b_work, cudaMemcpyHostToDevice, st), "H2D rays");
    cuda_ok(cudaMemcpyAsync(d + b_work, off.data(), (n + 1) * 4, cudaMemcpyHostToDevice, st), "H2D rejected");
    if (!items.empty())
      cuda_ok(cudaMemcpyAsync(d + b_work + b_off, items.data(), items.size() * sizeof(uint2), cudaMemcpyHostToDevice,
                              st), "H2D rejected");
    gb::TraceParams P{};
    P.nodes = bvh.nodes;
    P.tris = bvh.tris;
    P.rays = d;
    P.stride = sizeof(RTCRayHit);
    P.nrays = (uint32_t)n;
    P.ray_counter = c.dscratch;
    P.err = c.dscratch + 1;
    P.counters = reinterpret_cast<gb::TraceCounters*>(c.dscratch + 2);
    P.max_iters = 4 * bvh.num_nodes + 64;
    P.num_nodes = bvh.num_nodes;
    P.num_tris = bvh.num_tris;
    P.robust = bvh.robust;
    P.excl_off = reinterpret_cast<const uint32_t*>(d + b_work);
    P.excl = reinterpret_cast<const uint2*>(d + b_work + b_off);
    cuda_ok(cudaMemsetAsync(c.dscratch, 0, 64, st), "memset");
    cuda_ok(cudaEventRecord(c.e1, st), "event");
    cuda_ok(gb::launch_trace(P, false, false, st), "traversal launch");
    cuda_ok(cudaEventRecord(c.e2, st), "event");
    launches += 2;
    cuda_ok(cudaMemcpyAsync(work.data(), d, b_work, cudaMemcpyDeviceToHost, st), "D2H rays");
    cuda_ok(cudaMemcpyAsync(c.hscratch, c.dscratch, 64, cudaMemcpyDeviceToHost, st), "D2H status");
    cuda_ok(cudaStreamSynchronize(st), "traversal");
    float k_ms = 0.0f;
    cudaEventElapsedTime(&k_ms, c.e1, c.e2);
    k_ms_total += k_ms;
    const unsigned err = c.hscratch[1];
    if (err & gb::kErrStackOverflow) fail(RTC_ERROR_UNKNOWN, "traversal stack overflow");
    if (err & gb::kErrIterationLimit) fail(RTC_ERROR_UNKNOWN, "traversal iteration limit reached");
    if (err & gb::kErrBuild) fail(RTC_ERROR_UNKNOWN, "traversal found an invalid BVH reference");
    // callbacks on this round's hits
    size_t keep = 0;
    next_off.assign(1, 0u);
    next_items.clear();
    for (size_t j = 0; j < n; j++) {
      const RTCRayHit& w = work[j];
      if (w.hit.geomID == RTC_INVALID_GEOMETRY_ID) continue;  // no further hit: done
      char* rec = host + (size_t)pend[j] * stride;
      const Geometry* g = w.hit.geomID < scene->geoms.size() ? scene->geoms[w.hit.geomID] : nullptr;
      const RTCFilterFunctionN gf = g ? (anyhit ? g->ofilter : g->ifilter) : nullptr;
      const RTCFilterFunctionN cf = uctx ? uctx->filter : nullptr;
      RTCRayHit tmp;
      std::memcpy(&tmp.ray, rec, sizeof(RTCRay));
      tmp.ray.tfar = w.ray.tfar;  // the hit distance
      tmp.hit = w.hit;
      tmp.hit.instID[0] = inst0;
      bool accepted = true;
      if (gf || cf) {
        int valid = -1;
        RTCFilterFunctionNArguments args;
        args.valid = &valid;
        args.geometryUserPtr = g ? g->user : nullptr;
        args.context = const_cast<RTCIntersectContext*>(uctx);
        args.ray = reinterpret_cast<RTCRayN*>(&tmp.ray);
        args.hit = reinterpret_cast<RTCHitN*>(&tmp.hit);
        args.N = 1;
        if (gf) {
          gf(&args);
          accepted = valid != 0;
        }
        if (accepted && cf) {
          cf(&args);
          accepted = valid != 0;
        }
      }
      if (accepted) {
        if (anyhit) {
          const float ninf = -INFINITY;
          std::memcpy(rec + 32, &ninf, 4);
        } else {
          std::memcpy(rec, &tmp, sizeof(RTCRayHit));  // copyHitToRay (kernels/common/ray.h)
        }
        continue;
      }
      next_items.insert(next_items.end(), items.begin() + off[j], items.begin() + off[j + 1]);
      next_items.push_back(make_uint2(w.hit.primID, w.hit.geomID));
      next_off.push_back((uint32_t)next_items.size());
      pend[keep++] = pend[j];
    }
    pend.resize(keep);
    off.swap(next_off);
    items.swap(next_items);
  }
  if (on_device) {
    cuda_ok(cudaMemcpyAsync(rays, host, span, cudaMemcpyHostToDevice, st), "H2D results");
    cuda_ok(cudaStreamSynchronize(st), "H2D results");
  }
  gb::note_launches(launches);
  c.last.kernel_ms = k_ms_total;
  c.last.h2d_bytes = span;
  c.last.d2h_bytes = span;
}

void run_query(Scene* scene, void* rays, unsigned M, size_t stride, bool anyhit, size_t recsize,
               ProposerObj* prop = nullptr, const BatchArgs* batch = nullptr,
               const RTCIntersectContext* uctx = nullptr) {
  VERIFY_HANDLE(scene);
  if (!scene->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  if (M == 0) return;
  if (!rays) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (((size_t)rays & 0x3) || (stride & 0x3)) fail(RTC_ERROR_INVALID_ARGUMENT, "ray not aligned to 4 bytes");
  if (stride < recsize) fail(RTC_ERROR_INVALID_ARGUMENT, "byteStride smaller than the ray record");
  ThreadCtx& c = t_ctx;
  c.last = RTCGBQueryStats{};
  const gb::DeviceBVH& bvh = scene->bvh;
  if (bvh.num_nodes == 0) return;  // empty scene: nothing is hit
  if (scene->batched != (batch != nullptr))
    fail(RTC_ERROR_INVALID_OPERATION, scene->batched ? "batched scene: use rtcgbIntersect1MBatched / rtcgbOccluded1MBatched"
                                                     : "not a batched scene (rtcgbSetSceneBatched)");
  if (prop && scene->batched) fail(RTC_ERROR_INVALID_OPERATION, "the proposer does not support batched scenes");
  if (prop && scene->ninsts) fail(RTC_ERROR_INVALID_OPERATION, "the proposer does not support scenes with instances");
  if (scene->filters) {
    if (prop || batch) fail(RTC_ERROR_INVALID_OPERATION, "learned and batched queries do not call filter callbacks");
    if (scene->ninsts || !scene->inst_refs.empty())
      fail(RTC_ERROR_INVALID_OPERATION, "filter callbacks in scenes with instances are not supported");
    run_filtered(scene, uctx, rays, M, stride, anyhit, recsize);
    return;
  }
  // the BVHs the instance leaves point to must be those of this scene's commit
  for (const auto& r : scene->inst_refs)
    if (!r.first->committed || r.first->commit_serial != r.second)
      fail(RTC_ERROR_INVALID_OPERATION, "an instanced scene changed: commit the instancing scene again");
  if (prop && prop->scene != scene) fail(RTC_ERROR_INVALID_ARGUMENT, "proposer belongs to another scene");
  // seeded traversal needs 16-byte aligned records; otherwise the plain one runs
  if (prop && (!prop->current() || (stride % 16) != 0)) prop = nullptr;
  std::unique_lock<std::mutex> prop_lock;
  if (prop) prop_lock = std::unique_lock<std::mutex>(prop->mtx);
  Device* dev = scene->device;
  dev->set_current();
  c.ensure(dev->cuda_device);
  cudaStream_t st = c.stream();
  const size_t span = (size_t)(M - 1) * stride + recsize;
  const cudaMemoryType mt = pointer_type(rays);
  const bool on_device = mt == cudaMemoryTypeDevice || mt == cudaMemoryTypeManaged;
  // host memory the kernel may address directly (NVLink-C2C / ATS)
  const bool direct = !on_device && dev->host_mode == 2 &&
                      ((mt == cudaMemoryTypeHost && dev->host_ptr_registered) ||
                       (mt == cudaMemoryTypeUnregistered && dev->pageable_access));
  gb::TraceParams P{};
  P.nodes = bvh.nodes;
  P.tris = bvh.tris;
  P.stride = stride;
  P.ray_counter = c.dscratch;
  P.err = c.dscratch + 1;
  P.counters = reinterpret_cast<gb::TraceCounters*>(c.dscratch + 2);
  P.max_iters = 4 * bvh.num_nodes + 64;  // node visits, triangle phases and pops per ray
  if (scene->ninsts) {
    P.insts = scene->d_insts;
    P.ninsts = scene->ninsts;
    P.max_iters = (uint32_t)std::min<uint64_t>(0x7FFFFFFFull, 4 * ((uint64_t)bvh.num_nodes + scene->inst_nodes) + 64);
  }
  P.num_nodes = bvh.num_nodes;
  P.num_tris = bvh.num_tris;
  P.robust = bvh.robust;
  P.shape = scene->trace_shape.load(std::memory_order_relaxed);
  // batched: the batch boundaries on the device, validated on the host
  std::unique_ptr<uint32_t, void (*)(uint32_t*)> d_start(nullptr, [](uint32_t* p) { if (p) cudaFree(p); });
  if (batch) {
    if (!batch->start || batch->nbatches == 0 || batch->nbatches > scene->nroots)
      fail(RTC_ERROR_INVALID_ARGUMENT, "invalid batches");
    std::vector<uint32_t> hs(batch->nbatches + 1);
    cuda_ok(cudaMemcpy(hs.data(), batch->start, hs.size() * sizeof(uint32_t), cudaMemcpyDefault), "batches");
    if (hs[0] != 0 || hs.back() != M) fail(RTC_ERROR_INVALID_ARGUMENT, "batches must cover the rays exactly");
    for (size_t b = 1; b < hs.size(); b++)
      if (hs[b] < hs[b - 1]) fail(RTC_ERROR_INVALID_ARGUMENT, "batch boundaries must not decrease");
    uint32_t* p = nullptr;
    cuda_ok(cudaMalloc((void**)&p, hs.size() * sizeof(uint32_t)), "cudaMalloc batches");
    d_start.reset(p);
    cuda_ok(cudaMemcpyAsync(p, hs.data(), hs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st), "batches");
    P.batch_start = p;
    P.batch_root = scene->d_roots;
    P.nbatches = batch->nbatches;
  }
  cuda_ok(cudaEventRecord(c.e0, st), "event");
  cuda_ok(cudaMemsetAsync(c.dscratch, 0, 64, st), "memset");
  unsigned launches = 1;
  const uint32_t kChunk = 1u << 21;  // rays per pipeline stage
  // ray reordering (gpu.reorder=1): fetch order by direction octant and origin Morton code
  auto reorder = [&](gb::TraceParams& Pq) {
    if (!dev->reorder || Pq.nrays < (1u << 16)) return;
    const size_t n = Pq.nrays, hist = gb::sort_hist_entries(Pq.nrays);
    char* b = c.order_buffer(n * 24 + hist * 4 + 64);
    uint64_t* keys = reinterpret_cast<uint64_t*>(b);
    uint64_t* kb = keys + n;
    uint32_t* vals = reinterpret_cast<uint32_t*>(kb + n);
    uint32_t* vb = vals + n;
    uint32_t* h = vb + n;
    cuda_ok(gb::order_rays(Pq.rays, stride, Pq.nrays, bvh.lo, bvh.hi, keys, vals, kb, vb, h, st), "ray order");
    Pq.order = vals;
    launches += 19;
  };
  // learned queries: proposals for every ray, then the seeded traversal
  auto propose = [&](gb::TraceParams& Pq) {
    if (!prop) return;
    uint4* seeds = c.seed_buffer(Pq.nrays);
    cuda_ok(prop->net.predict(Pq.rays, stride, Pq.nrays, seeds, nullptr, st, nullptr, c.dscratch + 1),
            "proposer inference");
    Pq.seeds = seeds;
    Pq.max_iters = 8 * bvh.num_nodes + 64;  // proposed subtrees are searched again by the full search
    launches++;
  };
  if (prop && ((uintptr_t)rays % 16) != 0 && (on_device || direct)) {
    prop = nullptr;
    prop_lock = std::unique_lock<std::mutex>();
  }
  if (on_device || direct) {
    P.rays = (char*)rays;
    P.nrays = M;
    cuda_ok(cudaEventRecord(c.e1, st), "event");
    reorder(P);
    propose(P);
    cuda_ok(gb::launch_trace(P, anyhit, c.counting, st), "traversal launch");
    launches++;
    cuda_ok(cudaEventRecord(c.e2, st), "event");
    if (direct) {
      c.last.h2d_bytes = (unsigned long long)M * 48;                     // ray records read by the kernel
      c.last.d2h_bytes = (unsigned long long)M * (anyhit ? 4 : 36);      // at most tfar (+ hit) written
    }
  } else if (dev->host_mode >= 1 && M > kChunk && !prop && !batch) {
    // chunked pipeline: H2D of chunk i+1 and D2H of chunk i-1 overlap the trace of chunk i
    c.ensure_pipeline();
    char* d_rays = c.buffer(span);
    const uint32_t nchunks = std::min<uint32_t>((M + kChunk - 1) / kChunk, ThreadCtx::kMaxChunks);
    const uint32_t per = (M + nchunks - 1) / nchunks;
    cuda_ok(cudaEventRecord(c.e3, st), "event");
    cuda_ok(cudaStreamWaitEvent(c.s_in, c.e3, 0), "wait");
    for (uint32_t i = 0; i < nchunks; i++) {
      const uint32_t first = i * per, n = std::min(per, M - first);
      const size_t off = (size_t)first * stride, bytes = (size_t)(n - 1) * stride + recsize;
      cuda_ok(cudaMemcpyAsync(d_rays + off, (char*)rays + off, bytes, cudaMemcpyHostToDevice, c.s_in), "H2D rays");
      cuda_ok(cudaEventRecord(c.ev_in[i], c.s_in), "event");
    }
    cuda_ok(cudaEventRecord(c.e1, st), "event");
    for (uint32_t i = 0; i < nchunks; i++) {
      const uint32_t first = i * per, n = std::min(per, M - first);
      const size_t off = (size_t)first * stride, bytes = (size_t)(n - 1) * stride + recsize;
      cuda_ok(cudaStreamWaitEvent(st, c.ev_in[i], 0), "wait");
      cuda_ok(cudaMemsetAsync(c.dscratch, 0, sizeof(unsigned int), st), "memset");  // fetch counter only
      gb::TraceParams Pi = P;
      Pi.rays = d_rays + off;
      Pi.nrays = n;
      cuda_ok(gb::launch_trace(Pi, anyhit, c.counting, st), "traversal launch");
      launches += 2;
      cuda_ok(cudaEventRecord(c.ev_tr[i], st), "event");
      cuda_ok(cudaStreamWaitEvent(c.s_out, c.ev_tr[i], 0), "wait");
      cuda_ok(cudaMemcpyAsync((char*)rays + off, d_rays + off, bytes, cudaMemcpyDeviceToHost, c.s_out), "D2H rays");
    }
    cuda_ok(cudaEventRecord(c.e2, st), "event");
    cuda_ok(cudaEventRecord(c.e3, c.s_out), "event");
    cuda_ok(cudaStreamWaitEvent(st, c.e3, 0), "wait");
    c.last.h2d_bytes = span;
    c.last.d2h_bytes = span;
  } else {
    char* d_rays = c.buffer(span);
    cuda_ok(cudaMemcpyAsync(d_rays, rays, span, cudaMemcpyHostToDevice, st), "H2D rays");
    P.rays = d_rays;
    P.nrays = M;
    cuda_ok(cudaEventRecord(c.e1, st), "event");
    reorder(P);
    propose(P);
    cuda_ok(gb::launch_trace(P, anyhit, c.counting, st), "traversal launch");
    launches++;
    cuda_ok(cudaEventRecord(c.e2, st), "event");
    cuda_ok(cudaMemcpyAsync(rays, d_rays, span, cudaMemcpyDeviceToHost, st), "D2H rays");
    c.last.h2d_bytes = span;
    c.last.d2h_bytes = span;
  }
  gb::note_launches(launches);
  cuda_ok(cudaMemcpyAsync(c.hscratch, c.dscratch, 64, cudaMemcpyDeviceToHost, st), "D2H status");
  cuda_ok(cudaEventRecord(c.e3, st), "event");
  cuda_ok(cudaStreamSynchronize(st), "traversal");
  float k_ms = 0, t_ms = 0;
  cudaEventElapsedTime(&k_ms, c.e1, c.e2);
  cudaEventElapsedTime(&t_ms, c.e0, c.e3);
  c.last.kernel_ms = k_ms;
  c.last.total_ms = t_ms;
  const gb::TraceCounters* tc = reinterpret_cast<const gb::TraceCounters*>(c.hscratch + 2);
  if (c.counting) {
    c.last.nodes = tc->nodes;
    c.last.tris = tc->tris;
    c.last.rays = tc->rays;
  }
  if (prop) c.last.proposal_hits = tc->proposal_hits;
  const unsigned err = c.hscratch[1];
  if (err & gb::kErrStackOverflow) fail(RTC_ERROR_UNKNOWN, "traversal stack overflow");
  if (err & gb::kErrIterationLimit) fail(RTC_ERROR_UNKNOWN, "traversal iteration limit reached");
  if (err & gb::kErrBuild) fail(RTC_ERROR_UNKNOWN, "traversal found an invalid BVH reference");
}

// array-of-pointers variants gather into a packed host array first
template <typename Rec>
void run_query_pointers(Scene* scene, Rec** recs, unsigned M, bool anyhit, const RTCIntersectContext* uctx) {
  VERIFY_HANDLE(scene);
  if (M == 0) return;
  if (!recs) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  std::vector<Rec> tmp(M);
  for (unsigned i = 0; i < M; i++) tmp[i] = *recs[i];
  run_query(scene, tmp.data(), M, sizeof(Rec), anyhit, sizeof(Rec), nullptr, nullptr, uctx);
  for (unsigned i = 0; i < M; i++) *recs[i] = tmp[i];
}

// SOA layouts (packets RTCRayHit4/8/16, RTCRayHitN streams, RTCRayHitNp pointer streams).
// Field numbering follows the SOA order of include/embree3/rtcore_ray.h:222-248: ray fields
// 0..11, hit fields 12..19 (Ng_x, Ng_y, Ng_z, u, v, primID, geomID, instID[0]).
enum SoaField {
  kOrgX, kOrgY, kOrgZ, kTnear, kDirX, kDirY, kDirZ, kTime, kTfar, kMask, kId, kFlags,
  kNgX, kNgY, kNgZ, kU, kV, kPrimID, kGeomID, kInstID, kNumSoaFields
};

// The lanes are gathered into packed AOS records, traced by the stream path and scattered
// back.  Lane selection is the reference's: valid[i] == -1 for packets
// (kernels/bvh/bvh_intersector_hybrid.cpp:131, 623) and tnear <= tfar for every layout
// (kernels/common/ray.h:622-627, 922-927); a missing tnear reads as 0, a missing
// time as 0, missing mask/id/flags as all ones (ray.h:938-980).  A closest-hit lane is
// written only when it hit something, an occlusion lane only when it is occluded
// (ray.h:903-911, 988-1010), and null Ng/instID pointers are skipped.
template <typename Addr>
void run_query_soa(Scene* scene, size_t count, const int* valid, bool anyhit, const RTCIntersectContext* uctx,
                   Addr addr) {
  VERIFY_HANDLE(scene);
  if (count == 0) return;
  if (count > 0xffffffffull) fail(RTC_ERROR_INVALID_ARGUMENT, "too many rays");
  auto f32 = [&](int f, size_t i, float dflt) {
    const float* p = (const float*)addr(f, i);
    return p ? *p : dflt;
  };
  auto u32 = [&](int f, size_t i, unsigned dflt) {
    const unsigned* p = (const unsigned*)addr(f, i);
    return p ? *p : dflt;
  };
  std::vector<uint32_t> lane;
  lane.reserve(count);
  for (size_t i = 0; i < count; i++) {
    if (valid && valid[i] != -1) continue;
    if (!(f32(kTnear, i, 0.0f) <= f32(kTfar, i, 0.0f))) continue;
    lane.push_back((uint32_t)i);
  }
  if (lane.empty()) return;
  const unsigned M = (unsigned)lane.size();
  auto load_ray = [&](RTCRay& r, size_t i) {
    r.org_x = f32(kOrgX, i, 0.0f); r.org_y = f32(kOrgY, i, 0.0f); r.org_z = f32(kOrgZ, i, 0.0f);
    r.tnear = f32(kTnear, i, 0.0f);
    r.dir_x = f32(kDirX, i, 0.0f); r.dir_y = f32(kDirY, i, 0.0f); r.dir_z = f32(kDirZ, i, 0.0f);
    r.time = f32(kTime, i, 0.0f);
    r.tfar = f32(kTfar, i, 0.0f);
    r.mask = u32(kMask, i, 0xffffffffu); r.id = u32(kId, i, 0xffffffffu); r.flags = u32(kFlags, i, 0xffffffffu);
  };
  if (anyhit) {
    std::vector<RTCRay> tmp(M);
    for (unsigned j = 0; j < M; j++) load_ray(tmp[j], lane[j]);
    run_query(scene, tmp.data(), M, sizeof(RTCRay), true, sizeof(RTCRay), nullptr, nullptr, uctx);
    for (unsigned j = 0; j < M; j++)
      if (tmp[j].tfar < 0.0f) *(float*)addr(kTfar, lane[j]) = tmp[j].tfar;
    return;
  }
  std::vector<RTCRayHit> tmp(M);
  for (unsigned j = 0; j < M; j++) {
    load_ray(tmp[j].ray, lane[j]);
    tmp[j].hit.geomID = RTC_INVALID_GEOMETRY_ID;
    tmp[j].hit.primID = RTC_INVALID_GEOMETRY_ID;
    tmp[j].hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
  }
  run_query(scene, tmp.data(), M, sizeof(RTCRayHit), false, sizeof(RTCRayHit), nullptr, nullptr, uctx);
  for (unsigned j = 0; j < M; j++) {
    const RTCRayHit& h = tmp[j];
    if (h.hit.geomID == RTC_INVALID_GEOMETRY_ID) continue;
    const size_t i = lane[j];
    const float fv[6] = {h.ray.tfar, h.hit.Ng_x, h.hit.Ng_y, h.hit.Ng_z, h.hit.u, h.hit.v};
    const int ff[6] = {kTfar, kNgX, kNgY, kNgZ, kU, kV};
    for (int k = 0; k < 6; k++)
      if (float* p = (float*)addr(ff[k], i)) *p = fv[k];
    const unsigned uv[3] = {h.hit.primID, h.hit.geomID, h.hit.instID[0]};
    const int uf[3] = {kPrimID, kGeomID, kInstID};
    for (int k = 0; k < 3; k++)
      if (unsigned* p = (unsigned*)addr(uf[k], i)) *p = uv[k];
  }
}

// packets of K lanes / NM streams: field f of lane i of packet p sits at
// base + p * stride + (f * K + i) * 4 (rtcore_ray.h:222-248)
void run_query_packets(Scene* scene, void* base, unsigned K, size_t packets, size_t stride, const int* valid,
                       bool anyhit, const RTCIntersectContext* uctx) {
  if (!base) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (is_device_pointer(base)) fail(RTC_ERROR_INVALID_ARGUMENT, "ray packets must be in host memory");
  if (packets > 1 && stride < (size_t)(anyhit ? 12 : 20) * K * 4)
    fail(RTC_ERROR_INVALID_ARGUMENT, "byteStride smaller than one ray packet");
  char* b = (char*)base;
  run_query_soa(scene, (size_t)K * packets, valid, anyhit, uctx, [=](int f, size_t r) -> void* {
    const size_t p = r / K, i = r % K;
    return b + p * stride + ((size_t)f * K + i) * 4;
  });
}

// pointer-SOA streams (rtcore_ray.h:170-213); optional fields may be null
void run_query_pointer_soa(Scene* scene, const RTCRayHitNp* rh, const RTCRayNp* ray, unsigned N, bool anyhit,
                           const RTCIntersectContext* uctx) {
  if (!rh && !ray) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (N == 0) return;
  const RTCRayNp& r = rh ? rh->ray : *ray;
  void* fld[kNumSoaFields] = {r.org_x, r.org_y, r.org_z, r.tnear, r.dir_x, r.dir_y, r.dir_z, r.time,
                              r.tfar,  r.mask,  r.id,    r.flags};
  if (rh) {
    const RTCHitNp& h = rh->hit;
    void* hf[8] = {h.Ng_x, h.Ng_y, h.Ng_z, h.u, h.v, h.primID, h.geomID, h.instID[0]};
    for (int k = 0; k < 8; k++) fld[kNgX + k] = hf[k];
    if (!h.u || !h.v || !h.primID || !h.geomID) fail(RTC_ERROR_INVALID_ARGUMENT, "missing hit arrays");
  }
  if (!r.org_x || !r.org_y || !r.org_z || !r.dir_x || !r.dir_y || !r.dir_z || !r.tfar)
    fail(RTC_ERROR_INVALID_ARGUMENT, "missing ray arrays");
  for (int k = 0; k < kNumSoaFields; k++)
    if (fld[k] && is_device_pointer(fld[k])) fail(RTC_ERROR_INVALID_ARGUMENT, "ray arrays must be in host memory");
  run_query_soa(scene, N, nullptr, anyhit, uctx, [&](int f, size_t i) -> void* {
    return fld[f] ? (char*)fld[f] + i * 4 : nullptr;
  });
}

}  // namespace

namespace gb {
std::atomic<unsigned long long> g_launch_count{0};
void note_launches(unsigned n) { g_launch_count.fetch_add(n, std::memory_order_relaxed); }
}  // namespace gb

// ===========================================================================
// exported C ABI
// ===========================================================================

extern "C" {

RTC_API RTCDevice rtcNewDevice(const char* config) {
  API_BEGIN
  std::lock_guard<std::mutex> lk(g_mutex);
  Device* d = new Device(config);
  return (RTCDevice)d;
  API_END(nullptr)
  return nullptr;
}

RTC_API void rtcRetainDevice(RTCDevice hdevice) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  d->inc();
  API_END(nullptr)
}

RTC_API void rtcReleaseDevice(RTCDevice hdevice) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  d->dec();
  API_END(nullptr)
}

RTC_API ssize_t rtcGetDeviceProperty(RTCDevice hdevice, enum RTCDeviceProperty prop) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  switch (prop) {
    case RTC_DEVICE_PROPERTY_VERSION: return RTC_VERSION;
    case RTC_DEVICE_PROPERTY_VERSION_MAJOR: return RTC_VERSION_MAJOR;
    case RTC_DEVICE_PROPERTY_VERSION_MINOR: return RTC_VERSION_MINOR;
    case RTC_DEVICE_PROPERTY_VERSION_PATCH: return RTC_VERSION_PATCH;
    case RTC_DEVICE_PROPERTY_NATIVE_RAY4_SUPPORTED:
    case RTC_DEVICE_PROPERTY_NATIVE_RAY8_SUPPORTED:
    case RTC_DEVICE_PROPERTY_NATIVE_RAY16_SUPPORTED: return 0;
    case RTC_DEVICE_PROPERTY_RAY_STREAM_SUPPORTED: return 1;
    case RTC_DEVICE_PROPERTY_BACKFACE_CULLING_CURVES_ENABLED:
    case RTC_DEVICE_PROPERTY_RAY_MASK_SUPPORTED:
    case RTC_DEVICE_PROPERTY_BACKFACE_CULLING_ENABLED:
    case RTC_DEVICE_PROPERTY_IGNORE_INVALID_RAYS_ENABLED:
    case RTC_DEVICE_PROPERTY_COMPACT_POLYS_ENABLED: return 0;
    case RTC_DEVICE_PROPERTY_TRIANGLE_GEOMETRY_SUPPORTED: return 1;
    case RTC_DEVICE_PROPERTY_FILTER_FUNCTION_SUPPORTED: return 1;
    case RTC_DEVICE_PROPERTY_QUAD_GEOMETRY_SUPPORTED:
    case RTC_DEVICE_PROPERTY_SUBDIVISION_GEOMETRY_SUPPORTED:
    case RTC_DEVICE_PROPERTY_CURVE_GEOMETRY_SUPPORTED:
    case RTC_DEVICE_PROPERTY_USER_GEOMETRY_SUPPORTED:
    case RTC_DEVICE_PROPERTY_POINT_GEOMETRY_SUPPORTED: return 0;
    case RTC_DEVICE_PROPERTY_TASKING_SYSTEM: return 0;
    case RTC_DEVICE_PROPERTY_JOIN_COMMIT_SUPPORTED: return 1;
    case RTC_DEVICE_PROPERTY_PARALLEL_COMMIT_SUPPORTED: return 1;
    default: fail(RTC_ERROR_INVALID_ARGUMENT, "unknown readable property");
  }
  API_END(d)
  return 0;
}

RTC_API void rtcSetDeviceProperty(RTCDevice hdevice, const enum RTCDeviceProperty prop, ssize_t value) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  (void)prop;
  (void)value;
  fail(RTC_ERROR_INVALID_ARGUMENT, "unknown writable property");
  API_END(d)
}

RTC_API enum RTCError rtcGetDeviceError(RTCDevice hdevice) {
  Device* d = (Device*)hdevice;
  if (!d) {
    RTCError e = t_thread_error;
    t_thread_error = RTC_ERROR_NONE;
    return e;
  }
  auto it = t_device_error.find(d);
  if (it == t_device_error.end()) return RTC_ERROR_NONE;
  RTCError e = it->second;
  it->second = RTC_ERROR_NONE;
  return e;
}

RTC_API void rtcSetDeviceErrorFunction(RTCDevice hdevice, RTCErrorFunction error, void* userPtr) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  d->error_fn = error;
  d->error_user = userPtr;
  API_END(d)
}

RTC_API void rtcSetDeviceMemoryMonitorFunction(RTCDevice hdevice, RTCMemoryMonitorFunction fn, void* userPtr) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  d->mem_fn = fn;
  d->mem_user = userPtr;
  API_END(d)
}

// ---- buffers

RTC_API RTCBuffer rtcNewBuffer(RTCDevice hdevice, size_t byteSize) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  return (RTCBuffer) new Buffer(d, byteSize, nullptr);
  API_END(d)
  return nullptr;
}

RTC_API RTCBuffer rtcNewSharedBuffer(RTCDevice hdevice, void* ptr, size_t byteSize) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  return (RTCBuffer) new Buffer(d, byteSize, ptr);
  API_END(d)
  return nullptr;
}

RTC_API void* rtcGetBufferData(RTCBuffer hbuffer) {
  Buffer* b = (Buffer*)hbuffer;
  API_BEGIN
  VERIFY_HANDLE(hbuffer);
  return b->ptr;
  API_END(b ? b->device : nullptr)
  return nullptr;
}

RTC_API void rtcRetainBuffer(RTCBuffer hbuffer) {
  Buffer* b = (Buffer*)hbuffer;
  API_BEGIN
  VERIFY_HANDLE(hbuffer);
  b->inc();
  API_END(b ? b->device : nullptr)
}

RTC_API void rtcReleaseBuffer(RTCBuffer hbuffer) {
  Buffer* b = (Buffer*)hbuffer;
  API_BEGIN
  VERIFY_HANDLE(hbuffer);
  b->dec();
  API_END(nullptr)
}

// ---- geometry

RTC_API RTCGeometry rtcNewGeometry(RTCDevice hdevice, enum RTCGeometryType type) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  if (type != RTC_GEOMETRY_TYPE_TRIANGLE && type != RTC_GEOMETRY_TYPE_INSTANCE)
    fail(RTC_ERROR_UNKNOWN, "geometry type is not supported");
  return (RTCGeometry) new Geometry(d, type);
  API_END(d)
  return nullptr;
}

RTC_API void rtcRetainGeometry(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->inc();
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcReleaseGeometry(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->dec();
  API_END(nullptr)
}

RTC_API void rtcCommitGeometry(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcEnableGeometry(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->enabled = true;
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcDisableGeometry(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->enabled = false;
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryTimeStepCount(RTCGeometry hg, unsigned int timeStepCount) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (timeStepCount != 1) fail(RTC_ERROR_INVALID_OPERATION, "motion blur is not supported");
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryMask(RTCGeometry hg, unsigned int mask) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->mask = mask;
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryBuildQuality(RTCGeometry hg, enum RTCBuildQuality quality) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (quality != RTC_BUILD_QUALITY_LOW && quality != RTC_BUILD_QUALITY_MEDIUM && quality != RTC_BUILD_QUALITY_HIGH &&
      quality != RTC_BUILD_QUALITY_REFIT)
    fail(RTC_ERROR_INVALID_ARGUMENT, "invalid build quality");
  g->quality = quality;
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryBuffer(RTCGeometry hg, enum RTCBufferType type, unsigned int slot, enum RTCFormat format,
                                  RTCBuffer hbuffer, size_t byteOffset, size_t byteStride, size_t itemCount) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  VERIFY_HANDLE(hbuffer);
  Buffer* b = (Buffer*)hbuffer;
  if (g->device != b->device) fail(RTC_ERROR_INVALID_ARGUMENT, "inputs are from different devices");
  if (itemCount > 0xFFFFFFFFu) fail(RTC_ERROR_INVALID_ARGUMENT, "buffer too large");
  g->set_buffer(type, slot, format, b, byteOffset, byteStride, itemCount);
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetSharedGeometryBuffer(RTCGeometry hg, enum RTCBufferType type, unsigned int slot,
                                        enum RTCFormat format, const void* ptr, size_t byteOffset, size_t byteStride,
                                        size_t itemCount) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (itemCount > 0xFFFFFFFFu) fail(RTC_ERROR_INVALID_ARGUMENT, "buffer too large");
  Buffer* b = new Buffer(g->device, itemCount * byteStride, (char*)ptr + byteOffset);
  try {
    g->set_buffer(type, slot, format, b, 0, byteStride, itemCount);
  } catch (...) {
    b->dec();
    throw;
  }
  b->dec();
  API_END(g ? g->device : nullptr)
}

RTC_API void* rtcSetNewGeometryBuffer(RTCGeometry hg, enum RTCBufferType type, unsigned int slot,
                                      enum RTCFormat format, size_t byteStride, size_t itemCount) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (itemCount > 0xFFFFFFFFu) fail(RTC_ERROR_INVALID_ARGUMENT, "buffer too large");
  // vertex buffers are over-allocated to a 16-byte multiple, as in rtcore.cpp:1470-1486
  size_t bytes = itemCount * byteStride;
  if (type == RTC_BUFFER_TYPE_VERTEX || type == RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE) bytes += (16 - (byteStride % 16)) % 16;
  Buffer* b = new Buffer(g->device, bytes, nullptr);
  try {
    g->set_buffer(type, slot, format, b, 0, byteStride, itemCount);
  } catch (...) {
    b->dec();
    throw;
  }
  b->dec();
  return b->ptr;
  API_END(g ? g->device : nullptr)
  return nullptr;
}

RTC_API void* rtcGetGeometryBufferData(RTCGeometry hg, enum RTCBufferType type, unsigned int slot) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  return (void*)g->view(type, slot)->ptr;
  API_END(g ? g->device : nullptr)
  return nullptr;
}

RTC_API void rtcUpdateGeometryBuffer(RTCGeometry hg, enum RTCBufferType type, unsigned int slot) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->view(type, slot);  // validates; buffers are re-uploaded at every commit
  if (type == RTC_BUFFER_TYPE_INDEX) g->topo_version++;
  API_END(g ? g->device : nullptr)
}

// Geometry::setIntersectionFilterFunctionN / setOcclusionFilterFunctionN
// (kernels/common/geometry.cpp:136-150): triangle meshes take callbacks, instances do not
RTC_API void rtcSetGeometryIntersectFilterFunction(RTCGeometry hg, RTCFilterFunctionN filter) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (g->type != RTC_GEOMETRY_TYPE_TRIANGLE)
    fail(RTC_ERROR_INVALID_OPERATION, "filter functions not supported for this geometry");
  g->ifilter = filter;
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryOccludedFilterFunction(RTCGeometry hg, RTCFilterFunctionN filter) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  if (g->type != RTC_GEOMETRY_TYPE_TRIANGLE)
    fail(RTC_ERROR_INVALID_OPERATION, "filter functions not supported for this geometry");
  g->ofilter = filter;
  API_END(g ? g->device : nullptr)
}

// ---- instances (kernels/common/rtcore.cpp:996-1135, scene_instance.cpp)

RTC_API void rtcSetGeometryInstancedScene(RTCGeometry hg, RTCScene hs) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  VERIFY_HANDLE(hs);
  if (g->type != RTC_GEOMETRY_TYPE_INSTANCE) fail(RTC_ERROR_INVALID_OPERATION, "operation not supported for this geometry");
  Scene* s = (Scene*)hs;
  s->inc();
  if (g->inst_scene) g->inst_scene->dec();
  g->inst_scene = s;
  API_END(g ? g->device : nullptr)
}

// loadTransform / storeTransform (rtcore.cpp:1010-1069): 3x4 row-major, 3x4
// column-major and 4x4 column-major layouts
RTC_API void rtcSetGeometryTransform(RTCGeometry hg, unsigned int timeStep, enum RTCFormat format, const void* xfm) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  VERIFY_HANDLE(xfm);
  if (g->type != RTC_GEOMETRY_TYPE_INSTANCE) fail(RTC_ERROR_INVALID_OPERATION, "operation not supported for this geometry");
  if (timeStep >= g->time_steps) fail(RTC_ERROR_INVALID_OPERATION, "invalid timestep");
  const float* m = (const float*)xfm;
  float t[12];
  if (format == RTC_FORMAT_FLOAT3X4_ROW_MAJOR) {
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 3; r++) t[3 * c + r] = m[4 * r + c];
  } else if (format == RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR) {
    for (int k = 0; k < 12; k++) t[k] = m[k];
  } else if (format == RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR) {
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 3; r++) t[3 * c + r] = m[4 * c + r];
  } else {
    fail(RTC_ERROR_INVALID_OPERATION, "invalid matrix format");
  }
  std::memcpy(g->l2w, t, sizeof(t));
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcGetGeometryTransform(RTCGeometry hg, float time, enum RTCFormat format, void* xfm) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  (void)time;
  VERIFY_HANDLE(hg);
  VERIFY_HANDLE(xfm);
  if (g->type != RTC_GEOMETRY_TYPE_INSTANCE) fail(RTC_ERROR_INVALID_OPERATION, "operation not supported for this geometry");
  float* m = (float*)xfm;
  const float* t = g->l2w;
  if (format == RTC_FORMAT_FLOAT3X4_ROW_MAJOR) {
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 3; r++) m[4 * r + c] = t[3 * c + r];
  } else if (format == RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR) {
    for (int k = 0; k < 12; k++) m[k] = t[k];
  } else if (format == RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR) {
    for (int c = 0; c < 4; c++) {
      for (int r = 0; r < 3; r++) m[4 * c + r] = t[3 * c + r];
      m[4 * c + 3] = c == 3 ? 1.0f : 0.0f;
    }
  } else {
    fail(RTC_ERROR_INVALID_OPERATION, "invalid matrix format");
  }
  API_END(g ? g->device : nullptr)
}

RTC_API void rtcSetGeometryUserData(RTCGeometry hg, void* ptr) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  g->user = ptr;
  API_END(g ? g->device : nullptr)
}

RTC_API void* rtcGetGeometryUserData(RTCGeometry hg) {
  Geometry* g = (Geometry*)hg;
  API_BEGIN
  VERIFY_HANDLE(hg);
  return g->user;
  API_END(g ? g->device : nullptr)
  return nullptr;
}

// ---- scene

RTC_API RTCScene rtcNewScene(RTCDevice hdevice) {
  Device* d = (Device*)hdevice;
  API_BEGIN
  VERIFY_HANDLE(hdevice);
  return (RTCScene) new Scene(d);
  API_END(d)
  return nullptr;
}

RTC_API RTCDevice rtcGetSceneDevice(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->device->inc();
  return (RTCDevice)s->device;
  API_END(s ? s->device : nullptr)
  return nullptr;
}

RTC_API void rtcRetainScene(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->inc();
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcReleaseScene(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->dec();
  API_END(nullptr)
}

RTC_API unsigned int rtcAttachGeometry(RTCScene hs, RTCGeometry hg) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  VERIFY_HANDLE(hg);
  Geometry* g = (Geometry*)hg;
  if (s->device != g->device) fail(RTC_ERROR_INVALID_ARGUMENT, "inputs are from different devices");
  return s->attach(g, RTC_INVALID_GEOMETRY_ID);
  API_END(s ? s->device : nullptr)
  return RTC_INVALID_GEOMETRY_ID;
}

RTC_API void rtcAttachGeometryByID(RTCScene hs, RTCGeometry hg, unsigned int geomID) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  VERIFY_HANDLE(hg);
  if (geomID == RTC_INVALID_GEOMETRY_ID) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  Geometry* g = (Geometry*)hg;
  if (s->device != g->device) fail(RTC_ERROR_INVALID_ARGUMENT, "inputs are from different devices");
  s->attach(g, geomID);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcDetachGeometry(RTCScene hs, unsigned int geomID) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (geomID == RTC_INVALID_GEOMETRY_ID) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  s->detach(geomID);
  API_END(s ? s->device : nullptr)
}

RTC_API RTCGeometry rtcGetGeometry(RTCScene hs, unsigned int geomID) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  std::lock_guard<std::mutex> lk(s->mtx);
  if (geomID >= s->geoms.size()) return nullptr;
  return (RTCGeometry)s->geoms[geomID];
  API_END(s ? s->device : nullptr)
  return nullptr;
}

RTC_API void rtcCommitScene(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->commit();
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcJoinCommitScene(RTCScene hs) { rtcCommitScene(hs); }

RTC_API void rtcSetSceneProgressMonitorFunction(RTCScene hs, RTCProgressMonitorFunction progress, void* ptr) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->progress = progress;
  s->progress_ptr = ptr;
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcSetSceneBuildQuality(RTCScene hs, enum RTCBuildQuality quality) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (quality != RTC_BUILD_QUALITY_LOW && quality != RTC_BUILD_QUALITY_MEDIUM && quality != RTC_BUILD_QUALITY_HIGH)
    fail(RTC_ERROR_UNKNOWN, "invalid build quality");
  s->quality = quality;
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcSetSceneFlags(RTCScene hs, enum RTCSceneFlags flags) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  s->flags = flags;
  API_END(s ? s->device : nullptr)
}

RTC_API enum RTCSceneFlags rtcGetSceneFlags(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  return s->flags;
  API_END(s ? s->device : nullptr)
  return RTC_SCENE_FLAG_NONE;
}

RTC_API void rtcGetSceneBounds(RTCScene hs, struct RTCBounds* b) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  b->lower_x = s->bvh.lo[0];
  b->lower_y = s->bvh.lo[1];
  b->lower_z = s->bvh.lo[2];
  b->align0 = 0;
  b->upper_x = s->bvh.hi[0];
  b->upper_y = s->bvh.hi[1];
  b->upper_z = s->bvh.hi[2];
  b->align1 = 0;
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcGetSceneLinearBounds(RTCScene hs, struct RTCLinearBounds* b) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!b) fail(RTC_ERROR_INVALID_OPERATION, "invalid destination pointer");
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  RTCBounds one{};
  one.lower_x = s->bvh.lo[0]; one.lower_y = s->bvh.lo[1]; one.lower_z = s->bvh.lo[2];
  one.upper_x = s->bvh.hi[0]; one.upper_y = s->bvh.hi[1]; one.upper_z = s->bvh.hi[2];
  b->bounds0 = one;
  b->bounds1 = one;
  API_END(s ? s->device : nullptr)
}

// ---- queries

RTC_API void rtcIntersect1(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRayHit* rayhit) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!rayhit) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  // rtcore.cpp:609-612: a single ray is traced only when tnear <= tfar
  if (!(rayhit->ray.tnear <= rayhit->ray.tfar)) return;
  run_query(s, rayhit, 1, sizeof(RTCRayHit), false, sizeof(RTCRayHit), nullptr, nullptr, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcIntersect1M(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRayHit* rayhit, unsigned int M,
                            size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  run_query(s, rayhit, M, byteStride, false, sizeof(RTCRayHit), nullptr, nullptr, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcIntersect1Mp(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRayHit** rayhit, unsigned int M) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  run_query_pointers<RTCRayHit>(s, rayhit, M, false, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcOccluded1(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRay* ray) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!ray) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (!(ray->tnear <= ray->tfar)) return;
  run_query(s, ray, 1, sizeof(RTCRay), true, sizeof(RTCRay), nullptr, nullptr, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcOccluded1M(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRay* ray, unsigned int M,
                           size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  run_query(s, ray, M, byteStride, true, sizeof(RTCRay), nullptr, nullptr, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcOccluded1Mp(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRay** ray, unsigned int M) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  run_query_pointers<RTCRay>(s, ray, M, true, ctx);
  API_END(s ? s->device : nullptr)
}

#define GB_PACKET_QUERY(NAME, REC, K, ANYHIT)                                                     \
  RTC_API void NAME(const int* valid, RTCScene hs, struct RTCIntersectContext* ctx, struct REC* r) { \
    Scene* s = (Scene*)hs;                                                                         \
    API_BEGIN                                                                                      \
    VERIFY_HANDLE(hs);                                                                             \
    if (!valid) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid valid mask");                            \
    run_query_packets(s, r, K, 1, sizeof(struct REC), valid, ANYHIT, ctx);                         \
    API_END(s ? s->device : nullptr)                                                               \
  }
GB_PACKET_QUERY(rtcIntersect4, RTCRayHit4, 4, false)
GB_PACKET_QUERY(rtcIntersect8, RTCRayHit8, 8, false)
GB_PACKET_QUERY(rtcIntersect16, RTCRayHit16, 16, false)
GB_PACKET_QUERY(rtcOccluded4, RTCRay4, 4, true)
GB_PACKET_QUERY(rtcOccluded8, RTCRay8, 8, true)
GB_PACKET_QUERY(rtcOccluded16, RTCRay16, 16, true)
#undef GB_PACKET_QUERY

RTC_API void rtcIntersectNM(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRayHitN* rayhit, unsigned int N,
                            unsigned int M, size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  // rtcore.cpp:672-686: N == 1 is an AOS stream of RTCRayHit records
  if (N == 1) {
    if (M == 1 && rayhit && !(((RTCRayHit*)rayhit)->ray.tnear <= ((RTCRayHit*)rayhit)->ray.tfar)) return;
    run_query(s, rayhit, M, byteStride, false, sizeof(RTCRayHit), nullptr, nullptr, ctx);
  } else if (N != 0 && M != 0) {
    run_query_packets(s, rayhit, N, M, byteStride, nullptr, false, ctx);
  }
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcIntersectNp(RTCScene hs, struct RTCIntersectContext* ctx, const struct RTCRayHitNp* rayhit,
                            unsigned int N) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!rayhit) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  run_query_pointer_soa(s, rayhit, nullptr, N, false, ctx);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcOccludedNM(RTCScene hs, struct RTCIntersectContext* ctx, struct RTCRayN* ray, unsigned int N,
                           unsigned int M, size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (N == 1) {
    if (M == 1 && ray && !(((RTCRay*)ray)->tnear <= ((RTCRay*)ray)->tfar)) return;
    run_query(s, ray, M, byteStride, true, sizeof(RTCRay), nullptr, nullptr, ctx);
  } else if (N != 0 && M != 0) {
    run_query_packets(s, ray, N, M, byteStride, nullptr, true, ctx);
  }
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcOccludedNp(RTCScene hs, struct RTCIntersectContext* ctx, const struct RTCRayNp* ray, unsigned int N) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!ray) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  run_query_pointer_soa(s, nullptr, ray, N, true, ctx);
  API_END(s ? s->device : nullptr)
}

// ---- extensions

RTC_API void rtcgbGetSceneBuildStats(RTCScene hs, RTCGBBuildStats* out) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!out) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  memset(out, 0, sizeof(*out));
  out->sah = s->stats.sah;
  out->sah_exact = s->stats.sah_exact;
  out->leaf_max = s->stats.leaf_max;
  out->build_ms = s->stats.build_ms;
  out->num_nodes = s->stats.num_nodes;
  out->num_leaves = s->stats.num_leaves;
  out->num_prims = s->stats.num_prims;
  out->depth = s->stats.depth;
  out->ploc_iterations = s->stats.ploc_iterations;
  out->refit = s->stats.refit;
  out->bvh_bytes = (unsigned long long)s->bvh.num_nodes * sizeof(gb::WideNode) +
                   (unsigned long long)s->bvh.num_tris * sizeof(gb::TriRecord);
  API_END(s ? s->device : nullptr)
}

RTC_API unsigned int rtcgbGetSceneBuildPhases(RTCScene hs, double* us, unsigned int max_phases) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  const unsigned n = s->stats.nphases;
  for (unsigned k = 0; us && k < n && k < max_phases; k++) us[k] = s->stats.phase_us[k];
  return n;
  API_END(s ? s->device : nullptr)
  return 0;
}

RTC_API void rtcgbGetLastQueryStats(RTCGBQueryStats* out) {
  if (out) *out = t_ctx.last;
}

RTC_API void rtcgbSetQueryCounting(int enable) { t_ctx.counting = enable != 0; }

RTC_API unsigned long long rtcgbGetKernelLaunchCount(void) { return gb::g_launch_count.load(); }

RTC_API void rtcgbSetThreadStream(void* cuda_stream) {
  t_ctx.user = (cudaStream_t)cuda_stream;
  t_ctx.user_set = cuda_stream != nullptr;
}

RTC_API unsigned int rtcgbGetSceneBVH(RTCScene hs, void* nodes, unsigned int max_nodes, void* tris,
                                      unsigned int max_tris, unsigned int* num_tris) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  s->device->set_current();
  const unsigned nn = std::min(max_nodes, s->bvh.num_nodes), nt = std::min(max_tris, s->bvh.num_tris);
  if (nodes && nn) cuda_ok(cudaMemcpy(nodes, s->bvh.nodes, (size_t)nn * sizeof(gb::WideNode), cudaMemcpyDeviceToHost), "copy nodes");
  if (tris && nt) cuda_ok(cudaMemcpy(tris, s->bvh.tris, (size_t)nt * sizeof(gb::TriRecord), cudaMemcpyDeviceToHost), "copy tris");
  if (num_tris) *num_tris = s->bvh.num_tris;
  return s->bvh.num_nodes;
  API_END(s ? s->device : nullptr)
  return 0;
}

RTC_API void rtcgbIntersect1MNoAlloc(RTCScene hs, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride,
                                     void* cuda_stream) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  if (M == 0) return;
  if (!rayhit) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  if (((size_t)rayhit & 0x3) || (byteStride & 0x3)) fail(RTC_ERROR_INVALID_ARGUMENT, "ray not aligned to 4 bytes");
  if (byteStride < sizeof(RTCRayHit)) fail(RTC_ERROR_INVALID_ARGUMENT, "byteStride smaller than the ray record");
  // the no-allocation query runs the plain traversal only: scenes whose queries need
  // more (filter callbacks on the host, instance leaves, per-geometry batch roots) are
  // refused rather than traced as if they were plain triangle scenes
  if (s->filters) fail(RTC_ERROR_INVALID_OPERATION, "rtcgbIntersect1MNoAlloc: scene has filter callbacks");
  if (s->ninsts || !s->inst_refs.empty())
    fail(RTC_ERROR_INVALID_OPERATION, "rtcgbIntersect1MNoAlloc: scene has instances");
  if (s->batched) fail(RTC_ERROR_INVALID_OPERATION, "rtcgbIntersect1MNoAlloc: batched scene");
  if (s->bvh.num_nodes == 0) return;
  s->device->set_current();
  const bool on_device = is_device_pointer(rayhit);
  const size_t span = (size_t)(M - 1) * byteStride + sizeof(RTCRayHit);
  if (!on_device && span > gb::kNoAllocStagingBytes)
    fail(RTC_ERROR_INVALID_ARGUMENT,
         "rtcgbIntersect1MNoAlloc: host rays span more than its 32 MiB staging area; pass device memory or "
         "split the stream");
  uint32_t flags = 0;
  cuda_ok(gb::noalloc_closest(s->bvh, (char*)rayhit, on_device, M, byteStride, (cudaStream_t)cuda_stream, &flags),
          "rtcgbIntersect1MNoAlloc");
  gb::note_launches(2);  // memset + traversal
  if (flags & gb::kErrStackOverflow) fail(RTC_ERROR_UNKNOWN, "traversal stack overflow");
  if (flags & gb::kErrIterationLimit) fail(RTC_ERROR_UNKNOWN, "traversal iteration limit reached");
  if (flags & gb::kErrBuild) fail(RTC_ERROR_UNKNOWN, "traversal found an invalid BVH reference");
  API_END(s ? s->device : nullptr)
}

// ---- traversal launch shapes and their tuner

RTC_API unsigned int rtcgbGetTraversalShapes(RTCGBTraversalShape* shapes, unsigned int max_shapes) {
  for (unsigned i = 0; shapes && i < max_shapes && i < (unsigned)gb::kNumTraceShapes; i++) {
    shapes[i].threads = (unsigned)gb::kTraceShapes[i].threads;
    shapes[i].ctas_per_sm = (unsigned)gb::kTraceShapes[i].ctas;
    shapes[i].shared_stack = (unsigned)gb::kTraceShapes[i].shared_stack;
    shapes[i].refill = (unsigned)gb::kTraceShapes[i].refill;
  }
  return (unsigned)gb::kNumTraceShapes;
}

RTC_API void rtcgbSetSceneTraversalShape(RTCScene hs, unsigned int shape) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (shape >= (unsigned)gb::kNumTraceShapes) fail(RTC_ERROR_INVALID_ARGUMENT, "no such traversal launch shape");
  s->trace_shape = (int)shape;
  API_END(s ? s->device : nullptr)
}

RTC_API unsigned int rtcgbGetSceneTraversalShape(RTCScene hs) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  return (unsigned)s->trace_shape.load();
  API_END(s ? s->device : nullptr)
  return 0;
}

RTC_API unsigned int rtcgbTuneSceneTraversal(RTCScene hs, const struct RTCRayHit* rayhit, unsigned int M,
                                             size_t byteStride, const unsigned int* batch_start,
                                             unsigned int num_batches, unsigned int flags, unsigned int repeats,
                                             double* ms_per_shape) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  if (!rayhit || M == 0) fail(RTC_ERROR_INVALID_ARGUMENT, "rtcgbTuneSceneTraversal: no rays");
  if (byteStride < sizeof(RTCRayHit) || (byteStride % 16) != 0)
    fail(RTC_ERROR_INVALID_ARGUMENT, "rtcgbTuneSceneTraversal: byteStride must be a multiple of 16, >= 80");
  if (s->filters || s->ninsts || !s->inst_refs.empty())
    fail(RTC_ERROR_INVALID_OPERATION,
         "rtcgbTuneSceneTraversal: queries of scenes with filter callbacks or instances use the default shape");
  if (s->batched != (batch_start != nullptr))
    fail(RTC_ERROR_INVALID_ARGUMENT, s->batched ? "batched scene: pass its batch boundaries" : "not a batched scene");
  if (repeats == 0) repeats = 5;
  repeats = std::min(repeats, 64u);
  Device* dev = s->device;
  dev->set_current();
  ThreadCtx& c = t_ctx;
  c.ensure(dev->cuda_device);
  cudaStream_t st = c.stream();
  // the rays in device memory twice: a pristine copy and the records each timed query overwrites
  const size_t span = (size_t)(M - 1) * byteStride + sizeof(RTCRayHit);
  char* mem = nullptr;
  cuda_ok(cudaMalloc((void**)&mem, 2 * ((span + 255) & ~size_t(255))), "cudaMalloc tuning rays");
  std::unique_ptr<char, void (*)(char*)> hold(mem, [](char* p) { cudaFree(p); });
  char* pristine = mem;
  char* work = mem + ((span + 255) & ~size_t(255));
  cuda_ok(cudaMemcpyAsync(pristine, rayhit, span, cudaMemcpyDefault, st), "copy tuning rays");
  BatchArgs b;
  b.start = batch_start;
  b.nbatches = num_batches;
  const int queries = (flags & RTCGB_TUNE_OCCLUDED) ? 2 : 1;
  const int before = s->trace_shape.load();
  std::vector<std::vector<double>> ms(gb::kNumTraceShapes);
  try {
    // round 0 loads each shape's kernels and warms the caches; shapes take turns
    // within every round so that clock changes spread over all of them
    for (unsigned r = 0; r <= repeats; r++)
      for (int sh = 0; sh < gb::kNumTraceShapes; sh++) {
        double t = 0;
        for (int q = 0; q < queries; q++) {
          cuda_ok(gb::copy_device(work, pristine, span, st), "restore tuning rays");
          s->trace_shape = sh;
          run_query(s, work, M, byteStride, q == 1, q == 1 ? sizeof(RTCRay) : sizeof(RTCRayHit), nullptr,
                    s->batched ? &b : nullptr);
          t += c.last.kernel_ms;
        }
        if (r > 0) ms[sh].push_back(t);
      }
  } catch (...) {
    s->trace_shape = before;
    throw;
  }
  // median per shape; a shape other than the default must beat it by 1 %
  std::vector<double> med(gb::kNumTraceShapes);
  for (int sh = 0; sh < gb::kNumTraceShapes; sh++) {
    std::vector<double>& v = ms[sh];
    std::sort(v.begin(), v.end());
    med[sh] = v.size() % 2 ? v[v.size() / 2] : 0.5 * (v[v.size() / 2 - 1] + v[v.size() / 2]);
    if (ms_per_shape) ms_per_shape[sh] = med[sh];
  }
  int pick = 0;
  for (int sh = 1; sh < gb::kNumTraceShapes; sh++)
    if (med[sh] < med[pick] && med[sh] <= 0.99 * med[0]) pick = sh;
  s->trace_shape = pick;
  return (unsigned)pick;
  API_END(s ? s->device : nullptr)
  return 0;
}

RTC_API int rtcgbGetDeviceHostAccess(RTCDevice hdevice) {
  Device* d = (Device*)hdevice;
  if (!d) return -1;
  return (d->pageable_access ? 1 : 0) | (d->host_ptr_registered ? 2 : 0);
}

RTC_API int rtcgbRadixSortPairs(unsigned long long* keys, unsigned int* values, unsigned int n) {
  if (n == 0) return 0;
  if (!keys || !values) return 1;
  t_ctx.ensure(0);
  cudaStream_t st = t_ctx.stream();
  uint64_t* dk = nullptr;
  uint32_t* dv = nullptr;
  if (cudaMalloc((void**)&dk, (size_t)n * 8) != cudaSuccess) return 2;
  if (cudaMalloc((void**)&dv, (size_t)n * 4) != cudaSuccess) { cudaFree(dk); return 2; }
  int rc = 0;
  if (cudaMemcpyAsync(dk, keys, (size_t)n * 8, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dv, values, (size_t)n * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      gb::sort_pairs(dk, dv, n, st) != cudaSuccess ||
      cudaMemcpyAsync(keys, dk, (size_t)n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(values, dv, (size_t)n * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    rc = 3;
  cudaFree(dk);
  cudaFree(dv);
  return rc;
}

// ---- learned proposer

namespace {
// Device view of a caller buffer: device-accessible memory is used in place,
// host memory is staged in a temporary device allocation.
struct DevSpan {
  char* d = nullptr;
  void* host = nullptr;
  size_t bytes = 0;
  bool owned = false;
  DevSpan(const void* p, size_t n, cudaStream_t st, bool copy_in) {
    const cudaMemoryType mt = pointer_type(p);
    if (mt == cudaMemoryTypeDevice || mt == cudaMemoryTypeManaged) {
      d = (char*)p;
      return;
    }
    cuda_ok(cudaMalloc((void**)&d, std::max<size_t>(n, 16)), "cudaMalloc staging");
    owned = true;
    bytes = n;
    host = const_cast<void*>(p);
    if (copy_in) cuda_ok(cudaMemcpyAsync(d, p, n, cudaMemcpyHostToDevice, st), "H2D");
  }
  void copy_out(cudaStream_t st) {
    if (owned) cuda_ok(cudaMemcpyAsync(host, d, bytes, cudaMemcpyDeviceToHost, st), "D2H");
  }
  ~DevSpan() {
    if (owned) cudaFree(d);
  }
};

cudaStream_t proposer_stream(ProposerObj* p) {
  Device* dev = p->scene->device;
  dev->set_current();
  t_ctx.ensure(dev->cuda_device);
  return t_ctx.stream();
}
}  // namespace

RTC_API RTCGBProposer rtcgbNewProposer(RTCScene hs, unsigned int seed) {
  return rtcgbNewProposerEx(hs, seed, gb::kTreelets);
}

RTC_API RTCGBProposer rtcgbNewProposerEx(RTCScene hs, unsigned int seed, unsigned int max_treelets) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  if (max_treelets < 8 || max_treelets > (unsigned)gb::kTreelets)
    fail(RTC_ERROR_INVALID_ARGUMENT, "max_treelets must be within 8..4096");
  VERIFY_HANDLE(hs);
  std::lock_guard<std::mutex> lk(s->mtx);
  if (!s->committed) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed");
  if (s->batched) fail(RTC_ERROR_INVALID_OPERATION, "the proposer does not support batched scenes");
  s->device->set_current();
  t_ctx.ensure(s->device->cuda_device);
  cudaStream_t st = t_ctx.stream();
  ProposerObj* p = new ProposerObj(s);
  try {
    std::vector<uint32_t> prim, geom;
    cuda_ok(gb::choose_treelets(s->bvh, st, &p->roots, &p->record_treelet, &prim, &geom, max_treelets),
            "treelet cut");
    // primitive numbering of the labels: geometry slots in ID order
    std::vector<uint32_t> prefix(s->geoms.size(), gb::kInvalidID);
    uint64_t total = 0;
    for (size_t id = 0; id < s->geoms.size(); id++) {
      const Geometry* g = s->geoms[id];
      if (!g || !g->indices.ptr) continue;
      prefix[id] = (uint32_t)total;
      total += g->indices.num;
    }
    std::vector<uint32_t> prim_treelet((size_t)total, gb::kInvalidID);
    for (size_t r = 0; r < prim.size(); r++) {
      if (geom[r] >= prefix.size() || prefix[geom[r]] == gb::kInvalidID) continue;
      const uint64_t k = (uint64_t)prefix[geom[r]] + prim[r];
      if (k < total) prim_treelet[k] = p->record_treelet[r];
    }
    gb::GridSpec grid{};
    for (int a = 0; a < 3; a++) {
      const float lo = s->bvh.lo[a], ext = s->bvh.hi[a] - s->bvh.lo[a];
      const bool ok = std::isfinite(lo) && std::isfinite(ext) && ext > 0.0f;
      grid.lo[a] = ok ? lo : 0.0f;
      grid.scale[a] = ok ? 1.0f / ext : 1.0f;
    }
    p->net.use_mma_sync = s->device->proposer_mma;
    cuda_ok(p->net.init(p->roots, prim_treelet, prefix, grid, seed, st), "proposer initialisation");
  } catch (...) {
    p->dec();
    throw;
  }
  return (RTCGBProposer)p;
  API_END(s ? s->device : nullptr)
  return nullptr;
}

RTC_API void rtcgbRetainProposer(RTCGBProposer hp) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  p->inc();
  API_END(nullptr)
}

RTC_API void rtcgbReleaseProposer(RTCGBProposer hp) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  p->dec();
  API_END(nullptr)
}

RTC_API void rtcgbProposerTrain(RTCGBProposer hp, const struct RTCRayHit* records, unsigned int M, size_t byteStride,
                                unsigned int epochs, unsigned int batch, float learning_rate) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (M == 0) return;
  if (!records || byteStride < sizeof(RTCRayHit) || (byteStride % 4)) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid records");
  if (!(learning_rate > 0.0f)) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid learning rate");
  cudaStream_t st = proposer_stream(p);
  std::lock_guard<std::mutex> lk(p->mtx);
  DevSpan recs(records, (size_t)(M - 1) * byteStride + sizeof(RTCRayHit), st, true);
  cuda_ok(p->net.train(recs.d, byteStride, M, epochs, batch, learning_rate, st), "proposer training");
  cuda_ok(cudaStreamSynchronize(st), "proposer training");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbProposerPredict(RTCGBProposer hp, const struct RTCRay* rays, unsigned int M, size_t byteStride,
                                  unsigned int* treelets) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (M == 0) return;
  if (!rays || !treelets || byteStride < sizeof(RTCRay) || (byteStride % 4)) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  cudaStream_t st = proposer_stream(p);
  std::lock_guard<std::mutex> lk(p->mtx);
  DevSpan in(rays, (size_t)(M - 1) * byteStride + sizeof(RTCRay), st, true);
  DevSpan out(treelets, (size_t)M * 16, st, false);
  t_ctx.ensure(p->scene->device->cuda_device);
  cuda_ok(cudaMemsetAsync(t_ctx.dscratch + 1, 0, sizeof(uint32_t), st), "memset");
  cuda_ok(p->net.predict(in.d, byteStride, M, nullptr, (uint32_t*)out.d, st, nullptr, t_ctx.dscratch + 1),
          "proposer inference");
  out.copy_out(st);
  uint32_t perr = 0;
  cuda_ok(cudaMemcpyAsync(&perr, t_ctx.dscratch + 1, sizeof(perr), cudaMemcpyDeviceToHost, st), "status");
  cuda_ok(cudaStreamSynchronize(st), "proposer inference");
  if (perr) fail(RTC_ERROR_UNKNOWN, "proposer inference timed out");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbProposerGetStats(RTCGBProposer hp, RTCGBProposerStats* out) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (!out) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  RTCGBProposerStats r{};
  r.num_treelets = p->net.num_treelets;
  r.samples = p->net.stats.samples;
  r.steps = p->net.stats.steps;
  r.loss = p->net.stats.loss;
  r.top1 = p->net.stats.top1;
  r.top4 = p->net.stats.top4;
  *out = r;
  API_END(p ? p->scene->device : nullptr)
}

RTC_API size_t rtcgbProposerParamCount(void) { return gb::kNumParams; }

RTC_API void rtcgbProposerGetParams(RTCGBProposer hp, float* params) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (!params) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  cudaStream_t st = proposer_stream(p);
  std::lock_guard<std::mutex> lk(p->mtx);
  cuda_ok(p->net.get_params(params, st), "proposer parameters");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbProposerSetParams(RTCGBProposer hp, const float* params) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (!params) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  cudaStream_t st = proposer_stream(p);
  std::lock_guard<std::mutex> lk(p->mtx);
  cuda_ok(p->net.set_params(params, st), "proposer parameters");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API float rtcgbProposerGradients(RTCGBProposer hp, const struct RTCRay* rays, unsigned int B, size_t byteStride,
                                     const int* labels, float* grads) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (B == 0 || !rays || !labels || !grads || byteStride < sizeof(RTCRay) || (byteStride % 4))
    fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  cudaStream_t st = proposer_stream(p);
  std::lock_guard<std::mutex> lk(p->mtx);
  DevSpan in(rays, (size_t)(B - 1) * byteStride + sizeof(RTCRay), st, true);
  DevSpan lab(labels, (size_t)B * 4, st, true);
  DevSpan g(grads, gb::kNumParams * sizeof(float), st, false);
  float loss = 0.0f;
  cuda_ok(p->net.gradients(in.d, byteStride, (const int32_t*)lab.d, B, (float*)g.d, &loss, st), "proposer gradients");
  g.copy_out(st);
  cuda_ok(cudaStreamSynchronize(st), "proposer gradients");
  return loss;
  API_END(p ? p->scene->device : nullptr)
  return NAN;
}

RTC_API unsigned int rtcgbProposerGetTreelets(RTCGBProposer hp, unsigned int* roots, unsigned int* record_treelet,
                                              unsigned int max_records) {
  ProposerObj* p = (ProposerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (roots)
    for (unsigned i = 0; i < (unsigned)gb::kTreelets; i++) roots[i] = i < p->roots.size() ? p->roots[i] : gb::kInvalidID;
  if (record_treelet)
    for (unsigned i = 0; i < max_records && i < p->record_treelet.size(); i++) record_treelet[i] = p->record_treelet[i];
  return (unsigned)p->roots.size();
  API_END(p ? p->scene->device : nullptr)
  return 0;
}

RTC_API void rtcgbIntersect1MLearned(RTCScene hs, RTCGBProposer hp, struct RTCRayHit* rayhit, unsigned int M,
                                     size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hp);
  run_query(s, rayhit, M, byteStride, false, sizeof(RTCRayHit), (ProposerObj*)hp);
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcgbOccluded1MLearned(RTCScene hs, RTCGBProposer hp, struct RTCRay* ray, unsigned int M,
                                    size_t byteStride) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hp);
  run_query(s, ray, M, byteStride, true, sizeof(RTCRay), (ProposerObj*)hp);
  API_END(s ? s->device : nullptr)
}

// ---- animated path tracing

namespace {
struct PathTracerObj : RefCounted {
  Scene* scene;
  uint64_t build_serial;
  gb::PathTracer pt;
  gb::RefitScratch refit{};
  ProposerObj* prop = nullptr;
  explicit PathTracerObj(Scene* s) : scene(s), build_serial(s->build_serial) { scene->inc(); }
  ~PathTracerObj() override {
    scene->device->set_current();
    pt.release();
    gb::refit_release(&refit);
    if (prop) prop->dec();
    scene->dec();
  }
  cudaStream_t stream() {
    scene->device->set_current();
    t_ctx.ensure(scene->device->cuda_device);
    return t_ctx.stream();
  }
};
}  // namespace

RTC_API RTCGBPathTracer rtcgbNewPathTracer(RTCScene hs, unsigned int width, unsigned int height,
                                           unsigned int bounces, const float* camera) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  if (!camera || width == 0 || height == 0 || bounces == 0 || bounces > (unsigned)gb::kMaxBounces)
    fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  std::lock_guard<std::mutex> lk(s->mtx);
  if (!s->committed || s->bvh.num_nodes == 0) fail(RTC_ERROR_INVALID_OPERATION, "scene not committed or empty");
  if (s->bvh.robust || s->batched)
    fail(RTC_ERROR_INVALID_OPERATION, "robust and batched scenes are not supported by the path tracer");
  PathTracerObj* p = new PathTracerObj(s);
  try {
    gb::CameraSpec cam{};
    for (int a = 0; a < 3; a++) {
      cam.eye[a] = camera[a];
      cam.look[a] = camera[3 + a];
      cam.up[a] = camera[6 + a];
    }
    cam.fov_deg = camera[9];
    cuda_ok(p->pt.init(&s->bvh, width, height, bounces, cam, p->stream()), "path tracer");
  } catch (...) {
    p->dec();
    throw;
  }
  return (RTCGBPathTracer)p;
  API_END(s ? s->device : nullptr)
  return nullptr;
}

RTC_API void rtcgbRetainPathTracer(RTCGBPathTracer hp) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  p->inc();
  API_END(nullptr)
}

RTC_API void rtcgbReleasePathTracer(RTCGBPathTracer hp) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  p->dec();
  API_END(nullptr)
}

RTC_API void rtcgbPathTracerAnimateSoup(RTCGBPathTracer hp, unsigned int geomID, float amplitude, unsigned int seed) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  Scene* s = p->scene;
  std::lock_guard<std::mutex> lk(s->mtx);
  if (geomID >= s->geoms.size() || !s->geoms[geomID]) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid geometry ID");
  const gb::GeomDesc* d = nullptr;
  for (const gb::GeomDesc& x : s->descs)
    if (x.geomID == geomID) d = &x;
  if (!d) fail(RTC_ERROR_INVALID_ARGUMENT, "geometry is not part of the committed BVH");
  const Geometry* g = s->geoms[geomID];
  if (!is_device_pointer(g->vertices.ptr) || (const char*)g->vertices.ptr != d->verts)
    fail(RTC_ERROR_INVALID_OPERATION, "the animated geometry needs a shared vertex buffer in device memory");
  cudaStream_t st = p->stream();
  gb::refit_release(&p->refit);
  cuda_ok(gb::refit_prepare(s->descs.data(), (int)s->descs.size(), s->bvh, &p->refit, st), "refit setup");
  gb::SoupAnimation a{};
  a.verts = (float*)d->verts;
  a.vstride = d->vstride;
  a.idx = d->idx;
  a.istride = d->istride;
  a.ntris = d->ntris;
  a.nverts = d->nverts;
  a.amplitude = amplitude;
  a.seed = seed;
  cuda_ok(p->pt.animate(a, &p->refit, st), "animation setup");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbPathTracerSetProposer(RTCGBPathTracer hp, RTCGBProposer hprop) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  ProposerObj* q = (ProposerObj*)hprop;
  if (q && q->scene != p->scene) fail(RTC_ERROR_INVALID_ARGUMENT, "proposer belongs to another scene");
  if (q) q->inc();
  if (p->prop) p->prop->dec();
  p->prop = q;
  p->pt.set_proposer(q ? &q->net : nullptr);
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbPathTracerRenderFrame(RTCGBPathTracer hp, unsigned int frame, int learned, RTCGBFrameStats* out) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  Scene* s = p->scene;
  if (!s->committed || s->build_serial != p->build_serial)
    fail(RTC_ERROR_INVALID_OPERATION, "the scene was rebuilt since the path tracer was made");
  const bool use = learned && p->prop && p->prop->current();
  std::unique_lock<std::mutex> plk;
  if (use) plk = std::unique_lock<std::mutex>(p->prop->mtx);
  gb::FrameStats fs;
  cuda_ok(p->pt.render(frame, use, p->stream(), &fs), "frame");
  if (out) {
    RTCGBFrameStats r{};
    r.frame_ms = fs.frame_ms;
    r.rays = fs.rays;
    r.proposal_hits = fs.proposal_hits;
    for (int b = 0; b < gb::kMaxBounces; b++) r.rays_per_bounce[b] = fs.rays_per_bounce[b];
    r.learned = fs.learned;
    r.errors = fs.errors;
    *out = r;
  }
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbPathTracerTrainProposer(RTCGBPathTracer hp, unsigned int epochs, unsigned int batch, float lr) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (!p->prop) fail(RTC_ERROR_INVALID_OPERATION, "no proposer attached");
  if (!(lr > 0.0f)) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid learning rate");
  std::lock_guard<std::mutex> lk(p->prop->mtx);
  cudaStream_t st = p->stream();
  cuda_ok(p->prop->net.train(p->pt.log_records(), 80, p->pt.log_count(), epochs, batch, lr, st), "proposer training");
  cuda_ok(cudaStreamSynchronize(st), "proposer training");
  API_END(p ? p->scene->device : nullptr)
}

RTC_API void rtcgbPathTracerGetImage(RTCGBPathTracer hp, float* rgb) {
  PathTracerObj* p = (PathTracerObj*)hp;
  API_BEGIN
  VERIFY_HANDLE(hp);
  if (!rgb) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  cuda_ok(p->pt.image(rgb, p->stream()), "image");
  API_END(p ? p->scene->device : nullptr)
}

// ---- batched scenes

RTC_API void rtcgbSetSceneBatched(RTCScene hs, int enable) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  std::lock_guard<std::mutex> lk(s->mtx);
  s->batched = enable != 0;
  s->committed = false;  // takes effect at the next commit
  s->built_sig.clear();
  API_END(s ? s->device : nullptr)
}

RTC_API void rtcgbIntersect1MBatched(RTCScene hs, struct RTCRayHit* rayhit, unsigned int M, size_t byteStride,
                                     const unsigned int* batch_start, unsigned int num_batches) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  BatchArgs b;
  b.start = batch_start;
  b.nbatches = num_batches;
  run_query(s, rayhit, M, byteStride, false, sizeof(RTCRayHit), nullptr, &b);
  API_END(s ? s->device : nullptr)
}

// ---------------------------------------------------------------------------
// batched frames: restore + build + batched closest-hit query of a batched
// scene, captured into one CUDA graph and replayed
// ---------------------------------------------------------------------------

struct BatchedFrame {
  Scene* scene;
  uint64_t commit_serial;
  gb::GraphBuild gbuild;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t* d_start = nullptr;
  unsigned int* scratch = nullptr;  // [0] ray counter, [1] error flags, [2..] counters
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  RTCGBBatchedFrameStats stats{};
  explicit BatchedFrame(Scene* s) : scene(s), commit_serial(s->commit_serial) { scene->inc(); }
  ~BatchedFrame() {
    scene->device->set_current();
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_start) cudaFree(d_start);
    if (scratch) cudaFree(scratch);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    gb::graph_build_release(&gbuild);
    scene->dec();
  }
};

RTC_API RTCGBBatchedFrame rtcgbNewBatchedFrame(RTCScene hs, struct RTCRayHit* rayhit, const struct RTCRayHit* pristine,
                                               unsigned int M, size_t byteStride, const unsigned int* batch_start,
                                               unsigned int num_batches) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  std::lock_guard<std::mutex> lk(s->mtx);
  if (!s->batched || !s->committed) fail(RTC_ERROR_INVALID_OPERATION, "a committed batched scene is required");
  if (s->ninsts) fail(RTC_ERROR_INVALID_OPERATION, "batched frames do not take instances");
  if (s->bvh.num_nodes == 0) fail(RTC_ERROR_INVALID_OPERATION, "empty scene");
  for (size_t k = 0; k < s->descs.size(); k++)
    if (s->descs[k].geomID != k)
      fail(RTC_ERROR_INVALID_OPERATION, "batched frames need geometry IDs 0..n-1 without gaps");
  if (!rayhit || M == 0 || num_batches == 0 || num_batches > s->descs.size() || byteStride < sizeof(RTCRayHit) ||
      byteStride % 4)
    fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  const cudaMemoryType mt = pointer_type(rayhit);
  if (mt != cudaMemoryTypeDevice && mt != cudaMemoryTypeManaged) fail(RTC_ERROR_INVALID_ARGUMENT, "rays must be device memory");
  if (pristine) {
    const cudaMemoryType mp = pointer_type(pristine);
    if (mp != cudaMemoryTypeDevice && mp != cudaMemoryTypeManaged)
      fail(RTC_ERROR_INVALID_ARGUMENT, "pristine rays must be device memory");
  }
  std::vector<uint32_t> hs_start(num_batches + 1);
  cuda_ok(cudaMemcpy(hs_start.data(), batch_start, hs_start.size() * sizeof(uint32_t), cudaMemcpyDefault), "batches");
  if (hs_start[0] != 0 || hs_start.back() != M) fail(RTC_ERROR_INVALID_ARGUMENT, "batches must cover the rays exactly");
  for (size_t b = 1; b < hs_start.size(); b++)
    if (hs_start[b] < hs_start[b - 1]) fail(RTC_ERROR_INVALID_ARGUMENT, "batch boundaries must not decrease");
  // the plan of the replayed build: this scene's last build, with margins
  gb::GraphBuildPlan plan;
  plan.valid_tris = s->stats.num_prims;
  plan.roots = 0;
  for (uint32_t r : s->bvh.roots) plan.roots += r != gb::kInvalidID ? 1u : 0u;
  plan.ploc_rounds = s->stats.ploc_rounds;
  plan.levels = s->stats.depth;
  plan.leaf_max = (int)s->stats.leaf_max;
  gb::BuildOptions opt = s->device->build_opt;
  opt.robust = (s->flags & RTC_SCENE_FLAG_ROBUST) != 0;
  opt.segmented = 1;
  opt.leaf_max = plan.leaf_max;
  Device* dev = s->device;
  dev->set_current();
  t_ctx.ensure(dev->cuda_device);
  cudaStream_t st = t_ctx.stream();
  BatchedFrame* f = new BatchedFrame(s);
  try {
    cuda_ok(gb::graph_build_prepare(s->descs.data(), (int)s->descs.size(), opt, plan, &f->gbuild), "frame build buffers");
    cuda_ok(cudaMalloc((void**)&f->d_start, hs_start.size() * sizeof(uint32_t)), "cudaMalloc batches");
    cuda_ok(cudaMemcpy(f->d_start, hs_start.data(), hs_start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
            "batches");
    cuda_ok(cudaMalloc((void**)&f->scratch, 64), "cudaMalloc scratch");
    cuda_ok(cudaEventCreate(&f->e0), "event");
    cuda_ok(cudaEventCreate(&f->e1), "event");
    gb::TraceParams P{};
    P.nodes = f->gbuild.nodes;
    P.tris = f->gbuild.tris;
    P.rays = (char*)rayhit;
    P.stride = byteStride;
    P.nrays = M;
    P.ray_counter = f->scratch;
    P.err = f->scratch + 1;
    P.counters = reinterpret_cast<gb::TraceCounters*>(f->scratch + 2);
    P.max_iters = 4 * f->gbuild.maxw + 64;
    P.num_nodes = f->gbuild.maxw;
    P.num_tris = plan.valid_tris;
    P.robust = opt.robust;
    P.batch_start = f->d_start;
    P.batch_root = f->gbuild.seg_index;  // geometry IDs are the segments
    P.nbatches = num_batches;
    P.shape = s->trace_shape.load(std::memory_order_relaxed);
    const size_t span = (size_t)(M - 1) * byteStride + sizeof(RTCRayHit);
    cuda_ok(cudaStreamSynchronize(st), "frame");
    cuda_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = cudaSuccess;
    if (pristine) e = gb::copy_device(rayhit, pristine, span, st);
    if (e == cudaSuccess) e = gb::graph_build_enqueue(f->gbuild, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->scratch, 0, 64, st);
    if (e == cudaSuccess) e = gb::launch_trace(P, false, false, st);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(st, &g);
    f->graph = g;
    cuda_ok(e, "frame capture");
    cuda_ok(e2, "end capture");
    cuda_ok(cudaGraphInstantiate(&f->exec, f->graph, 0), "instantiate frame");
    size_t nnodes = 0;
    cuda_ok(cudaGraphGetNodes(f->graph, nullptr, &nnodes), "graph nodes");
    f->stats.graph_nodes = (unsigned int)nnodes;
    f->stats.ploc_rounds = 0;  // set by each replay: the device decides
    f->stats.levels = 0;
  } catch (...) {
    delete f;
    throw;
  }
  return (RTCGBBatchedFrame)f;
  API_END(s ? s->device : nullptr)
  return nullptr;
}

RTC_API void rtcgbBatchedFrameReplay(RTCGBBatchedFrame hf) {
  BatchedFrame* f = (BatchedFrame*)hf;
  API_BEGIN
  if (!f) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid frame");
  Scene* s = f->scene;
  if (s->commit_serial != f->commit_serial)
    fail(RTC_ERROR_INVALID_OPERATION, "the scene was committed again: create a new frame");
  s->device->set_current();
  t_ctx.ensure(s->device->cuda_device);
  cudaStream_t st = t_ctx.stream();
  cuda_ok(cudaEventRecord(f->e0, st), "event");
  cuda_ok(cudaGraphLaunch(f->exec, st), "frame launch");
  cuda_ok(cudaEventRecord(f->e1, st), "event");
  gb::GraphBuildResult r;
  cuda_ok(gb::graph_build_result(f->gbuild, s->bvh.lo, s->bvh.hi, &r, st), "frame result");
  unsigned int err = 0;
  cuda_ok(cudaMemcpy(&err, f->scratch + 1, sizeof(err), cudaMemcpyDeviceToHost), "frame status");
  float ms = 0;
  cudaEventElapsedTime(&ms, f->e0, f->e1);
  f->stats.frame_ms = ms;
  f->stats.status = r.status;
  f->stats.num_nodes = r.num_nodes;
  f->stats.build_sah = r.sah;
  f->stats.ploc_rounds = r.ploc_rounds;
  f->stats.levels = r.depth;
  f->stats.replays++;
  if (r.status) fail(RTC_ERROR_UNKNOWN, "the replayed build failed (its status in rtcgbGetBatchedFrameStats)");
  if (err) fail(RTC_ERROR_UNKNOWN, "traversal error in a frame");
  API_END(f ? f->scene->device : nullptr)
}

RTC_API void rtcgbGetBatchedFrameStats(RTCGBBatchedFrame hf, RTCGBBatchedFrameStats* out) {
  BatchedFrame* f = (BatchedFrame*)hf;
  API_BEGIN
  if (!f || !out) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid argument");
  *out = f->stats;
  API_END(f ? f->scene->device : nullptr)
}

RTC_API void rtcgbReleaseBatchedFrame(RTCGBBatchedFrame hf) {
  BatchedFrame* f = (BatchedFrame*)hf;
  API_BEGIN
  if (!f) fail(RTC_ERROR_INVALID_ARGUMENT, "invalid frame");
  delete f;
  API_END(nullptr)
}

RTC_API void rtcgbOccluded1MBatched(RTCScene hs, struct RTCRay* ray, unsigned int M, size_t byteStride,
                                    const unsigned int* batch_start, unsigned int num_batches) {
  Scene* s = (Scene*)hs;
  API_BEGIN
  VERIFY_HANDLE(hs);
  BatchArgs b;
  b.start = batch_start;
  b.nbatches = num_batches;
  run_query(s, ray, M, byteStride, true, sizeof(RTCRay), nullptr, &b);
  API_END(s ? s->device : nullptr)
}

}  // extern "C"
