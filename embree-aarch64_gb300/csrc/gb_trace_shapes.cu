// gb_trace_shapes.cu -- the plain closest-hit and any-hit traversal kernels
// (plain and robust scenes, 16-byte aligned records) in the tuned launch
// shapes 1.. of kTraceShapes.  A translation unit of its own, so that these
// instantiations compile in parallel with the default ones (gb_trace.cu).
#include "gb_trace_kernel.cuh"

namespace gb {

template <int S>
using ShapeN = Shape<kTraceShapes[S].threads, kTraceShapes[S].ctas, kTraceShapes[S].shared_stack,
                     kTraceShapes[S].refill>;

template <class SH>
static cudaError_t launch_plain(const TraceParams& P, bool anyhit, cudaStream_t st) {
  if (P.robust)
    return anyhit ? launch_shaped<true, false, true, true, false, false, false, SH>(P, st)
                  : launch_shaped<false, false, true, true, false, false, false, SH>(P, st);
  return anyhit ? launch_shaped<true, false, true, false, false, false, false, SH>(P, st)
                : launch_shaped<false, false, true, false, false, false, false, SH>(P, st);
}

cudaError_t launch_tuned_shape(const TraceParams& P, bool anyhit, cudaStream_t st) {
  static_assert(kNumTraceShapes == 7, "one case per tuned shape");
  switch (P.shape) {
    case 1: return launch_plain<ShapeN<1>>(P, anyhit, st);
    case 2: return launch_plain<ShapeN<2>>(P, anyhit, st);
    case 3: return launch_plain<ShapeN<3>>(P, anyhit, st);
    case 4: return launch_plain<ShapeN<4>>(P, anyhit, st);
    case 5: return launch_plain<ShapeN<5>>(P, anyhit, st);
    case 6: return launch_plain<ShapeN<6>>(P, anyhit, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gb
