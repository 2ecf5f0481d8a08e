/* Build configuration for compiling the reference (Embree 3.12.1, embree-aarch64) from its
   sources with oracle/ref.mk, without its CMake build. The reference's build writes this
   file from kernels/config.h.in; the options chosen here are those of an x86 AVX2 build
   with internal tasking, triangle and instance geometry, ray packets and filter
   functions (the option defaults of the reference's CMakeLists.txt:155-172, with the
   other geometry types switched off because the triangle path does not use them).
   Test infrastructure only: the library this builds is the parity oracle and the CPU
   baseline, never part of the product. */
#define EMBREE_FILTER_FUNCTION
#define EMBREE_GEOMETRY_TRIANGLE
#define EMBREE_GEOMETRY_INSTANCE
#define EMBREE_RAY_PACKETS
#if defined(ORC_REF_STAT_COUNTERS)
#define EMBREE_STAT_COUNTERS
#endif

#define EMBREE_CURVE_SELF_INTERSECTION_AVOIDANCE_FACTOR 2.0

#define IF_ENABLED_TRIS(x) x
#define IF_ENABLED_QUADS(x)
#define IF_ENABLED_CURVES_OR_POINTS(x)
#define IF_ENABLED_CURVES(x)
#define IF_ENABLED_POINTS(x)
#define IF_ENABLED_SUBDIV(x)
#define IF_ENABLED_USER(x)
#define IF_ENABLED_INSTANCE(x) x
#define IF_ENABLED_GRIDS(x)
