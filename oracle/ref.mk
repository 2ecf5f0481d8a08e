# Compiles the reference (Embree 3.12.1 / embree-aarch64) from its own sources, in place,
# into oracle/_ref/ — without the reference's CMake build. It is the parity oracle's pin
# and the CPU baseline measured in this container; test infrastructure only.
#
#   make -f oracle/ref.mk REF=<reference source tree> -j8        (from the repository root)
#
# One ISA: the x86 AVX2 code path (the reference's "x86 SSE/AVX2 build" selects it on any
# AVX2 host; its runtime ISA dispatch is compiled out), internal tasking, the flags of the
# reference's common/cmake/gnu.cmake (Release: -O3 -DNDEBUG, no auto-vectoriser, default
# FP contraction, so `madd`/`msub` fuse as in the reference's own AVX2 build). The three
# headers the reference's CMake build generates come from oracle/ref_config/. The source
# list is the reference's kernels/CMakeLists.txt library list for a single-ISA AVX2 build,
# minus the curve, point, quad, grid, user and subdivision geometry (switched off in
# oracle/ref_config/config.h) and the algorithms' self-tests.
#
# REF_STAT=1 builds a second library, libembree3_ref_stat.so, with the reference's
# traversal counters (EMBREE_STAT_COUNTERS, kernels/common/stat.h:9-18) switched on.

REF ?= /root/reference
OUT ?= oracle/_ref
CXX ?= g++
CC ?= gcc

ISA_FLAGS := -mf16c -mavx2 -mfma -mlzcnt -mbmi -mbmi2 -DEMBREE_TARGET_AVX2
BASE_FLAGS := -O3 -DNDEBUG -std=c++11 -fPIC -fvisibility=hidden -fvisibility-inlines-hidden \
  -fno-strict-aliasing -fno-tree-vectorize -fno-strict-overflow -fno-delete-null-pointer-checks \
  -fwrapv -w -DTASKING_INTERNAL -DEMBREE_LOWEST_ISA \
  -Ioracle/ref_config/embree3 -I$(REF)/include -I$(REF)

COMMON_SRC := \
  common/sys/alloc.cpp common/sys/barrier.cpp common/sys/condition.cpp common/sys/filename.cpp \
  common/sys/library.cpp common/sys/mutex.cpp common/sys/regression.cpp common/sys/string.cpp \
  common/sys/sysinfo.cpp common/sys/thread.cpp common/math/constants.cpp common/simd/sse.cpp \
  common/lexers/stringstream.cpp common/lexers/tokenstream.cpp \
  common/tasking/taskschedulerinternal.cpp

KERNEL_SRC := \
  kernels/common/device.cpp kernels/common/stat.cpp kernels/common/acceln.cpp \
  kernels/common/accelset.cpp kernels/common/state.cpp kernels/common/rtcore.cpp \
  kernels/common/rtcore_builder.cpp kernels/common/scene.cpp kernels/common/alloc.cpp \
  kernels/common/geometry.cpp kernels/common/scene_user_geometry.cpp \
  kernels/common/scene_instance.cpp kernels/common/scene_triangle_mesh.cpp \
  kernels/common/scene_quad_mesh.cpp kernels/common/scene_curves.cpp \
  kernels/common/scene_line_segments.cpp kernels/common/scene_grid_mesh.cpp \
  kernels/common/scene_points.cpp kernels/common/motion_derivative.cpp \
  kernels/subdiv/bezier_curve.cpp kernels/subdiv/bspline_curve.cpp kernels/subdiv/catmullrom_curve.cpp \
  kernels/geometry/primitive4.cpp kernels/geometry/primitive8.cpp \
  kernels/geometry/instance_intersector.cpp kernels/builders/primrefgen.cpp \
  kernels/bvh/bvh.cpp kernels/bvh/bvh_statistics.cpp kernels/bvh/bvh4_factory.cpp \
  kernels/bvh/bvh8_factory.cpp kernels/bvh/bvh_collider.cpp kernels/bvh/bvh_rotate.cpp \
  kernels/bvh/bvh_refit.cpp kernels/bvh/bvh_builder.cpp kernels/bvh/bvh_builder_hair.cpp \
  kernels/bvh/bvh_builder_hair_mb.cpp kernels/bvh/bvh_builder_morton.cpp \
  kernels/bvh/bvh_builder_sah.cpp kernels/bvh/bvh_builder_sah_spatial.cpp \
  kernels/bvh/bvh_builder_sah_mb.cpp kernels/bvh/bvh_builder_twolevel.cpp \
  kernels/bvh/bvh_intersector1_bvh4.cpp kernels/bvh/bvh_intersector1_bvh8.cpp \
  kernels/bvh/bvh_intersector_hybrid4_bvh4.cpp kernels/bvh/bvh_intersector_hybrid8_bvh4.cpp \
  kernels/bvh/bvh_intersector_hybrid4_bvh8.cpp kernels/bvh/bvh_intersector_hybrid8_bvh8.cpp \
  kernels/bvh/bvh_intersector_stream_bvh4.cpp kernels/bvh/bvh_intersector_stream_bvh8.cpp \
  kernels/bvh/bvh_intersector_stream_filters.cpp

SRC := $(COMMON_SRC) $(KERNEL_SRC)
OBJ := $(patsubst %.cpp,$(OUT)/obj/%.o,$(SRC))
OBJ_STAT := $(patsubst %.cpp,$(OUT)/obj_stat/%.o,$(SRC))

LIBS := $(OUT)/libembree3_ref.so $(OUT)/libref_harness.so
ifeq ($(REF_STAT),1)
LIBS += $(OUT)/libembree3_ref_stat.so
endif

all: $(LIBS)

$(OUT)/libembree3_ref.so: $(OBJ)
	$(CXX) -shared -Wl,-soname,libembree3_ref.so -Wl,--version-script=$(REF)/kernels/export.linux.map \
	  -o $@ $^ -lpthread -ldl

$(OUT)/libembree3_ref_stat.so: $(OBJ_STAT)
	$(CXX) -shared -Wl,-soname,libembree3_ref_stat.so -Wl,--version-script=$(REF)/kernels/export.linux.map \
	  -o $@ $^ -lpthread -ldl

# the harness is compiled against this repository's own API header (include/embree3)
$(OUT)/libref_harness.so: oracle/ref_harness.c $(OUT)/libembree3_ref.so
	$(CC) -O2 -fPIC -shared -Iinclude -o $@ oracle/ref_harness.c -L$(OUT) -l:libembree3_ref.so \
	  -Wl,-rpath,'$$ORIGIN' -lpthread

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(BASE_FLAGS) $(ISA_FLAGS) -c $< -o $@

$(OUT)/obj_stat/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(BASE_FLAGS) $(ISA_FLAGS) -DORC_REF_STAT_COUNTERS -c $< -o $@

.PHONY: all
