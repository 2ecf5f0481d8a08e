/* Source-revision string the reference's device prints in verbose mode (its build writes
   it from kernels/hash.h.in). Here: the reference tree compiled in place by oracle/ref.mk. */
#define RTC_HASH "embree-aarch64 source tree, oracle/ref.mk"
