"""Python-side helpers of the GB300 triangle ray-query library.

The product is the C-ABI shared library `librtcore_gb300.so` (sources in
../csrc, declarations in include/rtcore_gb300.h).  This package holds the
ctypes binding used by tests and the benchmark (`api`), the record layouts
(`rays`), the seeded synthetic workloads (`workloads`) and the build step
(`build`).
"""
