"""ctypes bridge to the reference itself: the reference's sources compiled in place by
oracle/ref.mk into oracle/_ref/libembree3_ref.so, driven by oracle/ref_harness.c.

TEST INFRASTRUCTURE ONLY: generates the reference-made fixtures under tests/golden/,
pins the oracle restatement (oracle.c) to the reference, and times the reference's CPU
path. It needs the reference source tree to build, so it exists only where that tree
does; `available()` says whether it does.
"""
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libembree3_ref.so")
HARNESS = os.path.join(OUT, "libref_harness.so")
DEFAULT_SRC = "/root/reference"

_h = None


def source_tree():
    return os.environ.get("EMBREE_REF_SRC", DEFAULT_SRC)


def build(jobs=None):
    """Compiles the reference + harness with oracle/ref.mk (incremental). Returns True
    when the library exists afterwards; False when the reference tree is absent."""
    src = source_tree()
    if not os.path.isdir(os.path.join(src, "kernels")):
        return os.path.exists(HARNESS)
    jobs = jobs or os.cpu_count() or 4
    subprocess.run(["make", "-s", "-f", os.path.join("oracle", "ref.mk"), f"REF={src}", f"-j{jobs}"],
                   cwd=REPO, check=True)
    return os.path.exists(HARNESS)


def available():
    return os.path.exists(HARNESS) and os.path.exists(LIB)


def harness():
    global _h
    if _h is None:
        if not available():
            raise RuntimeError("reference library not built (oracle/ref.mk needs the reference source tree)")
        H = ctypes.CDLL(HARNESS)
        vp, u, i, d = ctypes.c_void_p, ctypes.c_uint, ctypes.c_int, ctypes.c_double
        H.refh_scene_new.restype = vp
        H.refh_scene_new.argtypes = [ctypes.c_char_p, i, i]
        H.refh_add_mesh.restype = i
        H.refh_add_mesh.argtypes = [vp, vp, u, vp, u]
        H.refh_commit.restype = d
        H.refh_commit.argtypes = [vp]
        H.refh_bounds.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
        H.refh_error.restype = u
        H.refh_error.argtypes = [vp]
        H.refh_free.argtypes = [vp]
        H.refh_query.restype = d
        H.refh_query.argtypes = [vp, vp, u, ctypes.c_size_t, i, u, i, i]
        _h = H
    return _h


class _CaptureStdout:
    """Redirects file descriptor 1 (the reference prints BENCHMARK_BUILD lines with
    std::cout) into a temporary file for the duration of a call."""

    def __enter__(self):
        sys.stdout.flush()
        self._tmp = tempfile.TemporaryFile(mode="w+b")
        self._saved = os.dup(1)
        os.dup2(self._tmp.fileno(), 1)
        return self

    def __exit__(self, *exc):
        try:
            libc = ctypes.CDLL(None)
            libc.fflush(None)
        except OSError:
            pass
        os.dup2(self._saved, 1)
        os.close(self._saved)
        self._tmp.seek(0)
        self.text = self._tmp.read().decode("utf-8", "replace")
        self._tmp.close()
        return False


BENCH_RE = re.compile(r"BENCHMARK_BUILD\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)")

RTC_SCENE_FLAG_ROBUST = 4
RTC_BUILD_QUALITY_MEDIUM = 1


class RefScene:
    """A committed scene of the reference library built from [(verts, idx)] meshes
    (geometry IDs 0, 1, ... in order). `threads` sets the reference's thread count
    (0 = all cores); `benchmark=True` makes the commit report the reference builder's
    own BENCHMARK_BUILD line (kernels/bvh/bvh.cpp:173-179) in self.build_stats."""

    def __init__(self, meshes, robust=False, threads=0, benchmark=True, quality=RTC_BUILD_QUALITY_MEDIUM):
        H = harness()
        cfg = f"verbose=0,benchmark={1 if benchmark else 0}"
        if threads:
            cfg += f",threads={threads}"
        self._s = ctypes.c_void_p(H.refh_scene_new(cfg.encode(), RTC_SCENE_FLAG_ROBUST if robust else 0, quality))
        if not self._s:
            raise RuntimeError("rtcNewDevice failed")
        self._keep = []
        for verts, idx in meshes:
            v = np.asarray(verts, np.float32).reshape(-1, 3)
            # shared vertex buffers are read with 16-byte loads: one float of padding
            vp = np.zeros(v.size + 1, np.float32)
            vp[:v.size] = v.ravel()
            ix = np.ascontiguousarray(np.asarray(idx, np.uint32).reshape(-1, 3))
            self._keep.append((vp, ix))
            gid = H.refh_add_mesh(self._s, vp.ctypes.data, v.shape[0], ix.ctypes.data, ix.shape[0])
            if gid < 0:
                raise RuntimeError(f"rtcNewGeometry/attach failed: error {H.refh_error(self._s)}")
        with _CaptureStdout() as cap:
            self.commit_s = H.refh_commit(self._s)
        if self.commit_s < 0:
            raise RuntimeError(f"rtcCommitScene failed: error {H.refh_error(self._s)}")
        self.build_stats = None
        m = BENCH_RE.search(cap.text)
        if m:
            self.build_stats = dict(builder_s=float(m.group(1)), prims_per_s=float(m.group(2)),
                                    sah=float(m.group(3)), bytes=int(float(m.group(4))), bvh=m.group(5))

    def bounds(self):
        b = (ctypes.c_float * 6)()
        harness().refh_bounds(self._s, b)
        return list(b)

    def intersect(self, rayhits, nthreads=0, chunk=1024, coherent=False):
        """rtcIntersect1M in place on an RTCRayHit array; returns wall seconds."""
        assert rayhits.dtype.itemsize == 80 and rayhits.flags.c_contiguous
        nthreads = nthreads or os.cpu_count()
        return harness().refh_query(self._s, rayhits.ctypes.data, rayhits.shape[0], 80, nthreads, chunk, 0,
                                    1 if coherent else 0)

    def occluded(self, rays, nthreads=0, chunk=1024, coherent=False):
        """rtcOccluded1M in place on RTCRay (or RTCRayHit) records; returns wall seconds."""
        assert rays.flags.c_contiguous
        nthreads = nthreads or os.cpu_count()
        return harness().refh_query(self._s, rays.ctypes.data, rays.shape[0], rays.dtype.itemsize, nthreads,
                                    chunk, 1, 1 if coherent else 0)

    def close(self):
        if self._s:
            harness().refh_free(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
