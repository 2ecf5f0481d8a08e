"""ctypes binding of librtcore_gb300.so (the reference-compatible C ABI).

This is how Python callers -- the tests and the benchmark -- reach the
library: through the same `rtc*` entry points a C++ host program links.
There is no other compute path: if the shared library cannot be loaded the
import fails loudly.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from .rays import RAYHIT_DTYPE, RAY_DTYPE

RTC_GEOMETRY_TYPE_TRIANGLE = 0
RTC_BUFFER_TYPE_INDEX = 0
RTC_BUFFER_TYPE_VERTEX = 1
RTC_FORMAT_UINT3 = 0x5003
RTC_FORMAT_FLOAT3 = 0x9003
RTC_INVALID_GEOMETRY_ID = 0xFFFFFFFF
RTC_SCENE_FLAG_ROBUST = 1 << 2
RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION = 1 << 3
RTC_BUILD_QUALITY_REFIT = 3
RTC_GEOMETRY_TYPE_INSTANCE = 121
RTC_FORMAT_FLOAT3X4_ROW_MAJOR = 0x9134
RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR = 0x9234
RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR = 0x9244

ERRORS = {0: "NONE", 1: "UNKNOWN", 2: "INVALID_ARGUMENT", 3: "INVALID_OPERATION", 4: "OUT_OF_MEMORY",
          5: "UNSUPPORTED_CPU", 6: "CANCELLED"}

# every entry point declared in include/rtcore_gb300.h and include/rtcore_gb300_ext.h
EXPORTS = """rtcNewDevice rtcRetainDevice rtcReleaseDevice rtcGetDeviceProperty rtcSetDeviceProperty
rtcGetDeviceError rtcSetDeviceErrorFunction rtcSetDeviceMemoryMonitorFunction rtcNewBuffer rtcNewSharedBuffer
rtcGetBufferData rtcRetainBuffer rtcReleaseBuffer rtcNewGeometry rtcRetainGeometry rtcReleaseGeometry
rtcCommitGeometry rtcEnableGeometry rtcDisableGeometry rtcSetGeometryTimeStepCount rtcSetGeometryMask
rtcSetGeometryBuildQuality rtcSetGeometryBuffer rtcSetSharedGeometryBuffer rtcSetNewGeometryBuffer
rtcGetGeometryBufferData rtcUpdateGeometryBuffer rtcSetGeometryIntersectFilterFunction
rtcSetGeometryOccludedFilterFunction rtcSetGeometryUserData rtcGetGeometryUserData rtcNewScene rtcGetSceneDevice
rtcRetainScene rtcReleaseScene rtcAttachGeometry rtcAttachGeometryByID rtcDetachGeometry rtcGetGeometry
rtcCommitScene rtcJoinCommitScene rtcSetSceneProgressMonitorFunction rtcSetSceneBuildQuality rtcSetSceneFlags
rtcGetSceneFlags rtcGetSceneBounds rtcGetSceneLinearBounds rtcIntersect1 rtcIntersect1M rtcIntersect1Mp
rtcOccluded1 rtcOccluded1M rtcOccluded1Mp rtcIntersect4 rtcIntersect8 rtcIntersect16 rtcIntersectNM
rtcIntersectNp rtcOccluded4 rtcOccluded8 rtcOccluded16 rtcOccludedNM rtcOccludedNp rtcgbGetSceneBuildStats rtcgbGetSceneBuildPhases rtcgbGetLastQueryStats rtcgbSetQueryCounting
rtcgbGetKernelLaunchCount rtcgbSetThreadStream rtcgbGetSceneBVH rtcgbRadixSortPairs rtcgbIntersect1MNoAlloc rtcgbGetDeviceHostAccess
rtcgbGetTraversalShapes rtcgbSetSceneTraversalShape rtcgbGetSceneTraversalShape rtcgbTuneSceneTraversal
rtcgbNewProposer rtcgbNewProposerEx rtcgbRetainProposer rtcgbReleaseProposer rtcgbProposerTrain rtcgbProposerPredict rtcgbProposerGetStats
rtcgbProposerParamCount rtcgbProposerGetParams rtcgbProposerSetParams rtcgbProposerGradients rtcgbProposerGetTreelets
rtcgbIntersect1MLearned rtcgbOccluded1MLearned rtcgbNewPathTracer rtcgbRetainPathTracer rtcgbReleasePathTracer
rtcgbPathTracerAnimateSoup rtcgbPathTracerSetProposer rtcgbPathTracerRenderFrame rtcgbPathTracerTrainProposer
rtcgbPathTracerGetImage rtcgbSetSceneBatched rtcgbIntersect1MBatched rtcgbOccluded1MBatched
rtcSetGeometryInstancedScene rtcSetGeometryTransform rtcGetGeometryTransform rtcgbNewBatchedFrame
rtcgbBatchedFrameReplay rtcgbGetBatchedFrameStats rtcgbReleaseBatchedFrame""".split()


class RTCBounds(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("lower_x", "lower_y", "lower_z", "align0",
                                              "upper_x", "upper_y", "upper_z", "align1")]


class RTCIntersectContext(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_int), ("filter", ctypes.c_void_p), ("instID", ctypes.c_uint * 1)]


class RTCFilterFunctionNArguments(ctypes.Structure):
    _fields_ = [("valid", ctypes.POINTER(ctypes.c_int)), ("geometryUserPtr", ctypes.c_void_p),
                ("context", ctypes.c_void_p), ("ray", ctypes.c_void_p), ("hit", ctypes.c_void_p),
                ("N", ctypes.c_uint)]


# void filter(const RTCFilterFunctionNArguments* args)
FILTER_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(RTCFilterFunctionNArguments))


def filter_callback(fn):
    """Wraps a Python callable fn(geomID, primID, u, v, t) -> bool (True keeps
    the hit) as an RTCFilterFunctionN for N = 1 calls."""
    def cb(args):
        a = args.contents
        hf = ctypes.cast(a.hit, ctypes.POINTER(ctypes.c_float))
        hu = ctypes.cast(a.hit, ctypes.POINTER(ctypes.c_uint))
        rf = ctypes.cast(a.ray, ctypes.POINTER(ctypes.c_float))
        for k in range(a.N):   # RTCHitN / RTCRayN: field f of lane k at f * N + k
            if a.valid[k] == 0:
                continue
            n = a.N
            if not fn(hu[6 * n + k], hu[5 * n + k], hf[3 * n + k], hf[4 * n + k], rf[8 * n + k]):
                a.valid[k] = 0
    return FILTER_FN(cb)


class RTCGBBuildStats(ctypes.Structure):
    _fields_ = [("sah", ctypes.c_double), ("build_ms", ctypes.c_double), ("num_nodes", ctypes.c_uint),
                ("num_leaves", ctypes.c_uint), ("num_prims", ctypes.c_uint), ("depth", ctypes.c_uint),
                ("ploc_iterations", ctypes.c_uint), ("refit", ctypes.c_uint), ("bvh_bytes", ctypes.c_ulonglong),
                ("sah_exact", ctypes.c_double), ("leaf_max", ctypes.c_uint), ("reserved", ctypes.c_uint)]


class RTCGBQueryStats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("rays", ctypes.c_ulonglong),
                ("nodes", ctypes.c_ulonglong), ("tris", ctypes.c_ulonglong), ("h2d_bytes", ctypes.c_ulonglong),
                ("d2h_bytes", ctypes.c_ulonglong), ("proposal_hits", ctypes.c_ulonglong)]


class RTCGBFrameStats(ctypes.Structure):
    _fields_ = [("frame_ms", ctypes.c_double), ("rays", ctypes.c_ulonglong), ("proposal_hits", ctypes.c_ulonglong),
                ("rays_per_bounce", ctypes.c_uint * 8), ("learned", ctypes.c_uint), ("errors", ctypes.c_uint)]


class RTCGBBatchedFrameStats(ctypes.Structure):
    _fields_ = [("frame_ms", ctypes.c_double), ("build_sah", ctypes.c_double), ("status", ctypes.c_uint),
                ("num_nodes", ctypes.c_uint), ("ploc_rounds", ctypes.c_uint), ("levels", ctypes.c_uint),
                ("graph_nodes", ctypes.c_uint), ("replays", ctypes.c_uint)]


class RTCGBProposerStats(ctypes.Structure):
    _fields_ = [("num_treelets", ctypes.c_uint), ("samples", ctypes.c_uint), ("steps", ctypes.c_uint),
                ("reserved", ctypes.c_uint), ("loss", ctypes.c_double), ("top1", ctypes.c_double),
                ("top4", ctypes.c_double)]


class RTCGBTraversalShape(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_uint), ("ctas_per_sm", ctypes.c_uint), ("shared_stack", ctypes.c_uint),
                ("refill", ctypes.c_uint)]


RTCGB_TUNE_OCCLUDED = 1

ERROR_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p)
MEMORY_FN = ctypes.CFUNCTYPE(ctypes.c_bool, ctypes.c_void_p, ctypes.c_ssize_t, ctypes.c_bool)
PROGRESS_FN = ctypes.CFUNCTYPE(ctypes.c_bool, ctypes.c_void_p, ctypes.c_double)

_lib = None


def load(build=True):
    """Loads (building first if needed) the shared library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"librtcore_gb300.so missing at {path}; run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    vp, u, sz, i = ctypes.c_void_p, ctypes.c_uint, ctypes.c_size_t, ctypes.c_int
    sig = {
        "rtcNewDevice": (vp, [ctypes.c_char_p]),
        "rtcReleaseDevice": (None, [vp]), "rtcRetainDevice": (None, [vp]),
        "rtcGetDeviceProperty": (ctypes.c_ssize_t, [vp, i]),
        "rtcSetDeviceProperty": (None, [vp, i, ctypes.c_ssize_t]),
        "rtcGetDeviceError": (i, [vp]),
        "rtcSetDeviceErrorFunction": (None, [vp, ERROR_FN, vp]),
        "rtcSetDeviceMemoryMonitorFunction": (None, [vp, MEMORY_FN, vp]),
        "rtcNewBuffer": (vp, [vp, sz]), "rtcNewSharedBuffer": (vp, [vp, vp, sz]),
        "rtcGetBufferData": (vp, [vp]), "rtcRetainBuffer": (None, [vp]), "rtcReleaseBuffer": (None, [vp]),
        "rtcNewGeometry": (vp, [vp, i]), "rtcRetainGeometry": (None, [vp]), "rtcReleaseGeometry": (None, [vp]),
        "rtcCommitGeometry": (None, [vp]), "rtcEnableGeometry": (None, [vp]), "rtcDisableGeometry": (None, [vp]),
        "rtcSetGeometryTimeStepCount": (None, [vp, u]), "rtcSetGeometryMask": (None, [vp, u]),
        "rtcSetGeometryBuildQuality": (None, [vp, i]),
        "rtcSetGeometryBuffer": (None, [vp, i, u, i, vp, sz, sz, sz]),
        "rtcSetSharedGeometryBuffer": (None, [vp, i, u, i, vp, sz, sz, sz]),
        "rtcSetNewGeometryBuffer": (vp, [vp, i, u, i, sz, sz]),
        "rtcGetGeometryBufferData": (vp, [vp, i, u]), "rtcUpdateGeometryBuffer": (None, [vp, i, u]),
        "rtcSetGeometryIntersectFilterFunction": (None, [vp, vp]),
        "rtcSetGeometryOccludedFilterFunction": (None, [vp, vp]),
        "rtcSetGeometryUserData": (None, [vp, vp]), "rtcGetGeometryUserData": (vp, [vp]),
        "rtcNewScene": (vp, [vp]), "rtcGetSceneDevice": (vp, [vp]),
        "rtcRetainScene": (None, [vp]), "rtcReleaseScene": (None, [vp]),
        "rtcAttachGeometry": (u, [vp, vp]), "rtcAttachGeometryByID": (None, [vp, vp, u]),
        "rtcDetachGeometry": (None, [vp, u]), "rtcGetGeometry": (vp, [vp, u]),
        "rtcCommitScene": (None, [vp]), "rtcJoinCommitScene": (None, [vp]),
        "rtcSetSceneProgressMonitorFunction": (None, [vp, PROGRESS_FN, vp]),
        "rtcSetSceneBuildQuality": (None, [vp, i]), "rtcSetSceneFlags": (None, [vp, i]),
        "rtcGetSceneFlags": (i, [vp]),
        "rtcGetSceneBounds": (None, [vp, ctypes.POINTER(RTCBounds)]),
        "rtcGetSceneLinearBounds": (None, [vp, vp]),
        "rtcIntersect1": (None, [vp, vp, vp]), "rtcIntersect1M": (None, [vp, vp, vp, u, sz]),
        "rtcIntersect1Mp": (None, [vp, vp, vp, u]),
        "rtcOccluded1": (None, [vp, vp, vp]), "rtcOccluded1M": (None, [vp, vp, vp, u, sz]),
        "rtcOccluded1Mp": (None, [vp, vp, vp, u]),
        "rtcIntersect4": (None, [vp, vp, vp, vp]), "rtcIntersect8": (None, [vp, vp, vp, vp]),
        "rtcIntersect16": (None, [vp, vp, vp, vp]), "rtcOccluded4": (None, [vp, vp, vp, vp]),
        "rtcOccluded8": (None, [vp, vp, vp, vp]), "rtcOccluded16": (None, [vp, vp, vp, vp]),
        "rtcIntersectNM": (None, [vp, vp, vp, u, u, sz]), "rtcOccludedNM": (None, [vp, vp, vp, u, u, sz]),
        "rtcIntersectNp": (None, [vp, vp, vp, u]), "rtcOccludedNp": (None, [vp, vp, vp, u]),
        "rtcgbGetSceneBuildStats": (None, [vp, ctypes.POINTER(RTCGBBuildStats)]),
        "rtcgbGetLastQueryStats": (None, [ctypes.POINTER(RTCGBQueryStats)]),
        "rtcgbGetSceneBuildPhases": (u, [vp, ctypes.POINTER(ctypes.c_double), u]),
        "rtcgbSetQueryCounting": (None, [i]),
        "rtcgbGetKernelLaunchCount": (ctypes.c_ulonglong, []),
        "rtcgbSetThreadStream": (None, [vp]),
        "rtcgbGetSceneBVH": (u, [vp, vp, u, vp, u, ctypes.POINTER(u)]),
        "rtcgbRadixSortPairs": (i, [vp, vp, u]),
        "rtcgbIntersect1MNoAlloc": (None, [vp, vp, u, sz, vp]),
        "rtcgbGetDeviceHostAccess": (i, [vp]),
        "rtcgbGetTraversalShapes": (u, [ctypes.POINTER(RTCGBTraversalShape), u]),
        "rtcgbSetSceneTraversalShape": (None, [vp, u]),
        "rtcgbGetSceneTraversalShape": (u, [vp]),
        "rtcgbTuneSceneTraversal": (u, [vp, vp, u, sz, vp, u, u, u, ctypes.POINTER(ctypes.c_double)]),
        "rtcgbNewProposer": (vp, [vp, u]), "rtcgbNewProposerEx": (vp, [vp, u, u]),
        "rtcgbRetainProposer": (None, [vp]),
        "rtcgbReleaseProposer": (None, [vp]),
        "rtcgbProposerTrain": (None, [vp, vp, u, sz, u, u, ctypes.c_float]),
        "rtcgbProposerPredict": (None, [vp, vp, u, sz, vp]),
        "rtcgbProposerGetStats": (None, [vp, ctypes.POINTER(RTCGBProposerStats)]),
        "rtcgbProposerParamCount": (sz, []),
        "rtcgbProposerGetParams": (None, [vp, vp]), "rtcgbProposerSetParams": (None, [vp, vp]),
        "rtcgbProposerGradients": (ctypes.c_float, [vp, vp, u, sz, vp, vp]),
        "rtcgbProposerGetTreelets": (u, [vp, vp, vp, u]),
        "rtcgbIntersect1MLearned": (None, [vp, vp, vp, u, sz]),
        "rtcgbOccluded1MLearned": (None, [vp, vp, vp, u, sz]),
        "rtcgbNewPathTracer": (vp, [vp, u, u, u, ctypes.POINTER(ctypes.c_float)]),
        "rtcgbRetainPathTracer": (None, [vp]), "rtcgbReleasePathTracer": (None, [vp]),
        "rtcgbPathTracerAnimateSoup": (None, [vp, u, ctypes.c_float, u]),
        "rtcgbPathTracerSetProposer": (None, [vp, vp]),
        "rtcgbPathTracerRenderFrame": (None, [vp, u, i, ctypes.POINTER(RTCGBFrameStats)]),
        "rtcgbPathTracerTrainProposer": (None, [vp, u, u, ctypes.c_float]),
        "rtcgbPathTracerGetImage": (None, [vp, vp]),
        "rtcgbSetSceneBatched": (None, [vp, i]),
        "rtcSetGeometryInstancedScene": (None, [vp, vp]),
        "rtcSetGeometryTransform": (None, [vp, u, i, vp]),
        "rtcGetGeometryTransform": (None, [vp, ctypes.c_float, i, vp]),
        "rtcgbIntersect1MBatched": (None, [vp, vp, u, sz, vp, u]),
        "rtcgbOccluded1MBatched": (None, [vp, vp, u, sz, vp, u]),
        "rtcgbNewBatchedFrame": (vp, [vp, vp, vp, u, sz, vp, u]),
        "rtcgbBatchedFrameReplay": (None, [vp]),
        "rtcgbGetBatchedFrameStats": (None, [vp, ctypes.POINTER(RTCGBBatchedFrameStats)]),
        "rtcgbReleaseBatchedFrame": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class RTCError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where}: RTC_ERROR_{ERRORS.get(code, code)}")
        self.code = code


class Device:
    def __init__(self, config=b""):
        self.L = load()
        self.h = ctypes.c_void_p(self.L.rtcNewDevice(config))
        if not self.h:
            raise RTCError(self.L.rtcGetDeviceError(None), "rtcNewDevice")

    def error(self):
        return self.L.rtcGetDeviceError(self.h)

    def check(self, where):
        e = self.error()
        if e:
            raise RTCError(e, where)

    def release(self):
        if self.h:
            self.L.rtcReleaseDevice(self.h)
            self.h = None


class Scene:
    """A scene of triangle meshes built with rtcCommitScene."""

    def __init__(self, device, flags=0):
        self.dev = device
        self.L = device.L
        self.h = ctypes.c_void_p(self.L.rtcNewScene(device.h))
        self._keep = []
        if flags:
            self.L.rtcSetSceneFlags(self.h, flags)
        device.check("rtcNewScene")

    def add_mesh(self, verts, idx, geom_id=None, quality=None):
        """Attaches a triangle mesh using shared buffers (kept alive here).
        quality: RTC_BUILD_QUALITY_* of the geometry (REFIT = 3)."""
        verts = np.array(verts, np.float32).reshape(-1, 3)
        idx = np.array(idx, np.uint32).reshape(-1, 3)
        self._keep.append((verts, idx))
        L = self.L
        g = ctypes.c_void_p(L.rtcNewGeometry(self.dev.h, RTC_GEOMETRY_TYPE_TRIANGLE))
        if quality is not None:
            L.rtcSetGeometryBuildQuality(g, quality)
        L.rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_VERTEX, 0, RTC_FORMAT_FLOAT3, _ptr(verts), 0, 12,
                                     verts.shape[0])
        L.rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_INDEX, 0, RTC_FORMAT_UINT3, _ptr(idx), 0, 12, idx.shape[0])
        L.rtcCommitGeometry(g)
        if geom_id is None:
            gid = L.rtcAttachGeometry(self.h, g)
        else:
            L.rtcAttachGeometryByID(self.h, g, geom_id)
            gid = geom_id
        L.rtcReleaseGeometry(g)
        self.dev.check("add_mesh")
        self._by_id = getattr(self, "_by_id", {})
        self._by_id[gid] = (verts, idx)
        return gid

    def add_mesh_device(self, verts_ptr, nverts, idx_ptr, ntris, quality=None):
        """Attaches a triangle mesh whose FLOAT3 / UINT3 buffers are CUDA device
        memory (used in place by the builder, the refit and the path tracer)."""
        L = self.L
        g = ctypes.c_void_p(L.rtcNewGeometry(self.dev.h, RTC_GEOMETRY_TYPE_TRIANGLE))
        if quality is not None:
            L.rtcSetGeometryBuildQuality(g, quality)
        L.rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_VERTEX, 0, RTC_FORMAT_FLOAT3, ctypes.c_void_p(verts_ptr), 0,
                                     12, nverts)
        L.rtcSetSharedGeometryBuffer(g, RTC_BUFFER_TYPE_INDEX, 0, RTC_FORMAT_UINT3, ctypes.c_void_p(idx_ptr), 0, 12,
                                     ntris)
        L.rtcCommitGeometry(g)
        gid = L.rtcAttachGeometry(self.h, g)
        L.rtcReleaseGeometry(g)
        self.dev.check("add_mesh_device")
        return gid

    def add_instance(self, scene, xfm, geom_id=None, fmt=RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR):
        """Attaches an instance of `scene` with the local-to-world map xfm (12 or 16
        floats in the given format)."""
        L = self.L
        g = ctypes.c_void_p(L.rtcNewGeometry(self.dev.h, RTC_GEOMETRY_TYPE_INSTANCE))
        L.rtcSetGeometryInstancedScene(g, scene.h)
        m = np.ascontiguousarray(xfm, np.float32).ravel()
        L.rtcSetGeometryTransform(g, 0, fmt, _ptr(m))
        L.rtcCommitGeometry(g)
        if geom_id is None:
            gid = L.rtcAttachGeometry(self.h, g)
        else:
            L.rtcAttachGeometryByID(self.h, g, geom_id)
            gid = geom_id
        L.rtcReleaseGeometry(g)
        self.dev.check("add_instance")
        return gid

    def set_filters(self, gid, intersect=None, occluded=None):
        """rtcSetGeometryIntersectFilterFunction / rtcSetGeometryOccludedFilterFunction
        on geometry gid with Python callables fn(geomID, primID, u, v, t) -> bool
        (None removes a callback); takes effect at the next commit."""
        g = ctypes.c_void_p(self.L.rtcGetGeometry(self.h, gid))
        cbs = [filter_callback(f) if f is not None else None for f in (intersect, occluded)]
        self._keep.append(cbs)
        as_ptr = lambda c: ctypes.cast(c, ctypes.c_void_p) if c is not None else None  # noqa: E731
        self.L.rtcSetGeometryIntersectFilterFunction(g, as_ptr(cbs[0]))
        self.L.rtcSetGeometryOccludedFilterFunction(g, as_ptr(cbs[1]))
        self.dev.check("rtcSetGeometry*FilterFunction")

    def update_vertices(self, gid, new_verts):
        """Writes new positions into geometry gid's shared vertex buffer and
        marks it updated (rtcUpdateGeometryBuffer); takes effect at commit."""
        verts, _ = self._by_id[gid]
        verts[:] = np.asarray(new_verts, np.float32).reshape(verts.shape)
        self.L.rtcUpdateGeometryBuffer(self.L.rtcGetGeometry(self.h, gid), RTC_BUFFER_TYPE_VERTEX, 0)
        self.dev.check("rtcUpdateGeometryBuffer")

    def update_indices(self, gid, new_idx):
        _, idx = self._by_id[gid]
        idx[:] = np.asarray(new_idx, np.uint32).reshape(idx.shape)
        self.L.rtcUpdateGeometryBuffer(self.L.rtcGetGeometry(self.h, gid), RTC_BUFFER_TYPE_INDEX, 0)
        self.dev.check("rtcUpdateGeometryBuffer")

    def commit(self):
        self.L.rtcCommitScene(self.h)
        self.dev.check("rtcCommitScene")

    def bounds(self):
        b = RTCBounds()
        self.L.rtcGetSceneBounds(self.h, ctypes.byref(b))
        self.dev.check("rtcGetSceneBounds")
        return np.array([b.lower_x, b.lower_y, b.lower_z]), np.array([b.upper_x, b.upper_y, b.upper_z])

    BUILD_PHASES = ("primitives_and_keys", "sort", "ploc_setup", "ploc_rounds", "ploc_finish", "collapse_setup",
                    "collapse_levels", "leaf_records")

    def build_phases(self):
        """Device microseconds of each phase of the last (replayed) build, as a dict;
        empty unless the device has gpu.build_phases=1 and the commit was replayed."""
        us = (ctypes.c_double * 8)()
        n = self.L.rtcgbGetSceneBuildPhases(self.h, us, 8)
        self.dev.check("rtcgbGetSceneBuildPhases")
        return {k: us[i] for i, k in enumerate(self.BUILD_PHASES[:n])}

    def build_stats(self):
        s = RTCGBBuildStats()
        self.L.rtcgbGetSceneBuildStats(self.h, ctypes.byref(s))
        self.dev.check("rtcgbGetSceneBuildStats")
        return {f: getattr(s, f) for f, _ in s._fields_}

    @staticmethod
    def _context(context_filter):
        cb = filter_callback(context_filter) if context_filter is not None else None
        ctx = RTCIntersectContext(0, ctypes.cast(cb, ctypes.c_void_p) if cb is not None else None,
                                  (ctypes.c_uint * 1)(RTC_INVALID_GEOMETRY_ID))
        return ctx, cb

    def intersect(self, rays, stride=None, count=None, context_filter=None):
        """rtcIntersect1M on a host RTCRayHit array (in place); context_filter:
        optional callable fn(geomID, primID, u, v, t) -> bool set as the
        intersect context's filter."""
        ctx, _cb = self._context(context_filter)
        n = rays.shape[0] if count is None else count
        self.L.rtcIntersect1M(self.h, ctypes.byref(ctx), _ptr(rays), n, stride or rays.dtype.itemsize)
        self.dev.check("rtcIntersect1M")
        return rays

    def occluded(self, rays, stride=None, count=None, context_filter=None):
        """rtcOccluded1M on a host RTCRay (or RTCRayHit) array (in place)."""
        ctx, _cb = self._context(context_filter)
        n = rays.shape[0] if count is None else count
        self.L.rtcOccluded1M(self.h, ctypes.byref(ctx), _ptr(rays), n, stride or rays.dtype.itemsize)
        self.dev.check("rtcOccluded1M")
        return rays

    def intersect_ptr(self, ptr, n, stride=80):
        """rtcIntersect1M on raw memory (host or CUDA device pointer)."""
        ctx = RTCIntersectContext(0, None, (ctypes.c_uint * 1)(RTC_INVALID_GEOMETRY_ID))
        self.L.rtcIntersect1M(self.h, ctypes.byref(ctx), ctypes.c_void_p(ptr), n, stride)
        self.dev.check("rtcIntersect1M")

    def occluded_ptr(self, ptr, n, stride=48):
        ctx = RTCIntersectContext(0, None, (ctypes.c_uint * 1)(RTC_INVALID_GEOMETRY_ID))
        self.L.rtcOccluded1M(self.h, ctypes.byref(ctx), ctypes.c_void_p(ptr), n, stride)
        self.dev.check("rtcOccluded1M")

    def set_batched(self, on=True):
        """One BVH per geometry; query with intersect_batched / occluded_batched."""
        self.L.rtcgbSetSceneBatched(self.h, 1 if on else 0)
        self.dev.check("rtcgbSetSceneBatched")

    def intersect_batched(self, rays, batch_start, ptr=None, count=None):
        """rays [batch_start[b], batch_start[b+1]) query geometry b (host array, or a
        device pointer `ptr` with `count` rays)."""
        bs = np.ascontiguousarray(batch_start, np.uint32)
        if ptr is None:
            self.L.rtcgbIntersect1MBatched(self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize, _ptr(bs),
                                           bs.shape[0] - 1)
        else:
            self.L.rtcgbIntersect1MBatched(self.h, ctypes.c_void_p(ptr), count, 80, _ptr(bs), bs.shape[0] - 1)
        self.dev.check("rtcgbIntersect1MBatched")
        return rays

    def occluded_batched(self, rays, batch_start, ptr=None, count=None):
        bs = np.ascontiguousarray(batch_start, np.uint32)
        if ptr is None:
            self.L.rtcgbOccluded1MBatched(self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize, _ptr(bs),
                                          bs.shape[0] - 1)
        else:
            self.L.rtcgbOccluded1MBatched(self.h, ctypes.c_void_p(ptr), count, 48, _ptr(bs), bs.shape[0] - 1)
        self.dev.check("rtcgbOccluded1MBatched")
        return rays

    @property
    def traversal_shape(self):
        """Launch shape of this scene's plain queries (index into traversal_shapes())."""
        v = self.L.rtcgbGetSceneTraversalShape(self.h)
        self.dev.check("rtcgbGetSceneTraversalShape")
        return v

    @traversal_shape.setter
    def traversal_shape(self, shape):
        self.L.rtcgbSetSceneTraversalShape(self.h, shape)
        self.dev.check("rtcgbSetSceneTraversalShape")

    def tune_traversal(self, rays=None, batch_start=None, occluded=False, repeats=5, ptr=None, count=None,
                       stride=80):
        """rtcgbTuneSceneTraversal on host RTCRayHit records `rays` (or device records at
        `ptr`): sets and returns the fastest launch shape, with the median milliseconds
        of every shape."""
        n = len(traversal_shapes())
        ms = (ctypes.c_double * n)()
        bs = None if batch_start is None else np.ascontiguousarray(batch_start, np.uint32)
        if ptr is None:
            ptr, count, stride = _ptr(rays), rays.shape[0], rays.dtype.itemsize
        else:
            ptr = ctypes.c_void_p(ptr)
        pick = self.L.rtcgbTuneSceneTraversal(self.h, ptr, count, stride, None if bs is None else _ptr(bs),
                                              0 if bs is None else bs.shape[0] - 1,
                                              RTCGB_TUNE_OCCLUDED if occluded else 0, repeats, ms)
        self.dev.check("rtcgbTuneSceneTraversal")
        return pick, list(ms)

    def bvh(self):
        """Copies the committed BVH: (nodes uint8 [n,80], tris float32 [m,12])."""
        nt = ctypes.c_uint()
        n = self.L.rtcgbGetSceneBVH(self.h, None, 0, None, 0, ctypes.byref(nt))
        nodes = np.zeros((max(n, 1), 80), np.uint8)
        tris = np.zeros((max(nt.value, 1), 12), np.float32)
        self.L.rtcgbGetSceneBVH(self.h, _ptr(nodes), n, _ptr(tris), nt.value, ctypes.byref(nt))
        self.dev.check("rtcgbGetSceneBVH")
        return nodes[:n], tris[:nt.value]

    def release(self):
        if self.h:
            self.L.rtcReleaseScene(self.h)
            self.h = None


def last_query_stats():
    L = load()
    s = RTCGBQueryStats()
    L.rtcgbGetLastQueryStats(ctypes.byref(s))
    return {f: getattr(s, f) for f, _ in s._fields_}


def set_counting(on):
    load().rtcgbSetQueryCounting(1 if on else 0)


def launch_count():
    return load().rtcgbGetKernelLaunchCount()


def radix_sort_pairs(keys, values):
    """GPU stable radix sort of uint64 keys with uint32 values (returns copies)."""
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.ascontiguousarray(values, np.uint32).copy()
    rc = load().rtcgbRadixSortPairs(_ptr(k), _ptr(v), k.shape[0])
    if rc:
        raise RuntimeError(f"rtcgbRadixSortPairs failed ({rc})")
    return k, v


def traversal_shapes():
    """The compiled launch shapes of the traversal kernels, shape 0 first (dicts)."""
    L = load()
    n = L.rtcgbGetTraversalShapes(None, 0)
    arr = (RTCGBTraversalShape * n)()
    L.rtcgbGetTraversalShapes(arr, n)
    return [{f: getattr(a, f) for f, _ in a._fields_} for a in arr]


def set_thread_stream(stream_ptr):
    load().rtcgbSetThreadStream(ctypes.c_void_p(stream_ptr) if stream_ptr else None)


class Proposer:
    """Learned hit proposer of a committed scene (rtcgbNewProposer)."""

    def __init__(self, scene, seed=1, max_treelets=None):
        self.scene = scene
        self.L = scene.L
        if max_treelets is None:
            self.h = ctypes.c_void_p(self.L.rtcgbNewProposer(scene.h, seed))
        else:
            self.h = ctypes.c_void_p(self.L.rtcgbNewProposerEx(scene.h, seed, max_treelets))
        scene.dev.check("rtcgbNewProposer")

    def train(self, records, epochs=1, batch=16384, lr=5e-3, count=None, stride=80):
        """records: host RTCRayHit array, or an int device pointer (then count is required)."""
        if isinstance(records, int):
            ptr, n = ctypes.c_void_p(records), count
        else:
            ptr, n = _ptr(records), records.shape[0] if count is None else count
        self.L.rtcgbProposerTrain(self.h, ptr, n, stride, epochs, batch, lr)
        self.scene.dev.check("rtcgbProposerTrain")
        return self.stats()

    def predict(self, rays):
        out = np.zeros((rays.shape[0], 4), np.uint32)
        self.L.rtcgbProposerPredict(self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize, _ptr(out))
        self.scene.dev.check("rtcgbProposerPredict")
        return out

    def stats(self):
        s = RTCGBProposerStats()
        self.L.rtcgbProposerGetStats(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def params(self):
        p = np.zeros(self.L.rtcgbProposerParamCount(), np.float32)
        self.L.rtcgbProposerGetParams(self.h, _ptr(p))
        self.scene.dev.check("rtcgbProposerGetParams")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape[0] == self.L.rtcgbProposerParamCount()
        self.L.rtcgbProposerSetParams(self.h, _ptr(p))
        self.scene.dev.check("rtcgbProposerSetParams")

    def gradients(self, rays, labels):
        labels = np.ascontiguousarray(labels, np.int32)
        g = np.zeros(self.L.rtcgbProposerParamCount(), np.float32)
        loss = self.L.rtcgbProposerGradients(self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize,
                                             _ptr(labels), _ptr(g))
        self.scene.dev.check("rtcgbProposerGradients")
        return loss, g

    def treelets(self, num_records):
        roots = np.zeros(4096, np.uint32)
        rec = np.zeros(max(num_records, 1), np.uint32)
        n = self.L.rtcgbProposerGetTreelets(self.h, _ptr(roots), _ptr(rec), num_records)
        return roots[:n], rec[:num_records]

    def intersect(self, rays):
        self.L.rtcgbIntersect1MLearned(self.scene.h, self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize)
        self.scene.dev.check("rtcgbIntersect1MLearned")
        return rays

    def occluded(self, rays):
        self.L.rtcgbOccluded1MLearned(self.scene.h, self.h, _ptr(rays), rays.shape[0], rays.dtype.itemsize)
        self.scene.dev.check("rtcgbOccluded1MLearned")
        return rays

    def intersect_ptr(self, ptr, n, stride=80):
        self.L.rtcgbIntersect1MLearned(self.scene.h, self.h, ctypes.c_void_p(ptr), n, stride)
        self.scene.dev.check("rtcgbIntersect1MLearned")

    def occluded_ptr(self, ptr, n, stride=48):
        self.L.rtcgbOccluded1MLearned(self.scene.h, self.h, ctypes.c_void_p(ptr), n, stride)
        self.scene.dev.check("rtcgbOccluded1MLearned")

    def release(self):
        if self.h:
            self.L.rtcgbReleaseProposer(self.h)
            self.h = None


class BatchedFrame:
    """Rebuild of a committed batched scene + batched closest-hit query on
    device rays, captured into one CUDA graph (rtcgbNewBatchedFrame)."""

    def __init__(self, scene, rays_ptr, count, batch_start, pristine_ptr=None, stride=80):
        self.scene = scene
        self.L = scene.L
        bs = np.ascontiguousarray(batch_start, np.uint32)
        self.h = ctypes.c_void_p(self.L.rtcgbNewBatchedFrame(scene.h, ctypes.c_void_p(rays_ptr),
                                                             ctypes.c_void_p(pristine_ptr) if pristine_ptr else None,
                                                             count, stride, _ptr(bs), bs.shape[0] - 1))
        scene.dev.check("rtcgbNewBatchedFrame")

    def replay(self):
        self.L.rtcgbBatchedFrameReplay(self.h)
        self.scene.dev.check("rtcgbBatchedFrameReplay")
        return self.stats()

    def stats(self):
        s = RTCGBBatchedFrameStats()
        self.L.rtcgbGetBatchedFrameStats(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def release(self):
        if self.h:
            self.L.rtcgbReleaseBatchedFrame(self.h)
            self.h = None


class PathTracer:
    """Wavefront diffuse path tracer whose frames run as CUDA graphs."""

    def __init__(self, scene, width, height, bounces=4, eye=(0.5, -1.2, 0.5), look=(0.5, 0.5, 0.5), up=(0, 0, 1),
                 fov=50.0):
        self.scene = scene
        self.L = scene.L
        self.width, self.height = width, height
        cam = (ctypes.c_float * 10)(*eye, *look, *up, fov)
        self.h = ctypes.c_void_p(self.L.rtcgbNewPathTracer(scene.h, width, height, bounces, cam))
        scene.dev.check("rtcgbNewPathTracer")

    def animate_soup(self, geom_id, amplitude=0.002, seed=14):
        self.L.rtcgbPathTracerAnimateSoup(self.h, geom_id, amplitude, seed)
        self.scene.dev.check("rtcgbPathTracerAnimateSoup")

    def set_proposer(self, proposer):
        self.L.rtcgbPathTracerSetProposer(self.h, proposer.h if proposer is not None else None)
        self.scene.dev.check("rtcgbPathTracerSetProposer")

    def render(self, frame, learned=False):
        st = RTCGBFrameStats()
        self.L.rtcgbPathTracerRenderFrame(self.h, frame, 1 if learned else 0, ctypes.byref(st))
        self.scene.dev.check("rtcgbPathTracerRenderFrame")
        out = {f: getattr(st, f) for f, _ in st._fields_}
        out["rays_per_bounce"] = list(st.rays_per_bounce)
        return out

    def train_proposer(self, epochs=1, batch=16384, lr=5e-3):
        self.L.rtcgbPathTracerTrainProposer(self.h, epochs, batch, lr)
        self.scene.dev.check("rtcgbPathTracerTrainProposer")

    def image(self):
        img = np.zeros((self.height, self.width, 3), np.float32)
        self.L.rtcgbPathTracerGetImage(self.h, _ptr(img))
        self.scene.dev.check("rtcgbPathTracerGetImage")
        return img

    def release(self):
        if self.h:
            self.L.rtcgbReleasePathTracer(self.h)
            self.h = None
