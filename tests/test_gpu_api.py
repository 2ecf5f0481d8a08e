"""API semantics of the C ABI on a GPU: error codes and callbacks, handle
ownership, geometry IDs, device properties, host-side fault injection
(memory-monitor veto, progress-monitor cancel) and concurrent queries."""
import ctypes
import threading

import numpy as np
import pytest

from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu

E_NONE, E_UNKNOWN, E_ARG, E_OP, E_OOM, E_CANCEL = 0, 1, 2, 3, 4, 6


def tri_geom(L, dev, verts, idx):
    g = L.rtcNewGeometry(dev.h, 0)
    L.rtcSetSharedGeometryBuffer(g, 1, 0, 0x9003, verts.ctypes.data, 0, 12, verts.shape[0])
    L.rtcSetSharedGeometryBuffer(g, 0, 0, 0x5003, idx.ctypes.data, 0, 12, idx.shape[0])
    L.rtcCommitGeometry(g)
    return g


def test_device_properties(rtc, device):
    L = rtc.load()
    assert L.rtcGetDeviceProperty(device.h, 0) == 31201
    assert L.rtcGetDeviceProperty(device.h, 35) == 1   # RAY_STREAM_SUPPORTED
    assert L.rtcGetDeviceProperty(device.h, 96) == 1   # TRIANGLE_GEOMETRY_SUPPORTED
    assert L.rtcGetDeviceProperty(device.h, 97) == 0
    assert device.error() == E_NONE
    L.rtcGetDeviceProperty(device.h, 12345)
    assert device.error() == E_ARG
    assert device.error() == E_NONE  # read-and-clear


def test_error_callback_and_null_handles(rtc, device):
    L = rtc.load()
    seen = []
    cb = rtc.ERROR_FN(lambda user, code, msg: seen.append((code, msg)))
    L.rtcSetDeviceErrorFunction(device.h, cb, None)
    L.rtcNewGeometry(device.h, 1)  # QUAD: not supported
    assert device.error() == E_UNKNOWN
    assert seen and seen[-1][0] == E_UNKNOWN
    L.rtcSetDeviceErrorFunction(device.h, rtc.ERROR_FN(), None)  # NULL callback
    L.rtcCommitScene(None)
    assert L.rtcGetDeviceError(None) == E_ARG


def test_query_on_uncommitted_scene(rtc, device):
    L = rtc.load()
    s = L.rtcNewScene(device.h)
    rays = W.sphere_rays(4)
    L.rtcIntersect1M(s, None, rays.ctypes.data, 4, 80)
    assert device.error() == E_OP
    L.rtcReleaseScene(s)


def test_buffer_alignment_rules(rtc, device):
    """BufferStrideTest (verify.cpp:922-1021) for triangle meshes."""
    L = rtc.load()
    g = L.rtcNewGeometry(device.h, 0)
    ib = np.zeros(8 + 16 * 6 * 4, np.uint8)
    vb = np.zeros(12 + 16 * 9 * 4 + 4, np.uint8)
    L.rtcSetSharedGeometryBuffer(g, 0, 0, 0x5003, ib.ctypes.data, 1, 12, 16)
    assert device.error() == E_OP
    L.rtcSetSharedGeometryBuffer(g, 1, 0, 0x9003, vb.ctypes.data, 1, 12, 16)
    assert device.error() == E_OP
    L.rtcSetSharedGeometryBuffer(g, 0, 0, 0x5003, ib.ctypes.data, 0, 15, 16)
    assert device.error() == E_OP
    L.rtcSetSharedGeometryBuffer(g, 1, 0, 0x9003, vb.ctypes.data, 0, 15, 16)
    assert device.error() == E_OP
    for off, stride, buf, t, f in ((0, 12, ib, 0, 0x5003), (0, 12, vb, 1, 0x9003), (8, 24, ib, 0, 0x5003),
                                   (12, 36, vb, 1, 0x9003), (0, 16, vb, 1, 0x9003)):
        L.rtcSetSharedGeometryBuffer(g, t, 0, f, buf.ctypes.data, off, stride, 16)
        assert device.error() == E_NONE
    L.rtcSetSharedGeometryBuffer(g, 0, 0, 0x9003, ib.ctypes.data, 0, 12, 16)  # wrong index format
    assert device.error() == E_OP
    L.rtcSetSharedGeometryBuffer(g, 0, 1, 0x5003, ib.ctypes.data, 0, 12, 16)  # index slot 1
    assert device.error() == E_ARG
    # filter callbacks: triangle meshes take them, instances do not (geometry.cpp:136-150)
    L.rtcSetGeometryIntersectFilterFunction(g, ctypes.c_void_p(1))
    assert device.error() == E_NONE
    L.rtcSetGeometryIntersectFilterFunction(g, None)
    assert device.error() == E_NONE
    gi = L.rtcNewGeometry(device.h, rtc.RTC_GEOMETRY_TYPE_INSTANCE)
    L.rtcSetGeometryOccludedFilterFunction(gi, ctypes.c_void_p(1))
    assert device.error() == E_OP
    L.rtcReleaseGeometry(gi)
    assert L.rtcGetDeviceProperty(device.h, 66) == 1   # RTC_DEVICE_PROPERTY_FILTER_FUNCTION_SUPPORTED
    L.rtcReleaseGeometry(g)
    assert device.error() == E_NONE


def test_geometry_ids_and_ownership(rtc, device):
    L = rtc.load()
    verts, idx = W.heightfield(4)
    s = L.rtcNewScene(device.h)
    ids = []
    for _ in range(3):
        g = tri_geom(L, device, verts, idx)
        ids.append(L.rtcAttachGeometry(s, g))
        L.rtcReleaseGeometry(g)  # the scene keeps its own reference
    assert ids == [0, 1, 2]
    L.rtcDetachGeometry(s, 1)
    g = tri_geom(L, device, verts, idx)
    assert L.rtcAttachGeometry(s, g) == 1  # smallest free ID is reused
    L.rtcAttachGeometryByID(s, g, 2)       # taken
    assert device.error() == E_ARG
    L.rtcAttachGeometryByID(s, g, 10)
    assert device.error() == E_NONE
    L.rtcReleaseGeometry(g)
    assert L.rtcGetGeometry(s, 10) is not None and L.rtcGetGeometry(s, 5) is None
    L.rtcCommitScene(s)
    assert device.error() == E_NONE
    b = rtc.RTCBounds()
    L.rtcGetSceneBounds(s, ctypes.byref(b))
    assert (b.lower_x, b.lower_y, b.upper_x, b.upper_y) == (0.0, 0.0, 1.0, 1.0)
    L.rtcReleaseScene(s)
    assert device.error() == E_NONE


def test_memory_monitor_veto_is_out_of_memory(rtc):
    """Host-side fault injection: the memory monitor refuses the build's
    allocation, rtcCommitScene reports RTC_ERROR_OUT_OF_MEMORY and the scene
    stays uncommitted (device.cpp:318-328)."""
    dev = rtc.Device(b"")
    L = dev.L
    calls = []

    def monitor(user, nbytes, post):
        calls.append(nbytes)
        return False

    cb = rtc.MEMORY_FN(monitor)
    L.rtcSetDeviceMemoryMonitorFunction(dev.h, cb, None)
    verts, idx = W.heightfield(8)
    s = L.rtcNewScene(dev.h)
    g = tri_geom(L, dev, verts, idx)
    L.rtcAttachGeometry(s, g)
    L.rtcReleaseGeometry(g)
    L.rtcCommitScene(s)
    assert dev.error() == E_OOM and calls
    rays = W.sphere_rays(4)
    L.rtcIntersect1M(s, None, rays.ctypes.data, 4, 80)
    assert dev.error() == E_OP
    L.rtcReleaseScene(s)
    dev.release()


def test_progress_monitor_cancel(rtc, device):
    L = rtc.load()
    cb = rtc.PROGRESS_FN(lambda ptr, n: False)
    verts, idx = W.heightfield(8)
    s = L.rtcNewScene(device.h)
    g = tri_geom(L, device, verts, idx)
    L.rtcAttachGeometry(s, g)
    L.rtcReleaseGeometry(g)
    L.rtcSetSceneProgressMonitorFunction(s, cb, None)
    L.rtcCommitScene(s)
    assert device.error() == E_CANCEL
    ok_cb = rtc.PROGRESS_FN(lambda ptr, n: True)  # must outlive the commit below
    L.rtcSetSceneProgressMonitorFunction(s, ok_cb, None)
    L.rtcCommitScene(s)
    assert device.error() == E_NONE
    L.rtcReleaseScene(s)


def test_concurrent_queries_from_host_threads(rtc, device):
    """rtcIntersect1M is re-entrant: host threads tracing disjoint slices give
    the same bytes as one call (each thread uses its own CUDA stream)."""
    verts, idx = W.gaussian_soup(100_000, seed=4)
    rays = W.sphere_rays(200_000, seed=8)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    ref = rays.copy()
    sc.intersect(ref)
    work = rays.copy()
    chunks = np.array_split(np.arange(work.shape[0]), 8)
    errors = []

    def run(ix):
        try:
            sub = work[ix[0]:ix[-1] + 1]
            sc.intersect_ptr(sub.ctypes.data, sub.shape[0], 80)
        except Exception as e:  # pragma: no cover
            errors.append(e)

    th = [threading.Thread(target=run, args=(c,)) for c in chunks]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors
    assert (work.view(np.uint8) == ref.view(np.uint8)).all()


def test_pointer_stream_entry_points(rtc, device):
    """rtcIntersect1Mp / rtcOccluded1Mp (arrays of record pointers)."""
    L = rtc.load()
    verts, idx = W.gaussian_soup(20000, seed=6)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    rays = W.sphere_rays(3000, seed=1)
    ref = rays.copy()
    sc.intersect(ref)
    work = rays.copy()
    ptrs = (ctypes.c_void_p * rays.shape[0])(*[work.ctypes.data + 80 * i for i in range(rays.shape[0])][::-1])
    L.rtcIntersect1Mp(sc.h, None, ptrs, rays.shape[0])
    assert device.error() == E_NONE
    assert (work.view(np.uint8) == ref.view(np.uint8)).all()


def test_launch_counter_and_query_stats(rtc, device):
    verts, idx = W.heightfield(32)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    before = rtc.launch_count()
    sc.commit()
    mid = rtc.launch_count()
    assert mid - before >= 5
    rtc.set_counting(True)
    rays = W.camera_rays(64, 64)
    sc.intersect(rays)
    rtc.set_counting(False)
    st = rtc.last_query_stats()
    assert rtc.launch_count() >= mid + 1
    assert st["rays"] == rays.shape[0] and st["nodes"] > 0 and st["tris"] > 0
    # pageable host rays are read in place where the device can address pageable
    # host memory (48 B of ray record per ray), otherwise copied whole
    direct = rtc.load().rtcgbGetDeviceHostAccess(device.h) & 1
    assert st["h2d_bytes"] == (rays.shape[0] * 48 if direct else rays.nbytes) and st["kernel_ms"] > 0
