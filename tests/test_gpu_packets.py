"""Packet and SOA query entry points (rtcIntersect4/8/16, rtcOccluded4/8/16,
rtcIntersectNM/Np, rtcOccludedNM/Np) against the AOS stream path.

Lane semantics follow kernels/common/rtcore.cpp:498-590, 657-750, 749-960: packets
trace lanes with valid[i] == -1 and tnear <= tfar, NM streams with N == 1 are AOS
streams, Np streams may leave tnear/time/mask/id/flags/Ng/instID null; a lane that
misses (or is not occluded) is left untouched."""
import ctypes

import numpy as np
import pytest

from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu

E_NONE = 0


@pytest.fixture(scope="module")
def soup_scene(rtc, device):
    sc = rtc.Scene(device)
    sc.add_mesh(*W.heightfield(64))
    sc.add_mesh(*W.gaussian_soup(30000, seed=21))
    sc.commit()
    return sc


def _rays(n, seed):
    r = W.sphere_rays(n, seed=seed)
    rng = np.random.default_rng(seed)
    # a few lanes that must not be traced: tnear > tfar
    bad = rng.random(n) < 0.05
    r["tnear"][bad] = 2.0
    r["tfar"][bad] = 1.0
    # some lanes miss because their interval is short
    short = rng.random(n) < 0.1
    r["tfar"][short] = 1e-3
    return r


def _expected(sc, rays, active, anyhit):
    ref = rays.copy()
    sub = ref[active].copy()
    if anyhit:
        sc.occluded(sub)
    else:
        sc.intersect(sub)
    ref[active] = sub
    return ref


def _as_rays(rh):
    r = np.zeros(rh.shape[0], R.RAY_DTYPE)
    for name in R.RAY_DTYPE.names:
        r[name] = rh[name]
    return r


@pytest.mark.parametrize("K", [4, 8, 16])
@pytest.mark.parametrize("anyhit", [False, True])
def test_packets(rtc, device, soup_scene, K, anyhit):
    L = rtc.load()
    n = 64 * K
    rh = _rays(n, seed=K)
    rays = _as_rays(rh) if anyhit else rh
    rng = np.random.default_rng(100 + K)
    # valid masks: -1 active; 0 and other non -1 values inactive
    valid = np.where(rng.random(n) < 0.7, -1, rng.choice([0, 1, 7], n)).astype(np.int32)
    expected = _expected(soup_scene, rays, valid == -1, anyhit)
    packets = R.to_soa(rays, K)
    fn = {(4, False): L.rtcIntersect4, (8, False): L.rtcIntersect8, (16, False): L.rtcIntersect16,
          (4, True): L.rtcOccluded4, (8, True): L.rtcOccluded8, (16, True): L.rtcOccluded16}[(K, anyhit)]
    for p in range(packets.shape[0]):
        v = np.ascontiguousarray(valid[p * K:(p + 1) * K])
        pk = np.ascontiguousarray(packets[p])
        fn(v.ctypes.data, soup_scene.h, None, pk.ctypes.data)
        assert device.error() == E_NONE
        packets[p] = pk
    got = R.from_soa(packets, K, n, rays.dtype)
    assert (got.view(np.uint8) == expected.view(np.uint8)).all()
    if not anyhit:
        assert (got["geomID"][valid == -1] != R.RTC_INVALID_GEOMETRY_ID).sum() > n // 20


@pytest.mark.parametrize("N,pad_words", [(1, 0), (1, 4), (3, 0), (5, 7), (32, 0)])
@pytest.mark.parametrize("anyhit", [False, True])
def test_nm_streams(rtc, device, soup_scene, N, pad_words, anyhit):
    """M packets of N SOA rays, byteStride apart (N == 1: AOS records, any stride)."""
    L = rtc.load()
    n = 1000 if N > 1 else 777
    rh = _rays(n, seed=N + pad_words)
    rays = _as_rays(rh) if anyhit else rh
    expected = _expected(soup_scene, rays, np.ones(n, bool), anyhit)
    nf = rays.dtype.itemsize // 4
    packets = R.to_soa(rays, N, stride_words=nf * N + pad_words)
    M = packets.shape[0]
    fn = L.rtcOccludedNM if anyhit else L.rtcIntersectNM
    fn(soup_scene.h, None, packets.ctypes.data, N, M, packets.shape[1] * 4)
    assert device.error() == E_NONE
    lanes = M * N
    got = R.from_soa(packets, N, lanes, rays.dtype)[:n]
    assert (got.view(np.uint8) == expected.view(np.uint8)).all()
    # padding lanes of the last packet (all-zero rays: tnear 0 <= tfar 0) are traced but
    # have an empty interval, so nothing is written
    assert (R.from_soa(packets, N, lanes, rays.dtype)[n:].view(np.uint8) == 0).all()


class _RayNp(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f in ("org_x", "org_y", "org_z", "tnear", "dir_x", "dir_y", "dir_z",
                                                "time", "tfar", "mask", "id", "flags")]


class _HitNp(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f in ("Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID0")]


class _RayHitNp(ctypes.Structure):
    _fields_ = [("ray", _RayNp), ("hit", _HitNp)]


@pytest.mark.parametrize("optional", [True, False])
@pytest.mark.parametrize("anyhit", [False, True])
def test_np_streams(rtc, device, soup_scene, optional, anyhit):
    """Pointer-SOA streams; optional=False leaves tnear/time/mask/id/flags/Ng/instID null."""
    L = rtc.load()
    n = 2500
    rh = _rays(n, seed=33)
    if not optional:
        rh["tnear"] = 0.0  # a null tnear array reads as 0
    rays = _as_rays(rh) if anyhit else rh
    expected = _expected(soup_scene, rays, np.ones(n, bool), anyhit)
    cols = {name: np.ascontiguousarray(rays[name]) for name in rays.dtype.names}
    ray = _RayNp()
    for f, _ in _RayNp._fields_:
        setattr(ray, f, cols[f].ctypes.data)
    if not optional:
        for f in ("tnear", "time", "mask", "id", "flags"):
            setattr(ray, f, None)
    if anyhit:
        L.rtcOccludedNp(soup_scene.h, None, ctypes.byref(ray), n)
    else:
        hit = _HitNp()
        for f, _ in _HitNp._fields_:
            setattr(hit, f, cols["instID" if f == "instID0" else f].ctypes.data)
        if not optional:
            for f in ("Ng_x", "Ng_y", "Ng_z", "instID0"):
                setattr(hit, f, None)
        rhn = _RayHitNp(ray, hit)
        L.rtcIntersectNp(soup_scene.h, None, ctypes.byref(rhn), n)
    assert device.error() == E_NONE
    written = ("tfar",) if anyhit else ("tfar", "u", "v", "primID", "geomID") + (
        ("Ng_x", "Ng_y", "Ng_z", "instID") if optional else ())
    for name in rays.dtype.names:
        want = expected[name] if name in written else rays[name]
        assert (cols[name].view(np.uint32) == want.view(np.uint32)).all(), name


def test_packet_argument_errors(rtc, device, soup_scene):
    L = rtc.load()
    rays = R.to_soa(_rays(4, seed=1), 4)
    L.rtcIntersect4(None, soup_scene.h, None, rays.ctypes.data)
    assert device.error() == 2
    v = np.full(4, -1, np.int32)
    L.rtcIntersect4(v.ctypes.data, soup_scene.h, None, None)
    assert device.error() == 2
    # a byteStride smaller than one packet of N rays
    pk = R.to_soa(_rays(12, seed=2), 3)
    L.rtcIntersectNM(soup_scene.h, None, pk.ctypes.data, 3, pk.shape[0], 16)
    assert device.error() == 2
    L.rtcIntersectNp(soup_scene.h, None, None, 10)
    assert device.error() == 2
    # empty streams are no-ops
    L.rtcIntersectNM(soup_scene.h, None, pk.ctypes.data, 3, 0, 240)
    L.rtcIntersectNp(soup_scene.h, None, ctypes.byref(_RayHitNp()), 0)
    assert device.error() == E_NONE
