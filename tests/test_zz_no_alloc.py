"""rtcgbIntersect1MNoAlloc: the closest-hit query for callers that must not
allocate device memory while querying (a process whose memory its own
allocator already holds, a real-time loop that cannot absorb cudaMalloc's
implicit synchronisation, a service held to a fixed memory budget).

It is checked against rtcIntersect1M on the same rays, bit for bit, on two
calls in a row (the shared static scratch keeps the previous call's contents,
so the second call proves the state is cleared), for host rays staged through
the 32 MiB static area and for rays already in device memory; device memory
use must not change across calls; host rays beyond the staging area are
rejected.  This file is collected last so that a run stopping at its first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from rtcgb import workloads as W

pytestmark = pytest.mark.gpu

STAGING = 32 << 20


def _noalloc(L, scene, ptr, n, stride=80):
    L.rtcgbIntersect1MNoAlloc(scene.h, ctypes.c_void_p(ptr), n, stride, None)


def test_no_alloc_matches_rtcIntersect1M(rtc, device):
    L = rtc.load()
    verts, idx = W.gaussian_soup(200_000, seed=31)
    rays = W.sphere_rays(300_000, seed=32)          # 24 MB of records: fits the staging area
    assert rays.nbytes <= STAGING
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    ref = rays.copy()
    sc.intersect(ref)                               # the existing entry point
    assert np.mean(ref["geomID"] != 0xFFFFFFFF) > 0.05

    # host rays, two calls in a row
    for _ in range(2):
        got = rays.copy()
        _noalloc(L, sc, got.ctypes.data, got.shape[0])
        device.check("rtcgbIntersect1MNoAlloc")
        assert (got.view(np.uint8) == ref.view(np.uint8)).all()

    # device-resident rays (any size), two calls in a row, no device memory change
    torch = pytest.importorskip("torch")
    big = W.sphere_rays(1_000_000, seed=33)         # 80 MB: beyond the staging area, fine in device memory
    big_ref = big.copy()
    sc.intersect(big_ref)
    pristine = torch.from_numpy(big.view(np.uint8).copy()).cuda()
    work = torch.empty_like(pristine)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        work.copy_(pristine)
        torch.cuda.synchronize()
        _noalloc(L, sc, work.data_ptr(), big.shape[0])
        device.check("rtcgbIntersect1MNoAlloc")
        got = work.cpu().numpy().view(big_ref.dtype)
        assert (got.view(np.uint8) == big_ref.view(np.uint8)).all()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    sc.release()


def test_no_alloc_rejects_host_rays_beyond_staging(rtc, device):
    L = rtc.load()
    verts, idx = W.heightfield(32)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    rays = W.camera_rays(640, 660)                  # 422,400 records = 33.8 MB > 32 MiB
    assert rays.nbytes > STAGING
    before = rays.copy()
    _noalloc(L, sc, rays.ctypes.data, rays.shape[0])
    assert device.error() == 2                      # RTC_ERROR_INVALID_ARGUMENT
    assert (rays.view(np.uint8) == before.view(np.uint8)).all()
    # the same rays in slices that fit are traced, matching rtcIntersect1M
    ref = before.copy()
    sc.intersect(ref)
    half = rays.shape[0] // 2
    for part in (rays[:half], rays[half:]):
        _noalloc(L, sc, part.ctypes.data, part.shape[0])
        device.check("rtcgbIntersect1MNoAlloc")
    assert (rays.view(np.uint8) == ref.view(np.uint8)).all()
    sc.release()
