"""rtcgbIntersect1MNoAlloc: the closest-hit query for callers that must not
allocate device memory while querying (a process whose memory its own
allocator already holds, a real-time loop that cannot absorb cudaMalloc's
implicit synchronisation, a service held to a fixed memory budget).

It is checked against rtcIntersect1M on the same rays, bit for bit, on two
calls in a row (the shared static scratch keeps the previous call's contents,
so the second call proves the state is cleared), for host rays staged through
the 32 MiB static area and for rays already in device memory, on plain and
robust scenes, with 16-byte aligned (80 B) and unaligned (84 B) record strides;
device memory use must not change across calls, including the very first call
of a fresh process; host rays beyond the staging area are rejected, and so are
scenes the call does not trace (filter callbacks, instances, batched scenes).
This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu

STAGING = 32 << 20
RTC_ERROR_INVALID_ARGUMENT = 2
RTC_ERROR_INVALID_OPERATION = 3
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _noalloc(L, scene, ptr, n, stride=80):
    L.rtcgbIntersect1MNoAlloc(scene.h, ctypes.c_void_p(ptr), n, stride, None)


def _strided(rays, stride):
    """The records of `rays` at byte stride `stride` (>= 80) in one uint8 buffer."""
    buf = np.zeros(rays.shape[0] * stride, np.uint8)
    buf.reshape(-1, stride)[:, :80] = rays.view(np.uint8).reshape(-1, 80)
    return buf


def _records(buf, stride):
    return np.ascontiguousarray(buf.reshape(-1, stride)[:, :80]).view(R.RAYHIT_DTYPE).reshape(-1)


@pytest.mark.parametrize("robust", [False, True], ids=["plain", "robust"])
@pytest.mark.parametrize("stride", [80, 84])
def test_no_alloc_matches_rtcIntersect1M(rtc, device, robust, stride):
    L = rtc.load()
    verts, idx = W.gaussian_soup(200_000, seed=31)
    rays = W.sphere_rays(300_000, seed=32)          # 24-25 MB of records: fits the staging area
    assert rays.shape[0] * stride <= STAGING
    sc = rtc.Scene(device, flags=rtc.RTC_SCENE_FLAG_ROBUST if robust else 0)
    sc.add_mesh(verts, idx)
    sc.commit()
    ref = rays.copy()
    sc.intersect(ref)                               # the existing entry point
    assert np.mean(ref["geomID"] != 0xFFFFFFFF) > 0.05

    # host rays, two calls in a row
    for _ in range(2):
        buf = _strided(rays, stride)
        _noalloc(L, sc, buf.ctypes.data, rays.shape[0], stride)
        device.check("rtcgbIntersect1MNoAlloc")
        assert (_records(buf, stride).view(np.uint8) == ref.view(np.uint8)).all()

    # device-resident rays (any size), two calls in a row, no device memory change
    torch = pytest.importorskip("torch")
    big = W.sphere_rays(1_000_000, seed=33)         # 80 MB: beyond the staging area, fine in device memory
    big_ref = big.copy()
    sc.intersect(big_ref)
    pristine = torch.from_numpy(_strided(big, stride)).cuda()
    work = torch.empty_like(pristine)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        work.copy_(pristine)
        torch.cuda.synchronize()
        _noalloc(L, sc, work.data_ptr(), big.shape[0], stride)
        device.check("rtcgbIntersect1MNoAlloc")
        got = _records(work.cpu().numpy(), stride)
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
    assert device.error() == RTC_ERROR_INVALID_ARGUMENT
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


def _refused(rtc, device, sc):
    L = rtc.load()
    rays = W.sphere_rays(1000, seed=35)
    before = rays.copy()
    _noalloc(L, sc, rays.ctypes.data, rays.shape[0])
    assert device.error() == RTC_ERROR_INVALID_OPERATION
    assert (rays.view(np.uint8) == before.view(np.uint8)).all()


def test_no_alloc_refuses_scenes_it_does_not_trace(rtc, device):
    """Filter callbacks, instances and batched scenes need more than the plain
    traversal; the call refuses them (RTC_ERROR_INVALID_OPERATION, rays untouched)
    instead of tracing them as plain triangle scenes."""
    verts, idx = W.gaussian_soup(20_000, seed=34)
    filt = rtc.Scene(device)
    gid = filt.add_mesh(verts, idx)
    filt.set_filters(gid, intersect=lambda g, p, u, v, t: p % 2 == 0)
    filt.commit()
    _refused(rtc, device, filt)
    child = rtc.Scene(device)
    child.add_mesh(verts, idx)
    child.commit()
    top = rtc.Scene(device)
    top.add_instance(child, np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.1, 0.2, 0.3], np.float32))
    top.commit()
    _refused(rtc, device, top)
    batched = rtc.Scene(device)
    batched.set_batched()
    batched.add_mesh(verts, idx)
    batched.add_mesh(*W.heightfield(16))
    batched.commit()
    _refused(rtc, device, batched)
    for s in (filt, top, child, batched):
        s.release()


FIRST_CALL = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, {pkg!r})
    from rtcgb import api, workloads as W
    dev = api.Device(b"")
    sc = api.Scene(dev)
    sc.add_mesh(*W.gaussian_soup(50_000, seed=36))
    sc.commit()
    rays = W.sphere_rays(200_000, seed=37)
    work = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    # the first query of this process
    api.load().rtcgbIntersect1MNoAlloc(sc.h, ctypes.c_void_p(work.data_ptr()), rays.shape[0], 80, None)
    dev.check("rtcgbIntersect1MNoAlloc")
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    ref = rays.copy()
    sc.intersect(ref)
    same = bool((work.cpu().numpy() == ref.view(np.uint8)).all())
    print("RESULT", free_before, free_after, same)
""")


def test_no_alloc_first_call_of_a_process_takes_no_memory():
    """In a fresh process whose first query is this call, free device memory is the
    same before and after it: the scratch and the kernels were loaded with the device."""
    pytest.importorskip("torch")
    code = FIRST_CALL.format(pkg=os.path.join(REPO, "embree-aarch64_gb300"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("RESULT")][-1].split()
    assert int(line[1]) == int(line[2]), line
    assert line[3] == "True"
