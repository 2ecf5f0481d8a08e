"""Filter callbacks (rtcSetGeometryIntersectFilterFunction,
rtcSetGeometryOccludedFilterFunction, RTCIntersectContext::filter).

The reference offers every candidate hit to the callbacks inside its traversal
(kernels/geometry/intersector_epilog.h:237-276, 397-435) and keeps the nearest
accepted hit; an occlusion query stops at the first accepted one.  The oracle
restates that epilog; its result is pinned here against scenes in which the
rejected triangles are made degenerate (never hit).  The GPU library traces on
the device and calls the callbacks on the host between launches; its results
must equal the oracle's under the parity rules.
"""
import os

import numpy as np
import pytest

from rtcgb import rays as R

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
INVALID = 0xFFFFFFFF


def prim_rejected(p):
    """A quarter of the primitives, by a multiplicative hash of primID."""
    return ((int(p) * 2654435761) & 0xFFFFFFFF) >> 30 == 0


def cutout(g, p, u, v, t):
    """An alpha-cutout-like callback: rejects the hashed quarter of the
    primitives and every hit with u < 0.2 (depends on the hit, not only on the
    primitive)."""
    return not (prim_rejected(p) or u < 0.2)


def soup():
    d = np.load(os.path.join(GOLDEN, "soup_camera40_sphere.npz"))
    rays = d["rays"].view(R.RAYHIT_DTYPE).copy()
    shadow = d["shadow_rays"].view(R.RAY_DTYPE).copy()
    return d["verts"].copy(), d["idx"].copy(), rays, shadow


def degenerate(idx):
    """The index buffer with the rejected primitives collapsed to a point."""
    out = idx.copy()
    for p in range(idx.shape[0]):
        if prim_rejected(p):
            out[p] = 0
    return out


@pytest.mark.parametrize("robust", [False, True], ids=["moeller", "pluecker"])
def test_oracle_filter_equals_scene_without_rejected_triangles(oracle, robust):
    verts, idx, rays, shadow = soup()
    filt = oracle.OracleScene([(0, verts, idx)], robust=robust)
    filt.set_filters(intersect=lambda g, p, u, v, t: not prim_rejected(p),
                     occluded=lambda g, p, u, v, t: not prim_rejected(p))
    got = filt.intersect(rays.copy(), nthreads=4)
    sh = filt.occluded(shadow.copy(), nthreads=4)
    cut = oracle.OracleScene([(0, verts, degenerate(idx))], robust=robust)
    want = cut.intersect(rays.copy(), nthreads=4)
    sh_want = cut.occluded(shadow.copy(), nthreads=4)
    assert (got.view(np.uint8) == want.view(np.uint8)).all()
    assert np.array_equal(sh["tfar"] == -np.inf, sh_want["tfar"] == -np.inf)
    # the callback did remove hits
    plain = oracle.OracleScene([(0, verts, idx)], robust=robust).intersect(rays.copy(), nthreads=4)
    assert (plain["primID"] != got["primID"]).sum() > 100
    for s in (filt, cut):
        s.close()


def test_oracle_hit_dependent_filter(oracle):
    """With a callback that depends on u: every reported hit passes it, a ray
    whose unfiltered hit passes keeps that hit bit for bit, and the others end
    no nearer than their unfiltered hit."""
    verts, idx, rays, shadow = soup()
    plain = oracle.OracleScene([(0, verts, idx)])
    ref = plain.intersect(rays.copy(), nthreads=4)
    filt = oracle.OracleScene([(0, verts, idx)])
    filt.set_filters(intersect=cutout, occluded=cutout)
    got = filt.intersect(rays.copy(), nthreads=4)
    hit = got["geomID"] != INVALID
    assert hit.sum() > 500
    assert all(cutout(0, p, u, 0, 0) for p, u in zip(got["primID"][hit], got["u"][hit]))
    ref_hit = ref["geomID"] != INVALID
    keeps = ref_hit & np.array([cutout(0, p, u, 0, 0) for p, u in zip(ref["primID"], ref["u"])])
    assert (got[keeps].view(np.uint8) == ref[keeps].view(np.uint8)).all()
    moved = ref_hit & ~keeps & hit
    assert (got["tfar"][moved] >= ref["tfar"][moved]).all()
    # occlusion: never more occluded than without callbacks
    sh_plain = plain.occluded(shadow.copy(), nthreads=4)["tfar"] == -np.inf
    sh = filt.occluded(shadow.copy(), nthreads=4)["tfar"] == -np.inf
    assert not (sh & ~sh_plain).any() and (sh_plain & ~sh).any()
    plain.close()
    filt.close()


# ---------------------------------------------------------------- GPU path


def gpu_scene(rtc, device, verts, idx, flags=0):
    sc = rtc.Scene(device, flags=flags)
    gid = sc.add_mesh(verts, idx)
    return sc, gid


def counted(fn, calls):
    def f(g, p, u, v, t):
        calls.append((g, p))
        return fn(g, p, u, v, t)
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("robust", [False, True], ids=["moeller", "pluecker"])
def test_gpu_geometry_filters_match_oracle(rtc, device, oracle, robust):
    from parity import assert_clean, compare_closest
    verts, idx, rays, shadow = soup()
    sc, gid = gpu_scene(rtc, device, verts, idx, flags=rtc.RTC_SCENE_FLAG_ROBUST if robust else 0)
    calls_i, calls_o = [], []
    sc.set_filters(gid, intersect=counted(cutout, calls_i), occluded=counted(cutout, calls_o))
    sc.commit()
    got = sc.intersect(rays.copy())
    orc = oracle.OracleScene([(0, verts, idx)], robust=robust)
    orc.set_filters(intersect=cutout, occluded=cutout)
    ref = orc.intersect(rays.copy(), nthreads=4)
    rep = compare_closest(orc, rays, got, ref)
    assert_clean(rep)
    assert rep["id_mismatch"] <= 5
    hit = got["geomID"] != INVALID
    assert all(cutout(0, p, u, 0, 0) for p, u in zip(got["primID"][hit], got["u"][hit]))
    assert len(calls_i) >= int(hit.sum())   # every accepted hit went through the callback
    sh = sc.occluded(shadow.copy())
    sh_ref = orc.occluded(shadow.copy(), nthreads=4)
    assert np.array_equal(sh["tfar"] == -np.inf, sh_ref["tfar"] == -np.inf)
    assert len(calls_o) >= int((sh["tfar"] == -np.inf).sum())
    orc.close()
    sc.release()


@pytest.mark.gpu
def test_gpu_context_filter(rtc, device, oracle):
    """RTCIntersectContext::filter is called when the scene has
    RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION, and ignored without it (the
    reference selects its filtering intersectors at commit)."""
    from parity import assert_clean, compare_closest
    verts, idx, rays, shadow = soup()
    orc = oracle.OracleScene([(0, verts, idx)])
    plain_ref = orc.intersect(rays.copy(), nthreads=4)
    orc.set_filters(intersect=cutout, occluded=cutout)
    ref = orc.intersect(rays.copy(), nthreads=4)
    sh_ref = orc.occluded(shadow.copy(), nthreads=4)
    sc, _ = gpu_scene(rtc, device, verts, idx, flags=rtc.RTC_SCENE_FLAG_CONTEXT_FILTER_FUNCTION)
    sc.commit()
    got = sc.intersect(rays.copy(), context_filter=cutout)
    rep = compare_closest(orc, rays, got, ref)
    assert_clean(rep)
    sh = sc.occluded(shadow.copy(), context_filter=cutout)
    assert np.array_equal(sh["tfar"] == -np.inf, sh_ref["tfar"] == -np.inf)
    sc.release()
    # without the flag the context's callback is not called
    sc2, _ = gpu_scene(rtc, device, verts, idx)
    sc2.commit()
    calls = []
    got2 = sc2.intersect(rays.copy(), context_filter=counted(cutout, calls))
    assert calls == []
    assert np.array_equal(got2["primID"], plain_ref["primID"])
    sc2.release()
    orc.close()


@pytest.mark.gpu
def test_gpu_filter_on_one_geometry_only(rtc, device, oracle):
    """Hits on a geometry without a callback are kept without a call; the
    other geometry's callback rejects everything, so its triangles are never
    reported."""
    verts, idx, rays, _ = soup()
    half = idx.shape[0] // 2
    a_idx, b_idx = idx[:half], idx[half:]
    sc = rtc.Scene(device)
    ga = sc.add_mesh(verts, a_idx)
    gb = sc.add_mesh(verts, b_idx)
    calls = []
    sc.set_filters(gb, intersect=counted(lambda g, p, u, v, t: False, calls))
    sc.commit()
    got = sc.intersect(rays.copy())
    orc = oracle.OracleScene([(0, verts, a_idx)])   # geometry b removed
    ref = orc.intersect(rays.copy(), nthreads=4)
    assert (got["geomID"][got["geomID"] != INVALID] == ga).all()
    assert np.array_equal(got["primID"], ref["primID"])
    same = got["geomID"] != INVALID
    assert np.array_equal(got["tfar"][same].view(np.uint32), ref["tfar"][same].view(np.uint32))
    assert calls and all(g == gb for g, _ in calls)
    orc.close()
    sc.release()


@pytest.mark.gpu
def test_gpu_filter_device_rays_and_reject_all(rtc, device):
    import torch
    verts, idx, rays, _ = soup()
    sc, gid = gpu_scene(rtc, device, verts, idx)
    sc.set_filters(gid, intersect=cutout)
    sc.commit()
    host = sc.intersect(rays.copy())
    dev_rays = torch.from_numpy(rays.copy().view(np.uint8)).cuda()
    sc.intersect_ptr(dev_rays.data_ptr(), rays.shape[0])
    torch.cuda.synchronize()
    assert (dev_rays.cpu().numpy() == host.view(np.uint8)).all()
    sc.release()
    # a callback that rejects every hit: nothing is reported, records untouched
    sc, gid = gpu_scene(rtc, device, verts, idx)
    sc.set_filters(gid, intersect=lambda g, p, u, v, t: False)
    sc.commit()
    got = sc.intersect(rays[:400].copy())
    assert (got.view(np.uint8) == rays[:400].view(np.uint8)).all()
    sc.release()
