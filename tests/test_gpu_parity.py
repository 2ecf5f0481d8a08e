"""GPU library vs the CPU oracle, through the C ABI (rtcCommitScene,
rtcIntersect1M, rtcOccluded1M).  Small and medium cases are compared ray by
ray; the full-size soup is compared on a seeded sample plus size-independent
properties of every hit."""
import numpy as np
import pytest

from parity import assert_clean, compare_closest, compare_occluded
from rtcgb import rays as R
from rtcgb import workloads as W
from test_oracle import _single_triangle_rays, check_triangle_hit

pytestmark = pytest.mark.gpu


def gpu_scene(rtc, device, meshes):
    sc = rtc.Scene(device)
    for gid, v, i in meshes:
        sc.add_mesh(v, i, gid)
    sc.commit()
    return sc


def run_pair(rtc, device, oracle, meshes, rays, nthreads=0):
    sg = gpu_scene(rtc, device, meshes)
    so = oracle.OracleScene(meshes)
    g, r = rays.copy(), rays.copy()
    sg.intersect(g)
    so.intersect(r, nthreads=nthreads)
    return sg, so, g, r


def test_triangle_hit_known_answer(rtc, device):
    verts, idx, rays, u, v = _single_triangle_rays()
    sc = gpu_scene(rtc, device, [(0, verts, idx)])
    sc.intersect(rays)
    check_triangle_hit(rays, u, v, verts)


def test_triangle_hit_single_ray_entry(rtc, device):
    import ctypes
    verts, idx, rays, u, v = _single_triangle_rays(8)
    sc = gpu_scene(rtc, device, [(0, verts, idx)])
    ctx = rtc.RTCIntersectContext(0, None, (ctypes.c_uint * 1)(0xFFFFFFFF))
    for k in range(8):
        one = rays[k:k + 1].copy()
        rtc.load().rtcIntersect1(sc.h, ctypes.byref(ctx), ctypes.c_void_p(one.ctypes.data))
        device.check("rtcIntersect1")
        rays[k] = one[0]
    check_triangle_hit(rays, u, v, verts)


def test_triangle_occluded_known_answer(rtc, device):
    verts, idx, rays, _, _ = _single_triangle_rays()
    sc = gpu_scene(rtc, device, [(0, verts, idx)])
    r = np.ascontiguousarray(rays)
    sc.occluded(r, stride=80)
    assert np.all(r["tfar"] == -np.inf)
    shadow = np.zeros(256, R.RAY_DTYPE)
    for n in R.RAY_DTYPE.names:
        shadow[n] = rays[n]
    shadow["tfar"] = 1.0
    sc.occluded(shadow)
    assert np.all(shadow["tfar"] == -np.inf)


def test_inactive_and_empty(rtc, device, oracle):
    verts, idx = W.triangle_sphere((0, 0, 0), 2.0, 50)
    sc = gpu_scene(rtc, device, [(0, verts, idx)])
    rng = np.random.default_rng(3)
    n = 4000
    rays = R.make_rayhits(2 * rng.random((n, 3)) - 1, 2 * rng.random((n, 3)) - 1)
    inactive = rng.random(n) < 0.5
    rays["tnear"][inactive] = np.inf
    rays["tfar"][inactive] = 0.0
    before = rays.copy()
    sc.intersect(rays)
    assert (rays[inactive].view(np.uint8) == before[inactive].view(np.uint8)).all()
    assert np.all(rays["geomID"][~inactive] == 0)
    empty = gpu_scene(rtc, device, [])
    r2 = W.sphere_rays(1000)
    b2 = r2.copy()
    empty.intersect(r2)
    assert (r2.view(np.uint8) == b2.view(np.uint8)).all()
    lo, hi = empty.bounds()
    assert np.all(lo == np.inf) and np.all(hi == -np.inf)


@pytest.mark.parametrize("model", ["sphere", "plane"])
def test_watertight(rtc, device, model):
    """WatertightTest (verify.cpp:2898-2979) on the GPU: miss rate <= 2e-5."""
    rng = np.random.default_rng(11)
    n = 200000
    if model == "sphere":
        verts, idx = W.triangle_sphere((0, 0, 0), 2.0, 500)
        org = 2 * rng.random((n, 3), dtype=np.float32) - 1
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
    else:
        verts, idx = W.triangle_plane((0, -6, -6), (0, 0, 12), (0, 12, 0), 500, 500)
        org = np.broadcast_to(np.array([-3, 0, 0], np.float32), (n, 3))
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
        d[:, 0] = 1.0
    sc = gpu_scene(rtc, device, [(0, verts, idx)])
    rays = R.make_rayhits(org, d)
    sc.intersect(rays)
    assert np.mean(rays["geomID"] == 0xFFFFFFFF) <= 2e-5


def test_heightfield_config_parity(rtc, device, oracle):
    """Heightfield 256x256 (131,072 tris) with 1024x1024 primary rays: every ray
    compared with the oracle."""
    verts, idx = W.heightfield(256)
    rays = W.camera_rays(1024, 1024)
    sg, so, g, r = run_pair(rtc, device, oracle, [(0, verts, idx)], rays)
    rep = compare_closest(so, rays, g, r)
    print(rep)
    assert_clean(rep)
    assert rep["hits"] > 300000
    # same arithmetic as the oracle: every differing id is a classified tie, and
    # same-triangle hits are bit-identical
    assert rep["id_mismatch"] <= 8
    assert rep["same_hit_bit_differs"] == 0


def test_soup_parity(rtc, device, oracle):
    verts, idx = W.gaussian_soup(200_000, seed=21)
    rays = W.sphere_rays(400_000, seed=22)
    sg, so, g, r = run_pair(rtc, device, oracle, [(0, verts, idx)], rays)
    rep = compare_closest(so, rays, g, r)
    print(rep)
    assert_clean(rep)
    assert rep["hits"] > 10000
    # shadow rays from the hits toward a point light
    shadow, _ = W.shadow_rays(r, seed=23)
    sgo, soo = shadow.copy(), shadow.copy()
    sg.occluded(sgo)
    so.occluded(soo)
    rep2 = compare_occluded(so, shadow, sgo, soo, sg)
    print(rep2)
    assert_clean(rep2)
    assert rep2["occluded"] > 1000


def test_reordered_rays_parity(rtc, oracle):
    """gpu.reorder=1: the traversal fetches rays in direction-octant + origin-Morton
    order; every ray's result is still the oracle's (device and host rays)."""
    dev = rtc.Device(b"gpu.reorder=1")
    verts, idx = W.gaussian_soup(200_000, seed=31)
    sg = rtc.Scene(dev)
    sg.add_mesh(verts, idx)
    sg.commit()
    so = oracle.OracleScene([(0, verts, idx)])
    rays = W.sphere_rays(300_000, seed=32)
    g, r = rays.copy(), rays.copy()
    sg.intersect(g)
    so.intersect(r)
    rep = compare_closest(so, rays, g, r)
    assert_clean(rep)
    assert rep["hits"] > 5000
    shadow, _ = W.shadow_rays(r, seed=33)
    sgo, soo = shadow.copy(), shadow.copy()
    sg.occluded(sgo)
    so.occluded(soo)
    assert_clean(compare_occluded(so, shadow, sgo, soo, sg))
    sg.release()
    dev.release()


def test_multi_geometry_ids(rtc, device, oracle):
    """Several meshes with explicit geometry IDs; disabled and detached
    geometry is excluded from the next commit."""
    a = W.heightfield(16)
    b = W.gaussian_soup(3000, seed=2)
    c = W.triangle_sphere((0.5, 0.5, 0.5), 0.2, 20)
    meshes = [(3, *a), (7, *b), (12, *c)]
    rays = W.sphere_rays(50000, seed=5)
    sg, so, g, r = run_pair(rtc, device, oracle, meshes, rays)
    rep = compare_closest(so, rays, g, r)
    assert_clean(rep)
    assert set(np.unique(g["geomID"])) == {3, 7, 12, 0xFFFFFFFF}
    # detach 7, disable 12 -> only mesh 3 remains
    L = rtc.load()
    L.rtcDetachGeometry(sg.h, 7)
    L.rtcDisableGeometry(L.rtcGetGeometry(sg.h, 12))
    sg.commit()
    g2 = rays.copy()
    sg.intersect(g2)
    so3 = oracle.OracleScene([meshes[0]])
    r3 = rays.copy()
    so3.intersect(r3)
    assert_clean(compare_closest(so3, rays, g2, r3))


def test_strides_and_unaligned_records(rtc, device, oracle):
    """byteStride > sizeof(RTCRayHit) and a 4-byte (not 16-byte) aligned base
    select the scalar load path; results equal the packed call's."""
    verts, idx = W.gaussian_soup(20000, seed=9)
    rays = W.sphere_rays(20000, seed=10)
    sg = gpu_scene(rtc, device, [(0, verts, idx)])
    packed = rays.copy()
    sg.intersect(packed)
    for stride, offset in ((96, 0), (84, 4), (80, 4)):
        buf = np.zeros(offset + stride * rays.shape[0] + 16, np.uint8)
        view = np.ndarray(rays.shape, R.RAYHIT_DTYPE, buf, offset, (stride,))
        view[:] = rays
        import ctypes
        sg.intersect_ptr(buf.ctypes.data + offset, rays.shape[0], stride)
        got = np.ndarray(rays.shape, R.RAYHIT_DTYPE, buf, offset, (stride,)).copy()
        assert (got.view(np.uint8) == packed.view(np.uint8)).all(), (stride, offset)


def test_device_pointer_rays(rtc, device):
    """Rays already in HBM are traced in place (no host copies)."""
    torch = pytest.importorskip("torch")
    verts, idx = W.gaussian_soup(50000, seed=3)
    rays = W.sphere_rays(100000, seed=4)
    sg = gpu_scene(rtc, device, [(0, verts, idx)])
    host = rays.copy()
    sg.intersect(host)
    t = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    sg.intersect_ptr(t.data_ptr(), rays.shape[0], 80)
    st = rtc.last_query_stats()
    assert st["h2d_bytes"] == 0 and st["d2h_bytes"] == 0
    got = t.cpu().numpy().view(R.RAYHIT_DTYPE)
    assert (got.view(np.uint8) == host.view(np.uint8)).all()


def test_invalid_and_degenerate_triangles(rtc, device, oracle):
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2e18, 0, 0], [np.nan, 0, 0], [1, 1, 0]], np.float32)
    idx = np.array([[0, 1, 2], [0, 1, 9], [0, 1, 3], [0, 4, 2], [2, 1, 5], [0, 0, 0], [1, 1, 2]], np.uint32)
    sg = gpu_scene(rtc, device, [(2, verts, idx)])
    assert sg.build_stats()["num_prims"] == 4
    rng = np.random.default_rng(1)
    rays = R.make_rayhits(np.c_[rng.random((5000, 2)) * 1.2 - 0.1, -np.ones(5000)], np.tile([0, 0, 1], (5000, 1)))
    so = oracle.OracleScene([(2, verts, idx)])
    g, r = rays.copy(), rays.copy()
    sg.intersect(g)
    so.intersect(r)
    assert_clean(compare_closest(so, rays, g, r))


def test_overlapping_geometry(rtc, device, oracle):
    """OverlappingGeometryTest (verify.cpp:1216): thousands of identical triangles."""
    verts, idx = W.triangle_plane((0, 0, 0), (1, 0, 0), (0, 1, 0), 1, 1)
    idx = np.concatenate([idx, np.repeat(idx[-1:], 20000, 0)])
    sg = gpu_scene(rtc, device, [(0, verts, idx)])
    st = sg.build_stats()
    assert st["num_prims"] == idx.shape[0]
    rng = np.random.default_rng(2)
    rays = R.make_rayhits(np.c_[rng.random((2000, 2)), -np.ones(2000)], np.tile([0, 0, 1], (2000, 1)))
    so = oracle.OracleScene([(0, verts, idx)])
    g, r = rays.copy(), rays.copy()
    sg.intersect(g)
    so.intersect(r)
    rep = compare_closest(so, rays, g, r)
    assert_clean(rep)
    assert np.all(g["geomID"] == 0)


def test_full_size_soup_sample(rtc, device, oracle):
    """4M-triangle soup with 16M rays traced in HBM; a seeded 100k-ray sample
    is checked against the oracle, every hit against size-independent
    properties (t inside the ray interval, barycentrics inside the triangle,
    hit point on the triangle's plane)."""
    torch = pytest.importorskip("torch")
    verts, idx = W.gaussian_soup(4_000_000)
    rays = W.sphere_rays(16_000_000)
    sg = gpu_scene(rtc, device, [(0, verts, idx)])
    t = torch.from_numpy(rays.view(np.uint8)).cuda()
    sg.intersect_ptr(t.data_ptr(), rays.shape[0], 80)
    out = t.cpu().numpy().view(R.RAYHIT_DTYPE)
    hit = out["geomID"] == 0
    assert hit.mean() > 0.05
    assert np.all(out["tfar"][hit] > 0)
    u, v = out["u"][hit], out["v"][hit]
    assert u.min() >= 0 and v.min() >= 0 and (u + v).max() <= 1 + 1e-5
    p = verts.reshape(-1, 3, 3)[out["primID"][hit]]
    o = np.stack([out["org_x"], out["org_y"], out["org_z"]], -1)[hit]
    d = np.stack([out["dir_x"], out["dir_y"], out["dir_z"]], -1)[hit]
    P = o.astype(np.float64) + out["tfar"][hit][:, None].astype(np.float64) * d
    p = p.astype(np.float64)
    Q = p[:, 0] + u[:, None] * (p[:, 1] - p[:, 0]) + v[:, None] * (p[:, 2] - p[:, 0])
    err = np.abs(P - Q).max(1)
    # FP32 barycentrics of grazing rays are ill-conditioned: bound the tail loosely
    assert np.quantile(err, 0.999) < 1e-6 and err.max() < 1e-4
    # seeded sample against the oracle
    sel = np.sort(np.random.default_rng(99).choice(rays.shape[0], 100_000, replace=False))
    so = oracle.OracleScene([(0, verts, idx)])
    r = np.ascontiguousarray(rays[sel])
    so.intersect(r)
    rep = compare_closest(so, rays[sel], out[sel].copy(), r)
    print(rep)
    assert_clean(rep)


def test_radix_sort_bit_exact_vs_host_stable_sort(rtc):
    rng = np.random.default_rng(5)
    # 300k and 2M keys: the digit histograms (256 per 4096-key tile) take the
    # multi-CTA scan (3 and 16 scan tiles)
    for n in (1, 1000, 4097, 300_000, 2_000_000, 9_000_000):
        keys = rng.integers(0, 1 << 20, n, dtype=np.uint64) << np.uint64(rng.integers(0, 40))
        keys[rng.random(n) < 0.1] = np.uint64(0xFFFFFFFFFFFFFFFF)
        vals = np.arange(n, dtype=np.uint32)
        k, v = rtc.radix_sort_pairs(keys, vals)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(k, keys[order])
        assert np.array_equal(v, vals[order])


@pytest.mark.parametrize("mode", ["copy", "pipeline", "direct"])
def test_host_ray_modes(rtc, mode):
    """Host-resident rays through each host path (copy all, chunked copy/trace
    pipeline, direct access where the device can address host memory) give the bytes of tracing the
    same rays in device memory, for pageable and pinned host buffers, 16-byte
    aligned (stride 80) and not (stride 84), closest hit and occlusion."""
    torch = pytest.importorskip("torch")
    dev = rtc.Device(f"gpu.host_rays={mode}".encode())
    access = rtc.load().rtcgbGetDeviceHostAccess(dev.h)
    verts, idx = W.gaussian_soup(50_000, seed=41)
    rays = W.sphere_rays(2_500_000, seed=42)        # more than one 2M-ray pipeline chunk
    sc = rtc.Scene(dev)
    sc.add_mesh(verts, idx)
    sc.commit()
    t = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    sc.intersect_ptr(t.data_ptr(), rays.shape[0], 80)
    ref = t.cpu().numpy().view(R.RAYHIT_DTYPE)
    pageable = rays.copy()
    sc.intersect(pageable)
    assert (pageable.view(np.uint8) == ref.view(np.uint8)).all()
    pinned = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
    sc.intersect_ptr(pinned.data_ptr(), rays.shape[0], 80)
    assert (pinned.numpy() == ref.view(np.uint8)).all()
    st = rtc.last_query_stats()
    if mode == "direct" and access & 2:
        assert st["h2d_bytes"] == rays.shape[0] * 48
    else:
        assert st["h2d_bytes"] == rays.nbytes
    # unaligned records (stride 84) in pinned memory
    n = 300_000
    buf = np.zeros(n * 84, np.uint8)
    buf.reshape(n, 84)[:, :80] = rays[:n].view(np.uint8).reshape(n, 80)
    pin84 = torch.from_numpy(buf).pin_memory()
    sc.intersect_ptr(pin84.data_ptr(), n, 84)
    got84 = np.ascontiguousarray(pin84.numpy().reshape(n, 84)[:, :80])
    assert (got84 == ref[:n].view(np.uint8).reshape(n, 80)).all()
    # occlusion through the same paths, pageable and pinned
    shadow, _ = W.shadow_rays(ref, seed=43)
    a = shadow.copy()
    sc.occluded(a)
    ts = torch.from_numpy(shadow.view(np.uint8).copy()).cuda()
    sc.occluded_ptr(ts.data_ptr(), shadow.shape[0], 48)
    assert (a.view(np.uint8) == ts.cpu().numpy()).all()
    ps = torch.from_numpy(shadow.view(np.uint8).copy()).pin_memory()
    sc.occluded_ptr(ps.data_ptr(), shadow.shape[0], 48)
    assert (ps.numpy() == ts.cpu().numpy()).all()
    sc.release()
    dev.release()


def test_robust_mode_parity(rtc, device, oracle):
    """RTC_SCENE_FLAG_ROBUST (Triangle4v + Pluecker): GPU vs the oracle's
    robust path on a heightfield, a soup and the verify suite's far-away
    watertight sphere, whose rays must not leak (miss rate <= 2e-5)."""
    from test_oracle import WATERTIGHT_FAR, watertight_rays
    cases = [(W.heightfield(128), W.camera_rays(256, 256)),
             (W.gaussian_soup(100_000, seed=51), W.sphere_rays(200_000, seed=52))]
    vs, ix, wr = watertight_rays("sphere", WATERTIGHT_FAR, 100_000, 53)
    cases.append(((vs, ix), wr))
    for (verts, idx), rays in cases:
        sg = rtc.Scene(device, flags=rtc.RTC_SCENE_FLAG_ROBUST)
        sg.add_mesh(verts, idx)
        sg.commit()
        so = oracle.OracleScene([(0, verts, idx)], robust=True)
        g, r = rays.copy(), rays.copy()
        sg.intersect(g)
        so.intersect(r)
        rep = compare_closest(so, rays, g, r)
        print(rep)
        assert_clean(rep)
        shadow, _ = W.shadow_rays(r, seed=54)
        a, b = shadow.copy(), shadow.copy()
        sg.occluded(a)
        so.occluded(b)
        assert_clean(compare_occluded(so, shadow, a, b, sg))
        sg.release()
    assert np.mean(g["geomID"] == 0xFFFFFFFF) <= 2e-5


def test_update_buffers_then_commit_rebuilds(rtc, device, oracle):
    """rtcUpdateGeometryBuffer on a default-quality geometry (vertices, then
    indices) followed by rtcCommitScene rebuilds the BVH (no refit), and the
    hits are the oracle's on the new buffers (the reference's UpdateTest)."""
    verts, idx = W.gaussian_soup(40_000, seed=71)
    rays = W.sphere_rays(100_000, seed=72)
    sc = rtc.Scene(device)
    gid = sc.add_mesh(verts, idx)
    sc.commit()
    rng = np.random.default_rng(73)
    for step in range(2):
        if step == 0:
            sc.update_vertices(gid, verts + rng.normal(0, 0.01, verts.shape).astype(np.float32))
        else:
            sc.update_indices(gid, idx[rng.permutation(idx.shape[0])])
        sc.commit()
        assert sc.build_stats()["refit"] == 0
        v_now, i_now = sc._by_id[gid]
        g = rays.copy()
        sc.intersect(g)
        orc = oracle.OracleScene([(gid, v_now.copy(), i_now.copy())])
        r = rays.copy()
        orc.intersect(r)
        assert (r["geomID"] != 0xFFFFFFFF).sum() > 1000
        assert_clean(compare_closest(orc, rays, g, r))
        orc.close()
    sc.release()
