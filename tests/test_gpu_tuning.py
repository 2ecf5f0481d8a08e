"""The autotuner and the traversal's launch shapes (rtcgbGetTraversalShapes,
rtcgbSetSceneTraversalShape, rtcgbTuneSceneTraversal, gpu.trace_shape), and the
proposer's treelet budget (rtcgbNewProposerEx).

Every launch shape must return records bit-identical to the default shape's
(only the speed may differ); the tuner's pick must be no slower than the
default on the heightfield view (1024x1024 pinhole rays on the 256x256-cell
heightfield) and on a sample of batched scenes built like the 512-scene batch
(heightfields and soups of log-uniform size, a pinhole + sphere ray mix)."""
import math
import statistics

import numpy as np
import pytest

from rtcgb import workloads as W

pytestmark = pytest.mark.gpu

RTC_ERROR_INVALID_ARGUMENT = 2
RTC_ERROR_INVALID_OPERATION = 3


def _scene(rtc, device, meshes, robust=False, batched=False):
    sc = rtc.Scene(device, flags=rtc.RTC_SCENE_FLAG_ROBUST if robust else 0)
    if batched:
        sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    sc.commit()
    return sc


def _strided(rays, stride):
    buf = np.zeros(rays.shape[0] * stride, np.uint8)
    buf.reshape(-1, stride)[:, :80] = rays.view(np.uint8).reshape(-1, 80)
    return buf


def test_shape_table(rtc):
    shapes = rtc.traversal_shapes()
    assert len(shapes) >= 4
    assert shapes[0] == {"threads": 128, "ctas_per_sm": 9, "shared_stack": 8, "refill": 4}
    assert len({tuple(s.values()) for s in shapes}) == len(shapes)
    for s in shapes:
        assert s["threads"] % 32 == 0 and s["threads"] * s["ctas_per_sm"] <= 2048
        assert 1 <= s["shared_stack"] <= 64 and 1 <= s["refill"] <= 32


@pytest.mark.parametrize("robust", [False, True], ids=["plain", "robust"])
@pytest.mark.parametrize("stride", [80, 96, 84])
def test_every_shape_returns_identical_records(rtc, device, robust, stride):
    """Closest hit and occlusion in every shape: records bit-identical to shape 0's
    (a stride of 84 bytes is not 16-byte aligned and runs shape 0 whatever is set)."""
    verts, idx = W.gaussian_soup(150_000, seed=41)
    rays = W.sphere_rays(200_000, seed=42)
    sc = _scene(rtc, device, [(verts, idx)], robust=robust)
    out = {}
    for s in range(len(rtc.traversal_shapes())):
        sc.traversal_shape = s
        assert sc.traversal_shape == s
        buf = _strided(rays, stride)
        sc.intersect_ptr(buf.ctypes.data, rays.shape[0], stride)
        shadow = _strided(rays, stride)
        sc.occluded_ptr(shadow.ctypes.data, rays.shape[0], stride)
        out[s] = (buf, shadow)
    hits = np.mean(out[0][0].reshape(-1, stride)[:, 72:76].view(np.uint32) != 0xFFFFFFFF)
    assert hits > 0.05
    for s, (b, sh) in out.items():
        assert np.array_equal(b, out[0][0]), s
        assert np.array_equal(sh, out[0][1]), s
    sc.release()


def test_every_shape_batched_identical(rtc, device):
    meshes = [W.heightfield(60, seed=5), W.gaussian_soup(30_000, seed=6), W.heightfield(20, seed=7)]
    parts, start = [], [0]
    for k in range(3):
        r = W.sphere_rays(30_000, seed=50 + k)
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    rays = np.concatenate(parts)
    sc = _scene(rtc, device, meshes, batched=True)
    ref = None
    for s in range(len(rtc.traversal_shapes())):
        sc.traversal_shape = s
        got = sc.intersect_batched(rays.copy(), start)
        if ref is None:
            ref = got
            assert np.mean(got["geomID"] != 0xFFFFFFFF) > 0.05
        assert (got.view(np.uint8) == ref.view(np.uint8)).all(), s
    sc.release()


def _alternate(fns, rounds):
    """Median time of each callable, the callables taking turns each round."""
    t = [[] for _ in fns]
    for _ in range(rounds):
        for k, f in enumerate(fns):
            t[k].append(f())
    return [statistics.median(x) for x in t]


def test_tuner_pick_no_slower_than_default_heightfield(rtc, device):
    """Heightfield 256x256 cells, 1024x1024 pinhole rays (closest hit + occlusion
    on the same records): the tuned shape, re-measured against shape 0 in turns,
    is no slower (3 % for timing noise)."""
    from rtcgb import autotune
    import torch
    sc = _scene(rtc, device, [W.heightfield(256)])
    rays = W.camera_rays(1024, 1024)
    rec = autotune.tune_scene(sc, rays, occluded=True, repeats=5)
    assert sc.traversal_shape == rec["pick"]
    assert rec["pick_ms"] <= rec["default_ms"]
    print("heightfield shapes (ms):", [round(x, 4) for x in rec["ms_per_shape"]], "pick", rec["pick"])
    pristine = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    work = torch.empty_like(pristine)

    def run(shape):
        def f():
            sc.traversal_shape = shape
            work.copy_(pristine)
            sc.intersect_ptr(work.data_ptr(), rays.shape[0], 80)
            t = rtc.last_query_stats()["kernel_ms"]
            work.copy_(pristine)
            sc.occluded_ptr(work.data_ptr(), rays.shape[0], 80)
            return t + rtc.last_query_stats()["kernel_ms"]
        return f

    t_pick, t_default = _alternate([run(rec["pick"]), run(0)], 9)
    device.check("queries")
    print("re-measured: pick", t_pick, "default", t_default)
    assert t_pick <= 1.03 * t_default
    sc.release()


def _batched_sample(nscenes=12, seed=21, rays_per_tri=4):
    """Scenes drawn like the 512-scene batch (log-uniform 1k-200k triangles,
    heightfields and soups in turn) with a pinhole + sphere mix of rays."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(1000), math.log(200_000), nscenes)).astype(np.int64)
    meshes, parts, start = [], [], [0]
    for k, n in enumerate(counts):
        if k % 2 == 0:
            meshes.append(W.heightfield(max(8, int(round(math.sqrt(n / 2)))), seed=int(rng.integers(1, 10 ** 6))))
            eye, look = (0.5, -0.5, 0.6), (0.5, 0.5, 0.0)
        else:
            meshes.append(W.gaussian_soup(int(n), seed=int(rng.integers(1, 10 ** 6))))
            eye, look = (0.5, -1.0, 0.5), (0.5, 0.5, 0.5)
        m = rays_per_tri * meshes[-1][1].shape[0]
        side = max(8, int(math.sqrt(m // 2)))
        cam = W.camera_rays(side, side, eye=eye, look=look)
        sph = W.sphere_rays(m - cam.shape[0] if m > cam.shape[0] else 1000, seed=200 + k)
        r = np.concatenate([cam, sph])
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    return meshes, np.concatenate(parts), np.array(start, np.uint32)


def test_tuner_pick_no_slower_than_default_batched_sample(rtc):
    """Batched sample: the tuned configuration (build options + launch shape),
    re-measured against the device defaults in turns, takes no longer to build and
    trace (5 % for timing noise on these ~1-ms phases)."""
    from rtcgb import autotune
    meshes, rays, start = _batched_sample()
    best, results = autotune.tune(meshes, rays, start, shape_repeats=3)
    print("chosen", best)
    assert results[0]["config"] == autotune.DEFAULT
    devs = [rtc.Device(autotune.config_string(best).encode()), rtc.Device(b"")]
    scenes = []
    for d in devs:
        sc = rtc.Scene(d)
        sc.set_batched()
        for v, i in meshes:
            sc.add_mesh(v, i)
        sc.commit()
        scenes.append(sc)
    assert scenes[0].traversal_shape == best["gpu.trace_shape"] and scenes[1].traversal_shape == 0

    def run(sc):
        def f():
            sc.commit()
            b = sc.build_stats()["build_ms"]
            sc.intersect_batched(rays.copy(), start)
            return b + rtc.last_query_stats()["kernel_ms"]
        return f

    t_best, t_default = _alternate([run(scenes[0]), run(scenes[1])], 7)
    print("re-measured build + trace: chosen", t_best, "default", t_default)
    assert t_best <= 1.05 * t_default
    for sc in scenes:
        sc.release()
    for d in devs:
        d.release()


def test_shape_keys_and_errors(rtc, device):
    with pytest.raises(rtc.RTCError) as e:
        rtc.Device(b"gpu.trace_shape=99")
    assert e.value.code == RTC_ERROR_INVALID_ARGUMENT
    d2 = rtc.Device(b"gpu.trace_shape=2")
    sc = _scene(rtc, d2, [W.heightfield(16)])
    assert sc.traversal_shape == 2
    rtc.load().rtcgbSetSceneTraversalShape(sc.h, 99)
    assert d2.error() == RTC_ERROR_INVALID_ARGUMENT
    assert sc.traversal_shape == 2
    rays = W.camera_rays(64, 64)
    # records must be 16-byte aligned for the tuned shapes
    buf = _strided(rays, 84)
    rtc.load().rtcgbTuneSceneTraversal(sc.h, buf.ctypes.data, rays.shape[0], 84, None, 0, 0, 1, None)
    assert d2.error() == RTC_ERROR_INVALID_ARGUMENT
    # batched scenes need their batches, other scenes none
    rtc.load().rtcgbTuneSceneTraversal(sc.h, rays.ctypes.data, rays.shape[0], 80,
                                       np.array([0, rays.shape[0]], np.uint32).ctypes.data, 1, 0, 1, None)
    assert d2.error() == RTC_ERROR_INVALID_ARGUMENT
    # filter callbacks run the default shape only: tuning is refused
    filt = rtc.Scene(d2)
    gid = filt.add_mesh(*W.heightfield(16))
    filt.set_filters(gid, intersect=lambda g, p, u, v, t: True)
    filt.commit()
    rtc.load().rtcgbTuneSceneTraversal(filt.h, rays.ctypes.data, rays.shape[0], 80, None, 0, 0, 1, None)
    assert d2.error() == RTC_ERROR_INVALID_OPERATION
    # a tuned scene answers like before, and the records given to the tuner are untouched
    before = rays.copy()
    pick, ms = sc.tune_traversal(rays, repeats=1)
    assert (rays.view(np.uint8) == before.view(np.uint8)).all()
    assert 0 <= pick < len(rtc.traversal_shapes()) and all(x > 0 for x in ms)
    for s in (filt, sc):
        s.release()
    d2.release()


def test_treelet_budget(rtc, device):
    """rtcgbNewProposerEx: the cut respects the budget, learned queries keep the
    plain traversal's hits under every budget, and tune_treelets returns one of
    its candidates."""
    from rtcgb import autotune
    sc = _scene(rtc, device, [W.heightfield(128)])
    rays = W.camera_rays(256, 256)
    plain = sc.intersect(rays.copy())
    for nt in (64, 512):
        p = rtc.Proposer(sc, seed=3, max_treelets=nt)
        st = p.train(plain, epochs=1)
        assert 1 <= st["num_treelets"] <= nt
        got = p.intersect(rays.copy())
        assert (got.view(np.uint8) == plain.view(np.uint8)).all()
        p.release()
    with pytest.raises(rtc.RTCError):
        rtc.Proposer(sc, seed=3, max_treelets=5000)

    def q(prop):
        prop.intersect(rays.copy())
        return rtc.last_query_stats()["kernel_ms"]

    pick, res = autotune.tune_treelets(sc, plain, [q], candidates=(64, 512), epochs=1, repeats=1)
    assert pick in (64, 512) and len(res) == 2
    sc.release()
