"""Batched scenes (rtcgbSetSceneBatched): many independent scenes built in one
segmented pass and queried in one launch, each batch of rays against its own
geometry only, checked against one oracle scene per batch."""
import numpy as np
import pytest

from parity import assert_clean, compare_closest, compare_occluded
from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu


def _scenes(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        if k % 2 == 0:
            out.append(W.heightfield(int(rng.integers(8, 60)), seed=int(rng.integers(1, 1000))))
        else:
            out.append(W.gaussian_soup(int(rng.integers(1000, 30000)), seed=int(rng.integers(1, 1000))))
    return out


def _rays_for(meshes, per_tri, seed):
    """Half camera rays, half uniform-sphere rays per scene; returns (rays, start)."""
    rng = np.random.default_rng(seed)
    parts, start = [], [0]
    for v, i in meshes:
        n = max(64, per_tri * i.shape[0] // 8)
        side = max(4, int(np.sqrt(n // 2)))
        cam = W.camera_rays(side, side)
        sph = W.sphere_rays(n // 2, seed=int(rng.integers(1, 10 ** 6)))
        r = np.concatenate([cam, sph])
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    return np.concatenate(parts), np.array(start, np.uint32)


def test_batched_closest_and_occluded_match_oracle(rtc, device, oracle):
    meshes = _scenes(3, 7)
    sc = rtc.Scene(device)
    sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    sc.commit()
    rays, start = _rays_for(meshes, 2, 5)
    gpu = rays.copy()
    sc.intersect_batched(gpu, start)
    sh = np.zeros(rays.shape[0], R.RAY_DTYPE)
    for name in R.RAY_DTYPE.names:
        sh[name] = rays[name]
    sh["tfar"] = 0.3
    gsh = sh.copy()
    sc.occluded_batched(gsh, start)
    for b, (v, i) in enumerate(meshes):
        lo, hi = start[b], start[b + 1]
        orc = oracle.OracleScene([(b, v, i)])
        ref = rays[lo:hi].copy()
        orc.intersect(ref)
        g = gpu[lo:hi]
        assert set(np.unique(g["geomID"])) <= {b, 0xFFFFFFFF}
        assert (g["geomID"] == b).sum() > 0
        assert_clean(compare_closest(orc, rays[lo:hi], g, ref))
        rs = sh[lo:hi].copy()
        orc.occluded(rs)
        assert_clean(compare_occluded(orc, sh[lo:hi], gsh[lo:hi], rs))
    sc.release()


def test_batched_empty_batch_and_errors(rtc, device):
    sc = rtc.Scene(device)
    sc.set_batched()
    v, i = W.heightfield(16)
    sc.add_mesh(v, i)
    bad = v.copy()
    bad[:] = np.nan  # every triangle invalid: this batch has no tree
    sc.add_mesh(bad, i)
    sc.add_mesh(*W.gaussian_soup(2000, seed=2))
    sc.commit()
    rays = W.camera_rays(32, 32)
    start = np.array([0, 400, 700, rays.shape[0]], np.uint32)
    out = rays.copy()
    sc.intersect_batched(out, start)
    assert (out["geomID"][400:700] == 0xFFFFFFFF).all()
    assert (out["geomID"][:400] == 0).sum() > 0
    L = rtc.load()
    with pytest.raises(rtc.RTCError):
        sc.intersect_batched(rays.copy(), np.array([0, 10, 20], np.uint32))  # does not cover M
    with pytest.raises(rtc.RTCError):
        sc.intersect(rays.copy())  # plain query on a batched scene
    L.rtcGetDeviceError(device.h)
    sc.release()


def test_batched_refit(rtc, device, oracle):
    meshes = [W.gaussian_soup(5000, seed=s) for s in (1, 2, 3)]
    sc = rtc.Scene(device)
    sc.set_batched()
    gids = [sc.add_mesh(v, i, quality=rtc.RTC_BUILD_QUALITY_REFIT) for v, i in meshes]
    sc.commit()
    moved = [W.displace_soup(v, 9, seed=4, amplitude=0.01) for v, _ in meshes]
    for g, mv in zip(gids, moved):
        sc.update_vertices(g, mv)
    sc.commit()
    assert sc.build_stats()["refit"] == 1
    rays = W.sphere_rays(9000, seed=8)
    start = np.array([0, 3000, 6000, 9000], np.uint32)
    gpu = rays.copy()
    sc.intersect_batched(gpu, start)
    for b in range(3):
        orc = oracle.OracleScene([(b, moved[b], meshes[b][1])])
        ref = rays[start[b]:start[b + 1]].copy()
        orc.intersect(ref)
        assert_clean(compare_closest(orc, rays[start[b]:start[b + 1]], gpu[start[b]:start[b + 1]], ref))
    sc.release()


def test_autotuner_picks_the_fastest_candidate(rtc):
    """The autotuner runs every candidate configuration through the C ABI on a
    sample of batched scenes and returns the one with the least build + trace
    time, with the timings of all."""
    from rtcgb import autotune
    meshes = [W.heightfield(40, seed=3), W.gaussian_soup(20_000, seed=4)]
    parts, start = [], [0]
    for k in range(2):
        r = W.sphere_rays(20_000, seed=10 + k)
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    rays = np.concatenate(parts)
    cands = autotune.CANDIDATES[:3] + [c for c in autotune.CANDIDATES if c["gpu.morton_bits"] == 30][:1]
    best, results = autotune.tune(meshes, rays, np.array(start, np.uint32), candidates=cands, shape_repeats=2)
    shapes = results.pop()["shapes"]
    assert [r["config"] for r in results] == [autotune.DEFAULT] + cands
    assert all(r["build_ms"] > 0 and r["trace_ms"] > 0 for r in results)
    chosen = dict(best)
    assert chosen.pop("gpu.trace_shape") == shapes["pick"]
    assert chosen == min(results, key=lambda r: r["total_ms"])["config"]
    assert len(shapes["ms"]) == len(rtc.traversal_shapes()) and min(shapes["ms"]) > 0


@pytest.mark.parametrize("config", [b"", b"gpu.morton_bits=63"], ids=["key30", "key63"])
def test_batched_frame_graph_matches_separate_calls(rtc, config):
    """A batched frame -- the rebuild of every BVH of the scene and the batched
    closest-hit query, captured into one CUDA graph with the copy that restores
    the rays -- gives the bytes of rtcCommitScene + rtcgbIntersect1MBatched on
    the same rays, replay after replay; a new commit invalidates it.  With 63-bit
    and 30-bit sort keys."""
    torch = pytest.importorskip("torch")
    device = rtc.Device(config)
    meshes = [W.heightfield(32, seed=5), W.gaussian_soup(30_000, seed=6), W.heightfield(20, seed=7),
              W.gaussian_soup(8_000, seed=8)]
    parts, start = [], [0]
    for k in range(len(meshes)):
        cam = W.camera_rays(64, 64) if k % 2 == 0 else W.camera_rays(64, 64, eye=(0.5, -1.0, 0.5), look=(0.5, 0.5, 0.5))
        r = np.concatenate([cam, W.sphere_rays(8000, seed=30 + k)])
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    rays = np.concatenate(parts)
    sc = rtc.Scene(device)
    sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    sc.commit()
    ref = rays.copy()
    sc.intersect_batched(ref, start)
    assert (ref["geomID"] != 0xFFFFFFFF).sum() > 5000
    pristine = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    work = torch.zeros_like(pristine)
    frame = rtc.BatchedFrame(sc, work.data_ptr(), rays.shape[0], start, pristine_ptr=pristine.data_ptr())
    for _ in range(2):
        st = frame.replay()
        got = work.cpu().numpy()
        assert np.array_equal(got, ref.view(np.uint8))
    assert st["status"] == 0 and st["replays"] == 2 and st["graph_nodes"] > 10 and st["frame_ms"] > 0
    # the build's loops ran on the device as often as the data needed
    assert st["levels"] == sc.build_stats()["depth"] and st["ploc_rounds"] > 0
    assert st["num_nodes"] == sc.build_stats()["num_nodes"]
    sc.commit()
    with pytest.raises(rtc.RTCError):
        frame.replay()
    frame.release()
    sc.release()
    device.release()
