"""Animated wavefront path tracing with frames captured as CUDA graphs
(rtcgbNewPathTracer / rtcgbPathTracerRenderFrame): graph replays are
deterministic, learned frames produce the plain frames' images bit for bit,
and the refit inside the frame graph leaves a BVH whose hits match the oracle
on the moved vertices."""
import numpy as np
import pytest

from parity import assert_clean, compare_closest
from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def path_scene(rtc, device):
    sc = rtc.Scene(device)
    sc.add_mesh(*W.heightfield(48))
    sc.add_mesh(*W.gaussian_soup(60000, seed=5))
    sc.commit()
    return sc


def test_graph_replay_deterministic(rtc, path_scene):
    pt = rtc.PathTracer(path_scene, 160, 120, bounces=4)
    s1 = pt.render(3)
    a = pt.image()
    pt.render(9)
    s2 = pt.render(3)
    b = pt.image()
    assert (a.view(np.uint32) == b.view(np.uint32)).all()
    assert s1["rays_per_bounce"] == s2["rays_per_bounce"]
    rpb = s1["rays_per_bounce"]
    assert rpb[0] == 160 * 120 and rpb[0] >= rpb[1] >= rpb[2] >= rpb[3] > 0
    assert s1["rays"] == sum(rpb) and s1["errors"] == 0 and s1["frame_ms"] > 0
    assert np.isfinite(a).all() and a.max() > 0.1
    pt.release()


def test_learned_frames_match_plain_frames(rtc, path_scene):
    pt = rtc.PathTracer(path_scene, 160, 120, bounces=4)
    prop = rtc.Proposer(path_scene, seed=9)
    pt.set_proposer(prop)
    for f in range(3):  # logs of plain frames train the proposer
        pt.render(f)
        pt.train_proposer(epochs=4, batch=2048, lr=5e-3)
    plain = pt.render(5, learned=False)
    img_plain = pt.image()
    learned = pt.render(5, learned=True)
    img_learned = pt.image()
    assert learned["learned"] == 1 and plain["learned"] == 0
    assert (img_plain.view(np.uint32) == img_learned.view(np.uint32)).all()
    assert plain["rays_per_bounce"] == learned["rays_per_bounce"]
    assert learned["proposal_hits"] > 0 and learned["errors"] == 0
    assert prop.stats()["samples"] > 0
    pt.release()
    prop.release()


def test_animated_refit_in_graph_matches_oracle(rtc, device, oracle):
    torch = pytest.importorskip("torch")
    verts, idx = W.gaussian_soup(30000, seed=8)
    dv = torch.from_numpy(verts.copy()).cuda()
    di = torch.from_numpy(idx.view(np.int32).copy()).cuda()
    sc = rtc.Scene(device)
    gid = sc.add_mesh_device(dv.data_ptr(), verts.shape[0], di.data_ptr(), idx.shape[0], quality=rtc.RTC_BUILD_QUALITY_REFIT)
    sc.commit()
    pt = rtc.PathTracer(sc, 96, 64, bounces=3)
    pt.animate_soup(gid, amplitude=0.01, seed=14)
    st = pt.render(17)
    assert st["errors"] == 0
    moved = dv.cpu().numpy()
    # every triangle moved rigidly by at most the amplitude
    d = (moved - verts).reshape(-1, 3, 3)
    assert np.abs(d - d[:, :1, :]).max() < 1e-6
    assert np.linalg.norm(d[:, 0, :], axis=1).max() <= 0.01 + 1e-6
    assert np.linalg.norm(d[:, 0, :], axis=1).mean() > 1e-3
    # queries on the refitted BVH against the oracle built from the moved vertices
    rays = W.sphere_rays(20000, seed=19)
    gpu = rays.copy()
    sc.intersect(gpu)
    orc = oracle.OracleScene([(gid, moved, idx)])
    ref = rays.copy()
    orc.intersect(ref)
    assert_clean(compare_closest(orc, rays, gpu, ref))
    pt.release()
    sc.release()
