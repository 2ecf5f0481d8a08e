"""The learned hit proposer on the GPU: gradients and inference against the CPU
restatement (oracle/proposer_oracle.py), exactness of the learned queries
against the plain traversal, and what training gains over an untrained
network and over the plain method."""
import numpy as np
import pytest

import proposer_oracle as PO
from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu


def _grid(scene):
    """The proposer's origin normalisation, computed as the library does (float32)."""
    lo, hi = scene.bounds()
    lo = lo.astype(np.float32)
    ext = (hi.astype(np.float32) - lo).astype(np.float32)
    return lo, (np.float32(1.0) / ext).astype(np.float32)


@pytest.fixture(scope="module")
def small_scene(rtc, device):
    sc = rtc.Scene(device)
    sc.add_mesh(*W.heightfield(48))
    sc.add_mesh(*W.gaussian_soup(20000, seed=3))
    sc.commit()
    return sc


def _random_rays(n, seed, lo=0.05, hi=0.95):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return R.make_rays(rng.uniform(lo, hi, (n, 3)), d)


def test_treelet_cut(rtc, small_scene):
    prop = rtc.Proposer(small_scene, seed=1)
    n_rec = small_scene.build_stats()["num_prims"]
    roots, rec = prop.treelets(n_rec)
    assert 500 < roots.shape[0] <= 4096
    assert np.unique(roots).shape[0] == roots.shape[0]
    assigned = rec != 0xFFFFFFFF
    assert assigned.mean() > 0.9
    assert rec[assigned].max() < roots.shape[0]
    prop.release()


def test_gradients_match_oracle(rtc, small_scene):
    """GPU forward + backward (mma.sync BF16 kernels, softmax cross-entropy,
    hash-grid scatter) against the float64 restatement with the same BF16
    rounding points."""
    prop = rtc.Proposer(small_scene, seed=2)
    ntl = prop.stats()["num_treelets"]
    params = PO.random_params(seed=5)
    prop.set_params(params)
    B = 384
    rays = _random_rays(B, 6)
    labels = np.random.default_rng(7).integers(-1, ntl, B).astype(np.int32)
    loss_gpu, g_gpu = prop.gradients(rays, labels)
    lo, scale = _grid(small_scene)
    loss_ref, g_ref = PO.loss_and_grad(params, rays, labels, lo, scale)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * abs(loss_ref)
    for name, a, b in PO.segments():
        x, y = g_ref[a:b], g_gpu[a:b].astype(np.float64)
        nx = np.linalg.norm(x)
        assert nx > 0, name
        # BF16 rounding points may flip by one unit between the FP32 GPU sums
        # and the float64 restatement; the gradients agree to ~1e-2
        assert np.linalg.norm(y - x) <= 2e-2 * nx, (name, np.linalg.norm(y - x) / nx)
    prop.release()


def test_inference_matches_oracle(rtc, small_scene):
    """Fused top-4 inference: the proposed treelets are the oracle's top 4 up to
    near-ties of the logits."""
    prop = rtc.Proposer(small_scene, seed=3)
    ntl = prop.stats()["num_treelets"]
    params = PO.random_params(seed=11)
    prop.set_params(params)
    rays = _random_rays(1000, 12)
    top = prop.predict(rays).astype(np.int64)
    lo, scale = _grid(small_scene)
    Z = PO.logits(params, rays, lo, scale)
    Z[:, ntl:] = -np.inf
    order = np.argsort(-Z, axis=1, kind="stable")[:, :4]
    exact = (np.sort(order, 1) == np.sort(top, 1)).all(1)
    assert exact.mean() > 0.97
    # every proposal is within a near-tie of the oracle's 4th best logit
    fourth = np.take_along_axis(Z, order[:, 3:4], 1)[:, 0]
    picked = np.take_along_axis(Z, top, 1)
    assert (picked >= (fourth - 1e-3 * np.maximum(1.0, np.abs(fourth)))[:, None]).all()
    assert all(len(set(r)) == 4 for r in top.tolist())
    prop.release()


@pytest.fixture(scope="module")
def ao_setup(rtc, device):
    sc = rtc.Scene(device)
    for v, i in W.ao_scene(cells=160, soup_tris=40000, seed=3):
        sc.add_mesh(v, i)
    sc.commit()
    prim = W.camera_rays(192, 192)
    sc.intersect(prim)
    return sc, prim


def _logged(sc, prim, seed, per_hit=64):
    """Training log: closest hits of ambient-occlusion rays from the primary hits."""
    log, _ = W.hemisphere_rays(prim, per_hit, seed=seed, tfar=0.05)
    sc.intersect(log)
    return log


def test_learned_queries_exact_and_gain(rtc, ao_setup):
    """Trained on logs of the plain traversal, the proposer changes no result
    (occlusion bits identical; closest hits identical up to exact distance ties)
    and answers far more rays inside its proposed treelets, with fewer node
    visits, than the same network untrained.  On this small scene the seeded
    traversal still visits a few percent more nodes than the plain one on the
    occluded rays (wrong proposals cost a visit each); the ratio is printed."""
    sc, prim = ao_setup
    log = _logged(sc, prim, 31)
    trained = rtc.Proposer(sc, seed=4)
    untrained = rtc.Proposer(sc, seed=4)
    st = trained.train(log, epochs=20, batch=1024, lr=5e-3)
    labelled = int((log["geomID"] != 0xFFFFFFFF).sum())
    assert st["samples"] > 0.9 * labelled and st["samples"] > 5000, (st, labelled)
    assert st["top4"] > 0.3, st
    ao, _ = W.hemisphere_rays(prim, 8, seed=41, tfar=0.05, record=R.RAY_DTYPE)
    bounce, _ = W.hemisphere_rays(prim, 4, seed=42)

    def run(fn, rays):
        rtc.set_counting(True)
        out = rays.copy()
        fn(out)
        rtc.set_counting(False)
        return out, rtc.last_query_stats()

    plain_ao, s_plain = run(sc.occluded, ao)
    learn_ao, s_learn = run(trained.occluded, ao)
    _, s_untr = run(untrained.occluded, ao)
    assert (plain_ao.view(np.uint8) == learn_ao.view(np.uint8)).all()
    occ = plain_ao["tfar"] < 0
    assert occ.sum() > 300
    # what the trained network gains over the untrained one
    assert s_learn["proposal_hits"] > 0.25 * occ.sum(), (s_learn["proposal_hits"], int(occ.sum()))
    assert s_learn["proposal_hits"] > 4 * max(1, s_untr["proposal_hits"])
    # node visits on the occluded rays: trained vs untrained network, and vs the plain method
    _, s_plain_occ = run(sc.occluded, ao[occ])
    _, s_learn_occ = run(trained.occluded, ao[occ])
    _, s_untr_occ = run(untrained.occluded, ao[occ])
    assert s_learn_occ["nodes"] < s_untr_occ["nodes"], (s_learn_occ["nodes"], s_untr_occ["nodes"])
    print(f"occluded rays: {int(occ.sum())}, answered by a proposal: {s_learn['proposal_hits']} "
          f"(untrained {s_untr['proposal_hits']}); node visits trained/plain "
          f"{s_learn_occ['nodes'] / s_plain_occ['nodes']:.3f}, untrained/plain {s_untr_occ['nodes'] / s_plain_occ['nodes']:.3f}")
    plain_b, _ = run(sc.intersect, bounce)
    learn_b, s_lb = run(trained.intersect, bounce)
    same = R.hits_equal_bits(plain_b, learn_b)
    tie = (~same) & (plain_b["tfar"].view(np.uint32) == learn_b["tfar"].view(np.uint32))
    assert (same | tie).all(), int((~(same | tie)).sum())
    assert s_lb["proposal_hits"] > 0
    trained.release()
    untrained.release()


def test_learned_queries_fall_back_after_rebuild(rtc, device):
    """A proposer keeps its treelets only while the scene keeps its BVH: after a
    full rebuild the learned queries run the plain traversal (same results)."""
    sc = rtc.Scene(device)
    v, i = W.heightfield(32)
    gid = sc.add_mesh(v, i)
    sc.commit()
    prop = rtc.Proposer(sc, seed=5)
    sc.update_indices(gid, i[::-1].copy())  # new topology: full rebuild at commit
    sc.commit()
    rays = W.camera_rays(64, 64)
    a, b = rays.copy(), rays.copy()
    sc.intersect(a)
    prop.intersect(b)
    assert (a.view(np.uint8) == b.view(np.uint8)).all()
    assert rtc.last_query_stats()["proposal_hits"] == 0
    prop.release()


def test_tensor_core_inference_matches_mma_sync(rtc, small_scene):
    """The tcgen05 inference kernel (default) and the mma.sync one (device key
    gpu.proposer=mma) propose the same treelets up to FP32 accumulation-order ties."""
    dev_mma = rtc.Device(b"gpu.proposer=mma")
    sc2 = rtc.Scene(dev_mma)
    sc2.add_mesh(*W.heightfield(48))
    sc2.add_mesh(*W.gaussian_soup(20000, seed=3))
    sc2.commit()
    params = PO.random_params(seed=13)
    a = rtc.Proposer(small_scene, seed=1)
    b = rtc.Proposer(sc2, seed=1)
    a.set_params(params)
    b.set_params(params)
    rays = _random_rays(5000, 14)
    ta, tb = a.predict(rays), b.predict(rays)
    same = (np.sort(ta, 1) == np.sort(tb, 1)).all(1)
    assert same.mean() > 0.99, same.mean()
    a.release()
    b.release()
    sc2.release()
    dev_mma.release()
