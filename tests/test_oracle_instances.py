"""The oracle's instance path (orc_intersect_instanced / orc_occluded_instanced),
pinned without a GPU: an identity instance gives exactly the instanced scene's
hits, and a translated instance agrees with the translated mesh."""
import numpy as np

from rtcgb import workloads as W

IDENT = [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]


def test_identity_instance_equals_scene(oracle):
    v, i = W.gaussian_soup(20000, seed=4)
    sc = oracle.OracleScene([(0, v, i)])
    rays = W.sphere_rays(20000, seed=5)
    direct, inst = rays.copy(), rays.copy()
    sc.intersect(direct)
    oracle.instanced(None, [(sc, IDENT, 9)], inst)
    hit = direct["geomID"] != 0xFFFFFFFF
    assert hit.sum() > 100
    for f in ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "primID", "geomID"):
        assert (direct[f].view(np.uint32) == inst[f].view(np.uint32)).all(), f
    assert (inst["instID"][hit] == 9).all() and (inst["instID"][~hit] == 0xFFFFFFFF).all()
    sh = np.zeros(rays.shape[0], np.dtype(rays.dtype.descr[:12]))
    for f in sh.dtype.names:
        sh[f] = rays[f]
    sh["tfar"] = 0.2
    a, b = sh.copy(), sh.copy()
    sc.occluded(a)
    oracle.instanced(None, [(sc, IDENT, 9)], b, anyhit=True)
    assert (a["tfar"].view(np.uint32) == b["tfar"].view(np.uint32)).all()


def test_translated_instance_matches_translated_mesh(oracle):
    v, i = W.heightfield(24)
    off = np.array([0.25, -0.125, 0.5], np.float32)  # exact in binary: vertices move exactly
    moved = oracle.OracleScene([(0, v + off, i)])
    base = oracle.OracleScene([(0, v, i)])
    rays = W.sphere_rays(20000, seed=6)
    rays["org_x"] += 0.25
    rays["org_y"] -= 0.125
    rays["org_z"] += 0.5
    a, b = rays.copy(), rays.copy()
    moved.intersect(a)
    oracle.instanced(None, [(base, IDENT[:9] + list(off), 3)], b)
    same = (a["geomID"] == b["geomID"]) & (a["primID"] == b["primID"])
    assert same.mean() > 0.999
    hit = same & (a["geomID"] != 0xFFFFFFFF)
    assert hit.sum() > 100
    # the origins round differently when shifted by the offset: absolute ~1e-7 in t
    assert np.allclose(a["tfar"][hit], b["tfar"][hit], rtol=1e-5, atol=1e-6)
