"""Loads the reference-made fixtures of tests/golden/ (written by
tests/golden/make_golden.py from the reference library itself) and rebuilds their
inputs from the seeded generators.

Each loader returns a dict with the scene meshes, the input records (`rays`), the
reference's closest-hit records (`expected`), the shadow rays made from those hits
(`shadow`) and the reference's occlusion flags for them (`occluded`).
"""
import json
import os

import numpy as np

from rtcgb import rays as R
from rtcgb import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INVALID = 0xFFFFFFFF
SMALL = ("terrain_camera48.npz", "soup_camera40_sphere.npz")
HIT_FIELDS = ("tfar", "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID")


def build_stats():
    with open(os.path.join(GOLDEN, "ref_build_stats.json")) as f:
        return json.load(f)


def small(name):
    d = np.load(os.path.join(GOLDEN, name))
    rays = d["rays"].view(R.RAYHIT_DTYPE).copy()
    shadow = d["shadow_rays"].view(R.RAY_DTYPE).copy()
    expected = rays.copy()
    for f in HIT_FIELDS:
        expected[f] = d["hit_" + f]
    return dict(meshes=[(d["verts"].copy(), d["idx"].copy())], rays=rays, expected=expected, shadow=shadow,
                occluded=d["occluded"].copy(), robust=False)


def _expand(d, rays):
    """Reference closest-hit records: the input records with the fixture's hits filled in."""
    n = rays.shape[0]
    hit = np.unpackbits(d["hit_bits"])[:n].astype(bool)
    assert int(d["n"]) == n and hit.sum() == d["primID"].shape[0]
    exp = rays.copy()
    exp["geomID"][hit] = d["geomID"]
    exp["primID"][hit] = d["primID"]
    tuv = d["tuv"]
    for k, f in enumerate(("tfar", "u", "v")):
        exp[f][hit] = tuv[:, k].view(np.float32)
    ng = d["Ng"]
    for k, f in enumerate(("Ng_x", "Ng_y", "Ng_z")):
        exp[f][hit] = ng[:, k].view(np.float32)
    return exp


def _with_shadow(out, d, light_seed):
    shadow, _ = W.shadow_rays(out["expected"], seed=light_seed)
    out["shadow"] = shadow
    out["occluded"] = np.unpackbits(d["occluded_bits"])[:shadow.shape[0]].astype(bool)
    return out


def heightfield256(robust=False):
    """Config 0: heightfield 256^2, every pinhole ray of the 1024^2 view (robust: every
    16th ray of a RTC_SCENE_FLAG_ROBUST scene)."""
    name = "ref_robust_heightfield256.npz" if robust else "ref_heightfield256.npz"
    d = np.load(os.path.join(GOLDEN, name))
    rays = W.camera_rays(1024, 1024)
    if robust:
        rays = np.ascontiguousarray(rays[::int(d["every"])])
    out = dict(meshes=[W.heightfield(256)], rays=rays, expected=_expand(d, rays), robust=robust)
    return _with_shadow(out, d, int(d["light_seed"]))


def soup4M_sample(verts_idx=None, rays_all=None):
    """Config 1: the 4M soup and the fixture's 100k-ray sample of its 16M rays
    (`rays_all`: the 16M rays when the caller has them already)."""
    d = np.load(os.path.join(GOLDEN, "ref_soup4M_sample.npz"))
    sel = d["sel"]
    rays_all = W.sphere_rays(16_000_000) if rays_all is None else rays_all
    rays = np.ascontiguousarray(rays_all[sel])
    meshes = [verts_idx if verts_idx is not None else W.gaussian_soup(4_000_000)]
    out = dict(meshes=meshes, rays=rays, expected=_expand(d, rays), robust=False, sel=sel)
    return _with_shadow(out, d, int(d["light_seed"]))
