"""Writes the golden fixtures of this directory.

The reference cannot be built here (it needs its CMake build and generated
headers) and is not a Python package, so these vectors are produced by the
oracle (oracle/oracle.c, the C restatement of the reference path, itself
pinned by the reference's known-answer tests in tests/test_oracle.py).  They
freeze, for small seeded scenes, the scene buffers, the input rays and the
expected closest-hit records and occlusion flags, so that the GPU library and
the oracle are both checked against fixed data.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "embree-aarch64_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle_ffi  # noqa: E402
from rtcgb import rays as R  # noqa: E402
from rtcgb import workloads as W  # noqa: E402

HIT_FIELDS = ("tfar", "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID")


def case(name, verts, idx, rays):
    orc = oracle_ffi.OracleScene([(0, verts, idx)])
    hits = rays.copy()
    orc.intersect(hits)
    shadow, _ = W.shadow_rays(hits, seed=5)
    occ = shadow.copy()
    orc.occluded(occ)
    orc.close()
    out = {"verts": verts, "idx": idx, "rays": rays.view(np.uint8), "shadow_rays": shadow.view(np.uint8),
           "occluded": (occ["tfar"] == -np.inf)}
    for f in HIT_FIELDS:
        out["hit_" + f] = hits[f]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    n_hit = int((hits["geomID"] != 0xFFFFFFFF).sum())
    print(f"{path}: {idx.shape[0]} triangles, {rays.shape[0]} rays, {n_hit} hits, {int(out['occluded'].sum())} occluded")


def grown_soup(n, seed, factor=30.0):
    """A Gaussian-mixture soup whose triangles are scaled about their centroids
    (the generator's edge lengths suit millions of triangles; a few thousand
    need larger ones to be hit)."""
    v, i = W.gaussian_soup(n, seed=seed)
    t = v[i].astype(np.float64)                     # (n, 3 vertices, 3)
    c = t.mean(axis=1, keepdims=True)
    t = c + factor * (t - c)
    return t.reshape(-1, 3).astype(np.float32), np.arange(3 * n, dtype=np.uint32).reshape(n, 3)


def main():
    # heightfield with soup clusters above it: camera rays hit both, and the
    # clusters occlude part of the shadow rays
    hv, hi = W.heightfield(24, seed=1)
    sv, si = grown_soup(1500, seed=3)
    sv[:, 2] = sv[:, 2] * 0.3 + 0.15
    v = np.concatenate([hv, sv]).astype(np.float32)
    i = np.concatenate([hi, si + hv.shape[0]]).astype(np.uint32)
    case("terrain_camera48", v, i, W.camera_rays(48, 48))
    # a soup seen from outside, plus uniform-sphere rays from inside its box
    v, i = grown_soup(2500, seed=11)
    cam = W.camera_rays(40, 40, eye=(0.5, -1.0, 0.5), look=(0.5, 0.5, 0.5))
    case("soup_camera40_sphere", v, i, np.concatenate([cam, W.sphere_rays(1000, seed=12)]))


if __name__ == "__main__":
    main()
