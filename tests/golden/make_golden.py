"""Writes the golden fixtures of this directory from the reference itself.

The reference's own sources (Embree 3.12.1 / embree-aarch64, x86 AVX2 path, internal
tasking) are compiled in place by oracle/ref.mk into oracle/_ref/libembree3_ref.so and
driven through their public C API by oracle/ref_harness.c (oracle/ref_ffi.py):
rtcNewDevice -> rtcNewScene -> rtcNewGeometry(TRIANGLE) -> rtcSetSharedGeometryBuffer ->
rtcCommitScene -> rtcIntersect1M / rtcOccluded1M on 1024-ray chunks with an INCOHERENT
context (kernels/common/rtcore.cpp:595-624, 848-875). Every expected output below is
what that library returned; the inputs are regenerated from seeds (rtcgb/workloads.py)
by the tests and stored only where they are small.

  terrain_camera48.npz, soup_camera40_sphere.npz
      two small scenes with their buffers, rays and the full expected RTCRayHit
      records + occlusion flags of shadow rays built from the expected hits.
  ref_heightfield256.npz
      the 256x256-cell heightfield (131,072 triangles) and all 1,048,576 pinhole
      rays of the 1024x1024 view: hit mask, primID, t/u/v and Ng bits of every hit,
      and the occlusion flags of the shadow rays built from those hits.
  ref_soup4M_sample.npz
      the 4M-triangle Gaussian-mixture soup with its 16M uniform-sphere rays: a
      seeded sample of 100,000 of the rays (their indices), their geomID/primID, t/u/v
      and Ng bits, and the occlusion flags of their shadow rays.
  ref_robust_heightfield256.npz
      RTC_SCENE_FLAG_ROBUST (Pluecker test, kernels/common/scene.cpp:119-125) on the
      heightfield, every 16th pinhole ray.
  ref_build_stats.json
      the reference builder's own BENCHMARK_BUILD line (kernels/bvh/bvh.cpp:173-179:
      SAH, bytes, build time at the host's thread count) for the benchmark scenes.

Run from the repository root (needs the reference source tree; EMBREE_REF_SRC
overrides its default location):   python tests/golden/make_golden.py
"""
import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "embree-aarch64_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import ref_ffi  # noqa: E402
from rtcgb import workloads as W  # noqa: E402

HIT_FIELDS = ("tfar", "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID")
SOUP_SAMPLE_SEED = 99
SOUP_SAMPLE = 100_000
ROBUST_EVERY = 16
# the heightfield's shadow rays go to a low light, (0.694, 0.641, 0.129), so that the
# terrain shadows itself (the soup's light, seed 13, is above every hill)
HF_LIGHT_SEED = 23


def grown_soup(n, seed, factor=30.0):
    """A Gaussian-mixture soup whose triangles are scaled about their centroids
    (the generator's edge lengths suit millions of triangles; a few thousand
    need larger ones to be hit)."""
    v, i = W.gaussian_soup(n, seed=seed)
    t = v[i].astype(np.float64)                     # (n, 3 vertices, 3)
    c = t.mean(axis=1, keepdims=True)
    t = c + factor * (t - c)
    return t.reshape(-1, 3).astype(np.float32), np.arange(3 * n, dtype=np.uint32).reshape(n, 3)


def small_scenes():
    """The two small fixture scenes: (name, verts, idx, rays)."""
    # heightfield with soup clusters above it: camera rays hit both, and the
    # clusters occlude part of the shadow rays
    hv, hi = W.heightfield(24, seed=1)
    sv, si = grown_soup(1500, seed=3)
    sv[:, 2] = sv[:, 2] * 0.3 + 0.15
    v = np.concatenate([hv, sv]).astype(np.float32)
    i = np.concatenate([hi, si + hv.shape[0]]).astype(np.uint32)
    yield "terrain_camera48", v, i, W.camera_rays(48, 48)
    # a soup seen from outside, plus uniform-sphere rays from inside its box
    v, i = grown_soup(2500, seed=11)
    cam = W.camera_rays(40, 40, eye=(0.5, -1.0, 0.5), look=(0.5, 0.5, 0.5))
    yield "soup_camera40_sphere", v, i, np.concatenate([cam, W.sphere_rays(1000, seed=12)])


def soup_sample_indices(n_rays=16_000_000):
    rng = np.random.default_rng(SOUP_SAMPLE_SEED)
    return np.sort(rng.choice(n_rays, SOUP_SAMPLE, replace=False)).astype(np.uint32)


def _hits_compact(hits):
    """Hit mask + per-hit fields of a closest-hit result (as uint32 bit patterns)."""
    hit = hits["geomID"] != 0xFFFFFFFF
    out = {"hit_bits": np.packbits(hit), "n": np.uint32(hits.shape[0])}
    out["geomID"] = hits["geomID"][hit]
    out["primID"] = hits["primID"][hit]
    out["tuv"] = np.stack([hits[f][hit].view(np.uint32) for f in ("tfar", "u", "v")], -1)
    out["Ng"] = np.stack([hits[f][hit].view(np.uint32) for f in ("Ng_x", "Ng_y", "Ng_z")], -1)
    return out


def _stats(sc):
    st = dict(sc.build_stats or {})
    st["commit_s"] = sc.commit_s
    return st


def main():
    assert ref_ffi.build(), "the reference source tree is needed (EMBREE_REF_SRC)"
    threads = os.cpu_count()
    stats = {"host": platform.processor() or platform.machine(), "threads": threads,
             "isa": "AVX2 (x86, oracle/ref.mk)", "version": "3.12.1", "scenes": {}}

    for name, v, i, rays in small_scenes():
        sc = ref_ffi.RefScene([(v, i)])
        hits = rays.copy()
        sc.intersect(hits)
        shadow, _ = W.shadow_rays(hits, seed=5)
        occ = shadow.copy()
        sc.occluded(occ)
        out = {"verts": v, "idx": i, "rays": rays.view(np.uint8), "shadow_rays": shadow.view(np.uint8),
               "occluded": (occ["tfar"] == -np.inf)}
        for f in HIT_FIELDS:
            out["hit_" + f] = hits[f]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: {i.shape[0]} tris, {rays.shape[0]} rays, {int((hits['geomID'] != 0xFFFFFFFF).sum())} hits,"
              f" {int(out['occluded'].sum())} occluded")
        sc.close()

    # config 0: heightfield 256^2, 1024^2 pinhole rays, every ray
    v, i = W.heightfield(256)
    rays = W.camera_rays(1024, 1024)
    sc = ref_ffi.RefScene([(v, i)])
    stats["scenes"]["heightfield256"] = _stats(sc)
    hits = rays.copy()
    sc.intersect(hits)
    shadow, _ = W.shadow_rays(hits, seed=HF_LIGHT_SEED)
    occ = shadow.copy()
    sc.occluded(occ)
    out = _hits_compact(hits)
    out["occluded_bits"] = np.packbits(occ["tfar"] == -np.inf)
    out["light_seed"] = np.uint32(HF_LIGHT_SEED)
    np.savez_compressed(os.path.join(HERE, "ref_heightfield256.npz"), **out)
    print(f"heightfield256: {len(out['primID'])} hits, {int((occ['tfar'] == -np.inf).sum())} occluded; "
          f"{stats['scenes']['heightfield256']}")
    sc.close()

    # robust mode on the same scene, every 16th ray
    sc = ref_ffi.RefScene([(v, i)], robust=True)
    stats["scenes"]["heightfield256_robust"] = _stats(sc)
    sub = np.ascontiguousarray(rays[::ROBUST_EVERY])
    hits = sub.copy()
    sc.intersect(hits)
    shadow, _ = W.shadow_rays(hits, seed=HF_LIGHT_SEED)
    occ = shadow.copy()
    sc.occluded(occ)
    out = _hits_compact(hits)
    out["occluded_bits"] = np.packbits(occ["tfar"] == -np.inf)
    out["every"] = np.uint32(ROBUST_EVERY)
    out["light_seed"] = np.uint32(HF_LIGHT_SEED)
    np.savez_compressed(os.path.join(HERE, "ref_robust_heightfield256.npz"), **out)
    print(f"robust heightfield256: {len(out['primID'])} hits of {sub.shape[0]}")
    sc.close()

    # config 1: 4M soup, a seeded sample of its 16M uniform-sphere rays
    v, i = W.gaussian_soup(4_000_000)
    sel = soup_sample_indices()
    rays = W.sphere_rays(16_000_000)[sel]
    sc = ref_ffi.RefScene([(v, i)])
    stats["scenes"]["soup4M"] = _stats(sc)
    hits = rays.copy()
    sc.intersect(hits)
    shadow, _ = W.shadow_rays(hits)
    occ = shadow.copy()
    sc.occluded(occ)
    out = _hits_compact(hits)
    out["sel"] = sel
    out["light_seed"] = np.uint32(13)
    out["occluded_bits"] = np.packbits(occ["tfar"] == -np.inf)
    np.savez_compressed(os.path.join(HERE, "ref_soup4M_sample.npz"), **out)
    print(f"soup4M sample: {len(out['primID'])} hits of {rays.shape[0]}; {stats['scenes']['soup4M']}")
    sc.close()

    # SAH yardsticks of the other benchmark scenes
    for key, meshes in (("soup1M", [W.gaussian_soup(1_000_000)]),
                        ("heightfield724", [W.heightfield(724)]),
                        ("ao_scene", W.ao_scene())):
        sc = ref_ffi.RefScene(meshes)
        stats["scenes"][key] = _stats(sc)
        print(key, stats["scenes"][key])
        sc.close()

    with open(os.path.join(HERE, "ref_build_stats.json"), "w") as f:
        json.dump(stats, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
