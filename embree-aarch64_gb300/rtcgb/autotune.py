"""Autotuner: picks, per workload, the knobs that change speed but not results,
by running candidates through the library's C ABI on the GPU.

  * build options of a scene (rtcNewDevice keys): triangles per leaf
    (gpu.leaf_max), the sort key -- its scaling (gpu.morton axis / cube) and its
    width (gpu.morton_bits 63 or 30: 8 or 4 sort passes; batched scenes put the
    geometry ID above it) -- and the PLOC search radius (gpu.ploc_radius);
  * the traversal's launch shape (threads per CTA, resident CTAs per SM,
    shared-memory stack depth, refill threshold): rtcgbTuneSceneTraversal
    times every compiled shape on the workload's rays and sets the fastest on
    the scene; the pick is also a device key (gpu.trace_shape) for scenes
    made later;
  * the learned proposer's treelet count (rtcgbNewProposerEx).

`tune` (batched scenes) tunes the build options on a sample of the batch and
then the launch shape on the sample built with the chosen options; `tune_scene`
tunes the launch shape of one committed scene; `tune_treelets` the treelet
budget of a proposer."""
import statistics
import time

import numpy as np

from . import api

CANDIDATES = [
    {"gpu.leaf_max": 1, "gpu.morton": "axis", "gpu.ploc_radius": 1, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 2, "gpu.morton": "axis", "gpu.ploc_radius": 1, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 1, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 4, "gpu.morton": "cube", "gpu.ploc_radius": 1, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 1, "gpu.morton": "axis", "gpu.ploc_radius": 4, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 4, "gpu.morton_bits": 63},
    {"gpu.leaf_max": 1, "gpu.morton": "axis", "gpu.ploc_radius": 1, "gpu.morton_bits": 30},
    {"gpu.leaf_max": 2, "gpu.morton": "axis", "gpu.ploc_radius": 1, "gpu.morton_bits": 30},
    {"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 1, "gpu.morton_bits": 30},
]

# the device's own defaults: always measured first, so the pick is never a
# configuration that measured slower than running untuned
DEFAULT = {}

TREELET_CANDIDATES = (1024, 2048, 4096)


def config_string(cand, base=""):
    toks = [f"{k}={v}" for k, v in cand.items()]
    return ",".join(([base] if base else []) + toks)


def _batched_scene(dev, meshes):
    sc = api.Scene(dev)
    sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    sc.commit()
    return sc


def measure_build_options(meshes, rays, start, cand, base_config="", repeats=2):
    """Median device build time and batched closest-hit kernel time (ms) of the
    sample scenes under one candidate's build options (default launch shape)."""
    dev = api.Device(config_string(cand, base_config).encode())
    sc = _batched_scene(dev, meshes)
    build = []
    for _ in range(repeats):
        sc.commit()  # every commit of an unchanged scene rebuilds
        build.append(sc.build_stats()["build_ms"])
    trace = []
    for _ in range(repeats + 1):
        work = rays.copy()
        sc.intersect_batched(work, start)
        trace.append(api.last_query_stats()["kernel_ms"])
    sc.release()
    dev.release()
    return float(np.median(build)), float(np.median(trace[1:]))


def tune(meshes, rays, start, base_config="", repeats=2, candidates=CANDIDATES, shape_repeats=5):
    """Batched scenes.  meshes: [(verts, idx)] of the sample scenes; rays: host
    RTCRayHit array of their rays, start: batch boundaries.  Returns (the chosen
    device configuration as a dict -- build options plus gpu.trace_shape -- and
    the per-candidate timings in ms -- the device defaults first -- with the
    launch-shape timings of the chosen build options last, under "shapes")."""
    results = []
    for cand in [DEFAULT] + [c for c in candidates if c != DEFAULT]:
        b, t = measure_build_options(meshes, rays, start, cand, base_config, repeats)
        results.append({"config": cand, "build_ms": b, "trace_ms": t, "total_ms": b + t})
    best = dict(min(results, key=lambda r: r["total_ms"])["config"])
    # launch shape on the sample built with the chosen options
    dev = api.Device(config_string(best, base_config).encode())
    sc = _batched_scene(dev, meshes)
    pick, ms = sc.tune_traversal(rays, batch_start=start, repeats=shape_repeats)
    sc.release()
    dev.release()
    best["gpu.trace_shape"] = pick
    return best, results + [{"shapes": {"ms": ms, "pick": pick}}]


def tune_scene(scene, rays=None, occluded=True, repeats=5, ptr=None, count=None, stride=80):
    """Launch shape of one committed scene for its rays (host RTCRayHit array, or
    device records at `ptr`): closest-hit plus, with `occluded`, any-hit time on
    the same records.  Sets the pick on the scene; returns a record of the pick
    and of every shape's median time."""
    pick, ms = scene.tune_traversal(rays, occluded=occluded, repeats=repeats, ptr=ptr, count=count, stride=stride)
    shapes = api.traversal_shapes()
    return {"pick": pick, "shape": shapes[pick], "default_ms": ms[0], "pick_ms": ms[pick],
            "ms_per_shape": ms, "shapes": shapes, "objective": "closest + occluded" if occluded else "closest"}


def tune_treelets(scene, records, queries, count=None, candidates=TREELET_CANDIDATES, seed=7, epochs=2,
                  batch=16384, lr=5e-3, repeats=2):
    """Treelet budget of the scene's learned proposer.  For each candidate a
    proposer is cut and trained on `records` (closest-hit records, host array or
    device pointer with `count`), then `queries` -- a list of callables
    q(proposer) -> kernel ms, each one learned query of the workload -- are
    timed.  Returns (the budget with the least total time, per-candidate
    results).  Proposers are released."""
    results = []
    for nt in candidates:
        prop = api.Proposer(scene, seed=seed, max_treelets=nt)
        t = time.perf_counter()
        if isinstance(records, int):
            st = prop.train(records, epochs=epochs, batch=batch, lr=lr, count=count)
        else:
            st = prop.train(records, epochs=epochs, batch=batch, lr=lr)
        train_s = time.perf_counter() - t
        times = []
        for _ in range(repeats):
            times.append(sum(q(prop) for q in queries))
        results.append({"max_treelets": nt, "treelets": st["num_treelets"], "top4": st["top4"], "train_s": train_s,
                        "query_ms": float(statistics.median(times))})
        prop.release()
    best = min(results, key=lambda r: r["query_ms"])
    return best["max_treelets"], results
