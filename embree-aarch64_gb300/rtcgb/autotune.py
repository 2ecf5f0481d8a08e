"""Autotuner for batched scenes: picks the build parameters (triangles per
leaf, Morton scaling of the sort key, PLOC search radius) that give the
shortest build + trace time on a sample of the batch, by running each
candidate through the library's C ABI on the GPU.

Candidates are device configurations (rtcNewDevice keys gpu.leaf_max,
gpu.morton and gpu.ploc_radius); the traversal's launch shape is sized by the
library from the kernel's occupancy and needs no tuning."""
import numpy as np

from . import api

CANDIDATES = [
    {"gpu.leaf_max": 1, "gpu.morton": "axis", "gpu.ploc_radius": 1},
    {"gpu.leaf_max": 2, "gpu.morton": "axis", "gpu.ploc_radius": 1},
    {"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 1},
    {"gpu.leaf_max": 4, "gpu.morton": "cube", "gpu.ploc_radius": 1},
    {"gpu.leaf_max": 1, "gpu.morton": "axis", "gpu.ploc_radius": 4},
    {"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 4},
]


def config_string(cand, base=""):
    toks = [f"{k}={v}" for k, v in cand.items()]
    return ",".join(([base] if base else []) + toks)


def tune(meshes, rays, start, base_config="", repeats=2, candidates=CANDIDATES):
    """meshes: [(verts, idx)] of the sample scenes; rays: host RTCRayHit array of
    their rays, start: batch boundaries.  Returns (best candidate, per-candidate
    timings in ms)."""
    results = []
    for cand in candidates:
        dev = api.Device(config_string(cand, base_config).encode())
        sc = api.Scene(dev)
        sc.set_batched()
        for v, i in meshes:
            sc.add_mesh(v, i)
        sc.commit()
        build = []
        for _ in range(repeats):
            sc.commit()  # every commit of an unchanged scene rebuilds
            build.append(sc.build_stats()["build_ms"])
        trace = []
        for _ in range(repeats + 1):
            work = rays.copy()
            sc.intersect_batched(work, start)
            trace.append(api.last_query_stats()["kernel_ms"])
        res = {"config": cand, "build_ms": float(np.median(build)), "trace_ms": float(np.median(trace[1:]))}
        res["total_ms"] = res["build_ms"] + res["trace_ms"]
        results.append(res)
        sc.release()
        dev.release()
    best = min(results, key=lambda r: r["total_ms"])
    return best["config"], results
