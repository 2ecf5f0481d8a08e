"""Times the reference (its own sources compiled by oracle/ref.mk: x86 AVX2 path, internal
tasking) and the oracle port (oracle/oracle.c, scalar C) on identical rays, on the same
host cores with the same thread count, and writes oracle/ref_rates.json.

TEST / MEASUREMENT INFRASTRUCTURE. The benchmark's CPU arm runs the reference where it
is built (this x86 container). The GPU host is an aarch64 machine without the
reference's source tree, so there the arm times the port and scales it by the
reference/port rate ratio measured here, and says so in its output.

Reference timing follows the plan of the reference's benchmarks (tutorials/verify/
verify.cpp:4867-5016): T host threads, each calling rtcIntersect1M / rtcOccluded1M on
disjoint 1024-ray chunks with an INCOHERENT context; median of 5 runs, rays reset
between runs. Build: the reference builder's own BENCHMARK_BUILD time at T threads
(kernels/bvh/bvh.cpp:173-179) against the port's single-threaded builder.

Run from the repository root:   python oracle/measure_ref_rates.py
"""
import json
import os
import platform
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "embree-aarch64_gb300"))
sys.path.insert(0, HERE)

import oracle_ffi  # noqa: E402
import ref_ffi  # noqa: E402
from rtcgb import workloads as W  # noqa: E402

RUNS = 5


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def timed(fn, rays, runs=RUNS):
    ts = []
    for _ in range(runs):
        r = rays.copy()
        t = time.perf_counter()
        fn(r)
        ts.append(time.perf_counter() - t)
    return rays.shape[0] / statistics.median(ts) / 1e6, r


def measure(name, meshes, rays, threads, light_seed):
    ref = ref_ffi.RefScene(meshes, threads=threads)
    t = time.perf_counter()
    orc = oracle_ffi.OracleScene([(g, v, i) for g, (v, i) in enumerate(meshes)])
    port_build_s = time.perf_counter() - t
    ntris = sum(i.shape[0] for _, i in meshes)
    out = {"rays": int(rays.shape[0]), "tris": int(ntris)}
    rc, hits = timed(lambda r: ref.intersect(r, nthreads=threads), rays)
    pc, _ = timed(lambda r: orc.intersect(r, nthreads=threads), rays)
    shadow, _ = W.shadow_rays(hits, seed=light_seed)
    active = shadow["tnear"] <= shadow["tfar"]
    rs, _ = timed(lambda r: ref.occluded(r, nthreads=threads), shadow)
    ps, _ = timed(lambda r: orc.occluded(r, nthreads=threads), shadow)
    frac = float(active.mean())
    out["closest"] = {"reference_Mrays_per_s": rc, "port_Mrays_per_s": pc, "ref_over_port": rc / pc}
    # shadow rates count active rays only (the benchmark's convention)
    out["shadow"] = {"reference_Mrays_per_s": rs * frac, "port_Mrays_per_s": ps * frac, "ref_over_port": rs / ps,
                     "active_rays": int(active.sum())}
    b = ref.build_stats or {}
    out["build"] = {"reference_builder_s": b.get("builder_s"), "reference_commit_s": ref.commit_s,
                    "reference_threads": threads, "port_build_s": port_build_s, "port_threads": 1,
                    "reference_Mtris_per_s": ntris / b["builder_s"] / 1e6 if b.get("builder_s") else None,
                    "port_Mtris_per_s": ntris / port_build_s / 1e6}
    ref.close()
    orc.close()
    print(name, json.dumps(out))
    return out


def main():
    assert ref_ffi.build(), "the reference source tree is needed (EMBREE_REF_SRC)"
    threads = os.cpu_count()
    res = {"host": cpu_model(), "machine": platform.machine(), "threads": threads,
           "reference": "Embree 3.12.1 (embree-aarch64) own sources, x86 AVX2 path, internal tasking (oracle/ref.mk)",
           "port": "oracle/oracle.c (scalar C restatement)", "runs": RUNS, "workloads": {}}
    v, i = W.gaussian_soup(4_000_000)
    rays = np.ascontiguousarray(W.sphere_rays(16_000_000)[:1_000_000])
    res["workloads"]["soup4M"] = measure("soup4M", [(v, i)], rays, threads, 13)
    res["workloads"]["soup4M"]["sample"] = "first 1,000,000 of the 16M uniform-sphere rays"
    v, i = W.heightfield(256)
    res["workloads"]["heightfield256"] = measure("heightfield256", [(v, i)], W.camera_rays(1024, 1024), threads, 23)
    res["workloads"]["heightfield256"]["sample"] = "all 1,048,576 pinhole rays of the 1024x1024 view"
    with open(os.path.join(HERE, "ref_rates.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
