"""Benchmark of the GB300 triangle ray-query path (one JSON line on stdout).

Workload (default): the 4M-triangle Gaussian-mixture soup with 16M
uniform-sphere rays -- closest hit through rtcIntersect1M -- plus the shadow
rays from those hits through rtcOccluded1M and the GPU build through
rtcCommitScene.  A step is one rtcIntersect1M over the 16M rays with the rays
already in HBM (the rays are restored from a pristine HBM copy inside the
step, since the query writes them in place).  The rays (1.28 GB per step) are
larger than the 129 MB L2.

Arms:
  --impl gb (default)   the GPU library through its C ABI
  --impl reference      the reference path's CPU implementation on the host
                        cores (the oracle port: the reference itself cannot be
                        built here without its cmake build system)

Multi-GPU (torchrun): every rank builds the same scene and traces its own 16M
rays (weak scaling, no collective on the data path); the time is the maximum
over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "embree-aarch64_gb300"))

import numpy as np  # noqa: E402

METRIC = "Mrays/s closest/shadow, learned vs plain GPU, exact hits; build Mtris/s"
RAY_BYTES_CLOSEST = 84   # read 48 B RTCRay, write 4 B tfar + 32 B RTCHit
RAY_BYTES_SHADOW = 52    # read 48 B RTCRay, write 4 B tfar
NODE_BYTES = 80
TRI_BYTES = 48


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--workload", default="soup", choices=["soup", "heightfield"])
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the full workload (tests only)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--robust", action="store_true", help="RTC_SCENE_FLAG_ROBUST scene (Pluecker test)")
    ap.add_argument("--config", default="", help="extra rtcNewDevice config tokens, e.g. gpu.leaf_max=2")
    return ap.parse_args()


def workload(name, scale, rank=0):
    from rtcgb import workloads as W
    if name == "soup":
        ntris = max(64, int(4_000_000 * scale))
        nrays = max(1024, int(16_000_000 * scale))
        verts, idx = W.gaussian_soup(ntris)
        rays = W.sphere_rays(nrays, seed=12 + 1000 * rank)
        label = f"gaussian-mixture soup {ntris} tris, {nrays} uniform-sphere closest-hit rays + shadow rays"
    else:
        cells = max(8, int(round(256 * math.sqrt(scale))))
        res = max(16, int(round(1024 * math.sqrt(scale))))
        verts, idx = W.heightfield(cells)
        rays = W.camera_rays(res, res)
        label = f"value-noise heightfield {idx.shape[0]} tris, {res}x{res} primary closest-hit rays + shadow rays"
    return verts, idx, rays, label


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


# ---------------------------------------------------------------------------
# CPU arm (the oracle port of the reference path)
# ---------------------------------------------------------------------------

def cpu_rate(verts, idx, rays, budget_s, shadow=False, orc=None, robust=False):
    """Mrays/s of the oracle on all host threads over a bounded sample."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_ffi
    t0 = time.perf_counter()
    if orc is None:
        orc = oracle_ffi.OracleScene([(0, verts, idx)], robust=robust)
    build_s = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    n0 = min(rays.shape[0], 65536)
    probe = rays[:n0].copy()
    t = time.perf_counter()
    (orc.occluded if shadow else orc.intersect)(probe)
    rate = n0 / max(time.perf_counter() - t, 1e-6)
    n = int(min(rays.shape[0], max(n0, rate * budget_s)))
    sample = np.ascontiguousarray(rays[:n].copy())
    t = time.perf_counter()
    (orc.occluded if shadow else orc.intersect)(sample)
    dt = time.perf_counter() - t
    return dict(value=n / dt / 1e6, unit="Mrays/s", cores=cores, kind="port",
                sample=f"first {n} of {rays.shape[0]} rays of the same workload, all {cores} host threads",
                build_s=build_s), orc, sample


def run_reference(args, rank, world):
    if rank != 0:
        return
    verts, idx, rays, label = workload(args.workload, args.scale)
    per = []
    base, orc, _ = cpu_rate(verts, idx, rays, 1.0, robust=args.robust)
    for s in range(args.warmup + args.steps):
        r, orc, sample = cpu_rate(verts, idx, rays, max(1.0, args.cpu_seconds / max(1, args.steps)), orc=orc)
        if s >= args.warmup:
            per.append(r)
    value = statistics.median(p["value"] for p in per)
    st = orc.stats()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(sample.shape[0]) / (value * 1e6) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": label, "rays_per_step": int(sample.shape[0])},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": per[-1]["cores"], "kind": "port",
                         "sample": per[-1]["sample"]},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "build": {"seconds": base["build_s"], "Mtris_per_s": st.num_prims / base["build_s"] / 1e6,
                  "sah": st.sah, "threads": 1},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_gpu(args, rank, world):
    import torch
    from rtcgb import api
    from rtcgb import rays as R
    from rtcgb import workloads as W

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    verts, idx, rays, label = workload(args.workload, args.scale, rank)
    nrays = rays.shape[0]
    dev = api.Device(f"gpu.device={local}{',' + args.config if args.config else ''}".encode())
    stream = torch.cuda.current_stream()
    api.set_thread_stream(stream.cuda_stream)
    sc = api.Scene(dev, flags=api.RTC_SCENE_FLAG_ROBUST if args.robust else 0)
    if args.robust:
        label += " (robust scene: Pluecker test)"
    sc.add_mesh(verts, idx)
    t = time.perf_counter()
    sc.commit()
    build_wall = time.perf_counter() - t
    builds = []
    for _ in range(3):  # rebuilds: the first commit includes one-time setup
        t = time.perf_counter()
        sc.commit()
        builds.append((time.perf_counter() - t, sc.build_stats()["build_ms"]))
    bst = sc.build_stats()
    build_ms = statistics.median(b[1] for b in builds)
    build_wall_ms = statistics.median(b[0] for b in builds) * 1e3

    pristine = torch.from_numpy(rays.view(np.uint8)).cuda()
    work = torch.empty_like(pristine)

    def step():
        work.copy_(pristine)
        sc.intersect_ptr(work.data_ptr(), nrays, 80)
        return api.last_query_stats()["kernel_ms"]

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = api.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    kms = [step() for _ in range(args.steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = api.launch_count() - launches0
    clk = clocks.stop()
    total_ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    ms_per_step = total_ms / args.steps
    value = world * nrays / (ms_per_step * 1e-3) / 1e6
    kernel_ms = statistics.mean(kms)

    # counting run (untimed): traversal work for the algorithmic byte model
    api.set_counting(True)
    step()
    cnt = api.last_query_stats()
    api.set_counting(False)
    out = work.cpu().numpy().view(R.RAYHIT_DTYPE)
    alg_bytes = RAY_BYTES_CLOSEST * cnt["rays"] + NODE_BYTES * cnt["nodes"] + TRI_BYTES * cnt["tris"]
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9
    compulsory = RAY_BYTES_CLOSEST * nrays / (kernel_ms * 1e-3) / 1e9
    peak, peak_src = peaks()

    # shadow rays from the closest hits
    shadow, _ = W.shadow_rays(out, seed=13)
    active = int(np.sum(shadow["tnear"] <= shadow["tfar"]))
    sh_pristine = torch.from_numpy(shadow.view(np.uint8)).cuda()
    sh_work = torch.empty_like(sh_pristine)
    sh_ms = []
    for k in range(args.warmup + args.steps):
        sh_work.copy_(sh_pristine)
        sc.occluded_ptr(sh_work.data_ptr(), shadow.shape[0], 48)
        if k >= args.warmup:
            sh_ms.append(api.last_query_stats()["kernel_ms"])
    shadow_mrays = active / (statistics.median(sh_ms) * 1e-3) / 1e6
    api.set_counting(True)
    sh_work.copy_(sh_pristine)
    sc.occluded_ptr(sh_work.data_ptr(), shadow.shape[0], 48)
    scnt = api.last_query_stats()
    api.set_counting(False)
    sh_bytes = RAY_BYTES_SHADOW * scnt["rays"] + NODE_BYTES * scnt["nodes"] + TRI_BYTES * scnt["tris"]

    # end to end: the public call on pinned host memory (H2D + trace + D2H)
    e2e = None
    if not args.no_e2e:
        host = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
        src = torch.from_numpy(rays.view(np.uint8))
        times = []
        for k in range(args.warmup + args.steps):
            host.copy_(src)
            t = time.perf_counter()
            sc.intersect_ptr(host.data_ptr(), nrays, 80)
            dt = time.perf_counter() - t
            if k >= args.warmup:
                times.append(dt)
        q = api.last_query_stats()
        e2e_s = statistics.median(times)
        if dist:
            t = torch.tensor([e2e_s], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": world * nrays / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": int(q["h2d_bytes"]),
               "d2h_bytes_per_step": int(q["d2h_bytes"]), "ms_per_step": e2e_s * 1e3,
               "host_buffer": "pinned", "host_access": int(api.load().rtcgbGetDeviceHostAccess(dev.h)),
               "path": "rtcIntersect1M on host memory (" + (args.config or "gpu.host_rays default") + ")"}

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": label, "tris": int(idx.shape[0]), "rays_per_gpu": int(nrays),
                       "step": "restore rays from a pristine HBM copy + rtcIntersect1M over all rays",
                       "l2": "inputs larger than L2 (1.28 GB of rays per step)" if nrays * 80 > 129e6 else
                       "inputs smaller than L2"},
            "clocks": clk, "e2e": e2e, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                         "kernel": "k_trace<closest> (gb_trace.cu)", "kernel_ms": kernel_ms,
                         "bytes_per_launch": alg_bytes, "compulsory_GBps": compulsory,
                         "nodes_per_ray": cnt["nodes"] / max(1, cnt["rays"]),
                         "tris_per_ray": cnt["tris"] / max(1, cnt["rays"])},
            "closest": {"Mrays_per_s_kernel": nrays / (kernel_ms * 1e-3) / 1e6,
                        "hit_rate": float(np.mean(out["geomID"] != 0xFFFFFFFF))},
            "shadow": {"Mrays_per_s": shadow_mrays, "active_rays": active, "kernel_ms": statistics.median(sh_ms),
                       "achieved_GBps": sh_bytes / (statistics.median(sh_ms) * 1e-3) / 1e9,
                       "occluded_rate": float(np.mean(sh_work.cpu().numpy().view(R.RAY_DTYPE)["tfar"] == -np.inf))},
            "build": {"device_ms": build_ms, "wall_ms": build_wall_ms, "first_commit_wall_ms": build_wall * 1e3,
                      "Mtris_per_s": bst["num_prims"] / (build_ms * 1e-3) / 1e6, "sah": bst["sah"],
                      "nodes": bst["num_nodes"], "depth": bst["depth"], "ploc_iterations": bst["ploc_iterations"],
                      "bvh_MB": bst["bvh_bytes"] / 1e6},
            "learned": None,
        }

    if rank == 0 and not args.no_cpu:
        base, orc, sample = cpu_rate(verts, idx, rays, args.cpu_seconds, robust=args.robust)
        st = orc.stats()
        line["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line["build"]["sah_reference_builder"] = st.sah
        line["build"]["sah_ratio"] = bst["sah"] / st.sah
        line["build"]["reference_builder_s_1thread"] = base["build_s"]
        # exact-hit check of the sampled rays against the oracle
        n = sample.shape[0]
        same = (out["geomID"][:n] == sample["geomID"]) & (out["primID"][:n] == sample["primID"])
        line["parity"] = {"rays": int(n), "identical_ids": int(same.sum()), "differing_ids": int((~same).sum())}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    sc.release()
    dev.release()


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
