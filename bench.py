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
                        cores: the reference library compiled from its own
                        sources (oracle/ref.mk) where its source tree is present;
                        elsewhere the oracle port, scaled by the reference/port
                        rate ratio measured on identical rays
                        (oracle/ref_rates.json), both rates reported

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
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-proposer comparison")
    ap.add_argument("--learned-scale", type=float, default=1.0, help="fraction of the learned workload (tests only)")
    ap.add_argument("--no-animated", action="store_true", help="skip the animated path-tracing run")
    ap.add_argument("--animated-scale", type=float, default=1.0, help="fraction of the animated workload (tests only)")
    ap.add_argument("--frames", type=int, default=64, help="frames of the animated path-tracing run")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-scenes run")
    ap.add_argument("--no-heightfield", action="store_true", help="skip the heightfield-view run")
    ap.add_argument("--batched-scale", type=float, default=1.0, help="fraction of the batched workload (tests only)")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default traversal launch shape (skip rtcgbTuneSceneTraversal)")
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


TRAFFIC_SUMMARY = os.path.join("profiles", "trace_closest_soup4M.md")


def profiled_traffic():
    """DRAM bytes (read + written) per launch of the closest-hit traversal on
    the 4M-soup / 16M-ray workload, from the committed ncu summary of that
    kernel and workload (its `traffic_bytes_per_launch = N` line); None
    without it."""
    try:
        with open(os.path.join(REPO, TRAFFIC_SUMMARY)) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch"):
                    return int(line.split("=")[1].strip().replace(",", ""))
    except (OSError, ValueError):
        pass
    return None


def max_over_ranks(x, dist=None, device="cpu"):
    """The maximum of a per-rank float over all ranks (the slowest rank sets
    the job's time); x itself without a process group."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds):
    """Whole-job rate in millions of units per second: every rank processed
    units_per_rank units (weak scaling) in at most `seconds`."""
    return world * units_per_rank / seconds / 1e6


# ---------------------------------------------------------------------------
# CPU arm: the reference itself where it is built, else the oracle port scaled
# by the reference/port rate ratio measured on identical rays
# ---------------------------------------------------------------------------

REF_RATES = os.path.join(REPO, "oracle", "ref_rates.json")


def _ref_ffi():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ref_ffi
    return ref_ffi if ref_ffi.available() else None


def ref_over_port(workload_key, query):
    """Rate ratio reference / port measured on identical rays and threads on the host
    that has the reference built (oracle/measure_ref_rates.py -> oracle/ref_rates.json)."""
    try:
        with open(REF_RATES) as f:
            d = json.load(f)
        w = d["workloads"][workload_key][query]
        return float(w["ref_over_port"]), (f"{REF_RATES.split(REPO + os.sep)[1]}: reference and port on identical "
                                           f"rays, {d['threads']} threads of {d['host']} ({d['machine']})")
    except (OSError, KeyError, ValueError):
        return None, "no measured ratio"


def cpu_rate(verts, idx, rays, budget_s, shadow=False, orc=None, robust=False, workload_key="soup4M"):
    """Mrays/s of the reference path on all host threads over a bounded sample of
    `rays`: the reference library itself (1024-ray chunks, INCOHERENT context) where
    oracle/_ref is built; otherwise the oracle port, whose rate is reported as
    measured and, in `value`, scaled by the measured reference/port ratio."""
    cores = os.cpu_count() or 1
    ref = _ref_ffi() if not robust else None
    if orc is None:
        t0 = time.perf_counter()
        if ref is not None:
            orc = ref.RefScene([(verts, idx)], threads=cores)
        else:
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import oracle_ffi
            orc = oracle_ffi.OracleScene([(0, verts, idx)], robust=robust)
        orc._build_wall_s = time.perf_counter() - t0
    is_ref = not hasattr(orc, "stats")
    query = orc.occluded if shadow else orc.intersect
    n0 = min(rays.shape[0], 65536)
    probe = rays[:n0].copy()
    t = time.perf_counter()
    query(probe)
    rate = n0 / max(time.perf_counter() - t, 1e-6)
    n = int(min(rays.shape[0], max(n0, rate * budget_s)))
    sample = np.ascontiguousarray(rays[:n].copy())
    t = time.perf_counter()
    query(sample)
    dt = time.perf_counter() - t
    measured = n / dt / 1e6
    out = dict(unit="Mrays/s", cores=cores, build_s=getattr(orc, "_build_wall_s", 0.0),
               sample=f"first {n} of {rays.shape[0]} rays of the same workload, all {cores} host threads")
    if is_ref:
        out.update(value=measured, kind="reference",
                   isa="x86 AVX2 build of the reference's own sources (oracle/ref.mk), internal tasking, "
                       "1024-ray chunks, INCOHERENT context")
        if orc.build_stats:
            out["reference_builder"] = orc.build_stats
    else:
        factor, src = ref_over_port(workload_key, "shadow" if shadow else "closest")
        out.update(kind="port", port_measured=measured, value=measured * factor if factor else measured,
                   scaled_by_ref_over_port=factor, factor_source=src,
                   note="the reference's sources are not on this host; value = the port's measured rate x the "
                        "reference/port ratio measured on identical rays where the reference is built")
    return out, orc, sample


def run_reference(args, rank, world):
    if rank != 0:
        return
    verts, idx, rays, label = workload(args.workload, args.scale)
    key = "soup4M" if args.workload == "soup" else "heightfield256"
    per = []
    base, orc, _ = cpu_rate(verts, idx, rays, 1.0, robust=args.robust, workload_key=key)
    for s in range(args.warmup + args.steps):
        r, orc, sample = cpu_rate(verts, idx, rays, max(1.0, args.cpu_seconds / max(1, args.steps)), orc=orc,
                                  workload_key=key)
        if s >= args.warmup:
            per.append(r)
    value = statistics.median(p["value"] for p in per)
    cb = {k: per[-1][k] for k in per[-1] if k not in ("build_s", "reference_builder")}
    cb["value"] = value
    if "port_measured" in cb:
        cb["port_measured"] = statistics.median(p["port_measured"] for p in per)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(sample.shape[0]) / (value * 1e6) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": label, "rays_per_step": int(sample.shape[0])},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if cb["kind"] == "reference":
        rb = base.get("reference_builder") or {}
        line["build"] = {"commit_s": base["build_s"], "builder_s": rb.get("builder_s"), "sah": rb.get("sah"),
                         "threads": base["cores"], "source": "BENCHMARK_BUILD line of the reference builder"}
    else:
        st = orc.stats()
        line["build"] = {"seconds": base["build_s"], "Mtris_per_s": st.num_prims / base["build_s"] / 1e6,
                         "sah": st.sah, "threads": 1, "source": "oracle port builder (single thread)"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

MLP_FLOPS_PER_RAY = 2 * (32 * 64 + 64 * 64 + 64 * 64 + 64 * 4096)  # forward pass of the proposer


def run_learned(api, dev, torch, stream, scale, steps, warmup, cpu_seconds):
    """Learned proposer vs plain traversal on the ambient-occlusion workload:
    724x724 heightfield + 300k soup triangles, 1024x1024 primary view, 8
    cosine-weighted AO rays (tfar 0.05) and 8 diffuse bounce rays per primary
    hit.  The proposer is trained on ~10M closest-hit records the plain
    traversal logs for rays drawn with other seeds, with the treelet budget the
    autotuner picks for this workload.  Times include the
    proposer's inference (the learned calls' kernel time covers inference +
    seeded traversal)."""
    from rtcgb import rays as R
    from rtcgb import workloads as W
    cells = max(16, int(round(724 * math.sqrt(scale))))
    res = max(32, int(round(1024 * math.sqrt(scale))))
    soup = max(1000, int(300_000 * scale))
    sc = api.Scene(dev)
    for v, i in W.ao_scene(cells=cells, soup_tris=soup, seed=3):
        sc.add_mesh(v, i)
    sc.commit()
    ntris = sc.build_stats()["num_prims"]
    prim = W.camera_rays(res, res)
    sc.intersect(prim)
    nhit = int((prim["geomID"] != 0xFFFFFFFF).sum())
    # training log (other seeds than the measured rays): 5 AO + 5 bounce rays per hit
    ao_t, _ = W.hemisphere_rays(prim, 5, seed=31, tfar=0.05)
    b_t, _ = W.hemisphere_rays(prim, 5, seed=32)
    log = torch.from_numpy(np.concatenate([ao_t, b_t]).view(np.uint8)).cuda()
    nlog = log.numel() // 80
    del ao_t, b_t
    sc.intersect_ptr(log.data_ptr(), nlog, 80)
    # treelet budget for this workload, timed on 2 AO + 2 bounce rays per hit drawn
    # with other seeds (speed only: every budget returns the plain traversal's hits)
    from rtcgb import autotune
    tq = []
    for rec, stride, fn in ((W.hemisphere_rays(prim, 2, seed=51, tfar=0.05, record=R.RAY_DTYPE)[0], 48, "occluded_ptr"),
                            (W.hemisphere_rays(prim, 2, seed=52)[0], 80, "intersect_ptr")):
        tq.append((torch.from_numpy(rec.view(np.uint8)).cuda(), rec.shape[0], stride, fn))

    def tuning_query(q):
        src, n, stride, fn = q

        def run(p):
            w = src.clone()
            getattr(p, fn)(w.data_ptr(), n, stride)
            return api.last_query_stats()["kernel_ms"]
        return run

    max_treelets, treelet_tuning = autotune.tune_treelets(sc, log.data_ptr(), [tuning_query(q) for q in tq],
                                                          count=nlog)
    del tq
    prop = api.Proposer(sc, seed=7, max_treelets=max_treelets)
    torch.cuda.synchronize()
    t = time.perf_counter()
    st = prop.train(log.data_ptr(), epochs=2, batch=16384, lr=5e-3, count=nlog)
    train_s = time.perf_counter() - t
    del log
    ao, _ = W.hemisphere_rays(prim, 8, seed=41, tfar=0.05, record=R.RAY_DTYPE)
    bounce, _ = W.hemisphere_rays(prim, 8, seed=42)

    def timed(fn, pristine, n, stride):
        work = torch.empty_like(pristine)
        ms = []
        for k in range(warmup + steps):
            work.copy_(pristine)
            fn(work.data_ptr(), n, stride)
            if k >= warmup:
                ms.append(api.last_query_stats()["kernel_ms"])
        q = api.last_query_stats()
        return work, statistics.median(ms), q

    out = {"workload": f"heightfield {cells}x{cells} + {soup} soup triangles ({ntris} tris), {res}x{res} view, "
                       f"8 AO rays (tfar 0.05) + 8 bounce rays per hit",
           "train": {"records": int(nlog), "labelled": int(st["samples"]), "epochs": 2, "batch": 16384,
                     "seconds": train_s, "loss": st["loss"], "top1": st["top1"], "top4": st["top4"],
                     "treelets": int(st["num_treelets"])},
           "autotune": {"max_treelets": max_treelets, "candidates": treelet_tuning,
                        "objective": "learned AO + bounce kernel time on 2 + 2 rays per hit (other seeds)"}}
    total_plain = total_learned = 0.0
    for name, rays, stride, plain_fn, learned_fn in (
            ("ao", ao, 48, sc.occluded_ptr, prop.occluded_ptr),
            ("bounce", bounce, 80, sc.intersect_ptr, prop.intersect_ptr)):
        n = rays.shape[0]
        pristine = torch.from_numpy(rays.view(np.uint8)).cuda()
        w_plain, ms_plain, _ = timed(plain_fn, pristine, n, stride)
        w_learn, ms_learn, q = timed(learned_fn, pristine, n, stride)
        a = w_plain.cpu().numpy().view(rays.dtype)
        b = w_learn.cpu().numpy().view(rays.dtype)
        if stride == 48:
            mism = int((a.view(np.uint8).reshape(n, 48) != b.view(np.uint8).reshape(n, 48)).any(1).sum())
            answered = int((a["tfar"] < 0).sum())
        else:
            same = R.hits_equal_bits(a, b)
            tie = (~same) & (a["tfar"].view(np.uint32) == b["tfar"].view(np.uint32))
            mism = int((~(same | tie)).sum())
            answered = int((a["geomID"] != 0xFFFFFFFF).sum())
        # proposer inference alone
        treelets = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        api.load().rtcgbProposerPredict(prop.h, ctypes_ptr(pristine.data_ptr()), n, stride,
                                        ctypes_ptr(treelets.data_ptr()))
        e0.record(stream)
        api.load().rtcgbProposerPredict(prop.h, ctypes_ptr(pristine.data_ptr()), n, stride,
                                        ctypes_ptr(treelets.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        inf_ms = e0.elapsed_time(e1)
        out[name] = {"rays": n, "plain_Mrays_per_s": n / (ms_plain * 1e-3) / 1e6,
                     "learned_Mrays_per_s": n / (ms_learn * 1e-3) / 1e6, "speedup": ms_plain / ms_learn,
                     "mismatches": mism, "answered_by_proposal": int(q["proposal_hits"]),
                     "hits_or_occluded": answered, "inference_ms": inf_ms,
                     "mlp_TFLOPs": MLP_FLOPS_PER_RAY * n / (inf_ms * 1e-3) / 1e12}
        total_plain += ms_plain
        total_learned += ms_learn
        del pristine, w_plain, w_learn, treelets
    out["speedup_all_rays"] = total_plain / total_learned
    out["mismatches"] = out["ao"]["mismatches"] + out["bounce"]["mismatches"]
    prop.release()
    sc.release()
    if cpu_seconds > 0:  # the oracle on the same two ray sets, all host threads
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_ffi
        orc = oracle_ffi.OracleScene([(g, v, i) for g, (v, i) in
                                      enumerate(W.ao_scene(cells=cells, soup_tris=soup, seed=3))])
        cpu = {}
        for name, rays, shadow in (("ao", ao, True), ("bounce", bounce, False)):
            r, _, _ = cpu_rate(None, None, rays, cpu_seconds / 2, shadow=shadow, orc=orc)
            cpu[name] = r["value"]
        orc.close()
        cores = os.cpu_count() or 1
        out["cpu_baseline"] = {"value": (ao.shape[0] + bounce.shape[0]) / (ao.shape[0] / cpu["ao"] / 1e6 +
                                                                           bounce.shape[0] / cpu["bounce"] / 1e6) / 1e6,
                               "unit": "Mrays/s", "cores": cores, "kind": "port",
                               "ao_Mrays_per_s": cpu["ao"], "bounce_Mrays_per_s": cpu["bounce"],
                               "sample": f"leading rays of the AO and bounce sets (~{cpu_seconds / 2:.0f} s each), "
                                         f"all {cores} host threads"}
    torch.cuda.empty_cache()
    return out


def run_animated(api, dev, torch, scale, frames):
    """Animated path tracing: the 4M-triangle soup moves every frame (0.002 *
    sin(2 pi (f/60 + x)) along per-triangle random normals), the BVH is refitted
    and 4-bounce diffuse paths are traced from a 1920x1080 camera with
    compaction between bounces, each frame one CUDA graph.  Run twice over the
    same frames: plain traversal only, and adaptive (learned proposer retrained
    every 8 frames from the frames' own closest-hit logs; the plain graph runs
    while the proposer's hit rate is below 20%)."""
    from rtcgb import workloads as W
    ntris = max(1000, int(4_000_000 * scale))
    width, height = max(64, int(1920 * math.sqrt(scale))), max(36, int(1080 * math.sqrt(scale)))
    verts, idx = W.gaussian_soup(ntris, seed=11)
    dv = torch.from_numpy(verts).cuda()
    di = torch.from_numpy(idx.view(np.int32)).cuda()
    sc = api.Scene(dev)
    gid = sc.add_mesh_device(dv.data_ptr(), verts.shape[0], di.data_ptr(), ntris, quality=api.RTC_BUILD_QUALITY_REFIT)
    sc.commit()
    out = {"workload": f"gaussian soup {ntris} tris animated, {width}x{height} camera, 4 diffuse bounces, {frames} frames",
           "frame": "one CUDA graph: displacement + refit + camera rays + 4 x (trace, shade, compact)"}
    images = {}
    for mode in ("plain", "adaptive"):
        dv.copy_(torch.from_numpy(verts))
        pt = api.PathTracer(sc, width, height, bounces=4)
        pt.animate_soup(gid, amplitude=0.002, seed=14)
        prop = None
        if mode == "adaptive":
            prop = api.Proposer(sc, seed=7)
            pt.set_proposer(prop)
        pt.render(0)  # captures the graph(s) outside the measured frames
        rays = ms = 0.0
        learned_frames, hit_rates, train_s = 0, [], 0.0
        use_learned = False
        launches0 = api.launch_count()
        for f in range(frames):
            st = pt.render(f, learned=use_learned)
            rays += st["rays"]
            ms += st["frame_ms"]
            if st["errors"]:
                raise RuntimeError(f"frame {f}: error flags {st['errors']:#x}")
            if prop is not None:
                if st["learned"]:
                    learned_frames += 1
                    rate = st["proposal_hits"] / max(1, st["rays"])
                    hit_rates.append(rate)
                    use_learned = rate >= 0.2
                if f % 8 == 0:  # online retraining from this frame's log
                    t = time.perf_counter()
                    pt.train_proposer(epochs=2, batch=16384, lr=5e-3)
                    train_s += time.perf_counter() - t
                    use_learned = True
        images[mode] = pt.image()
        out[mode] = {"Mrays_per_s": rays / (ms * 1e-3) / 1e6, "frames_per_s": frames / (ms * 1e-3),
                     "ms_per_frame": ms / frames, "rays": int(rays), "gpu_launches": int(api.launch_count() - launches0)}
        if prop is not None:
            out[mode].update({"learned_frames": learned_frames,
                              "mean_proposal_hit_rate": float(np.mean(hit_rates)) if hit_rates else None,
                              "training_s": train_s})
            prop.release()
        pt.release()
    out["speedup"] = out["adaptive"]["Mrays_per_s"] / out["plain"]["Mrays_per_s"]
    out["identical_last_image"] = bool((images["plain"].view(np.uint32) == images["adaptive"].view(np.uint32)).all())
    sc.release()
    del dv, di
    torch.cuda.empty_cache()
    return out


def _device_rays(torch, n_cam, n_sph, eye, look, seed):
    """RTCRayHit records on the device: an n_cam-ray pinhole view (60 degrees)
    and n_sph uniform-sphere rays from the unit cube."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    side = max(1, int(math.isqrt(n_cam)))
    n_cam = side * side
    rec = torch.zeros((n_cam + n_sph, 20), dtype=torch.float32, device="cuda")
    eye_t = torch.tensor(eye, dtype=torch.float32, device="cuda")
    w = torch.tensor(look, dtype=torch.float32, device="cuda") - eye_t
    w = w / w.norm()
    u = torch.linalg.cross(w, torch.tensor([0.0, 0.0, 1.0], device="cuda"))
    u = u / u.norm()
    v = torch.linalg.cross(u, w)
    th = math.tan(math.radians(30.0))
    px = (torch.arange(side, device="cuda", dtype=torch.float32) + 0.5) / side * 2 - 1
    sy, sx = torch.meshgrid(-px, px, indexing="ij")
    d = w + th * (sx.reshape(-1, 1) * u + sy.reshape(-1, 1) * v)
    rec[:n_cam, 0:3] = eye_t
    rec[:n_cam, 4:7] = d
    rec[n_cam:, 0:3] = torch.rand((n_sph, 3), generator=g, device="cuda")
    ds = torch.randn((n_sph, 3), generator=g, device="cuda")
    rec[n_cam:, 4:7] = ds / ds.norm(dim=1, keepdim=True)
    rec[:, 8] = float("inf")
    ints = rec.view(torch.int32)
    ints[:, 9] = -1
    ints[:, 17:20] = -1
    return rec


def flush_l2(torch, buf):
    """Writes a buffer larger than the 129 MB L2 so the next launch starts cold."""
    buf.fill_(0)


def run_heightfield(api, dev, torch, stream, steps, warmup, cpu_seconds, tune=True):
    """The heightfield view: a 256x256-cell value-noise heightfield (131,072
    triangles), 1024x1024 pinhole primary rays through rtcIntersect1M, then
    shadow rays from the hits through rtcOccluded1M.  The rays (80 MB) fit in
    L2, so a 256 MB buffer is written between timed launches.  The traversal's
    launch shape is tuned on the view's rays first.  Every ray is compared with
    the oracle, which is also timed as the CPU baseline."""
    from rtcgb import rays as R
    from rtcgb import workloads as W
    verts, idx = W.heightfield(256)
    rays = W.camera_rays(1024, 1024)
    n = rays.shape[0]
    sc = api.Scene(dev)
    sc.add_mesh(verts, idx)
    t = time.perf_counter()
    sc.commit()
    first_s = time.perf_counter() - t
    builds = []
    for _ in range(3):
        sc.commit()
        builds.append(sc.build_stats()["build_ms"])
    bst = sc.build_stats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    pristine = torch.from_numpy(rays.view(np.uint8)).cuda()
    work = torch.empty_like(pristine)
    tuning = None
    if tune:
        from rtcgb import autotune
        tuning = autotune.tune_scene(sc, ptr=pristine.data_ptr(), count=n, occluded=True, repeats=5)
    kms = []
    for k in range(warmup + steps):
        work.copy_(pristine)
        flush_l2(torch, flush)
        sc.intersect_ptr(work.data_ptr(), n, 80)
        if k >= warmup:
            kms.append(api.last_query_stats()["kernel_ms"])
    out_rays = work.cpu().numpy().view(R.RAYHIT_DTYPE)
    shadow, _ = W.shadow_rays(out_rays, seed=13)
    active = int(np.sum(shadow["tnear"] <= shadow["tfar"]))
    sh_pristine = torch.from_numpy(shadow.view(np.uint8)).cuda()
    sh_work = torch.empty_like(sh_pristine)
    sms = []
    for k in range(warmup + steps):
        sh_work.copy_(sh_pristine)
        flush_l2(torch, flush)
        sc.occluded_ptr(sh_work.data_ptr(), n, 48)
        if k >= warmup:
            sms.append(api.last_query_stats()["kernel_ms"])
    sh_out = sh_work.cpu().numpy().view(R.RAY_DTYPE)
    # end to end through the public call on pinned host memory
    host = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
    src = torch.from_numpy(rays.view(np.uint8))
    e2e = []
    for k in range(warmup + steps):
        host.copy_(src)
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        t = time.perf_counter()
        sc.intersect_ptr(host.data_ptr(), n, 80)
        if k >= warmup:
            e2e.append(time.perf_counter() - t)
    kernel_ms, sh_ms = statistics.median(kms), statistics.median(sms)
    out = {"workload": f"value-noise heightfield 256x256 cells ({idx.shape[0]} tris), 1024x1024 pinhole closest-hit "
                       "rays + shadow rays from the hits",
           "l2": "rays fit in L2: a 256 MB buffer is written before every timed launch",
           "build": {"device_ms": float(statistics.median(builds)), "first_commit_wall_ms": first_s * 1e3,
                     "Mtris_per_s": float(bst["num_prims"] / (statistics.median(builds) * 1e-3) / 1e6),
                     "sah": bst["sah"], "sah_exact_boxes": bst["sah_exact"], "leaf_max": bst["leaf_max"]},
           "closest": {"kernel_ms": kernel_ms, "Mrays_per_s": n / (kernel_ms * 1e-3) / 1e6,
                       "hit_rate": float(np.mean(out_rays["geomID"] != 0xFFFFFFFF))},
           "shadow": {"kernel_ms": sh_ms, "Mrays_per_s": active / (sh_ms * 1e-3) / 1e6, "active_rays": active},
           "e2e": {"Mrays_per_s": n / statistics.median(e2e) / 1e6, "h2d_bytes_per_step": n * 80,
                   "d2h_bytes_per_step": n * 36, "host_buffer": "pinned"},
           "autotune": tuning}
    del pristine, work, sh_pristine, sh_work, flush, host
    torch.cuda.empty_cache()
    sc.release()
    if cpu_seconds > 0:
        base, cpu_scene, sample = cpu_rate(verts, idx, rays, cpu_seconds, workload_key="heightfield256")
        if cpu_scene is not None and not hasattr(cpu_scene, "stats"):
            cpu_scene.close()
        out["cpu_baseline"] = {k: v for k, v in base.items() if k not in ("build_s", "reference_builder")}
        # every ray against the oracle (same arithmetic: same-triangle hits bit-identical)
        orc = oracle_scene([(verts, idx)])
        ref = rays.copy()
        orc.intersect(ref)
        sh_ref = shadow.copy()
        orc.occluded(sh_ref)
        out["parity"] = classified_parity(orc, rays, out_rays, ref)
        out["parity"]["shadow_rays"] = n
        out["parity"]["identical_occlusion"] = int(((sh_out["tfar"] < 0) == (sh_ref["tfar"] < 0)).sum())
        # every ray against the reference's own outputs (tests/golden/ref_heightfield256.npz)
        out["parity_vs_reference"] = fixture_parity(orc, out_rays, "heightfield256")
        ref_sah = reference_sah("heightfield256")
        out["build"]["sah_oracle_restatement"] = orc.stats().sah
        out["build"]["sah_reference_builder"] = ref_sah or orc.stats().sah
        out["build"]["sah_ratio"] = bst["sah"] / out["build"]["sah_reference_builder"]
        out["build"]["sah_ratio_exact_boxes"] = bst["sah_exact"] / out["build"]["sah_reference_builder"]
        orc.close()
    return out


def run_batched(api, dev_config, torch, scale, steps, warmup, cpu_seconds):
    """512 independent scenes (log-uniform 1k-200k triangles, ~20M in total;
    even scenes noise heightfields of matching grid size, odd scenes Gaussian
    soups), 32 rays per triangle (half a pinhole view, half uniform-sphere
    rays), all built by one commit of a batched scene and traced by one
    persistent launch.  Build parameters come from the autotuner run on a
    sample of the scenes."""
    from rtcgb import autotune
    from rtcgb import rays as R
    from rtcgb import workloads as W
    rng = np.random.default_rng(21)
    nscenes = max(4, int(round(512 * scale)))
    counts = np.exp(rng.uniform(math.log(1000), math.log(200_000), nscenes)).astype(np.int64)
    t = time.perf_counter()
    meshes, kinds = [], []
    for k, n in enumerate(counts):
        if k % 2 == 0:
            cells = max(8, int(round(math.sqrt(n / 2))))
            meshes.append(W.heightfield(cells, seed=int(rng.integers(1, 10 ** 6))))
            kinds.append("heightfield")
        else:
            meshes.append(W.gaussian_soup(int(n), seed=int(rng.integers(1, 10 ** 6))))
            kinds.append("soup")
    gen_s = time.perf_counter() - t
    tris = np.array([i.shape[0] for _, i in meshes], np.int64)
    # autotune on 16 scenes with an eighth of their rays (host copies)
    sample = list(range(0, nscenes, max(1, nscenes // 16)))[:16]
    s_parts, s_start = [], [0]
    for k in sample:
        n = int(32 * tris[k] // 8)
        eye, look = ((0.5, -0.5, 0.6), (0.5, 0.5, 0.0)) if kinds[k] == "heightfield" else ((0.5, -1.0, 0.5), (0.5, 0.5, 0.5))
        r = _device_rays(torch, n // 2, n - n // 2, eye, look, 100 + k).cpu().numpy().view(R.RAYHIT_DTYPE).reshape(-1)
        s_parts.append(r)
        s_start.append(s_start[-1] + r.shape[0])
    best, tuning = autotune.tune([meshes[k] for k in sample], np.concatenate(s_parts), np.array(s_start, np.uint32),
                                 base_config=dev_config)
    dev = api.Device(autotune.config_string(best, dev_config).encode())
    sc = api.Scene(dev)
    sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    t = time.perf_counter()
    sc.commit()
    first_commit_s = time.perf_counter() - t
    builds = []
    for _ in range(2):
        sc.commit()
        builds.append(sc.build_stats()["build_ms"])
    bst = sc.build_stats()
    # rays on the device, batch by batch
    parts, start = [], [0]
    for k in range(nscenes):
        n = int(32 * tris[k])
        eye, look = ((0.5, -0.5, 0.6), (0.5, 0.5, 0.0)) if kinds[k] == "heightfield" else ((0.5, -1.0, 0.5), (0.5, 0.5, 0.5))
        r = _device_rays(torch, n // 2, n - n // 2, eye, look, 1000 + k)
        parts.append(r)
        start.append(start[-1] + r.shape[0])
    pristine = torch.cat(parts)
    del parts
    start = np.array(start, np.uint32)
    nrays = int(start[-1])
    work = torch.empty_like(pristine)
    kms = []
    for k in range(warmup + steps):
        work.copy_(pristine)
        sc.intersect_batched(None, start, ptr=work.data_ptr(), count=nrays)
        if k >= warmup:
            kms.append(api.last_query_stats()["kernel_ms"])
    kernel_ms = statistics.median(kms)
    out = {"workload": f"{nscenes} scenes ({kinds.count('heightfield')} heightfields, {kinds.count('soup')} soups), "
                       f"{int(tris.sum())} tris, {nrays} rays (32 per triangle: half pinhole view, half uniform sphere)",
           "build": {"device_ms": float(statistics.median(builds)), "first_commit_wall_s": first_commit_s,
                     "Mtris_per_s": float(bst["num_prims"] / (statistics.median(builds) * 1e-3) / 1e6),
                     "ploc_iterations": bst["ploc_iterations"], "nodes": bst["num_nodes"]},
           "trace": {"kernel_ms": kernel_ms, "Mrays_per_s": nrays / (kernel_ms * 1e-3) / 1e6, "launches_per_query": 1},
           "build_plus_trace_ms": float(statistics.median(builds)) + kernel_ms,
           "autotune": {"chosen": best, "candidates": tuning, "sample_scenes": len(sample)},
           "generation_s": gen_s}
    # CPU baseline and exact-hit check: the oracle builds and traces whole
    # scenes one after another (every 8th scene, then the rest, until the time
    # budget is spent), every ray of each compared with the GPU's result
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_ffi
    res = work.cpu().numpy().view(R.RAYHIT_DTYPE).reshape(-1)
    src = pristine.cpu().numpy().view(R.RAYHIT_DTYPE).reshape(-1)
    same = total = done_tris = 0
    classes = {"near_tie": 0, "fp32_tie": 0, "grazing": 0, "unexplained": 0}
    build_s = trace_s = 0.0
    order = list(range(0, nscenes, 8)) + [k for k in range(nscenes) if k % 8]
    scenes_done = 0
    for k in order:
        if build_s + trace_s > cpu_seconds and scenes_done >= 2:
            break
        lo, hi = int(start[k]), int(start[k + 1])
        t = time.perf_counter()
        orc = oracle_ffi.OracleScene([(k, meshes[k][0], meshes[k][1])])
        build_s += time.perf_counter() - t
        ref = src[lo:hi].copy()
        t = time.perf_counter()
        orc.intersect(ref)
        trace_s += time.perf_counter() - t
        ids = (ref["geomID"] == res["geomID"][lo:hi]) & (ref["primID"] == res["primID"][lo:hi])
        same += int(ids.sum())
        # every differing ray is classified (parity rule: near tie, FP32 order tie, grazing)
        for j in np.nonzero(~ids)[0]:
            g = res[lo + j]
            c = orc.classify(src[lo + j], (g["geomID"], g["primID"], g["tfar"]),
                             (ref["geomID"][j], ref["primID"][j], ref["tfar"][j]))
            classes[c if isinstance(c, str) else "unexplained"] += 1
        total += hi - lo
        done_tris += int(tris[k])
        scenes_done += 1
        orc.close()
    cores = os.cpu_count() or 1
    out["parity_sample"] = {"scenes": scenes_done, "rays": total, "identical_ids": same,
                            "differing": total - same, "classes": classes,
                            "rule": "differing ids must be near ties (FP64, 4 ulps), FP32 order ties or grazing"}
    out["cpu_baseline"] = {"value": total / (build_s + trace_s) / 1e6, "unit": "Mrays/s (build + trace)",
                           "cores": cores, "kind": "port",
                           "sample": f"{scenes_done} whole scenes ({done_tris} tris, {total} rays), built one after "
                                     f"another by the single-threaded oracle builder and traced on {cores} threads",
                           "build_Mtris_per_s": done_tris / build_s / 1e6, "trace_Mrays_per_s": total / trace_s / 1e6}
    out["gpu_build_plus_trace_Mrays_per_s"] = nrays / ((float(statistics.median(builds)) + kernel_ms) * 1e-3) / 1e6
    # the same step as one CUDA graph: ray restore copy + rebuild of every BVH +
    # batched closest-hit query (rtcgbNewBatchedFrame), replayed
    separate = work.clone()  # the separate calls' results, kept on the device for the comparison
    # the restore copy alone (part of every frame)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    copy_ms = []
    for _ in range(3):
        c0.record()
        work.copy_(pristine)
        c1.record()
        torch.cuda.synchronize()
        copy_ms.append(c0.elapsed_time(c1))
    frame = api.BatchedFrame(sc, work.data_ptr(), nrays, start, pristine_ptr=pristine.data_ptr())
    fms = []
    for k in range(warmup + steps):
        fst = frame.replay()
        if k >= warmup:
            fms.append(fst["frame_ms"])
    # bitwise: the records' integer fields (e.g. instID = 0xFFFFFFFF) are NaN as floats
    same = bool(torch.equal(work.view(torch.int32), separate.view(torch.int32)))
    del separate
    out["graph"] = {"frame": "ray restore copy + rebuild of all BVHs (PLOC rounds and collapse levels in two "
                             "cooperative launches that end them on the device) + batched closest-hit query, "
                             "one CUDA graph launch",
                    "ms_per_step": float(statistics.median(fms)),
                    "Mrays_per_s": nrays / (statistics.median(fms) * 1e-3) / 1e6,
                    "restore_copy_ms": float(statistics.median(copy_ms)),
                    "separate_parts_ms": float(statistics.median(copy_ms)) + float(statistics.median(builds)) + kernel_ms,
                    "graph_nodes": fst["graph_nodes"], "ploc_rounds_device_loop": fst["ploc_rounds"],
                    "levels_device_loop": fst["levels"], "build_status": fst["status"],
                    "identical_to_separate_calls": same}
    frame.release()
    sc.release()
    dev.release()
    del pristine, work
    torch.cuda.empty_cache()
    return out


REF_BUILD_STATS_NAME = os.path.join("tests", "golden", "ref_build_stats.json")


def reference_sah(scene_key):
    """SAH of the reference builder's own tree on a benchmark scene, from the committed
    BENCHMARK_BUILD record (tests/golden/make_golden.py ran the reference)."""
    try:
        with open(os.path.join(REPO, REF_BUILD_STATS_NAME)) as f:
            return float(json.load(f)["scenes"][scene_key]["sah"])
    except (OSError, KeyError, ValueError):
        return None


def oracle_scene(meshes, robust=False):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_ffi
    return oracle_ffi.OracleScene([(g, v, i) for g, (v, i) in enumerate(meshes)], robust=robust)


def classified_parity(orc, rays_in, got, ref):
    """geomID/primID of `got` against `ref` on the same input rays: identical, or a
    classified tie (FP64 near tie within 4 ulps, FP32 order tie, grazing); anything
    else is counted as unexplained. t/u/v: largest relative difference of same-triangle hits."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from parity import compare_closest
    rep = compare_closest(orc, rays_in, got, ref)
    out = {k: rep[k] for k in ("n", "hits", "id_mismatch", "near_tie", "fp32_tie", "grazing", "max_rel_tuv",
                               "same_hit_bit_identical")}
    out["unexplained"] = len(rep["failures"])
    out["identical_ids"] = rep["n"] - rep["id_mismatch"]
    return out


def fixture_parity(orc, got_all, which, rays_all=None):
    """The GPU's results on the rays of a reference-made fixture (tests/golden) against
    the reference's own outputs."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import refgold
    case = (refgold.soup4M_sample(verts_idx=(None, None), rays_all=rays_all) if which == "soup4M"
            else refgold.heightfield256())
    got = got_all[case["sel"]] if which == "soup4M" else got_all
    rep = classified_parity(orc, case["rays"], got, case["expected"])
    rep["fixture"] = os.path.join("tests", "golden", "ref_soup4M_sample.npz" if which == "soup4M"
                                  else "ref_heightfield256.npz")
    return rep


def ctypes_ptr(p):
    import ctypes
    return ctypes.c_void_p(p)


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
    # where the replayed build's time goes: the same build on a device that stamps its phases
    pdev = api.Device(f"gpu.device={local},gpu.build_phases=1{',' + args.config if args.config else ''}".encode())
    psc = api.Scene(pdev, flags=api.RTC_SCENE_FLAG_ROBUST if args.robust else 0)
    psc.add_mesh(verts, idx)
    for _ in range(4):
        psc.commit()
    build_phases = psc.build_phases()
    psc.release()
    pdev.release()

    pristine = torch.from_numpy(rays.view(np.uint8)).cuda()
    work = torch.empty_like(pristine)
    # the traversal's launch shape for this workload (closest + any hit on its rays)
    tuning = None
    if not args.no_tune:
        from rtcgb import autotune
        tuning = autotune.tune_scene(sc, ptr=pristine.data_ptr(), count=nrays, occluded=True, repeats=3)

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
    total_ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    if dist:
        dist.barrier()
    ms_per_step = total_ms / args.steps
    value = job_rate(nrays, world, ms_per_step * 1e-3)
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
        e2e_s = max_over_ranks(statistics.median(times), dist, "cuda")
        e2e = {"value": job_rate(nrays, world, e2e_s), "unit": "Mrays/s", "h2d_bytes_per_step": int(q["h2d_bytes"]),
               "d2h_bytes_per_step": int(q["d2h_bytes"]), "ms_per_step": e2e_s * 1e3,
               "host_buffer": "pinned", "host_access": int(api.load().rtcgbGetDeviceHostAccess(dev.h)),
               "path": "rtcIntersect1M on host memory (" + (args.config or "gpu.host_rays default") + ")"}

    # DRAM traffic of the same kernel on the same workload (ncu), when this is that workload
    traffic = profiled_traffic() if (args.workload == "soup" and args.scale == 1.0 and not args.robust
                                     and not args.config) else None
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
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "traffic_source": TRAFFIC_SUMMARY + " (ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                           "same kernel and workload)" if traffic else None,
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
                      "sah_exact_boxes": bst["sah_exact"], "leaf_max": bst["leaf_max"],
                      "nodes": bst["num_nodes"], "depth": bst["depth"], "ploc_iterations": bst["ploc_iterations"],
                      "bvh_MB": bst["bvh_bytes"] / 1e6,
                      "phases_us": build_phases or None,
                      "phases_source": "rtcgbGetSceneBuildPhases on a second device with gpu.build_phases=1 "
                                       "(device timestamps between the phases of the replayed build)"},
            "autotune": tuning,
            "learned": None, "animated": None, "batched": None, "heightfield": None,
        }

    # the other configurations (learned, animated, batched, heightfield) are
    # single-GPU workloads: they run at N = 1 only, so that under torchrun no
    # rank waits at the final barrier while rank 0 runs them; the CPU baseline
    # is rank 0's at N = 1 only as well
    single = world == 1
    if single and not args.no_learned:
        del pristine, work, sh_pristine, sh_work
        torch.cuda.empty_cache()
        line["learned"] = run_learned(api, dev, torch, stream, args.learned_scale, args.steps, args.warmup,
                                      0.0 if args.no_cpu else min(6.0, args.cpu_seconds))
    if single and not args.no_animated:
        line["animated"] = run_animated(api, dev, torch, args.animated_scale, args.frames)
    if single and not args.no_batched:
        line["batched"] = run_batched(api, f"gpu.device={local}{',' + args.config if args.config else ''}", torch,
                                      args.batched_scale, args.steps, args.warmup,
                                      0.0 if args.no_cpu else min(8.0, args.cpu_seconds))
    if single and not args.no_heightfield:
        line["heightfield"] = run_heightfield(api, dev, torch, stream, args.steps, args.warmup,
                                              0.0 if args.no_cpu else min(3.0, args.cpu_seconds),
                                              tune=not args.no_tune)

    if single and not args.no_cpu:
        key = "soup4M" if args.workload == "soup" else "heightfield256"
        base, cpu_scene, sample = cpu_rate(verts, idx, rays, args.cpu_seconds, robust=args.robust, workload_key=key)
        line["cpu_baseline"] = {k: v for k, v in base.items() if k not in ("build_s", "reference_builder")}
        orc = cpu_scene if hasattr(cpu_scene, "stats") else oracle_scene([(verts, idx)], args.robust)
        # the GPU builder's SAH over the reference builder's own (BENCHMARK_BUILD, committed)
        ref_sah = reference_sah(key) if args.scale == 1.0 and not args.robust else None
        orc_sah = orc.stats().sah
        line["build"]["sah_oracle_restatement"] = orc_sah
        line["build"]["sah_reference_builder"] = ref_sah if ref_sah else orc_sah
        line["build"]["sah_reference_source"] = (REF_BUILD_STATS_NAME + " (the reference builder's BENCHMARK_BUILD)"
                                                 if ref_sah else "oracle restatement of the reference builder")
        line["build"]["sah_ratio"] = bst["sah"] / line["build"]["sah_reference_builder"]
        line["build"]["sah_ratio_exact_boxes"] = bst["sah_exact"] / line["build"]["sah_reference_builder"]
        line["build"]["cpu_build_s"] = base["build_s"]
        # every sampled ray against the CPU arm's result, differences classified
        n = sample.shape[0]
        line["parity"] = classified_parity(orc, rays[:n], out[:n], sample)
        line["parity"]["against"] = base["kind"]
        if args.workload == "soup" and args.scale == 1.0 and not args.robust and rank == 0:
            line["parity_vs_reference"] = fixture_parity(orc, out, "soup4M", rays_all=rays)
        if orc is not cpu_scene:
            orc.close()
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
