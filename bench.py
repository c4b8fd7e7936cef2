"""Benchmark: ref-views/s of the full ACMP-style pipeline on the synthetic
room scene (20 views at 1600x1200, 10 source views per reference): random
pass, planar prior, prior pass, two geometric passes and fusion.

A step reconstructs the whole scene once (20 reference views).  `value` is
measured with the images already resident in HBM; `e2e` adds, every step,
the host->device copy of the 8-bit images from pinned memory and the
device->host copy of the fused depth/normal maps.  Inputs (20 x 7.7 MB
images, 2.5 GB of per-view state) exceed L2, so no flush is needed.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gmvs|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ref-views/s at 1600x1200x10 src vs plain GPU path; p50/p99 per-view latency"
UNIT = "ref-views/s"
WORKLOAD = "room scene: 20 views 1600x1200, 10 src/view, random + planar-prior + 2 geometric passes + fusion"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gmvs", choices=["gmvs", "reference"])
    ap.add_argument("--views", type=int, default=20)
    ap.add_argument("--height", type=int, default=1200)
    ap.add_argument("--width", type=int, default=1600)
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-view comparison step")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-serving", action="store_true", help="skip the served-stream latency measurement")
    ap.add_argument("--batching", action="store_true",
                    help="measure the batching form instead: reference views of uneven size and source count "
                         "from four scenes, one launch per stage against one launch chain per view")
    ap.add_argument("--split", action="store_true",
                    help="with --profile: run every half-sweep as two kernels (neighbours, then the rest)")
    ap.add_argument("--ref-views", type=int, default=0,
                    help="with --profile: reconstruct only the first K reference views of the scene (a smaller case "
                         "for detailed ncu captures; the full scene is still rendered)")
    ap.add_argument("--profile", action="store_true",
                    help="run the pipeline once (after one warm-up) and exit: the command profiled by ncu")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": max(maxs) if maxs else None,
                "reasons": sorted(reasons), "samples": len(sms)}


# ------------------------------------------------------------ CPU baseline --
def cpu_baseline(sc, threads: int):
    """The oracle's multi-view NCC evaluation of one full 1600x1200 reference
    view with 10 sources, timed on the host cores; a pipeline reference view
    costs 144 such evaluations (random and prior passes 1 + 14*3 each, two
    geometric passes 1 + 14*2 each), which gives ref-views/s."""
    import numpy as np

    import oracle

    ref, src = sc.problems[0]
    ids = [ref] + list(src)
    from gmvs_gb300 import synthetic

    cam_args = [synthetic.camera_args(sc, i) for i in ids]
    H, W = sc.hw
    K, R = sc.K[ref], sc.R[ref]
    d = sc.depths[ref].astype(np.float64)
    ys, xs = np.mgrid[0:H, 0:W]
    X = np.stack([(xs - K[0, 2]) / K[0, 0] * d, (ys - K[1, 2]) / K[1, 1] * d, d], -1)
    n = sc.normals[ref].astype(np.float64) @ R.T
    planes = np.concatenate([n, -np.sum(n * X, -1)[..., None]], -1).astype(np.float32)
    imgs = sc.images[ids].astype(np.float32)
    prm = oracle.make_params(sampler=0)
    oracle.ncc_costs(cam_args, imgs[:, :64], planes[:64], prm, nthreads=threads)  # warm the library
    t0 = time.perf_counter()
    oracle.ncc_costs(cam_args, imgs, planes, prm, nthreads=threads)
    dt = time.perf_counter() - t0
    evals_per_view = 2 * (1 + 14 * 3) + 2 * (1 + 14 * 2)
    return {"value": 1.0 / (evals_per_view * dt), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle fp32 multi-view NCC of one {W}x{H} view x {len(src)} sources "
                      f"({dt:.2f} s) x {evals_per_view} evaluations per pipeline view"}


# ------------------------------------------------------------------ main --
def serving_run(dev) -> dict:
    """A bounded served stream: 6 room-scene jobs of 8-12 views at 640x480 to
    1600x1200 with 4-10 sources, Poisson arrivals at 2 jobs/s, continuous
    batching with two jobs in flight under the default memory budget."""
    import torch

    from gmvs_gb300 import serving

    jobs = serving.poisson_stream(6, 2.0, seed=5, views=(8, 12), src=(4, 10), device=dev)
    torch.cuda.synchronize()
    srv = serving.ReconstructionServer(device=dev, max_active=2, prior_threads=min(16, os.cpu_count() or 1))
    for j in jobs:
        srv.submit(j)
    srv.run()
    srv.close()
    st = serving.latency_stats(jobs)
    st.update({"jobs": len(jobs), "rate_jobs_per_s": 2.0, "errors": sum(j.error is not None for j in jobs),
               "mix": [f"{j.num_views}x{j.images.shape[1]}x{j.images.shape[2]}" for j in jobs]})
    return st


def job_time_ms(ms: float, world: int, device) -> float:
    """Whole-job step time: the slowest rank's (replicas run the same
    workload, so the job ends with the last one)."""
    import torch

    if world <= 1:
        return float(ms)
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def segments_run(dev) -> dict:
    """The fusion scripts' superpixel statistics on one 1600x1200 view: the
    device kernels (CUDA events, inputs resident) beside the host routine
    that restates the reference's CPU code (one core)."""
    import torch

    from gmvs_gb300 import engine
    from gmvs_gb300 import planar_initer as pi
    from gmvs_gb300.synthetic import superpixel_case

    rows, cols = 1200, 1600
    seg, planar, n, var = superpixel_case(rows, cols, 1)
    t = lambda a: torch.from_numpy(a).to(dev)
    ds, dp, dn, dv = t(seg), t(planar), t(n), t(var)
    ms_id = int(seg.max())
    ws = engine.Workspace(dev)
    out = {"size": f"{cols}x{rows}", "segments": ms_id}
    for name, dev_fn, host_fn in (
            ("fusion_planar_mask",
             lambda: engine.fusion_planar_mask(ds, dp, dn, 100, max_seg_id=ms_id, workspace=ws),
             lambda: pi.fusion_planar_mask(seg, planar, n, rows, cols, 100)),
            ("filter_by_var_map",
             lambda: engine.filter_by_var_map(dv, ds, 0.3, max_seg_id=ms_id, workspace=ws),
             lambda: pi.filter_by_var_map(var, seg, 0.3)),
            ("sliding_window_normal_7", lambda: engine.sliding_window_normal(dp, dn, 7),
             lambda: pi.sliding_window_normal(planar, n, 7))):
        for _ in range(3):
            dev_fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            dev_fn()
        e1.record()
        torch.cuda.synchronize()
        host_fn()
        t0 = time.perf_counter()
        for _ in range(3):
            host_fn()
        host_ms = (time.perf_counter() - t0) / 3 * 1000.0
        out[name] = {"device_ms": e0.elapsed_time(e1) / 10, "host_ms": host_ms}
    return out


def superpixels_run(dev, n_images: int = 16, workers: int = 8) -> dict:
    """The segmentation preprocessing (extract_superpixel.py seg_func's
    segment-id map) on 1600x1200 BGR images from host memory: one image at a
    time and `workers` at a time (wall clock, host copies included), beside
    the oracle's CPU restatement of one image (numpy + a Python merge)."""
    import torch

    import oracle.superpixel as osp
    from gmvs_gb300 import superpixel as sp
    from gmvs_gb300.synthetic import indoor_image

    imgs = [indoor_image(1200, 1600, s) for s in range(n_images)]
    for b, g in imgs[:2]:
        sp.segment_ids(b, g)
    sp.extract_many([b for b, _ in imgs[:workers]], [g for _, g in imgs[:workers]], workers=workers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b, g in imgs:
        sp.segment_ids(b, g)
    one_ms = (time.perf_counter() - t0) / n_images * 1000.0
    t0 = time.perf_counter()
    sp.extract_many([b for b, _ in imgs], [g for _, g in imgs], workers=workers)
    many_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    osp.segment_ids(imgs[0][0], imgs[0][1])
    cpu_s = time.perf_counter() - t0
    return {"size": "1600x1200", "working_size": "384x288", "images": n_images,
            "ms_per_image_one_at_a_time": one_ms, "images_per_s": n_images / many_s, "workers": workers,
            "cpu_baseline": {"s_per_image": cpu_s, "kind": "port", "cores": 1,
                             "sample": "oracle segment-id map of one 1600x1200 image"}}


BATCH_SIZES = ((480, 640), (960, 1280), (1200, 1600), (1800, 2400), (2400, 3200))


def batching_run(dev, n_views: int = 16, seed: int = 0, sizes=BATCH_SIZES) -> dict:
    """Batching form: n_views reference views drawn from four room scenes
    (seeds 0-3), each scene at a resolution drawn from `sizes` (H, W), 4-12
    sources per view; the random pass (init + 3 iterations) as one launch
    per stage over all of them, and as one launch chain per view,
    CUDA-event timed on one stream."""
    import numpy as np
    import torch

    from gmvs_gb300 import _abi, engine, synthetic

    rng = np.random.default_rng(seed)
    views, mix = [], []
    per_scene = n_views // 4
    for sd in range(4):
        H, W = sizes[int(rng.integers(len(sizes)))]
        sc = synthetic.room_scene(sd, H=H, W=W, num_views=16, num_src=12, device=dev)
        imgs = torch.from_numpy(sc.images.astype(np.float32)).to(dev)
        cams = [engine.make_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
        for ref, src in sc.problems[:per_scene]:
            n = int(rng.integers(4, 13))
            ids = [ref] + list(src)[:n]
            v = engine.ViewInputs(cams=[cams[i] for i in ids], images=[imgs[i] for i in ids],
                                  depth_min=sc.depth_range[0] * 0.6, depth_max=sc.depth_range[1] * 1.2,
                                  stream_id=ref)
            v.allocate_outputs()
            views.append(v)
            mix.append(f"{W}x{H}/{len(ids) - 1}")
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX)
    ws = engine.Workspace(dev)
    batched = engine.Plan(views, p, ws)
    singles = [engine.Plan([v], p, engine.Workspace(dev)) for v in views]
    st = torch.cuda.current_stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    ms_batched = timed(lambda: batched.launch(st))
    batched_depth = [v.out_depth.clone() for v in views]
    ms_single = timed(lambda: [pl.launch(st) for pl in singles])
    # the batched launch and the per-view chains compute one thing
    same = all(torch.equal(a, v.out_depth) for a, v in zip(batched_depth, views))
    px = sum(v.height * v.width for v in views)
    for pl in singles + [batched]:
        pl.close()
    return {"views": len(views), "megapixels": round(px / 1e6, 2), "mix": mix,
            "random_pass_ms_one_launch_per_stage": ms_batched, "random_pass_ms_one_chain_per_view": ms_single,
            "speedup": ms_single / ms_batched, "outputs_equal": same}


def main():
    args = parse()
    rank, world, local = dist_info()
    import numpy as np
    import torch

    if args.batching:
        if rank == 0:
            dev = torch.device("cuda", local)
            print(json.dumps({"batching_form": {"all_sizes": batching_run(dev),
                                                "small_sizes": batching_run(dev, sizes=BATCH_SIZES[:2])}}))
        return

    if args.impl == "reference":
        if rank != 0:
            return
        from gmvs_gb300 import synthetic

        sc = synthetic.room_scene(0, H=args.height, W=args.width, num_views=args.views,
                                  device=torch.device("cuda") if torch.cuda.is_available() else None)
        threads = os.cpu_count() or 1
        vals = []
        for _ in range(max(1, args.steps)):
            vals.append(cpu_baseline(sc, threads))
        v = statistics.median([x["value"] for x in vals])
        cb = dict(vals[0])
        cb["value"] = v
        out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1000.0 / v * args.views, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": WORKLOAD, "views": args.views, "height": args.height, "width": args.width},
               "impl": "reference", "cpu_baseline": cb,
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    from gmvs_gb300 import build as gb

    gb.build()
    from gmvs_gb300 import _abi, synthetic
    from gmvs_gb300.pipeline import ScenePipeline, scene_inputs_from_synthetic

    sc = synthetic.room_scene(0, H=args.height, W=args.width, num_views=args.views, device=dev)
    inputs = scene_inputs_from_synthetic(sc, dev)
    if args.profile and args.ref_views > 0:
        inputs.problems = inputs.problems[:args.ref_views]
    from gmvs_gb300.autotune import Autotuner

    # batched form: one persistent launch per stage over all views, each
    # pass's launch chain replayed from a CUDA graph, launch shapes picked by
    # the autotuner during the first (untimed) run
    import types

    pipe = ScenePipeline(inputs, mode="batched", prior_threads=min(16, os.cpu_count() or 1),
                         graphs=not args.profile, autotuner=None if args.profile else Autotuner(reps=1, max_views=2),
                         params=types.SimpleNamespace(split_sweep=1) if (args.profile and args.split) else None)
    if args.profile:
        pipe.run()
        torch.cuda.synchronize()
        pipe.run()
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": "ok", "views": args.views, "ref_views": len(inputs.problems),
                          "height": args.height, "width": args.width}))
        return
    for _ in range(args.warmup):
        pipe.run()
    torch.cuda.synchronize()

    # timed region: batched pipeline, images resident
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            pipe.run()
        e1.record()
        torch.cuda.synchronize()
    barrier()
    ms = job_time_ms(e0.elapsed_time(e1) / args.steps, world, dev)
    value = world * args.views / (ms / 1000.0)

    # per-stage breakdown and the dominant kernel's launch time (one instrumented step)
    torch.cuda.synchronize()
    pipe.times.seconds.clear()
    pipe.run(timed=True)
    stages = dict(pipe.times.seconds)
    sweep_ms, sweep_bytes, launches = sweep_roofline(pipe, torch)
    samples = ncc_samples_per_step(pipe)

    # end-to-end through host buffers: pinned 8-bit images in, fused maps out
    host_imgs = torch.from_numpy(sc.images).pin_memory()
    out_d = torch.empty_like(pipe.fused_depth, device="cpu").pin_memory()
    out_n = torch.empty_like(pipe.fused_normal, device="cpu").pin_memory()
    h2d = host_imgs.numel() * host_imgs.element_size()
    d2h = out_d.numel() * 4 + out_n.numel() * 4
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record()
    for _ in range(args.steps):
        inputs.images.copy_(host_imgs.to(dev, non_blocking=True).to(torch.float32))
        pipe.run()
        out_d.copy_(pipe.fused_depth, non_blocking=True)
        out_n.copy_(pipe.fused_normal, non_blocking=True)
    e3.record()
    torch.cuda.synchronize()
    e2e_ms = e2.elapsed_time(e3) / args.steps

    plain = None
    if not args.no_plain and rank == 0:
        pp = ScenePipeline(inputs, mode="plain", prior_threads=min(16, os.cpu_count() or 1))
        pp.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pp.run()
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        plain = {"value": args.views / plain_s, "unit": UNIT, "steps": 1,
                 "mode": "one view per launch chain, fp32 images, synchronised after every kernel"}
        pp.close()

    served = None
    if not args.no_serving and rank == 0:
        served = serving_run(dev)
    segments = segments_run(dev) if rank == 0 else None
    superpixels = superpixels_run(dev) if rank == 0 else None

    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs")
    peak_note = "of measured" if hbm else "of fallback"
    hbm = hbm or 6800.0
    achieved = sweep_bytes / (sweep_ms / 1000.0) / 1e9 if sweep_ms else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "sweep_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    cpu = None if args.no_cpu else cpu_baseline(sc, os.cpu_count() or 1)
    clocks = clk.summary()  # reads and removes the sample file: once
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded room scene rendered on device)",
        "config": {"workload": WORKLOAD, "views": args.views, "height": args.height, "width": args.width,
                   "num_src": 10, "parallelism": f"replicas x{world}", "l2": "inputs larger than L2, no flush",
                   "cuda_graphs": True,
                   "launch_shapes": {k: {"tile_h": r.best[0], "ctas_per_sm": r.best[1],
                                         "split_sweep": r.best[2] if len(r.best) > 2 else 0}
                                     for k, r in pipe.tuned.items()}},
        "e2e": {"value": world * args.views / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        # pixels x source views evaluated per second (H * W * N * ref-views/s)
        "mpix_views_per_s": value * args.height * args.width * 10 / 1e6,
        "latency": ({"p50_ms_per_view": served["p50_ms"], "p99_ms_per_view": served["p99_ms"],
                     "note": "served Poisson stream (see serving): arrival to fused maps on the host, per view"}
                    if served else
                    {"p50_ms_per_view": ms / args.views, "p99_ms_per_view": ms / args.views,
                     "note": "batched: every view of the scene completes with the step"}),
        "serving": served,
        "segments": segments,
        "superpixels": superpixels,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "kernel": "k_sweep (half-sweep over all views)", "peak_source": peak_note,
                     "launch_ms": sweep_ms,
                     "note": "latency-bound texture/L1 gather, not HBM: ncu shows 36-47 % SM issue, 37 % of the "
                             "texture pipe and under 10 % of DRAM bandwidth"},
        "ncc_samples": ncc_samples_block(samples, ms, clocks),
        "stages_s": stages,
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
        "plain_path": plain,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out))


def ncc_samples_per_step(pipe) -> float:
    """Algorithmic NCC window samples of one pipeline step: per view and pass
    H * W * N * 36 * (1 + 14 * I) (the initial costs, then 8 neighbour and
    5 refinement hypotheses plus the current one per pixel and iteration)."""
    total = 0.0
    for key in pipe.plans:
        for plan in pipe.plans[key]:
            iters = (plan.num_stages - 4) // 2
            for v in plan.views:
                total += v.height * v.width * (len(v.images) - 1) * 36 * (1 + 14 * iters)
    return total


def ncc_samples_block(samples: float, ms: float, clocks: dict) -> dict:
    """Samples per second and per SM-clock.  A sample costs about 38 warp-lane
    instructions in the fp16-quad kernels (projection 8, clamp and corner 13,
    load 3, unpack 2, interpolation 4, weights 1, moments 4, loop 3); an SM
    issues at most 4 x 32 lane-instructions a clock, so about 3.4 samples per
    SM-clock is the issue ceiling."""
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    per_s = samples / (ms / 1000.0)
    per_sm_clk = per_s / (152 * mhz * 1e6)
    return {"per_step": samples, "per_s": per_s, "per_sm_clock": per_sm_clk, "issue_ceiling_per_sm_clock": 128 / 38,
            "frac_of_issue_ceiling": per_sm_clk / (128 / 38)}


def sweep_roofline(pipe, torch):
    """Average duration of the half-sweep launches (CUDA events on the
    launching stream) over one pipeline step, their algorithmic bytes (image
    reads + 36 B/pixel of state per half-sweep + src depths in the geometric
    passes) and the number of kernels one step launches."""
    import numpy as np

    durations, nbytes, launches = [], [], 0
    stream = torch.cuda.current_stream()
    V = pipe.V
    HW = pipe.H * pipe.W
    for key in sorted(pipe.plans):
        plans = pipe.plans[key]
        for plan in plans:
            n_st = plan.num_stages
            iters = (n_st - 4) // 2
            for s in range(n_st):
                is_sweep = 1 <= s <= 2 * iters
                if is_sweep:
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                plan.launch_stage(s)
                launches += 2 if (is_sweep and plan.params.split_sweep) else 1  # split: two kernels
                if is_sweep:
                    b.record(stream)
                    durations.append((a, b))
                    b_img = 2  # fp16 staged images (algorithmic 2 B/pixel)
                    if key.startswith(("random", "prior")):
                        b_img = 4  # fp32 textures
                    per_view = 0
                    for v in plan.views:
                        n = len(v.images)
                        per_view += n * HW * b_img + 36 * HW + (n * HW * 4 if key.startswith("geom") else 0)
                    nbytes.append(per_view)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in durations]
    # fusion launches 2 kernels per view; a geometric pass restages its
    # fp16 texel quads with one kernel per image at stage 0
    launches += 2 * V
    launches += sum(V for key in pipe.plans if key.startswith("geom"))
    if not ms:
        return None, 0, launches
    return float(np.mean(ms)), float(np.mean(nbytes)), launches


if __name__ == "__main__":
    main()
