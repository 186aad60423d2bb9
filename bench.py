#!/usr/bin/env python
"""Throughput of the Gaussian-splat training step on one GB300.

Workload (synthetic stand-in for the reference's COLMAP captures): N = 1M
Gaussians of SH degree 3 in 64 clusters, 16 pinhole cameras at 1920x1080 on
a radius-5 orbit, targets rendered from a separate seeded 300k-Gaussian
ground-truth scene, loss w_L2 = 1, w_L1 = 0.2.

A "train iteration" is one camera view rendered, back-propagated and applied
(the reference's train() loop does one view + one Adam step per iteration).
value = batched trainer, B views per sky_step (one Adam step per B views);
the plain per-view path (one view + one Adam step per sky_step) is timed
beside it.  Device time: CUDA events on the library's stream around exactly
K steps; e2e: wall clock around the same K sky_step calls through the C-ABI
with host camera arrays (per-step host->device step parameters, device->host
status with the loss).  Inputs (1M Gaussians, 16 x 33 MB targets, all step
buffers) are far larger than L2, so no flush is needed between steps.

--impl reference: the reference's path runs only as WGSL through WebGPU,
which no box here has; its CPU stand-in is the oracle port (oracle/), timed
on the host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
for _p in (str(REPO), str(REPO / "skyfall-viewer_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "train iters/s & Mpix/s @1M splats 1080p: batched vs plain, grads within 1e-3"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--views", type=int, default=16)
    ap.add_argument("--cameras", type=int, default=16)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--gt", type=int, default=300_000)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-views", type=int, default=1)
    ap.add_argument("--workload", default="train1080", choices=["train1080", "mixed", "stress4k"],
                    help="train1080: 1M SH-3 clusters, 16 orbit views 1920x1080 per step; "
                         "mixed: 16 views per step of 640x480 / 1280x720 / 1920x1080; "
                         "stress4k: 4M tightly clustered SH-3 Gaussians, one 3840x2160 view")
    ap.add_argument("--tile-size", type=int, default=16, choices=[8, 16, 32])
    ap.add_argument("--fwd-batch", type=int, default=0, choices=[0, 64, 128, 256],
                    help="forward splat-batch depth (0 = 256)")
    ap.add_argument("--bwd-batch", type=int, default=0, choices=[0, 32, 64, 128],
                    help="16x16-tile backward splat-batch depth (0 = 128)")
    ap.add_argument("--tile-cull", type=int, default=1, choices=[0, 1],
                    help="1: intersection lists of the training steps hold only the tiles each "
                         "Gaussian's alpha >= 1/255 ellipse reaches (bit-identical results)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the tile size from 8/16/32, then the splat-batch depths")
    ap.add_argument("--prune-after", action="store_true",
                    help="after the measurement, prune a seeded 10%% of the Gaussians once")
    args = ap.parse_args()
    if args.workload == "stress4k":
        if args.n == 1_000_000:
            args.n = 4_000_000
        args.views = args.cameras = 1
        args.width, args.height = 3840, 2160
    return args


def workload(args):
    from skyfall import scenes
    if args.workload == "stress4k":
        P = scenes.scene_clusters(args.n, seed=1005, cluster_sigma=0.05, logscale_mean=-5.0,
                                  logscale_sigma=0.5)
    else:
        P = scenes.scene_clusters(args.n, seed=1002)
    if args.workload == "mixed":
        cams = scenes.cameras_mixed(args.cameras, 5.0)
    else:
        cams = scenes.cameras_orbit(args.cameras, 5.0, args.width, args.height)
    return P, cams


def workload_name(args, n, B, C) -> str:
    if args.workload == "mixed":
        return (f"batched train, uneven resolutions: {n} Gaussians SH-3 (64 clusters), {B} views/step "
                f"from {C} cameras of 640x480 / 1280x720 / 1920x1080, tile {args.tile_size}; "
                f"1 iteration = 1 view")
    if args.workload == "stress4k":
        return (f"memory-stress train: {n} Gaussians SH-3 in 64 clusters of sigma 0.05, log-scales "
                f"N(-5, 0.5), one 3840x2160 view per step; 1 iteration = 1 view")
    return (f"batched train: {n} Gaussians SH-3 (64 clusters), {B} views/step of "
            f"{args.width}x{args.height} from {C} orbit cameras, targets rendered from a "
            f"{args.gt}-Gaussian scene; 1 iteration = 1 view")


def measured_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from an ncu capture
    recorded in profiles/traffic.json (null when none was taken)."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    e = d.get(kernel)
    if not e or e.get("workload") != workload:
        return None
    return float(e["bytes_per_launch"])


def measured_issue(kernel: str):
    """Issue-slot utilisation of `kernel` (smsp__issue_active, fraction of
    cycles a warp instruction issued) from its full ncu capture, recorded in
    profiles/traffic.json: the bound of the issue-bound raster kernels."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    e = json.loads(p.read_text()).get(kernel) or {}
    return e.get("issue_active")


def render_targets(sky, cams, args):
    """Targets: renders of a separate ground-truth scene."""
    from skyfall import scenes
    gt = scenes.scene_clusters(args.gt, seed=3002)
    out = []
    with sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0) as r:
        r.load_points(gt)
        r.setTrainingCameras(cams)
        for k in range(len(cams)):
            rgba, _ = r.render([k], with_alpha=False)
            out.append(rgba[:, :3].reshape(cams[k]["height"], cams[k]["width"], 3).copy())
    return out


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The largest `value` over the replicas (the slowest rank's time).  The
    replicas train independent copies: nothing else crosses ranks."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(views_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job views/s: every rank's views over the slowest rank's time."""
    return views_per_rank * world / (ms_max / 1000.0)


def time_steps(r, torch, view_sets, warmup):
    """Device time (CUDA events on the library stream) of len(view_sets)
    sky_step calls after `warmup` untimed ones; also wall clock."""
    stream = torch.cuda.ExternalStream(r.stream())
    for k in range(warmup):
        r.trainStep(view_sets[k % len(view_sets)])
    r.sync()
    r.enableProfiling(True)
    st0 = r.getStatus()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    t0 = time.perf_counter()
    isects = 0
    loss = 0.0
    for vs in view_sets:
        st = r.trainStep(vs)
        isects += st.num_intersections
        loss = st.loss
    t1 = time.perf_counter()
    e1.record(stream)
    torch.cuda.synchronize()
    st1 = r.getStatus()
    stages, nsteps = r.stageTimes()
    return dict(ms=e0.elapsed_time(e1), wall=t1 - t0, isects=isects, loss=loss, stages=stages,
                steps=nsteps, launches=st1.kernel_launches - st0.kernel_launches)


def cpu_baseline(args, P, cams, targets, threads):
    """Oracle (CPU port of the reference's WGSL) timed on the host cores for
    `cpu_sample_views` full view-iterations of the same workload."""
    from oracle import oracle as orc
    orc.build()
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0, nthreads=threads)
    Pc = P.copy()
    m1 = np.zeros_like(Pc)
    m2 = np.zeros_like(Pc)
    t0 = time.perf_counter()
    pixels = 0
    for k in range(args.cpu_sample_views):
        cam = cams[k % len(cams)]
        out = orc.view_pipeline(Pc, cam, targets[k % len(targets)], s, 3, mode=0)
        g = orc.geom(Pc, cam, s, 3, out["bw"]["gsum9"].astype(np.float32))
        for lo, hi, lr in [(0, 3, 1.6e-4), (3, 6, 5e-3), (6, 10, 1e-3), (10, 11, 2.5e-2)]:
            p, a, b = (np.ascontiguousarray(x[lo:hi]) for x in (Pc, m1, m2))
            orc.adam(p, a, b, np.ascontiguousarray(g[lo:hi]), lr, 0.9, 0.999, 1e-8, 10.0, 31.62)
            Pc[lo:hi], m1[lo:hi], m2[lo:hi] = p, a, b
        pixels += cam["width"] * cam["height"]
    dt = time.perf_counter() - t0
    return dict(value=args.cpu_sample_views / dt, seconds=dt, pixels=pixels)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        P, cams = workload(args)
        from skyfall import scenes
        targets = [scenes.target_uniform(c["width"], c["height"], seed=2001 + k)
                   for k, c in enumerate(cams[: args.cpu_sample_views])]
        threads = os.cpu_count() or 1
        vals = []
        for _ in range(max(1, args.steps)):
            vals.append(cpu_baseline(args, P, cams, targets, threads))
        v = float(np.median([x["value"] for x in vals]))
        line = {
            "metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": 0, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"train step, {args.n} Gaussians SH-3, {args.width}x{args.height}, "
                                   f"one view per iteration (oracle CPU port; the reference's WGSL "
                                   f"needs WebGPU, unavailable on this box)"},
            "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": f"{args.cpu_sample_views} full view-iteration(s) per step"},
            "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import skyfall as sky
    from skyfall import build
    build.build()

    P, cams = workload(args)
    targets = render_targets(sky, cams, args)
    B = args.views
    C = len(cams)
    rng = np.random.default_rng(1234 + rank)
    batched_sets = [list((np.arange(B) + k * B) % C) for k in range(args.steps)]
    warm_sets = [list(rng.integers(0, C, B)) for _ in range(args.warmup)]

    def make(ts):
        rr = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2,
                                  w_ssim=0.0, max_views_per_step=args.views, use_graph=1,
                                  tile_size=ts)
        rr.load_points(P)
        rr.setTrainingCameras(cams)
        rr.setTrainingImages(targets)
        rr.setTileCull(bool(args.tile_cull))
        return rr

    tune = None
    if args.autotune:
        from skyfall.autotune import autotune
        args.tile_size, args.fwd_batch, args.bwd_batch, tune = autotune(make, batched_sets[:3])
    r = make(args.tile_size)
    r.setBatchDepth(args.fwd_batch, args.bwd_batch)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    barrier()
    for vs in warm_sets:
        r.trainStep(vs)
    with Clocks(local) as clk:
        res = time_steps(r, torch, batched_sets, 0)
    barrier()
    ms = max_over_ranks(res["ms"], world)
    value = replica_throughput(args.steps * B, world, ms)
    px_step = [sum(cams[c]["width"] * cams[c]["height"] for c in vs) for vs in batched_sets]
    px_per_view = sum(px_step) / (len(px_step) * B)
    mpix = value * px_per_view / 1e6
    e2e_value = replica_throughput(args.steps * B, world, max_over_ranks(res["wall"] * 1000.0, world))
    device_bytes = int(r.getStatus().device_bytes)

    plain = None
    plain_stage_ms = None
    if not args.no_plain:
        # the plain per-view path: one view and one Adam step per sky_step,
        # launched directly with the host-side sizing read-back
        r.config.use_graph = 0
        sky._lib.check(r._L.sky_set_config(r._h, sky._lib.C.byref(r.config)))
        psets = [[k % C] for k in range(args.steps * B)]
        for k in range(args.warmup):
            r.trainStep([k % C])
        pr = time_steps(r, torch, psets, 0)
        plain = len(psets) / (pr["ms"] / 1000.0)
        plain_stage_ms = {k: v / max(pr["steps"], 1) for k, v in pr["stages"].items()}

    # roofline of the dominant stage
    steps = max(res["steps"], 1)
    stage_ms = {k: v / steps for k, v in res["stages"].items()}
    dom = max(stage_ms, key=stage_ms.get)
    isect = res["isects"] / steps
    pix = B * px_per_view
    n = args.n
    # algorithmic bytes per launch: per-unit figures x units.  Backward per
    # intersection: the 48-byte record, its 4-byte item index and the 48-byte
    # partial; per pixel: last index, transmittance, residual.
    algo_bytes = {
        "preprocess": n * 236 + B * n * 72,
        "scan": B * n * 16,
        "emit": isect * 8 + B * n * 20,
        "sort": isect * 36,
        "ranges": isect * 4,
        "forward": isect * 52 + pix * 60,
        "backward": isect * 100 + pix * 28,
        "geom_adam": n * 1652 + isect * 48,
    }
    peak, peak_kind = measured_peak()
    achieved = algo_bytes[dom] / (stage_ms[dom] / 1000.0) / 1e9
    clocks = clk.summary()
    wl_key = f"{args.workload}/ts{args.tile_size}" + ("/cull" if args.tile_cull else "")
    traffic = measured_traffic(dom, wl_key)

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        threads = os.cpu_count() or 1
        cb = cpu_baseline(args, P, cams, targets, threads)
        cpu = {"value": cb["value"], "unit": "iters/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample_views} view-iteration(s) of the same workload "
                         f"({cb['seconds']:.1f} s): oracle project/sort/forward/loss/backward/"
                         f"geometry/Adam"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "iters/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": workload_name(args, n, B, C),
            "views_per_step": B, "global_batch": B, "parallelism": "replicas" if world > 1 else "none",
            "tile_size": args.tile_size, "fwd_batch": args.fwd_batch or 256,
            "bwd_batch": (args.bwd_batch or 128) if args.tile_size == 16 else None,
            "tile_cull": bool(args.tile_cull),
            "autotune_ms_per_step": tune,
            "l2": "inputs > L2 (no flush)",
        },
        "device_bytes": device_bytes,
        "mpix_per_s": mpix,
        "plain_iters_per_s": plain,
        "plain_stage_ms": plain_stage_ms,
        "batched_over_plain": (value / world / plain) if plain else None,
        "stage_ms": stage_ms,
        "intersections_per_step": isect,
        "loss": res["loss"],
        "gpu_launches": int(res["launches"]),
        "e2e": {"value": e2e_value, "unit": "iters/s",
                "h2d_bytes_per_step": 13312, "d2h_bytes_per_step": 2 * 160},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes": algo_bytes[dom],
                     "traffic_source": "profiles/traffic.json (ncu dram__bytes_read.sum + "
                                       "dram__bytes_write.sum, same workload)" if traffic else None,
                     # the raster kernels are issue-bound: the fraction of cycles on
                     # which a warp instruction issued (full ncu capture of the kernel)
                     "issue_active": measured_issue(dom),
                     "issue_source": "profiles/traffic.json (ncu smsp__issue_active, "
                                     "profiles/raster_and_sort_4views_200k_1080p.md)"
                                     if measured_issue(dom) is not None else None},
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if args.prune_after:
        # After the timed region: one prune of a seeded 10 % of the Gaussians
        # through the public API (the compaction kernels an ncu capture of
        # this command measures); the wall time includes the host work.
        mask = np.random.default_rng(7).random(r.getGaussianCount()) < 0.1
        t0 = time.perf_counter()
        left = r.prune(minOpacity=0.0, mask=mask.astype(np.uint8))
        line["prune"] = {"removed": int(mask.sum()), "remaining": int(left),
                         "wall_ms": (time.perf_counter() - t0) * 1e3}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
