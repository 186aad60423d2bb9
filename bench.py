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
K steps, with per-stage profiling off; e2e: wall clock around the same K
sky_step calls through the C-ABI (per-step host->device step parameters,
device->host step status with the loss, both counted by the library).
Stage times and the rasterizers' pair counts come from separate runs of the
same steps afterwards.  Inputs (1M Gaussians, 16 x 33 MB targets, all step
buffers) are far larger than L2, so no flush is needed between steps.

Beside the headline the line carries: `matched_loss` (batched and plain
trainers from one initial state on uneven-resolution cameras, time to a
common loss), `mixed` (views/s at uneven resolutions with the autotuned
tile size), `configs` (the plain-step and forward-only configurations on
the GPU) and `cpu_legs` (the oracle on the host cores: the plain step at
N = 16,384 on all cores and on one, and a 1080p forward of the 1M scene).

--impl reference: the reference's path runs only as WGSL through WebGPU,
which no box here has; its CPU stand-in is the oracle port (oracle/), timed
on the host cores on a bounded sample of the same workload (the same
scene, cameras and rendered targets).
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
RASTER = ("forward", "backward")


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
    ap.add_argument("--no-extras", action="store_true",
                    help="skip matched_loss, mixed, configs and cpu_legs (profiling runs)")
    ap.add_argument("--cpu-sample-views", type=int, default=1)
    ap.add_argument("--workload", default="train1080",
                    choices=["train1080", "mixed", "stress4k", "train720"],
                    help="train1080: 1M SH-3 clusters, 16 orbit views 1920x1080 per step; "
                         "mixed: 16 views per step of 640x480 / 1280x720 / 1920x1080; "
                         "stress4k: 4M tightly clustered SH-3 Gaussians, one 3840x2160 view; "
                         "train720: a full training run (500k SH-3, 100 Fibonacci cameras "
                         "1280x720, --steps Adam steps, densify + prune every 100)")
    ap.add_argument("--tile-size", type=int, default=16, choices=[8, 16, 32])
    ap.add_argument("--fwd-batch", type=int, default=0, choices=[0, 64, 128, 256],
                    help="forward splat-batch depth (0 = 256)")
    ap.add_argument("--bwd-batch", type=int, default=0, choices=[0, 32, 64, 128],
                    help="16x16-tile backward splat-batch depth (0 = 64)")
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
    if args.workload == "train720" and "--views" not in sys.argv:
        args.views = 1  # the reference's train(n): one view per Adam step
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
                f"from {C} cameras of 640x480 / 1280x720 / 1920x1080, tile {args.tile_size}, "
                f"targets rendered from a {args.gt}-Gaussian scene; 1 iteration = 1 view")
    if args.workload == "stress4k":
        return (f"memory-stress train: {n} Gaussians SH-3 in 64 clusters of sigma 0.05, log-scales "
                f"N(-5, 0.5), one 3840x2160 view per step, targets rendered from a "
                f"{args.gt}-Gaussian scene; 1 iteration = 1 view")
    return (f"batched train: {n} Gaussians SH-3 (64 clusters), {B} views/step of "
            f"{args.width}x{args.height} from {C} orbit cameras, targets rendered from a "
            f"{args.gt}-Gaussian scene; 1 iteration = 1 view")


def algo_bytes(stage: str, n: int, B: int, isect: float, pix: float) -> float:
    """Algorithmic bytes of one launch of a stage (per-unit figures x units).
    Backward per intersection: the 48-byte record, its 4-byte item index and
    the 48-byte partial; per pixel: last index, transmittance, residual."""
    return {
        "preprocess": n * 236 + B * n * 72,
        "scan": B * n * 16,
        "emit": isect * 8 + B * n * 20,
        "sort": isect * 36,
        "ranges": isect * 4,
        "forward": isect * 60 + pix * 60,
        "backward": isect * 100 + pix * 28,
        "geom_adam": n * 1652 + isect * 48,
    }[stage]


def measured_traffic(stage: str, workload_key: str, n: int, B: int, isect: float, pix: float):
    """DRAM bytes per launch of the stage's kernel on this workload, scaled
    from an ncu capture of a small case (profiles/traffic.json: one kernel,
    a few launches, the 200k-Gaussian 4-view case): its measured bytes per
    launch times the ratio of the algorithmic bytes of the two launches (the
    kernel's traffic grows with the intersections and pixels it processes).
    Returns (bytes, source) or (None, None)."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    e = d.get(stage)
    if not e or e.get("bench_workload") != workload_key:
        return None, None
    small = e["small_case"]
    small_algo = algo_bytes(stage, small["n"], small["views"], small["isect_per_launch"],
                            small["pixels_per_launch"])
    scale = algo_bytes(stage, n, B, isect, pix) / small_algo
    src = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of {e['kernel']} on {small['name']} "
           f"({e['bytes_per_launch']:.4g} B per launch, {e['launches']} launches), scaled by the "
           f"algorithmic-byte ratio {scale:.3f} (profiles/traffic.json)")
    return e["bytes_per_launch"] * scale, src


def measured_issue(stage: str):
    """Issue-slot utilisation (smsp__issue_active) and lanes active per warp
    instruction of the stage's kernel, from its full ncu capture on the small
    case (profiles/traffic.json)."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return {}
    e = json.loads(p.read_text()).get(stage) or {}
    return {k: e[k] for k in ("issue_active", "lanes_per_warp_instruction") if k in e}


def render_targets(sky, cams, args, gt=None):
    """Targets: renders of a separate ground-truth scene."""
    from skyfall import scenes
    if gt is None:
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


def time_steps(r, torch, view_sets, profile: int = 0):
    """Device time (CUDA events on the library stream) of len(view_sets)
    sky_step calls; also their wall clock, launches and host<->device bytes.
    profile: 0 none, 1 per-stage events, 2 events + pair counts."""
    stream = torch.cuda.ExternalStream(r.stream())
    r.sync()
    r.enableProfiling(profile)
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
    pairs = r.read_buffer("pair_counts") if profile == 2 else None
    r.enableProfiling(0)
    return dict(ms=e0.elapsed_time(e1), wall=t1 - t0, isects=isects, loss=loss, stages=stages,
                steps=nsteps, launches=st1.kernel_launches - st0.kernel_launches,
                h2d=st1.step_h2d_bytes - st0.step_h2d_bytes, d2h=st1.step_d2h_bytes - st0.step_d2h_bytes,
                pairs=pairs)


def pair_stats(pairs, steps: int = 1):
    """The rasterizers' work per step from the counting variants (profiling
    level 2): pairs evaluated and composited / contributing, and the share of
    the warps' pixel slots that evaluated a pair."""
    if pairs is None or int(pairs[2]) == 0:
        return None
    f_eval, f_con, f_ent, b_eval, b_con, b_ent, b_idle = (int(x) / steps for x in pairs[:7])
    return {
        "forward": {"pairs_evaluated": f_eval, "pairs_contributing": f_con, "warp_entries": f_ent,
                    "lane_use": f_eval / (32.0 * f_ent) if f_ent else None,
                    "contributing_share": f_con / f_eval if f_eval else None},
        "backward": {"pairs_evaluated": b_eval, "pairs_contributing": b_con, "warp_entries": b_ent,
                     "slot_use": b_eval / (64.0 * b_ent) if b_ent else None,
                     "contributing_share": b_con / b_eval if b_eval else None,
                     "entries_without_contribution": b_idle / b_ent if b_ent else None},
    }


# ---------------------------------------------------------------------------
# CPU legs (the oracle: the reference's algorithm restated)
# ---------------------------------------------------------------------------
def cpu_view_iterations(orc, P, cams, targets, views: int, threads: int, deg: int = 3):
    """`views` full view-iterations of the oracle (project, sort, forward,
    loss, backward, geometry, Adam) at SH degree `deg`; returns (views/s,
    seconds)."""
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0, nthreads=threads)
    Pc = P.copy()
    m1 = np.zeros_like(Pc)
    m2 = np.zeros_like(Pc)
    t0 = time.perf_counter()
    for k in range(views):
        cam = cams[k % len(cams)]
        out = orc.view_pipeline(Pc, cam, targets[k % len(targets)], s, deg, mode=0)
        g = orc.geom(Pc, cam, s, deg, out["bw"]["gsum9"].astype(np.float32))
        for lo, hi, lr in [(0, 3, 1.6e-4), (3, 6, 5e-3), (6, 10, 1e-3), (10, 11, 2.5e-2)]:
            p, a, b = (np.ascontiguousarray(x[lo:hi]) for x in (Pc, m1, m2))
            orc.adam(p, a, b, np.ascontiguousarray(g[lo:hi]), lr, 0.9, 0.999, 1e-8, 10.0, 31.62)
            Pc[lo:hi], m1[lo:hi], m2[lo:hi] = p, a, b
    dt = time.perf_counter() - t0
    return views / dt, dt


def cpu_legs(orc, P1080, cams1080, threads: int):
    """The plain-step configuration (N = 16,384 SH-0, 256x256) on all host
    cores and on one, and a 1920x1080 forward of the 1M SH-3 scene on all
    cores (one view of the 8-view forward-only configuration)."""
    from skyfall import scenes
    Ps = scenes.scene_uniform(16384, seed=1001)
    cs = scenes.cameras_single(256, 256, 3.0)
    ts = [scenes.target_uniform(256, 256, seed=2001)]
    legs = []
    for th in (threads, 1):
        k = 40 if th > 1 else 10
        v, dt = cpu_view_iterations(orc, Ps, cs, ts, k, th, deg=0)
        legs.append({"config": "plain step: 16384 Gaussians SH-0, 256x256, 16x16 tiles", "cores": th,
                     "value": v, "unit": "iters/s", "sample": f"{k} iterations ({dt:.2f} s)"})
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0, nthreads=threads)
    t0 = time.perf_counter()
    out = orc.view_pipeline(P1080, cams1080[0], None, s, 3)
    dt = time.perf_counter() - t0
    px = cams1080[0]["width"] * cams1080[0]["height"]
    legs.append({"config": f"forward only: {P1080.shape[1]} Gaussians SH-3, 1920x1080", "cores": threads,
                 "value": px / dt / 1e6, "unit": "Mpix/s",
                 "sample": f"1 view ({dt:.2f} s, {int(out['pr']['counts'].sum())} intersections)"})
    return legs


def oracle_targets(orc, cams, count: int, gt_n: int):
    """The ground-truth renders the GPU arm trains against, made by the oracle
    on the CPU (the GPU's renders are bit-identical to the oracle's)."""
    from skyfall import scenes
    gt = scenes.scene_clusters(gt_n, seed=3002)
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    out = []
    for k in range(count):
        fw = orc.view_pipeline(gt, cams[k], None, s, 3)["fw"]
        out.append(fw["rgba"][:, :3].reshape(cams[k]["height"], cams[k]["width"], 3).copy())
    return out


# ---------------------------------------------------------------------------
# Extras of the GPU arm
# ---------------------------------------------------------------------------
def interp_time(curve, level):
    """First time the (time, loss) curve reaches `level`, linear between the
    evaluations around the crossing."""
    for (t0, l0), (t1, l1) in zip(curve, curve[1:]):
        if l1 <= level:
            if l0 <= level:
                return t0
            return t0 + (t1 - t0) * (l0 - level) / (l0 - l1)
    return None


def matched_loss(sky, torch, P, args, ts: int):
    """From one initial state, the batched trainer (all 16 uneven-resolution
    cameras per step, graph-captured) and the plain trainer (one camera per
    step, direct launches, cycling through a seeded permutation per epoch)
    train on the same targets for the same number of views.  The loss over
    all 16 cameras is evaluated every epoch (16 views) outside the timed
    steps; the result is the device time each needs to reach the lowest loss
    both reach.  Both use SH degree 3 from the start, SH planes updated every
    step and no position-learning-rate warm-up: the reference's schedules
    count steps, which would give the plain trainer 16x the warm-up
    progress.  The batched trainer runs twice: with batch-scaled Adam
    hyperparameters (SkyConfig.batch_scaling: learning rates x sqrt(16),
    betas^16; the headline ratio) and with those of one view."""
    from skyfall import scenes
    cams = scenes.cameras_mixed(16, 5.0)
    targets = render_targets(sky, cams, args)
    px_all = sum(c["width"] * c["height"] for c in cams)
    epochs = 40

    def make(graph, scaling=0):
        r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, sh_update_interval=1,
                                 lr_means_delay_mult=1.0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
                                 max_views_per_step=16, use_graph=graph, tile_size=ts,
                                 batch_scaling=scaling)
        r.load_points(P)
        r.setTrainingCameras(cams)
        r.setTrainingImages(targets)
        r.setTileCull(True)
        return r

    def run(batched, scaling=0):
        r = make(1 if batched else 0, scaling)
        stream = torch.cuda.ExternalStream(r.stream())
        rng = np.random.default_rng(77)
        curve = [(0.0, r.forward(list(range(16))) / (3 * px_all))]
        t = 0.0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for ep in range(epochs):
            order = [int(x) for x in rng.permutation(16)]
            sets = [order] if batched else [[v] for v in order]
            r.sync()
            e0.record(stream)
            for vs in sets:
                r.trainStep(vs)
            e1.record(stream)
            torch.cuda.synchronize()
            t += e0.elapsed_time(e1) / 1000.0
            curve.append((t, r.forward(list(range(16))) / (3 * px_all)))
        r.close()
        return curve

    cb = run(True, 1)
    cu = run(True, 0)
    cp = run(False)

    def at_matched(c):
        level = max(min(l for _, l in c), min(l for _, l in cp))
        tb, tp = interp_time(c, level), interp_time(cp, level)
        return level, tb, tp, ((tp / tb) if (tb and tp) else None)

    level, tb, tp, ratio = at_matched(cb)
    ulevel, utb, utp, uratio = at_matched(cu)
    return {
        "cameras": "16 on a Fibonacci sphere, 640x480 / 1280x720 / 1920x1080",
        "views_each": epochs * 16, "tile_size": ts,
        "loss": "sum over the 16 views of 0.5 r^2 + 0.2 |r| per channel, / (3 x pixels)",
        "initial_loss": cb[0][1],
        "batched": {"final_loss": cb[-1][1], "seconds": cb[-1][0], "adam_steps": epochs,
                    "adam": "batch_scaling 1: learning rates x 4, betas^16"},
        "plain": {"final_loss": cp[-1][1], "seconds": cp[-1][0], "adam_steps": epochs * 16},
        "common_loss": level,
        "batched_seconds_to_common_loss": tb, "plain_seconds_to_common_loss": tp,
        "batched_over_plain_at_matched_loss": ratio,
        "unscaled": {"adam": "batch_scaling 0: one view's hyperparameters", "final_loss": cu[-1][1],
                     "common_loss": ulevel, "batched_seconds_to_common_loss": utb,
                     "plain_seconds_to_common_loss": utp, "batched_over_plain_at_matched_loss": uratio},
        "curves": {"batched": [[round(a, 5), b] for a, b in cb],
                   "batched_unscaled": [[round(a, 5), b] for a, b in cu],
                   "plain": [[round(a, 5), b] for a, b in cp]},
    }


def mixed_throughput(sky, torch, P, args):
    """Views/s of the batched and the plain trainer on 16 uneven-resolution
    cameras (640x480 / 1280x720 / 1920x1080), with the tile size picked by the
    autotuner from 8 / 16 / 32 (default splat-batch depths)."""
    from skyfall import scenes
    from skyfall.autotune import pick_tile_size
    cams = scenes.cameras_mixed(16, 5.0)
    targets = render_targets(sky, cams, args)

    def make(ts, graph=1):
        r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
                                 max_views_per_step=16, use_graph=graph, tile_size=ts)
        r.load_points(P)
        r.setTrainingCameras(cams)
        r.setTrainingImages(targets)
        r.setTileCull(True)
        return r

    sets = [list(range(16))] * 3
    ts, tile_ms = pick_tile_size(make, sets, warmup=2)
    r = make(ts)
    for _ in range(3):
        r.trainStep(list(range(16)))
    b = time_steps(r, torch, [list(range(16))] * 8)
    r.close()
    r = make(ts, graph=0)
    for k in range(8):
        r.trainStep([k])
    p = time_steps(r, torch, [[k % 16] for k in range(64)])
    r.close()
    batched = 8 * 16 / (b["ms"] / 1000.0)
    plain = 64 / (p["ms"] / 1000.0)
    return {"tile_size": ts, "autotune_ms_per_step": tile_ms, "batched_views_per_s": batched,
            "plain_views_per_s": plain, "batched_over_plain": batched / plain}


def gpu_configs(sky, torch, P1080):
    """The plain training step at N = 16,384 (SH-0, 256x256, uniform target)
    and the forward-only configuration (1M SH-3, 8 views of 1920x1080),
    timed with CUDA events on the library stream."""
    from skyfall import scenes
    out = {}
    Ps = scenes.scene_uniform(16384, seed=1001)
    r = sky.GaussianRenderer(sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)
    r.load_points(Ps)
    r.setTrainingCameras(scenes.cameras_single(256, 256, 3.0))
    r.setTrainingImages([scenes.target_uniform(256, 256, seed=2001)])
    for _ in range(5):
        r.trainStep([0])
    t = time_steps(r, torch, [[0]] * 100)
    out["plain_step_16k_256"] = {"iters_per_s": 100 / (t["ms"] / 1000.0), "ms_per_step": t["ms"] / 100}
    r.close()
    cams = scenes.cameras_orbit(8, 5.0, 1920, 1080)
    r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
                             tile_size=16, max_views_per_step=8)
    r.load_points(P1080)
    r.setTrainingCameras(cams)
    r.setTrainingImages([scenes.target_uniform(1920, 1080, seed=2300 + k) for k in range(8)])
    stream = torch.cuda.ExternalStream(r.stream())

    def timed(view_sets, reps=3):
        for vs in view_sets:
            r.forward(vs)
        r.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            for vs in view_sets:
                r.forward(vs)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    px = 8 * 1920 * 1080
    ms_plain = timed([[v] for v in range(8)])
    ms_batched = timed([list(range(8))])
    out["forward_1M_8x1080p"] = {"plain_mpix_per_s": px / ms_plain / 1e3,
                                 "batched_mpix_per_s": px / ms_batched / 1e3,
                                 "what": "forward + loss epilogue, 8 views; plain = 8 passes of 1 view"}
    r.close()
    return out


def full_training_run(sky, torch, args):
    """A full training run through the public API: N = 500k Gaussians
    initialised as the plain-step scene (means U[-1,1]^3, log-scales
    N(-4, 0.3), logits N(0, 1), DC colours U[0,1]) with SH degree 3 (higher
    coefficients 0), targets rendered from the separate 300k-Gaussian scene,
    100 cameras 1280x720 on a Fibonacci sphere of radius 4, `steps` Adam steps
    of one seeded camera each (the reference's train(n)) with the
    TrainingController schedule set to densify (with its combined scored
    prune) every 100 steps from step 100 and prune opacities below 0.005.
    Device time of the whole run (CUDA events on the library stream);
    the loss over all 100 cameras before and after."""
    from skyfall import scenes
    n = args.n if args.n != 1_000_000 else 500_000
    P = scenes.scene_uniform(n, seed=1003)
    cams = scenes.cameras_fibonacci(100, 4.0, 1280, 720)
    targets = render_targets(sky, cams, args)
    r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
                             max_views_per_step=max(1, args.views), use_graph=1, tile_size=16)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(targets)
    r.setTileCull(True)
    r.setSchedule(densify_from=100, densify_until=args.steps, densify_interval=100,
                  prune_from=100, prune_until=args.steps, prune_interval=100,
                  opacity_reset_interval=100000, min_opacity=0.005)
    px_all = sum(c["width"] * c["height"] for c in cams)

    def loss_all():
        tot = 0.0
        for k in range(0, 100, 50):
            tot += r.forward(list(range(k, k + 50)))
        return tot / (3 * px_all)

    l0 = loss_all()
    stream = torch.cuda.ExternalStream(r.stream())
    r.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    r.train(args.steps, views_per_step=max(1, args.views))
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    st = r.getStatus()
    l1 = loss_all()
    views = args.steps * max(1, args.views)
    line = {
        "metric": METRIC, "value": views / (ms / 1000.0), "unit": "iters/s", "n_gpus": 1,
        "steps": args.steps, "warmup": 0, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"full training run: {n} Gaussians SH-3 (plain-step initialisation), "
                               f"100 Fibonacci cameras 1280x720 (r = 4), targets rendered from a "
                               f"{args.gt}-Gaussian scene, {args.steps} Adam steps of "
                               f"{max(1, args.views)} seeded view(s), densify + scored prune "
                               f"(min opacity 0.005) every 100 steps",
                   "tile_size": 16, "tile_cull": True, "schedule": "densify/prune every 100 from 100"},
        "initial_loss": l0, "final_loss": l1,
        "loss_def": "sum over the 100 views of 0.5 r^2 + 0.2 |r| per channel, / (3 x pixels)",
        "gaussians_initial": n, "gaussians_final": int(st.num_gaussians),
        "densify_runs": int(st.densify_runs), "prune_runs": int(st.prune_runs),
        "graph_replays": int(st.graph_replays), "seconds_device": ms / 1000.0, "seconds_wall": wall,
        "device_bytes": int(st.device_bytes),
    }
    r.close()
    print(json.dumps(line))
    return 0


def reference_arm(args):
    """The reference's path timed on the host cores: the oracle port, one
    full view-iteration per step, on the GPU arm's scene, cameras and
    rendered targets (made by the oracle: bit-identical to the GPU's)."""
    from oracle import oracle as orc
    orc.build()
    P, cams = workload(args)
    targets = oracle_targets(orc, cams, args.cpu_sample_views, args.gt)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(max(1, args.steps)):
        v, _ = cpu_view_iterations(orc, P, cams, targets, args.cpu_sample_views, threads)
        vals.append(v)
    v = float(np.median(vals))
    line = {
        "metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": 0, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": workload_name(args, args.n, args.views, len(cams)),
                   "views_per_step": 1, "l2": "inputs > L2 (no flush)",
                   "path": "oracle CPU port of the reference's WGSL (WebGPU unavailable on this box)"},
        "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
                         "sample": f"{args.cpu_sample_views} full view-iteration(s) of the workload per step"},
        "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return reference_arm(args) if rank == 0 else 0

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import skyfall as sky
    from skyfall import build
    build.build()
    if args.workload == "train720":
        return full_training_run(sky, torch, args) if rank == 0 else 0

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
    # per-stage times (events between the stages) and the rasterizers' work
    # counts, from separate runs of the same steps
    prof = time_steps(r, torch, batched_sets, 1)
    cnt = time_steps(r, torch, batched_sets[:1], 2)

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
        pp = time_steps(r, torch, psets[:C], 1)
        plain_stage_ms = {k: v / max(pp["steps"], 1) for k, v in pp["stages"].items()}

    # roofline of the dominant stage
    steps = max(prof["steps"], 1)
    stage_ms = {k: v / steps for k, v in prof["stages"].items()}
    dom = max(stage_ms, key=stage_ms.get)
    isect = res["isects"] / args.steps
    pix = B * px_per_view
    n = args.n
    peak, peak_kind = measured_peak()
    ab = algo_bytes(dom, n, B, isect, pix)
    achieved = ab / (stage_ms[dom] / 1000.0) / 1e9
    clocks = clk.summary()
    wl_key = f"{args.workload}/ts{args.tile_size}" + ("/cull" if args.tile_cull else "")
    traffic, traffic_src = measured_traffic(dom, wl_key, n, B, isect, pix)
    pairs = pair_stats(cnt["pairs"])
    roof = {"bound": "issue" if dom in RASTER else "hbm", "kernel": dom, "achieved": achieved,
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "frac_of": "measured HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "algorithmic_bytes": ab, "traffic_source": traffic_src}
    if dom in RASTER:
        # the rasterizers are issue-bound: the fraction of cycles on which a
        # warp instruction issued, and how much of the warps' work was pairs
        roof.update(measured_issue(dom))
        roof["issue_source"] = "ncu smsp__issue_active on the small case (profiles/traffic.json)"
        if pairs:
            roof["work"] = pairs[dom]

    threads = os.cpu_count() or 1
    cpu = None
    legs = None
    from oracle import oracle as orc
    if not args.no_cpu_baseline and rank == 0:
        orc.build()
        v, dt = cpu_view_iterations(orc, P, cams, targets, args.cpu_sample_views, threads)
        cpu = {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample_views} view-iteration(s) of the same workload "
                         f"({dt:.1f} s): oracle project/sort/forward/loss/backward/geometry/Adam"}
        if not args.no_extras:
            legs = cpu_legs(orc, P, cams, threads)

    extras = {}
    if not args.no_extras and rank == 0 and args.workload == "train1080":
        extras["matched_loss"] = matched_loss(sky, torch, P, args, args.tile_size)
        extras["mixed"] = mixed_throughput(sky, torch, P, args)
        extras["configs"] = gpu_configs(sky, torch, P)

    steps_t = len(batched_sets)
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
            "bwd_batch": (args.bwd_batch or 64) if args.tile_size == 16 else None,
            "tile_cull": bool(args.tile_cull),
            "autotune_ms_per_step": tune,
            "l2": "inputs > L2 (no flush)",
            "timed_region": "stage events off; stage_ms and pair counts from separate runs of the same steps",
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
                "h2d_bytes_per_step": res["h2d"] / steps_t, "d2h_bytes_per_step": res["d2h"] / steps_t},
        "roofline": roof,
        "raster_work": pairs,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "cpu_legs": legs,
    }
    line.update(extras)
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
