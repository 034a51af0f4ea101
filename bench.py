"""Benchmark: forward + adjoint samples/s of the ray marcher.

Workload (TF reconstruction): 256^3 volume of 32 seeded Gaussian blobs plus
0.02 uniform noise, 64-entry RGBA texture TF initialised U(0,1), 8 views at
256x256 on a Fibonacci sphere at radius 3 (FOV 45 deg), Beer-Lambert, step
0.25 voxel, trilinear.  One step = forward render of the 8 views (with
transmittance checkpoints) + L2-loss gradient against a target image + adjoint
render accumulating the TF gradient.  Samples per step S = sum of the forward
termination indices.  Synthetic data (seeded), as the reference has no public
dataset for this path.

Arms:
  default          the optimized kernels, volume stored in BF16, all 8 views
                   in one launch per pass, the step captured in a CUDA graph
                   (`value`, device-resident); `e2e` runs the same step
                   through pyrenderer.Renderer with the inputs copied from
                   pinned host memory every step and the loss and TF gradient
                   read back.  The plain FP32 kernels are timed beside it.
  --impl reference the reference's CPU implementation of the path on the host
                   cores (the reference's own CPU marcher where it was built
                   here, else the oracle port), on a bounded sample of rays.

Other configurations of the metric (`--workload`, not the default line):
absorption_recon_128 (volume gradient, 64 views into 128^3), large_mixed_512
(512^3 BF16, 16 views at 1024^2, ray + volume + TF gradients),
batched_uneven_32 (32 instances of different volume and image sizes through
the batched entry points, one CUDA graph per step) and plain_cpu_64 (the
CPU-sized case).

--method forward times the forward method of the same workload instead
(render_forward_gradients tracing one derivative per TF entry, and camera
rays where the workload optimises them, + L2-loss gradient +
forward_variables_to_gradients); its CPU baseline is the oracle's forward
mode (the reference's forward mode needs cudAD, absent from its sources).

Multi-GPU: rays and views shard without any exchange in a TF-only step except
the TF-gradient sum, so N GPUs run N replicas ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+adjoint samples/sec: batched-BF16 vs plain FP32, grad rel err ≤1e-3"
METRIC_FORWARD = "forward-mode samples/sec: render_forward_gradients + forward_variables_to_gradients"
# the headline workload (the default) and the other configurations of the metric
WORKLOADS = {
    "tf_reconstruction_256": {
        "desc": "tf_reconstruction_256: 256^3 blobs+noise, texture TF R=64, 8 views 256x256, step 0.25 voxel, TF grad",
        "camera": "frame", "interval": 16, "estimate": "target", "res": 256, "views": 8, "image": 256},
    "absorption_recon_128": {
        "desc": "absorption_recon_128: 128^3 ellipsoid target, estimate 0.1, identity TF (absorption 20), "
                "64 views 256x256, step 0.5 voxel, volume grad",
        "camera": "frame", "interval": 32, "estimate": "const0.1", "res": 128, "views": 64, "image": 256},
    "large_mixed_512": {
        "desc": "large_mixed_512: 512^3 blobs+band-limited noise, linear TF R=16, 16 views 1024x1024 as per-pixel "
                "rays, step 0.5 voxel, ray + volume + TF grads",
        "camera": "rays", "interval": 16, "estimate": "target", "res": 512, "views": 16, "image": 1024},
    "preshaded_256": {
        "desc": "preshaded_256: the tf_reconstruction_256 scene pre-shaded into a 4x256^3 colour volume, "
                "8 views 256x256, step 0.25 voxel, colour-volume grad against the full volume from half of it",
        "camera": "frame", "interval": 16, "estimate": "half", "res": 256, "views": 8, "image": 256},
    "plain_cpu_64": {
        "desc": "plain_cpu_64: 64^3 blobs, linear TF R=8, one 128x128 view, step 0.5 voxel, TF + volume grads",
        "camera": "frame", "interval": 16, "estimate": "target", "res": 64, "views": 1, "image": 128},
    "batched_uneven_32": {
        "desc": "batched_uneven_32: 32 instances in one batched call per pass, volume edges from "
                "{32,64,96,128,192,256}, images from {64,128,256,512}^2, 16 blobs, sum of 4 Gaussians TF, "
                "step 0.5 voxel, TF + volume grads",
        "camera": "rays", "interval": 16, "estimate": "target", "res": 256, "views": 1, "image": 512,
        "instances": 32},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="tf_reconstruction_256", choices=sorted(WORKLOADS))
    ap.add_argument("--res", type=int, default=None, help="volume edge (workload default)")
    ap.add_argument("--views", type=int, default=None, help="views (workload default)")
    ap.add_argument("--image", type=int, default=None, help="image edge (workload default)")
    ap.add_argument("--storage", choices=["bf16", "f16", "f32"], default="bf16", help="volume storage type")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparison arm")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline budget")
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline, the reference CUDA timing and the accuracy check (profiling runs)")
    ap.add_argument("--interval", type=int, default=0, help="transmittance checkpoint interval (workload default)")
    ap.add_argument("--method", choices=["adjoint", "forward"], default="adjoint",
                    help="gradient method: adjoint (the headline) or forward-mode derivatives")
    ap.add_argument("--gather", choices=["auto", "direct", "cells", "texture"], default="auto",
                    help="how the forward reads a trilinear sample's corners (pyrenderer.set_forward_gather)")
    ap.add_argument("--window", choices=["on", "off"], default="off",
                    help="volume gradients from the record through the window adjoint (on) or the general kernel "
                         "(off, the library's default)")
    ap.add_argument("--record", choices=["full", "auto", "none"], default="auto",
                    help="sample record: a pool for every ray; one for every ray if that fits in a quarter of "
                         "the free device memory, else as large as that; or none")
    a = ap.parse_args()
    spec = WORKLOADS[a.workload]
    for k in ("res", "views", "image"):
        if getattr(a, k) is None:
            setattr(a, k, spec[k])
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, world: int, device) -> list:
    """Each timing's maximum over the ranks: the job's step takes as long as
    its slowest replica.  device: where the collective's tensor lives (CUDA for
    NCCL, CPU for gloo)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def job_rate(samples_per_rank: int, world: int, ms: float) -> float:
    """Whole-job samples/s: every replica marches the same workload."""
    return samples_per_rank * world / (ms / 1e3)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        # 10 ms samples; the timed region starts once the first sample is out
        # (nvidia-smi takes a while to start), so it lies inside the record
        self.first = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "10"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            line = self.proc.stdout.readline()
            if line.strip():
                self.first.append(line)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in self.first + out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ workload
def make_workload(args):
    from diffdvr_gb300 import scenes
    if args.workload == "batched_uneven_32":
        return scenes.batched_uneven(seed=3, n=WORKLOADS[args.workload]["instances"])
    if args.workload == "absorption_recon_128":
        return scenes.absorption_recon_128(seed=2, views=args.views, image=args.image)
    if args.workload == "large_mixed_512":
        return scenes.large_mixed_512(seed=4, res=args.res, views=args.views, image=args.image)
    if args.workload == "plain_cpu_64":
        return scenes.plain_cpu_64(seed=0)
    if args.workload == "preshaded_256":
        return scenes.preshaded_256(seed=1, res=args.res, views=args.views, image=args.image)
    return scenes.tf_reconstruction_256(seed=1, res=args.res, views=args.views, image=args.image)


def l2_copy_peak(dev) -> dict:
    """Copy bandwidth inside L2, measured live: a 12 MB float buffer copied
    into another (24 MB of L2-resident traffic per copy, read + write), 200
    copies after 20 warm-up ones, CUDA events on the current stream.  The
    denominator of the gather model (per-sample corner bytes served from the
    caches)."""
    import torch
    n = 3 * 1024 * 1024
    a = torch.rand(n, device=dev)
    b = torch.empty_like(a)
    for _ in range(20):
        b.copy_(a)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(200):
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 200
    return {"GBps": 2 * n * 4 / (ms * 1e-3) / 1e9, "how": "torch copy of a 12 MB float buffer, 200 times, CUDA events"}


def gather_model(gather_bytes: float, ms: float, l2: dict) -> dict:
    """The gather model's bytes per second (every sample's corners, no
    reuse assumed) against the measured L2 copy bandwidth."""
    achieved = gather_bytes / (ms / 1e3) / 1e9
    return {"achieved_GBps": achieved, "l2_peak_GBps": l2["GBps"], "frac": achieved / l2["GBps"],
            "l2_peak_how": l2["how"], "bytes_per_step": int(gather_bytes)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


# ------------------------------------------------------------------ GPU arm
def algorithmic_bytes(w, s_v, V, P, S, ck_written, recorded, record_kernel, tf_numel):
    """Compulsory HBM bytes per forward and adjoint launch: volume once,
    per-ray outputs/inputs, checkpoints, the sample record (8 B per sample),
    gradients read-modify-written once."""
    grads = set(w.grads)
    fwd = V * s_v + P * (16 + 4) + ck_written * 4
    if recorded:
        fwd += P * 4 + S * 8
    if record_kernel:
        adj = P * (4 + 16 + 4) + S * 8 + tf_numel * 4 * 2
    else:
        regather = (not recorded) or ("camera" in grads)
        adj = (V * s_v if regather else 0) + P * (4 + 16)
        adj += (P * 4 + S * 8) if recorded else ck_written * 4
        if "tf" in grads:
            adj += tf_numel * 4 * 2
        if "volume" in grads:
            adj += V * 4 * 2
        if "camera" in grads:
            adj += P * 24 * 2
    return fwd, adj


def compulsory_bytes(w, s_v, V, P, ck_written, tf_numel, D=0):
    """Compulsory HBM bytes per forward and adjoint launch of the measurement
    plan: the volume read once per launch, colour (16 B) and termination index
    (4 B) written by the forward and read again by the adjoint with the output
    adjoint (16 B), gradients read-modify-written once (volume 4 B per voxel,
    rays 24 B per ray), the TF gradient, and the checkpoints (4 B each here)
    written by the forward and read by the adjoint.  The forward method adds
    its forward variables (16 B per derivative and ray), written once and read
    once."""
    grads = set(w.grads)
    fwd = V * s_v + P * (16 + 4) + ck_written * 4 + P * D * 16
    if D:  # the contraction: forward variables and the output adjoint in, gradients out
        adj = P * D * 16 + P * 16
    else:
        adj = V * s_v + P * (16 + 4 + 16) + ck_written * 4
    if "tf" in grads:
        adj += tf_numel * 4 * 2
    if "volume" in grads:
        adj += V * 4 * 2
    if "camera" in grads:
        adj += P * 24 * 2
    return fwd, adj


# warp-instruction issue rate of the GPU: 4 schedulers per SM, one warp
# instruction each per cycle
ISSUE_PER_SM_CLOCK = 4


def issue_bound(workload: str, kernel: str, samples: int, ms: float):
    """The issue-slot ceiling of the dominant kernel: warp instructions per
    sample from the committed ncu summary of the same workload
    (profiles/issue_rate.txt), the rate they were issued at in this run, and
    the GPU's peak issue rate at its maximum clock."""
    p = os.path.join(ROOT, "profiles", "issue_rate.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    per = d.get("warp_instructions_per_sample", {}).get(workload, {}).get(kernel)
    if per is None:
        return None
    peak = d["sms"] * ISSUE_PER_SM_CLOCK * d["sm_max_mhz"] * 1e6 / 1e12
    achieved = per * samples / (ms / 1e3) / 1e12
    return {"warp_instructions_per_sample": per, "achieved": achieved, "peak": peak, "unit": "T warp-instr/s",
            "frac": achieved / peak, "source": "profiles/issue_rate.txt"}


def reference_cuda(w, args, volume=None):
    """The reference's own CUDA forward + adjoint (its kernels compiled for
    sm_103a from its sources, launched as its backend launches them) on the
    workload, with the gradients the workload asks for, FP32 volume (the
    reference stores no other type; volume: the FP32 volume each step
    renders), L2 flushed before every step.  TF gradients are added by
    immediate atomics: the reference's default delayed accumulation is not
    run (its warp reduction passes the shuffle's value where the member mask
    belongs, renderer/cooperative_groups.cuh:206, and kernels built with it
    raised an illegal-instruction error on the GB300).  None for workloads
    it has no kernels for (pre-shaded volumes, the batched instances); a
    reason where the kernels are absent."""
    from oracle import ref_cuda as R
    if w.name not in R.TIMED_ADJOINTS:
        return None
    if not R.available():
        return {"unavailable": "the reference's kernels were not built (no reference sources where the repo was built)"}
    r = R.time_workload(w, volume=volume, steps=max(3, args.steps // 2), warmup=args.warmup)
    r["source"] = "reference kernels (renderer/renderer_kernels.cuh:92-106, :447-468) built from its sources"
    r["samples_per_s_best"] = r["samples_per_s"]
    if w.name == "tf_reconstruction_256" and (w.width, w.height, w.ray_start.shape[0]) == (256, 256, 8):
        # The reference's default TF adjoint (delayed accumulation) on this
        # workload, timed on a GB300 by this bench before its warp reduction
        # was found to fault (it is not run any more): the speed bar is the
        # faster of the two reference paths.
        r["delayed_recorded"] = dict(REFERENCE_CUDA_DELAYED_TF_RECONSTRUCTION)
        r["samples_per_s_best"] = max(r["samples_per_s"], r["delayed_recorded"]["samples_per_s"])
    return r


# The reference's CUDA forward + delayed-accumulation TF adjoint on the
# TF-reconstruction workload (256^3 FP32, 8 views of 256^2), as this bench
# timed it on a GB300 (2070 MHz, L2 flushed, median of 10 steps) before the
# kernel was retired; see reference_cuda.
REFERENCE_CUDA_DELAYED_TF_RECONSTRUCTION = {
    "forward_ms": 1.7237, "adjoint_ms": 10.6492, "samples_per_step": 89997698, "samples_per_s": 7.2738e9,
    "launch": {"forward": [152, 1024, 0], "adjoint": [912, 32, 32768]},
    "note": "recorded measurement, not re-run: the delayed accumulation's warp reduction passes the shuffle's "
            "value as its member mask (renderer/cooperative_groups.cuh:206)"}


def grad_check(w, spec, args, vol_s, tf, cam, t_inp, K, inputs):
    """The metric's accuracy gate on a bounded subset of the workload, through
    the same entry points and kernels as the timed step: the first two views
    (reference-frame cameras) or 8192 rays that hit the volume (per-pixel-ray
    cameras), rendered with a sample record as the step does, their L2-loss
    gradient against the target images, and the workload's gradients; then
    the FP64 oracle on the same inputs (the stored volume's rounded values)."""
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from oracle import check, oracle as O
    dev = vol_s.device
    if spec["camera"] == "frame":
        nv = min(2, cam[0].shape[0])
        sub = (cam[0][:nv].contiguous(),)
        W, H = w.width, w.height
        target_inputs = inputs(t_inp.volume, t_inp.tf, sub)
        what = f"first {nv} views"
    else:
        rs, rd = w.ray_start.reshape(-1, 3), w.ray_dir.reshape(-1, 3)
        t = -(rs * rd).sum(1)
        hit = np.nonzero(np.linalg.norm(rs + t[:, None] * rd, axis=1) < 0.866)[0]
        idx = np.sort(np.random.default_rng(0).choice(hit, size=min(8192, hit.size), replace=False))
        W, H = idx.size, 1
        sub = (torch.from_numpy(rs[idx].reshape(1, 1, -1, 3).copy()).to(dev),
               torch.from_numpy(rd[idx].reshape(1, 1, -1, 3).copy()).to(dev))
        target_inputs = inputs(t_inp.volume, t_inp.tf, sub)
        what = f"{idx.size} rays hitting the volume"

    def sized(inp):
        inp.screen_size = pr.int2(W, H)
        return inp

    inp = sized(inputs(vol_s, tf, sub))
    target_inputs = sized(target_inputs)
    B = sub[0].shape[0]
    color = torch.empty(B, H, W, 4, device=dev)
    term = torch.empty(B, H, W, dtype=torch.int32, device=dev)
    out = pr.RendererOutputs(color, term, torch.empty(B, H, W, pr.Renderer.checkpoint_slots(inp, K), device=dev), K)
    out.sample_density = torch.empty(pr.Renderer.sample_density_size(inp, B), device=dev)
    out.sample_offset = torch.empty(B, H, W, dtype=torch.int32, device=dev)
    pr.Renderer.render_forward(inp, out)
    target = torch.empty_like(color)
    pr.Renderer.render_forward(target_inputs, pr.RendererOutputs(target, torch.empty_like(term)))
    adj_color = (color - target) * (2.0 / color.numel())
    a = pr.AdjointOutputs()
    grads = {}
    if "tf" in w.grads:
        a.has_tf_derivatives = True
        a.tf_delayed_accumulation = True
        a.adj_tf = grads["adj_tf"] = torch.zeros(tf.shape, device=dev)
    if "volume" in w.grads:
        a.has_volume_derivatives = True
        a.adj_volume = grads["adj_volume"] = torch.zeros(vol_s.shape, device=dev)
    if "camera" in w.grads:
        a.has_camera_derivatives = True
        a.adj_camera_ray_start = grads["adj_ray_start"] = torch.zeros(B, H, W, 3, device=dev)
        a.adj_camera_ray_dir = grads["adj_ray_dir"] = torch.zeros(B, H, W, 3, device=dev)
    pr.Renderer.render_adjoint(inp, out, adj_color, a)
    torch.cuda.synchronize()
    vol_np = vol_s.float().cpu().numpy()
    sc = O.Scene(width=W, height=H, volume=vol_np, tf=tf.cpu().numpy(),
                 step_size=np.full((1, 1, 1), w.step_size, np.float32),
                 box_min=np.asarray([w.box_min], np.float32), box_size=np.asarray([w.box_size], np.float32),
                 filter_mode=w.filter_mode, tf_mode=w.tf_mode, blend_mode=w.blend_mode,
                 camera_mode=2 if spec["camera"] == "frame" else 0)
    if spec["camera"] == "frame":
        sc.camera_matrix = sub[0].cpu().numpy()
        sc.fov_y_radians = float(np.float32(w.fov_y))
    else:
        sc.ray_start, sc.ray_dir = sub[0].cpu().numpy(), sub[1].cpu().numpy()
    t0 = time.perf_counter()
    r = check.render_errors(sc, color.cpu().numpy(), term.cpu().numpy(), adj_color.cpu().numpy(),
                            {k: v.double().cpu().numpy() for k, v in grads.items()})
    r["oracle_s"] = round(time.perf_counter() - t0, 1)
    r["subset"] = what
    r["against"] = "FP64 oracle on the same inputs (stored volume values), L2-loss output adjoint"
    return r


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from diffdvr_gb300 import _abi, pyrenderer as pr

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _abi.load()

    w = make_workload(args)
    spec = WORKLOADS[args.workload]
    grads = set(w.grads)
    B, H, W = w.ray_start.shape[0], w.height, w.width
    vol_target32 = torch.from_numpy(w.volume).to(dev)
    # the absorption reconstruction renders its estimate (0.1 everywhere) against the target's images
    if spec["estimate"] == "const0.1":
        vol32 = torch.full_like(vol_target32, 0.1)
    elif spec["estimate"] == "half":  # the pre-shaded estimate: half the target's colour and absorption
        vol32 = vol_target32 * 0.5
    else:
        vol32 = vol_target32
    sdt = {"bf16": torch.bfloat16, "f16": torch.float16, "f32": torch.float32}[args.storage]
    vol_s = vol32.to(sdt)
    tf = torch.from_numpy(w.tf).to(dev)
    rays = spec["camera"] == "rays"
    if rays:
        cam = (torch.from_numpy(w.ray_start).to(dev), torch.from_numpy(w.ray_dir).to(dev))
    else:
        cam = (torch.from_numpy(w.viewport.astype(np.float32)).to(dev),)

    def inputs(volume, tf_t, cam_t):
        inp = pr.RendererInputs()
        inp.screen_size = pr.int2(W, H)
        inp.volume = volume
        inp.volume_filter_mode = pr.VolumeFilterMode(w.filter_mode)
        inp.box_min = pr.real3(*w.box_min)
        inp.box_size = pr.real3(*w.box_size)
        if rays:
            inp.camera_mode = pr.CameraMode.RayStartDir
            inp.camera = pr.CameraPerPixelRays(cam_t[0], cam_t[1])
        else:
            inp.camera_mode = pr.CameraMode.ReferenceFrame
            inp.camera = pr.CameraReferenceFrame(cam_t[0], float(w.fov_y))
        inp.step_size = float(w.step_size)
        inp.tf_mode = pr.TFMode(w.tf_mode)
        inp.tf = tf_t
        inp.blend_mode = pr.BlendMode(w.blend_mode)
        return inp

    inp_s = inputs(vol_s, tf, cam)
    K = args.interval or spec["interval"]
    slots = pr.Renderer.checkpoint_slots(inp_s, K)
    color = torch.empty(B, H, W, 4, device=dev)
    term = torch.empty(B, H, W, dtype=torch.int32, device=dev)
    ckpt = torch.empty(B, H, W, slots, device=dev)
    out = pr.RendererOutputs(color, term, ckpt, K)
    pool = 0
    record_mode = "none"
    # pre-shaded: the record only on request (the adjoint uses it when the rays are few)
    if args.record != "none" and args.method == "adjoint" and (w.filter_mode != 3 or args.record == "full"):
        full = pr.Renderer.sample_density_size(inp_s, B)
        pool = full
        if args.record == "auto":
            free, _ = torch.cuda.mem_get_info(dev)
            pool = min(full, free // 4 // 4) // 4 * 4
        record_mode = "full" if pool == full else "partial"
        out.sample_density = torch.empty(pool, device=dev)
        out.sample_offset = torch.empty(B, H, W, dtype=torch.int32, device=dev)
    adj = pr.AdjointOutputs()
    g_tensors = []
    if "tf" in grads:
        adj.has_tf_derivatives = True
        adj.tf_delayed_accumulation = True
        adj.adj_tf = torch.zeros(tf.shape, device=dev)
        g_tensors.append(adj.adj_tf)
    if "volume" in grads:
        adj.has_volume_derivatives = True
        adj.adj_volume = torch.zeros(vol32.shape, device=dev)
        g_tensors.append(adj.adj_volume)
    if "camera" in grads:
        adj.has_camera_derivatives = True
        adj.adj_camera_ray_start = torch.zeros(B, H, W, 3, device=dev)
        adj.adj_camera_ray_dir = torch.zeros(B, H, W, 3, device=dev)
        g_tensors += [adj.adj_camera_ray_start, adj.adj_camera_ray_dir]
    adj_color = torch.empty_like(color)
    record_kernel = pool > 0 and grads == {"tf"} and w.tf_mode == 1
    forward_method = args.method == "forward"
    fs = J = out_fg = None
    if forward_method:
        if "volume" in grads:
            raise SystemExit(f"the forward method has no volume derivatives ({args.workload} optimises the volume)")
        fs = pr.ForwardDifferencesSettings()
        D = 0
        if "camera" in grads:
            fs.d_rayStart, fs.d_rayDir = pr.int3(0, 1, 2), pr.int3(3, 4, 5)
            D = 6
        if "tf" in grads:
            _, R, C = tf.shape
            fs.d_tf = torch.arange(D, D + R * C, dtype=torch.int32, device=dev).reshape(1, R, C)
            fs.has_tf_derivatives = True
            D += R * C
        fs.D = D
        J = torch.empty(B, H, W, D, 4, device=dev)
        out_fg = pr.RendererOutputs(color, term)
        record_kernel = False

    # target image: the target volume (absorption reconstruction) or the TF perturbed
    target = torch.empty_like(color)
    pr.set_kernel_family("optimized")
    pr.set_window_adjoint(args.window == "on")
    pr.set_forward_gather(args.gather)
    if spec["estimate"] in ("const0.1", "half"):
        t_inp = inputs(vol_target32.to(sdt), tf, cam)
    else:
        g = torch.Generator(device="cpu").manual_seed(3)
        tf_target = (tf.cpu() + 0.05 * torch.randn(tf.shape, generator=g)).clamp_min(0).to(dev)
        if w.tf_mode == 2:  # keep the linear TF's positions
            tf_target[..., 4] = tf[..., 4]
        t_inp = inputs(vol_s, tf_target, cam)
    pr.Renderer.render_forward(t_inp, pr.RendererOutputs(target, torch.empty_like(term)))
    torch.cuda.synchronize()
    inv_n = 1.0 / color.numel()

    stream = torch.cuda.Stream(device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    fwd_ev, adj_ev = [], []

    def step(record=False):
        # forward + L2-loss gradient + adjoint
        if record:
            e = (ev(), ev(), ev(), ev())
            e[0].record()
        if forward_method:
            pr.Renderer.render_forward_gradients(inp_s, fs, out_fg, J)
        else:
            pr.Renderer.render_forward(inp_s, out)
        if record:
            e[1].record()
        torch.sub(color, target, out=adj_color)
        adj_color.mul_(2 * inv_n)
        for t in g_tensors:
            t.zero_()
        if record:
            e[2].record()
        if forward_method:
            pr.Renderer.forward_variables_to_gradients(J, adj_color, fs, adj)
        else:
            pr.Renderer.render_adjoint(inp_s, out, adj_color, adj)
        if record:
            e[3].record()
            fwd_ev.append((e[0], e[1]))
            adj_ev.append((e[2], e[3]))

    with torch.cuda.stream(stream):
        step()
    torch.cuda.synchronize()
    samples = int(term.to(torch.int64).sum().item())
    rays_hit = int((term > 0).sum().item())
    recorded_rays = int((out.sample_offset >= 0).sum().item()) if pool > 0 else 0

    # capture the step in a CUDA graph
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        step()
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=stream):
            step()
    torch.cuda.synchronize()

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def timed(fn, steps, warmup, pre=None):
        for _ in range(warmup):
            if pre:
                pre()
            fn()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        starts = [ev() for _ in range(steps)]
        stops = [ev() for _ in range(steps)]
        cur = torch.cuda.current_stream()
        for i in range(steps):
            flush.zero_()
            if pre:
                pre()
            starts[i].record(cur)
            fn()
            stops[i].record(cur)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return sum(a.elapsed_time(b) for a, b in zip(starts, stops)) / steps

    # ---- value: device-resident, graph replay
    with torch.cuda.stream(stream):
        with ClockSampler(local) as clocks:
            ms_graph = timed(lambda: graph.replay(), args.steps, args.warmup)
    clock_summary = clocks.summary()

    # ---- kernel durations for the roofline (same stream, events around launches)
    fwd_ev.clear()
    adj_ev.clear()
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.steps // 2)):
            flush.zero_()
            step(record=True)
        torch.cuda.synchronize()
    fwd_ms = float(np.mean([a.elapsed_time(b) for a, b in fwd_ev]))
    adj_ms = float(np.mean([a.elapsed_time(b) for a, b in adj_ev]))

    # ---- e2e: public API with host buffers
    vol_host = vol_s.cpu().pin_memory()
    tf_host = tf.cpu().pin_memory()
    cam_host = [c.cpu().pin_memory() for c in cam]
    target_host = target.cpu().pin_memory()
    loss_host = torch.empty(1, pin_memory=True)
    read_back = adj.adj_tf if "tf" in grads else None
    grad_host = torch.empty_like(read_back, device="cpu").pin_memory() if read_back is not None else None
    vol_d, tf_d, tgt_d = torch.empty_like(vol_s), torch.empty_like(tf), torch.empty_like(target)
    cam_d = [torch.empty_like(c) for c in cam]
    inp_e2e = inputs(vol_d, tf_d, cam_d)
    loss_d = torch.empty(1, device=dev)

    # the target image is needed only by the loss: its copy runs on a side
    # stream beside the forward, after the previous step's loss has read it
    copy_stream = torch.cuda.Stream(device=dev)
    target_in = torch.cuda.Event()

    def e2e_step():
        cur = torch.cuda.current_stream()
        copy_stream.wait_stream(cur)
        with torch.cuda.stream(copy_stream):
            tgt_d.copy_(target_host, non_blocking=True)
            target_in.record(copy_stream)
        vol_d.copy_(vol_host, non_blocking=True)
        tf_d.copy_(tf_host, non_blocking=True)
        for d, h in zip(cam_d, cam_host):
            d.copy_(h, non_blocking=True)
        if forward_method:
            pr.Renderer.render_forward_gradients(inp_e2e, fs, out_fg, J)
        else:
            pr.Renderer.render_forward(inp_e2e, out)
        cur.wait_event(target_in)
        torch.sub(color, tgt_d, out=adj_color)
        loss_d.copy_((adj_color * adj_color).sum().view(1))
        adj_color.mul_(2 * inv_n)
        for t in g_tensors:
            t.zero_()
        if forward_method:
            pr.Renderer.forward_variables_to_gradients(J, adj_color, fs, adj)
        else:
            pr.Renderer.render_adjoint(inp_e2e, out, adj_color, adj)
        loss_host.copy_(loss_d, non_blocking=True)
        if grad_host is not None:
            grad_host.copy_(read_back, non_blocking=True)

    with torch.cuda.stream(stream):
        ms_e2e = timed(e2e_step, args.steps, args.warmup)
    h2d = vol_host.numel() * vol_host.element_size() + tf_host.numel() * 4 + sum(c.numel() * 4 for c in cam_host) + \
        target_host.numel() * 4
    d2h = 4 + (grad_host.numel() * 4 if grad_host is not None else 0)

    # ---- plain FP32 arm (same workload, the reference's GPU algorithm)
    plain = None
    if not args.no_plain and not forward_method:
        inp32 = inputs(vol32, tf, cam)
        out32 = pr.RendererOutputs(torch.empty_like(color), torch.empty_like(term))

        def plain_step():
            pr.Renderer.render_forward(inp32, out32)
            torch.sub(out32.color, target, out=adj_color)
            adj_color.mul_(2 * inv_n)
            for t in g_tensors:
                t.zero_()
            pr.Renderer.render_adjoint(inp32, out32, adj_color, adj)

        pr.set_kernel_family("plain")
        with torch.cuda.stream(stream):
            ms_plain = timed(plain_step, max(2, args.steps // 4), 2)
        pr.set_kernel_family("optimized")
        samples32 = int(out32.terminationIndex.to(torch.int64).sum().item())
        plain = {"samples_per_s": samples32 / (ms_plain / 1e3), "ms_per_step": ms_plain,
                 "kernels": "plain FP32 (one thread per ray, blend inversion)"}

    # ---- memory-lean arm: no sample record, transmittance checkpoints only
    checkpoint_only = None
    if pool > 0 and not forward_method:
        out_ck = pr.RendererOutputs(color, term, ckpt, K)
        fwd_ev.clear()
        adj_ev.clear()

        def ck_step(record=False):
            e = (ev(), ev(), ev(), ev()) if record else None
            if record:
                e[0].record()
            pr.Renderer.render_forward(inp_s, out_ck)
            if record:
                e[1].record()
            torch.sub(color, target, out=adj_color)
            adj_color.mul_(2 * inv_n)
            for t in g_tensors:
                t.zero_()
            if record:
                e[2].record()
            pr.Renderer.render_adjoint(inp_s, out_ck, adj_color, adj)
            if record:
                e[3].record()
                fwd_ev.append((e[0], e[1]))
                adj_ev.append((e[2], e[3]))

        graph_ck = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            ck_step()
            torch.cuda.synchronize()
            with torch.cuda.graph(graph_ck, stream=stream):
                ck_step()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ms_ck = timed(lambda: graph_ck.replay(), max(3, args.steps // 2), args.warmup)
            for _ in range(3):
                flush.zero_()
                ck_step(record=True)
            torch.cuda.synchronize()
            ck_path = pr.last_adjoint_path()
        checkpoint_only = {
            "samples_per_s": samples / (ms_ck / 1e3), "ms_per_step": ms_ck,
            "forward_ms": float(np.mean([a_.elapsed_time(b_) for a_, b_ in fwd_ev])),
            "adjoint_ms": float(np.mean([a_.elapsed_time(b_) for a_, b_ in adj_ev])),
            "checkpoint_interval": K, "checkpoint_MB": round(ckpt.numel() * 4 / 1e6, 1),
            "adjoint_path": ck_path,
            "issue": issue_bound(args.workload, "adjoint_remarch", samples,
                                 float(np.mean([a_.elapsed_time(b_) for a_, b_ in adj_ev])))
            if ck_path == "remarch" else None,
            "path": "no sample record; the adjoint re-marches from the checkpoints (remarch: each warp re-marches its "
                    "ray in chunks of up to 512 samples into shared memory; general: per-ray K-sample segments)"}

    # ---- aggregate over ranks (max time)
    ms_graph, ms_e2e = max_over_ranks([ms_graph, ms_e2e], world, dev)
    value = job_rate(samples, world, ms_graph)
    e2e_value = job_rate(samples, world, ms_e2e)

    # ---- roofline of the dominant kernel (compulsory HBM bytes per launch)
    peak, peak_kind = measured_peaks()
    V = int(np.prod(w.volume.shape[1:])) * (4 if w.filter_mode == 3 else 1)  # pre-shaded: 4 channels
    P = B * H * W
    ck_per_ray = torch.clamp((term.to(torch.int64) - 1) // K, min=0).clamp_max(slots)
    if pool > 0:  # recorded rays write no checkpoints
        ck_per_ray = torch.where(out.sample_offset >= 0, torch.zeros_like(ck_per_ray), ck_per_ray)
    ck_written = int(ck_per_ray.sum().item())
    s_v = vol_s.element_size()
    if forward_method:
        # volume once, colour + termination, the forward variables written once and read once
        fwd_bytes = V * s_v + P * (16 + 4) + P * fs.D * 16
        adj_bytes = P * fs.D * 16 + P * 16 + tf.numel() * 4 * 2 + (P * 24 if "camera" in grads else 0)
        names = ("contraction", "forward gradients")
    else:
        fwd_bytes, adj_bytes = algorithmic_bytes(w, s_v, V, P, samples, ck_written, pool > 0, record_kernel,
                                                 tf.numel())
        if w.filter_mode == 3 and pool > 0:
            adj_bytes += V * s_v  # the pre-shaded record holds opacities only: colours are gathered again
        names = ("adjoint", "forward")
    dominant = (names[0], adj_bytes, adj_ms) if adj_ms >= fwd_ms else (names[1], fwd_bytes, fwd_ms)
    # the compulsory HBM model of the measurement plan: volume, per-ray outputs
    # and inputs, gradients and checkpoints, without the sample record this
    # design chooses to write
    comp_fwd, comp_adj = compulsory_bytes(w, s_v, V, P, ck_written, tf.numel(), fs.D if forward_method else 0)
    comp = comp_adj if dominant[0] == names[0] else comp_fwd
    achieved = comp / (dominant[2] / 1e3) / 1e9
    achieved_rec = dominant[1] / (dominant[2] / 1e3) / 1e9
    tr = profiled_traffic()
    traffic = None
    if tr and tr.get("workload") == args.workload and tr.get("record") == record_mode and tr.get("views") == B \
            and tr.get("method", "adjoint") == args.method:
        traffic = tr.get("dram_bytes_per_launch", {}).get(dominant[0])
    # 8 corner reads per sample in the forward, and in the adjoint unless it reads the record
    regather = pool == 0 or "camera" in grads
    gather_bytes = samples * 8 * s_v * (2 if regather else 1)
    # kernels of ours per step: forward = ray order (3) + march; adjoint = ray order (3) + the
    # record kernel and the general kernel over its leftovers, or the general kernel alone
    launches_per_step = 4 + (5 if record_kernel else 4)
    if forward_method:
        launches_per_step = 2  # forward-gradient march + contraction
    elif w.filter_mode == 3:
        # pre-shaded: forward; ray order (3) + the record kernel and the per-lane kernel over its leftovers
        launches_per_step = 1 + 3 + (2 if pool > 0 else 1)

    result = {
        "metric": METRIC_FORWARD if forward_method else METRIC,
        "value": value,
        "unit": "samples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_graph,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": f"{args.storage}-storage/f32-compute",
        "data": "synthetic (seeded, shapes and distributions of the workload)",
        "config": {"workload": spec["desc"], "volume_storage": args.storage,
                   "tf_storage": "f32", "views": B, "image": [H, W], "volume": list(w.volume.shape[1:]),
                   "gradients": sorted(grads), "samples_per_step": samples, "rays_hit": rays_hit,
                   "method": args.method, "forward_derivatives": fs.D if forward_method else None,
                   "checkpoint_interval": K, "sample_record": record_mode, "window_adjoint": args.window, "forward_gather": args.gather,
                   "recorded_rays": recorded_rays, "record_pool_MB": round(pool * 4 / 1e6, 1),
                   "l2": "flushed (256 MB write) before every timed step",
                   "graph": "forward+loss+adjoint captured in one CUDA graph",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
                "path": ("pyrenderer.Renderer.render_forward_gradients/forward_variables_to_gradients"
                         if forward_method else "pyrenderer.Renderer.render_forward/render_adjoint")
                + ", pinned host inputs"},
        "gpu_launches": launches_per_step * args.steps,
        "kernel_ms": {names[1]: fwd_ms, names[0]: adj_ms},
        "roofline": {"bound": "hbm", "kernel": dominant[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": int(comp),
                     "bytes_model": "compulsory: volume once, per-ray outputs and inputs, gradients, checkpoints",
                     "with_record": {"bytes_per_launch": int(dominant[1]), "achieved": achieved_rec,
                                     "frac": achieved_rec / peak},
                     "gather_model_GBps": gather_bytes / ((fwd_ms + adj_ms) / 1e3) / 1e9,
                     "gather_model": gather_model(gather_bytes, fwd_ms + adj_ms, l2_copy_peak(dev)),
                     "issue": issue_bound(args.workload, dominant[0], samples, dominant[2])},
        "plain_fp32": plain,
        "speedup_vs_plain_fp32": (value / plain["samples_per_s"]) if plain else None,
        "checkpoint_only": checkpoint_only,
        "clocks": clock_summary,
    }
    if rank == 0 and not args.no_cpu:
        # baselines and the accuracy check: the oracle and the reference's own kernels as checkers
        result["reference_cuda"] = reference_cuda(w, args, vol32.cpu().numpy())
        if result["reference_cuda"] and "samples_per_s" in result["reference_cuda"]:
            result["speedup_vs_reference_cuda"] = value / result["reference_cuda"]["samples_per_s_best"]
        if not forward_method and w.filter_mode != 3:
            chk = grad_check(w, spec, args, vol_s, tf, cam, t_inp, K, inputs)
            result["grad_check"] = chk
            result["grad_rel_err"] = chk.get("grad_rel_err")
    if rank == 0:
        result["cpu_baseline"] = None if args.no_cpu else cpu_baseline(w, args, vol32.cpu().numpy(), args.method)
        print(json.dumps(result))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_gpu_batched(args):
    """The batched-uneven workload: every instance's forward in one
    render_forward_batched call and every adjoint in one
    render_adjoint_batched call (one launch per 24 instances each), the
    per-instance L2-loss gradients between them, the step captured in one
    CUDA graph.  value = samples of all instances / step time."""
    import torch
    import torch.distributed as dist
    from diffdvr_gb300 import _abi, pyrenderer as pr

    if args.method != "adjoint":
        raise SystemExit("the batched entry points have no forward method")
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _abi.load()
    spec = WORKLOADS[args.workload]
    ws = make_workload(args)
    sdt = {"bf16": torch.bfloat16, "f16": torch.float16, "f32": torch.float32}[args.storage]
    K = args.interval or spec["interval"]
    pr.set_kernel_family("optimized")

    def inputs(w, volume, tf_t, rs, rd):
        inp = pr.RendererInputs()
        inp.screen_size = pr.int2(w.width, w.height)
        inp.volume = volume
        inp.volume_filter_mode = pr.VolumeFilterMode(w.filter_mode)
        inp.box_min = pr.real3(*w.box_min)
        inp.box_size = pr.real3(*w.box_size)
        inp.camera_mode = pr.CameraMode.RayStartDir
        inp.camera = pr.CameraPerPixelRays(rs, rd)
        inp.step_size = float(w.step_size)
        inp.tf_mode = pr.TFMode(w.tf_mode)
        inp.tf = tf_t
        inp.blend_mode = pr.BlendMode(w.blend_mode)
        return inp

    I = []  # per instance: device tensors, inputs, outputs, gradients
    g = torch.Generator(device="cpu").manual_seed(3)
    for w in ws:
        d = {"w": w}
        d["vol_s"] = torch.from_numpy(w.volume).to(dev).to(sdt)
        d["tf"] = torch.from_numpy(w.tf).to(dev)
        d["rs"], d["rd"] = torch.from_numpy(w.ray_start).to(dev), torch.from_numpy(w.ray_dir).to(dev)
        d["inp"] = inputs(w, d["vol_s"], d["tf"], d["rs"], d["rd"])
        slots = pr.Renderer.checkpoint_slots(d["inp"], K)
        d["color"] = torch.empty(1, w.height, w.width, 4, device=dev)
        d["term"] = torch.empty(1, w.height, w.width, dtype=torch.int32, device=dev)
        d["out"] = pr.RendererOutputs(d["color"], d["term"],
                                      torch.empty(1, w.height, w.width, slots, device=dev), K)
        d["slots"] = slots
        d["pool"] = pr.Renderer.sample_density_size(d["inp"], 1) if args.record != "none" else 0
        a = pr.AdjointOutputs()
        a.has_tf_derivatives = True
        a.tf_delayed_accumulation = True
        a.adj_tf = torch.zeros(d["tf"].shape, device=dev)
        a.has_volume_derivatives = True
        a.adj_volume = torch.zeros(d["vol_s"].shape, device=dev)
        d["adj"] = a
        d["adj_color"] = torch.empty_like(d["color"])
        # target image: the instance's TF perturbed by N(0, 0.05)
        tf_t = (d["tf"].cpu() + 0.05 * torch.randn(d["tf"].shape, generator=g)).clamp_min(0).to(dev)
        tf_t[..., 5] = d["tf"][..., 5]  # keep the Gaussians' widths positive as drawn
        d["target"] = torch.empty_like(d["color"])
        pr.Renderer.render_forward(inputs(w, d["vol_s"], tf_t, d["rs"], d["rd"]),
                                   pr.RendererOutputs(d["target"], torch.empty_like(d["term"])))
        d["inv_n"] = 1.0 / d["color"].numel()
        I.append(d)
    # sample records (every ray its fixed run of its instance's pool), when they fit
    pool_total = sum(d["pool"] for d in I)
    free, _ = torch.cuda.mem_get_info(dev)
    use_record = pool_total > 0 and (args.record == "full" or pool_total * 4 <= free // 4)
    if use_record:
        for d in I:
            d["out"].sample_density = torch.empty(d["pool"], device=dev)
            d["out"].sample_offset = torch.empty(1, d["w"].height, d["w"].width, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    ins, outs = [d["inp"] for d in I], [d["out"] for d in I]
    adjs, aos = [d["adj_color"] for d in I], [d["adj"] for d in I]

    stream = torch.cuda.Stream(device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    fwd_ev, adj_ev = [], []

    def loss_grads(targets=None):
        for j, d in enumerate(I):
            torch.sub(d["color"], d["target"] if targets is None else targets[j], out=d["adj_color"])
            d["adj_color"].mul_(2 * d["inv_n"])
            d["adj"].adj_tf.zero_()
            d["adj"].adj_volume.zero_()

    # tile shapes per size class from the autotuner (a fresh cache: every run searches)
    from diffdvr_gb300.autotune import SHAPE_NAMES, TileTuner
    import tempfile
    tuner = TileTuner(cache_path=os.path.join(tempfile.mkdtemp(prefix="dvr_tune_"), "tiles.json"))
    with torch.cuda.stream(stream):
        pr.Renderer.render_forward_batched(ins, outs)
        loss_grads()
        t0 = time.perf_counter()
        fwd_shapes, adj_shapes = tuner.tune(ins, outs, adjs, aos, storage=args.storage)
        torch.cuda.synchronize()
        tune_s = time.perf_counter() - t0
    shapes = {"forward": list(fwd_shapes), "adjoint": list(adj_shapes)}

    def step(record=False):
        if record:
            e = (ev(), ev(), ev(), ev())
            e[0].record()
        pr.Renderer.render_forward_batched(ins, outs, shapes["forward"])
        if record:
            e[1].record()
        loss_grads()
        if record:
            e[2].record()
        pr.Renderer.render_adjoint_batched(ins, outs, adjs, aos, shapes["adjoint"])
        if record:
            e[3].record()
            fwd_ev.append((e[0], e[1]))
            adj_ev.append((e[2], e[3]))

    with torch.cuda.stream(stream):
        step()
    torch.cuda.synchronize()
    samples = sum(int(d["term"].to(torch.int64).sum().item()) for d in I)

    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        step()
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=stream):
            step()
    torch.cuda.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        starts = [ev() for _ in range(steps)]
        stops = [ev() for _ in range(steps)]
        cur = torch.cuda.current_stream()
        for i in range(steps):
            flush.zero_()
            starts[i].record(cur)
            fn()
            stops[i].record(cur)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return sum(a.elapsed_time(b) for a, b in zip(starts, stops)) / steps

    with torch.cuda.stream(stream):
        with ClockSampler(local) as clocks:
            ms_graph = timed(lambda: graph.replay(), args.steps, args.warmup)
    clock_summary = clocks.summary()

    with torch.cuda.stream(stream):
        for _ in range(max(3, args.steps // 2)):
            flush.zero_()
            step(record=True)
        torch.cuda.synchronize()
    fwd_ms = float(np.mean([a.elapsed_time(b) for a, b in fwd_ev]))
    adj_ms = float(np.mean([a.elapsed_time(b) for a, b in adj_ev]))

    # ---- the same step with the fixed 16x8 tile, for the tuner's gain
    tuned = dict(shapes)
    shapes["forward"], shapes["adjoint"] = [0] * len(I), [0] * len(I)
    fwd_ev.clear()
    adj_ev.clear()
    graph_fixed = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        step()
        torch.cuda.synchronize()
        with torch.cuda.graph(graph_fixed, stream=stream):
            step()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ms_fixed = timed(lambda: graph_fixed.replay(), args.steps, args.warmup)
        for _ in range(3):
            flush.zero_()
            step(record=True)
        torch.cuda.synchronize()
    tile_tuning = {
        "classes": len(set(tuner.cache.get(tuner._device(), {}).keys())), "tuning_s": round(tune_s, 2),
        "search": tuner.report, "tuned_ms_per_step": ms_graph, "fixed_16x8_ms_per_step": ms_fixed,
        "gain": ms_fixed / ms_graph,
        "fixed_16x8_kernel_ms": {"forward": float(np.mean([a.elapsed_time(b) for a, b in fwd_ev])),
                                 "adjoint": float(np.mean([a.elapsed_time(b) for a, b in adj_ev]))},
        "forward_shapes": [SHAPE_NAMES[t] for t in tuned["forward"]],
        "adjoint_shapes": [SHAPE_NAMES[t] for t in tuned["adjoint"]]}
    shapes.update(tuned)

    # ---- e2e: the batched public API with every input copied from pinned host memory
    host = [{k: d[k].cpu().pin_memory() for k in ("vol_s", "tf", "rs", "rd", "target")} for d in I]
    devc = [{k: torch.empty_like(d[k]) for k in ("vol_s", "tf", "rs", "rd", "target")} for d in I]
    ins_e2e = [inputs(d["w"], c["vol_s"], c["tf"], c["rs"], c["rd"]) for d, c in zip(I, devc)]
    loss_d = torch.empty(len(I), device=dev)
    loss_host = torch.empty(len(I), pin_memory=True)
    grad_host = [torch.empty(d["tf"].shape, pin_memory=True) for d in I]

    def e2e_step():
        for h, c in zip(host, devc):
            for k in h:
                c[k].copy_(h[k], non_blocking=True)
        pr.Renderer.render_forward_batched(ins_e2e, outs, shapes["forward"])
        loss_grads([c["target"] for c in devc])
        for j, d in enumerate(I):
            loss_d[j] = (d["adj_color"] * d["adj_color"]).sum() / (4 * d["inv_n"] * d["inv_n"])
        pr.Renderer.render_adjoint_batched(ins_e2e, outs, adjs, aos, shapes["adjoint"])
        loss_host.copy_(loss_d, non_blocking=True)
        for gh, d in zip(grad_host, I):
            gh.copy_(d["adj"].adj_tf, non_blocking=True)

    with torch.cuda.stream(stream):
        ms_e2e = timed(e2e_step, args.steps, args.warmup)
    h2d = sum(sum(t.numel() * t.element_size() for t in h.values()) for h in host)
    d2h = loss_host.numel() * 4 + sum(gh.numel() * 4 for gh in grad_host)

    ms_graph, ms_e2e = max_over_ranks([ms_graph, ms_e2e], world, dev)
    value = job_rate(samples, world, ms_graph)
    e2e_value = job_rate(samples, world, ms_e2e)

    # ---- roofline: compulsory bytes summed over the instances of one batched launch pair
    peak, peak_kind = measured_peaks()
    fwd_bytes = adj_bytes = 0
    for d in I:
        w = d["w"]
        V = int(np.prod(w.volume.shape[1:]))
        P = w.width * w.height
        ck = int(torch.clamp((d["term"].to(torch.int64) - 1) // K, min=0).clamp_max(d["slots"]).sum().item())
        S = int(d["term"].to(torch.int64).sum().item())
        f, a = algorithmic_bytes(w, d["vol_s"].element_size(), V, P, S, ck, use_record, False, d["tf"].numel())
        fwd_bytes += f
        adj_bytes += a
    dominant = ("adjoint", adj_bytes, adj_ms) if adj_ms >= fwd_ms else ("forward", fwd_bytes, fwd_ms)
    achieved = dominant[1] / (dominant[2] / 1e3) / 1e9
    s_v = I[0]["vol_s"].element_size()
    launches = -(-len(I) // 24)  # one persistent launch per 24 instances and pass

    result = {
        "metric": METRIC,
        "value": value,
        "unit": "samples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_graph,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": f"{args.storage}-storage/f32-compute",
        "data": "synthetic (seeded, shapes and distributions of the workload)",
        "config": {"workload": spec["desc"], "volume_storage": args.storage, "instances": len(I),
                   "volume_edges": [int(d["w"].volume.shape[1]) for d in I],
                   "image_edges": [int(d["w"].width) for d in I], "gradients": ["tf", "volume"],
                   "samples_per_step": samples, "checkpoint_interval": K,
                   "sample_record": "full" if use_record else "none",
                   "record_pool_MB": round(pool_total * 4 / 1e6, 1) if use_record else 0,
                   "l2": "flushed (256 MB write) before every timed step",
                   "graph": "batched forward + loss gradients + batched adjoint captured in one CUDA graph",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
                "path": "pyrenderer.Renderer.render_forward_batched/render_adjoint_batched, pinned host inputs"},
        "gpu_launches": 2 * launches * args.steps,
        "kernel_ms": {"forward": fwd_ms, "adjoint": adj_ms},
        "tile_tuning": tile_tuning,
        "roofline": {"bound": "hbm", "kernel": dominant[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": int(dominant[1]),
                     "gather_model_GBps": samples * 8 * s_v * 2 / ((fwd_ms + adj_ms) / 1e3) / 1e9,
                     "gather_model": gather_model(samples * 8 * s_v * 2, fwd_ms + adj_ms, l2_copy_peak(dev))},
        "clocks": clock_summary,
    }
    if rank == 0:
        if args.no_cpu:
            result["cpu_baseline"] = None
        else:
            from oracle import oracle as O
            O.build(reference=True)
            kind = "reference" if O.reference_available() else "port"
            v, sample = time_cpu_instances(ws, args.cpu_seconds, kind)
            result["cpu_baseline"] = {"value": v, "unit": "samples/s", "cores": os.cpu_count(), "kind": kind,
                                      "sample": sample}
        print(json.dumps(result))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


# ------------------------------------------------------------------ CPU (reference) arm
def cpu_sample_scene(w, volume, n_rays: int, seed: int = 0):
    """A bounded sample of the workload: n_rays rays of its views, chosen
    among rays that hit the volume, as one 1 x n_rays 'image'."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    rs = w.ray_start.reshape(-1, 3)
    rd = w.ray_dir.reshape(-1, 3)
    # rays whose line passes within the box's circumsphere
    t = -(rs * rd).sum(1)
    closest = rs + t[:, None] * rd
    hit = np.nonzero(np.linalg.norm(closest, axis=1) < 0.866)[0]
    idx = rng.choice(hit, size=min(n_rays, hit.size), replace=False)
    sc = O.Scene(width=idx.size, height=1, volume=volume, tf=w.tf, step_size=np.full((1, 1, 1), w.step_size),
                 box_min=np.array([w.box_min]), box_size=np.array([w.box_size]), filter_mode=w.filter_mode,
                 camera_mode=0, tf_mode=w.tf_mode, blend_mode=w.blend_mode, ray_start=rs[idx][None, None],
                 ray_dir=rd[idx][None, None])
    return sc


def time_cpu(w, volume, budget_s: float, kind: str, method: str = "adjoint"):
    """Forward + adjoint (the workload's gradients) of a ray sample on the host
    cores, or the forward method (forward-mode derivatives + contraction);
    returns (samples/s, description)."""
    from oracle import oracle as O
    req = O.AdjointRequest(tf="tf" in w.grads, volume="volume" in w.grads, camera="camera" in w.grads)
    fs = None
    if method == "forward":
        req.volume = False
        D = 6 if "camera" in w.grads else 0
        kw = {"d_ray_start": (0, 1, 2), "d_ray_dir": (3, 4, 5)} if D else {}
        if "tf" in w.grads:
            _, R, C = w.tf.shape
            kw["d_tf"] = np.arange(D, D + R * C, dtype=np.int32).reshape(1, R, C)
            D += R * C
        fs = O.ForwardSettings(D=D, **kw)

    def one_pass(sc):
        if fs is not None:
            c, term, J = O.forward_gradients(sc, fs, "f32")
            O.forward_variables_to_gradients(J, np.full(c.shape, 1e-3, np.float32), fs, req, precision="f32")
        else:
            c, term = O.forward(sc, kind, "f32")
            O.adjoint(sc, c, term, np.full(c.shape, 1e-3, np.float32), req, kind, "f32")
        return term

    n = 512
    while True:
        sc = cpu_sample_scene(w, volume, n)
        t0 = time.perf_counter()
        one_pass(sc)
        dt = time.perf_counter() - t0
        if dt > budget_s / 6 or n >= 65536:
            break
        n *= 2
    reps, total, samples = 0, 0.0, 0
    while total < budget_s * 0.7 or reps < 2:
        t0 = time.perf_counter()
        term = one_pass(sc)
        total += time.perf_counter() - t0
        samples += int(term.sum())
        reps += 1
    what = "forward-mode + contraction" if fs is not None else "fwd+adj"
    return samples / total, f"{sc.width} rays of the workload (hitting the volume), {reps} {what} passes"


def cpu_baseline(w, args, volume, method: str = "adjoint"):
    from oracle import oracle as O
    O.build(reference=True)
    # the reference's forward mode needs cudAD, which its sources do not include: the oracle port times it
    kind = "reference" if O.reference_available() and method == "adjoint" else "port"
    value, sample = time_cpu(w, volume, args.cpu_seconds, kind, method)
    return {"value": value, "unit": "samples/s", "cores": os.cpu_count(), "kind": kind, "sample": sample}


def time_cpu_instances(ws, budget_s: float, kind: str):
    """time_cpu over the instances of a batched workload, an equal share of
    the budget each (at least 0.3 s); returns (mean samples/s, description)."""
    rates = [time_cpu(w, w.volume, max(0.3, budget_s / len(ws)), kind)[0] for w in ws]
    return float(np.mean(rates)), f"rays of each of the {len(ws)} instances (hitting the volume), fwd+adj passes"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(reference=True)
    kind = "reference" if O.reference_available() and args.method == "adjoint" else "port"
    w = make_workload(args)
    if isinstance(w, list):  # batched instances
        if args.method != "adjoint":
            raise SystemExit("the batched entry points have no forward method")
        timer = lambda budget: time_cpu_instances(w, budget, kind)
    else:
        est = WORKLOADS[args.workload]["estimate"]
        volume = np.full_like(w.volume, 0.1) if est == "const0.1" else (w.volume * 0.5 if est == "half" else w.volume)
        timer = lambda budget: time_cpu(w, volume, budget, kind, args.method)
    for _ in range(args.warmup):
        timer(1.0)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, sample = timer(max(1.0, args.cpu_seconds / max(args.steps, 1)))
        vals.append(v)
    wall = time.perf_counter() - t0
    value = float(np.median(vals))
    res = {"metric": METRIC_FORWARD if args.method == "forward" else METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": WORKLOADS[args.workload]["desc"], "sample": sample}, "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "samples/s", "cores": os.cpu_count(), "kind": kind,
                            "sample": sample},
           "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(res))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif "instances" in WORKLOADS[a.workload]:
        run_gpu_batched(a)
    else:
        run_gpu(a)
