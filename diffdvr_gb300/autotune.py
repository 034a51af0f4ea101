"""Autotuner of the batched launches: the tile shape per size class.

The batched entry points render instances of different volume and image
sizes in one launch of (instance, batch entry, tile) work items, one block of
128 rays per tile.  Which tile shape suits an instance depends on its size:
wide rows of rays (32x4) share more cache lines on short rays across a large
image, tall ones (8x16) or the square 16x8 tile keep a block's rays closer in
length.  The reference has no such choice: its batches share one volume and
image size and its only launch parameter is the occupancy block size
(renderer/renderer_cuda.cpp:97-108).

A size class groups instances that behave alike: the volume's largest edge
and the image's larger edge, each rounded up to a power of two, the sample
step in voxels (rounded to a power of two), the filter, TF and blend modes,
the volume storage type and the gradients the adjoint computes.  ``tune``
searches the shapes of every class of a batch in the batched call itself:
starting from 16x8 everywhere, it tries each other shape for one class at a
time in the full forward and the full adjoint launch (CUDA events on the
current stream, warm-up, median of repeats, on scratch outputs so the
caller's outputs and gradients are untouched; the scratch outputs carry
checkpoints and a sample record where the caller's do, so the adjoint is
timed on the path the caller's call takes) and keeps a shape only when it
beats the current choice by more than the noise margin.  Choices are cached
per device name and class in a JSON file, so later batches and later
processes reuse them without timing.
"""
from __future__ import annotations

import json
import math
import os
from typing import Callable, Dict, List, Optional, Sequence, Tuple

SHAPES = (0, 1, 2)  # DvrTileShape: 16x8, 32x4, 8x16
SHAPE_NAMES = {0: "16x8", 1: "32x4", 2: "8x16"}
MARGIN = 0.02       # a shape replaces the current one when it is this much faster


def _pow2_ceil(v: float) -> int:
    return 1 if v <= 1 else 1 << int(math.ceil(math.log2(v)))


def size_class(volume_shape: Sequence[int], width: int, height: int, step_voxels: float, modes: Sequence[int],
               storage: str, grads: Sequence[str]) -> str:
    """The class key of one instance (see the module docstring).  modes:
    (filter, TF, blend)."""
    edge = _pow2_ceil(max(int(v) for v in volume_shape[-3:]))
    image = _pow2_ceil(max(int(width), int(height)))
    step = 2.0 ** round(math.log2(step_voxels)) if step_voxels > 0 else 0.0
    return (f"vol{edge}-img{image}-step{step:g}-f{modes[0]}t{modes[1]}b{modes[2]}-{storage}-"
            + "+".join(sorted(grads)))


def search(classes: Sequence[str], time_pass: Callable[[Dict[str, int]], float],
           margin: float = MARGIN) -> Tuple[Dict[str, int], float, float]:
    """Coordinate search over the classes' shapes for one pass: time_pass(
    {class: shape}) -> ms of the whole launch.  Returns (choice, ms of the
    choice, ms with 16x8 everywhere)."""
    choice = {c: 0 for c in classes}
    base = best = time_pass(dict(choice))
    for c in classes:
        for shape in SHAPES[1:]:
            trial = dict(choice)
            trial[c] = shape
            ms = time_pass(trial)
            if ms < best * (1.0 - margin):
                best, choice = ms, trial
    return choice, best, base


class TileTuner:
    """Per-class tile shapes for the batched forward and adjoint.

    cache_path: JSON file of earlier choices (None: DIFFDVR_TUNE_CACHE, else
    ~/.cache/diffdvr_gb300/tiles.json).  device: the key under which choices
    are cached (the GPU's name).  timer(run) -> ms times one call of run();
    the default uses CUDA events with `warmup` calls first and the median of
    `repeats`."""

    def __init__(self, cache_path: Optional[str] = None, device: Optional[str] = None,
                 timer: Optional[Callable[[Callable[[], None]], float]] = None, warmup: int = 2, repeats: int = 5):
        self.cache_path = cache_path or os.environ.get("DIFFDVR_TUNE_CACHE") or os.path.join(
            os.path.expanduser("~"), ".cache", "diffdvr_gb300", "tiles.json")
        self.device = device
        self.timer = timer
        self.warmup, self.repeats = warmup, repeats
        self.cache: Dict[str, Dict[str, dict]] = {}
        self.timed = False        # whether the last tune() timed (or read the cache)
        self.report: dict = {}    # the last search's timings
        if os.path.exists(self.cache_path):
            try:
                with open(self.cache_path) as f:
                    self.cache = json.load(f)
            except (OSError, ValueError):
                self.cache = {}

    def _device(self) -> str:
        if self.device is None:
            import torch
            self.device = torch.cuda.get_device_name()
        return self.device

    def _time(self, run: Callable[[], None]) -> float:
        if self.timer is not None:
            return float(self.timer(run))
        import torch
        for _ in range(self.warmup):
            run()
        times = []
        for _ in range(self.repeats):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            run()
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b))
        times.sort()
        return times[len(times) // 2]

    def _save(self) -> None:
        d = os.path.dirname(self.cache_path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def choose(self, classes: Sequence[str], time_forward: Callable[[Dict[str, int]], float],
               time_adjoint: Callable[[Dict[str, int]], float]) -> Tuple[Dict[str, int], Dict[str, int]]:
        """The (forward, adjoint) shape of every class: from the cache when
        every class is there, else by searching the launch with the given
        timers ({class: shape} -> ms)."""
        dev = self._device()
        known = self.cache.get(dev, {})
        if all(c in known for c in classes):
            self.timed = False
            return ({c: int(known[c]["forward"]) for c in classes}, {c: int(known[c]["adjoint"]) for c in classes})
        fwd, fwd_ms, fwd_base = search(classes, time_forward)
        adj, adj_ms, adj_base = search(classes, time_adjoint)
        self.timed = True
        self.report = {"forward_ms": fwd_ms, "forward_16x8_ms": fwd_base, "adjoint_ms": adj_ms,
                       "adjoint_16x8_ms": adj_base}
        for c in classes:
            self.cache.setdefault(dev, {})[c] = {"forward": fwd[c], "adjoint": adj[c]}
        self._save()
        return fwd, adj

    def tune(self, inputs, outputs, adj_colors, adj_outputs, storage: str = "f32") -> Tuple[List[int], List[int]]:
        """Tile shapes (forward, adjoint) for every instance of a batched call:
        the arguments of render_forward_batched / render_adjoint_batched
        (pyrenderer objects with CUDA tensors)."""
        import torch
        from . import pyrenderer as pr
        keys = []
        for inp, adj in zip(inputs, adj_outputs):
            grads = [g for g, on in (("tf", adj.has_tf_derivatives), ("volume", adj.has_volume_derivatives)) if on]
            vs = tuple(inp.volume.shape)
            box = inp.box_size
            size = max(float(v) for v in ((box.x, box.y, box.z) if hasattr(box, "x") else box.flatten().tolist()))
            voxel = size / max(1, max(vs[-3:]) - 1)
            st = inp.step_size
            step = float(st.min()) if isinstance(st, torch.Tensor) else float(st)
            keys.append(size_class(vs, inp.screen_size.x, inp.screen_size.y, step / voxel,
                                   (int(inp.volume_filter_mode), int(inp.tf_mode), int(inp.blend_mode)), storage,
                                   grads))
        classes = sorted(set(keys))
        # scratch outputs of the same kind as the caller's: with a sample
        # record of their own where the caller's carry one, so the adjoint is
        # timed on the path (record or re-march) that the caller's call takes
        like = lambda o, name: None if getattr(o, name, None) is None else torch.empty_like(getattr(o, name))
        scratch_out = [pr.RendererOutputs(torch.empty_like(o.color), torch.empty_like(o.terminationIndex),
                                          like(o, "checkpoints"), o.checkpoint_interval,
                                          like(o, "sample_density"), like(o, "sample_offset")) for o in outputs]
        scratch_adj = []
        for a in adj_outputs:
            sa = pr.AdjointOutputs()
            for flag, name in (("has_tf_derivatives", "adj_tf"), ("has_volume_derivatives", "adj_volume")):
                if getattr(a, flag):
                    setattr(sa, flag, True)
                    setattr(sa, name, torch.zeros_like(getattr(a, name)))
            sa.tf_delayed_accumulation = a.tf_delayed_accumulation
            scratch_adj.append(sa)
        pr.Renderer.render_forward_batched(inputs, scratch_out)
        per_instance = lambda choice: [choice[k] for k in keys]
        fwd, adj = self.choose(
            classes,
            lambda choice: self._time(lambda: pr.Renderer.render_forward_batched(inputs, scratch_out,
                                                                                 per_instance(choice))),
            lambda choice: self._time(lambda: pr.Renderer.render_adjoint_batched(
                inputs, scratch_out, adj_colors, scratch_adj, per_instance(choice))))
        return per_instance(fwd), per_instance(adj)
