"""Accuracy report of a GPU render against the FP64 oracle — TEST
INFRASTRUCTURE ONLY.

Given the forward outputs and the gradients that the GPU kernels produced
for a scene, ``render_errors`` runs the oracle restatement on the same inputs
(FP64 for the ground truth, FP32 for the error the reference's own FP32
arithmetic makes on the same pixels; the restatement is bit-identical to the
reference's CPU templates, renderer/renderer_kernels.cuh:108-127, :470-496)
and returns the errors the metric's gates are stated in:

* image: per pixel, the reference's symmetric metric |a-b| / max(1, |a|+|b|)
  (unittests/testConsistencyTF.cpp:16-41), max over the four channels.  A
  pixel fails when the GPU's error against FP64 exceeds max(1e-5, 3 e32),
  e32 being the reference FP32 arithmetic's error against FP64 on that same
  pixel.  Every pixel is counted, including those whose sample count differs
  from the FP64 oracle's.
* termination: the number of pixels whose sample count differs from the
  FP64 oracle's (and, for comparison, from the FP32 arithmetic's).  A ray
  takes the samples k >= 0 with tmin + k step <= tmax
  (renderer/renderer_kernels.cuh:50-56), n = floor((tmax - tmin) / step) + 1
  without early termination; where (tmax - tmin) / step lies within 2e-3 of
  an integer, the last sample's inclusion is decided by the rounding of the
  box exit distance, and two FP32 implementations (the reference's CPU build
  without and its CUDA build with fused multiply-adds) can take one sample
  more or less.  A failing pixel whose count differs from FP64's by one on
  such a ray is reported as explained by the exit rounding; every other
  failing pixel is unexplained.
* gradients: relative L2 error of each gradient against the FP64 adjoint on
  the same output adjoint (renderer/renderer_kernels.cuh:315-444), beside
  the FP32 arithmetic's own.  Per-pixel ray gradients are also reported
  over the rays without a rounding-decided sample, with the number of rays
  left out.  A sample that lies on a cell boundary takes the trilinear
  position derivative of one cell or the other, as rounding decides (the
  derivative jumps there): a ray entering the box through the face at the
  upper end of an axis has its first sample on that face, in the last cell
  (whose upper corners are clamped onto it, derivative zero along the
  axis) or in the one before; and a ray whose (tmax - tmin) / step lies
  within 2e-3 of an integer may end with a sample on the exit face.  On
  such rays FP32 and FP64 arithmetic, and any two FP32 orders of
  operations, may each take a whole sample's derivative differently.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s checker leg
use this module.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

_REQUEST = {"adj_tf": "tf", "adj_volume": "volume", "adj_ray_start": "camera", "adj_ray_dir": "camera"}


def pixel_errors(a, b) -> np.ndarray:
    """Per-pixel symmetric error, max over the channel axis."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(1.0, np.abs(a) + np.abs(b)), axis=-1)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def _well_conditioned(got, g32, g64, decided) -> dict:
    """Relative L2 errors of a per-pixel vector gradient (..., 3) over the
    rays without a rounding-decided sample (decided: bool per pixel, see the
    module docstring), and the number of rays left out."""
    got, g32, g64 = (np.asarray(x, np.float64).reshape(-1, 3) for x in (got, g32, g64))
    ok = ~np.asarray(decided, bool).ravel()
    return {"rel_l2_unambiguous_rays": rel_l2(got[ok], g64[ok]),
            "rel_l2_f32_unambiguous_rays": rel_l2(g32[ok], g64[ok]),
            "rays_left_out": int((~ok).sum()), "rays": int(ok.size)}


def _ray_geometry(scene: O.Scene):
    """Per pixel in FP64: ray start, direction, box min and size, and the
    entry and exit distances (tmin clamped to 0); None for the
    inverse-view-matrix camera.  Rays from the reference-frame camera follow
    renderer/renderer_camera.cuh:40-57, the slab test
    renderer/renderer_utils.cuh:60-74."""
    B, H, W = scene.batch(), scene.height, scene.width
    if scene.camera_mode == 0:
        start = np.broadcast_to(np.asarray(scene.ray_start, np.float64), (B, H, W, 3))
        d = np.broadcast_to(np.asarray(scene.ray_dir, np.float64), (B, H, W, 3))
    elif scene.camera_mode == 2:
        vp = np.broadcast_to(np.asarray(scene.camera_matrix, np.float64), (B, 3, 3))
        eye, right, up = vp[:, 0], vp[:, 1], vp[:, 2]
        front = np.cross(up, right)
        fov_y = float(scene.fov_y_radians)
        tx, ty = np.tan(fov_y * W / H / 2), np.tan(fov_y / 2)
        fx = 2 * (np.arange(W) + 0.5) / W - 1
        fy = 2 * (np.arange(H) + 0.5) / H - 1
        d = (front[:, None, None] + (fx * tx)[None, None, :, None] * right[:, None, None]
             + (fy * ty)[None, :, None, None] * up[:, None, None])
        d = d / np.linalg.norm(d, axis=-1, keepdims=True)
        start = np.broadcast_to(eye[:, None, None], (B, H, W, 3))
    else:
        return None
    bmin = np.broadcast_to(np.asarray(scene.box_min, np.float64).reshape(-1, 1, 1, 3), (B, 1, 1, 3))
    bsize = np.broadcast_to(np.asarray(scene.box_size, np.float64).reshape(-1, 1, 1, 3), (B, 1, 1, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        t1 = (bmin - start) * inv
        t2 = (bmin + bsize - start) * inv
    tmin = np.maximum(np.max(np.minimum(t1, t2), axis=-1), 0.0)
    tmax = np.min(np.maximum(t1, t2), axis=-1)
    return start, d, bmin, bsize, tmin, tmax


def rounding_decided_rays(scene: O.Scene):
    """Per pixel, whether the ray has a sample whose trilinear cell rounding
    decides: its first sample on the face at the upper end of an axis
    (within 1e-3 voxel), or its last sample on the exit face (exit
    ambiguity below 2e-3); None for the inverse-view-matrix camera."""
    g = _ray_geometry(scene)
    if g is None:
        return None
    start, d, bmin, bsize, tmin, tmax = g
    size = np.asarray(np.asarray(scene.volume).shape[1:4], np.float64)
    entry = (start + tmin[..., None] * d - bmin) / bsize * (size - 1)
    hit = tmax >= tmin
    upper = np.any(np.abs(entry - (size - 1)) < 1e-3, axis=-1) & (tmin > 0)
    amb = exit_ambiguity(scene)
    return hit & (upper | (amb < 2e-3))


def exit_ambiguity(scene: O.Scene):
    """Per pixel, the distance of (tmax - tmin) / step, in FP64, from the
    nearest integer (inf where the ray misses the box); None for the
    inverse-view-matrix camera."""
    g = _ray_geometry(scene)
    if g is None:
        return None
    _, _, _, _, tmin, tmax = g
    B, H, W = scene.batch(), scene.height, scene.width
    step = np.broadcast_to(np.asarray(scene.step_size, np.float64), (B, H, W))
    r = (tmax - tmin) / step
    return np.where(tmax >= tmin, np.abs(r - np.round(r)), np.inf)


def render_errors(scene: O.Scene, color: np.ndarray, term: np.ndarray, adj_color: np.ndarray = None,
                  grads: dict = None, floor: float = 1e-5) -> dict:
    """Errors of a GPU forward (color, term) and, when given, of its
    gradients `grads` (any of adj_tf, adj_volume, adj_ray_start,
    adj_ray_dir) for the output adjoint adj_color, against the FP64 oracle
    on `scene` (see the module docstring).  grad_rel_err is the largest of
    the gradients' relative L2 errors."""
    c64, t64 = O.forward(scene, "port", "f64")
    c32, t32 = O.forward(scene, "port", "f32")
    e_gpu = pixel_errors(color, c64)
    e_32 = pixel_errors(c32, c64)
    tol = np.maximum(floor, 3.0 * e_32)
    fail = e_gpu > tol
    same = term == t64
    res = {
        "pixels": int(term.size),
        "samples": int(np.asarray(term, np.int64).sum()),
        "image_err_max": float(e_gpu.max()) if e_gpu.size else 0.0,
        "image_err_max_same_count": float(e_gpu[same].max()) if same.any() else 0.0,
        "image_err_f32_max": float(e_32.max()) if e_32.size else 0.0,
        "image_fail": int(fail.sum()),
        "image_fail_max_excess": float((e_gpu - tol)[fail].max()) if fail.any() else 0.0,
        "image_fail_unexplained": int(fail.sum()),
        "image_fail_exit_rounding": 0,
        "term_mismatch": int((~same).sum()),
        "term_mismatch_f32": int((t32 != t64).sum()),
        "term_mismatch_vs_f32": int((term != t32).sum()),
        "term_max_diff": int(np.abs(np.asarray(term, np.int64) - t64).max()) if term.size else 0,
    }
    amb = exit_ambiguity(scene)
    if amb is not None and fail.any():
        one_off = np.abs(np.asarray(term, np.int64) - t64) == 1
        explained = fail & ~same & one_off & (amb < 2e-3)
        res["image_fail_exit_rounding"] = int(explained.sum())
        res["image_fail_unexplained"] = int((fail & ~explained).sum())
    if grads:
        req = O.AdjointRequest(**{_REQUEST[k]: True for k in grads})
        g64 = O.adjoint(scene, c64, t64, adj_color, req, "port", "f64")
        g32 = O.adjoint(scene, c32, t32, adj_color, req, "port", "f32")
        res["grad"] = {k: {"rel_l2": rel_l2(v, g64[k]), "rel_l2_f32": rel_l2(g32[k], g64[k])}
                       for k, v in grads.items()}
        decided = rounding_decided_rays(scene) if scene.camera_mode == 0 else None
        for k in ("adj_ray_start", "adj_ray_dir"):
            if k in grads and decided is not None:
                res["grad"][k].update(_well_conditioned(grads[k], g32[k], g64[k], decided))
        res["grad_rel_err"] = max(e["rel_l2"] for e in res["grad"].values())
        res["grad_rel_err_f32"] = max(e["rel_l2_f32"] for e in res["grad"].values())
    return res
