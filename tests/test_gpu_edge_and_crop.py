"""GPU parity on degenerate inputs and the large mixed-precision
configuration's accuracy report.

* Degenerate inputs (the cases of dvr_cases.edge_cases, on which the oracle
  is pinned to the reference's own CPU code): 1x1 and empty images,
  one-voxel axes, rays that all miss the box, one sample per ray, early out
  at zero opacity.  Both kernel families against the FP64 oracle, forward
  and every gradient, with the tolerances of test_gpu_parity.py: colour
  within max(1e-5, 3 e32), gradients within relative L2 max(1e-3, 3 r32),
  sample counts agreeing on >= 98% of pixels.  Volumes with at least three
  voxels per axis get equal outer two layers on every face (as the camera
  tests of test_gpu_parity.py do): with one sample per ray every sample lies
  on the box face where the ray enters, where the reference's trilinear
  position derivative is one-sided and picks its cell by rounding, so ray
  gradients would otherwise compare two different one-sided derivatives.
* The large mixed-precision configuration's accuracy report: the 512^3
  scene stored in BF16 and, separately, in FP16, its volume, TF and ray
  gradients against the FP64 oracle on a 64^3 crop (same TF and rays of one
  view, the box shrunk to the sub-volume; the oracle gets the rounded
  voxels, so the comparison measures the arithmetic, not the storage).
"""
import functools

import numpy as np
import pytest
import torch

from dvr_cases import Case, edge_cases, gpu_adjoint, gpu_forward, pad_faces, rel_l2, symmetric_error

pytestmark = pytest.mark.gpu


def _compare(case, family, O, grads):
    """Forward and adjoint of one case against the FP64 oracle; returns a
    list of failed checks."""
    sc = case.oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    c32, t32 = O.forward(sc, "port", "f32")
    inp, out = gpu_forward(case, family, checkpoints=(family == "optimized"))
    color, term = out.color.cpu().numpy(), out.terminationIndex.cpu().numpy()
    bad = []
    if color.shape != c64.shape:
        return [f"colour shape {color.shape} != {c64.shape}"]
    if term.size == 0:
        return bad
    same = term == t64
    if np.mean(~same) > 0.02 or not np.all(np.abs(term - t64) <= 1):
        bad.append(f"sample counts differ on {np.mean(~same):.3f} of pixels")
    agree = t32 == t64
    tol = max(1e-5, 3 * symmetric_error(c32[agree], c64[agree]))
    if same.any() and symmetric_error(color[same], c64[same]) > tol:
        bad.append(f"colour error {symmetric_error(color[same], c64[same]):.2e} > {tol:.1e}")
    adj = np.random.default_rng(11).normal(size=color.shape).astype(np.float32)
    adj = np.where((same & agree)[..., None], adj, 0.0).astype(np.float32)
    req = O.AdjointRequest(**grads)
    ref = O.adjoint(sc, c64, t64, adj, req, "port", "f64")
    r32 = O.adjoint(sc, c32, t32, adj, req, "port", "f32")
    got = gpu_adjoint(case, inp, out, adj, family=family, **grads)
    for k in got:
        if not np.any(ref[k]):
            if np.any(got[k]):
                bad.append(f"{k}: nonzero where the oracle's gradient is zero")
            continue
        r = rel_l2(got[k], ref[k])
        lim = max(1e-3, 3 * rel_l2(r32[k], ref[k]))
        if r > lim:
            bad.append(f"{k}: relative L2 {r:.2e} > {lim:.1e}")
    return bad


@pytest.mark.parametrize("family", ["plain", "optimized"])
@pytest.mark.parametrize("filter_mode", [0, 1])
def test_degenerate_inputs(family, filter_mode, oracle_built, cuda_device):
    O = oracle_built
    failures = {}
    for name, case in edge_cases():
        case.filter_mode = filter_mode
        if min(case.volume.shape[1:]) >= 3:
            case.volume = pad_faces(case.volume)
        # the optimized family returns the full step-size derivative, the oracle only the last blend term
        grads = dict(volume=True, tf=True, camera=True, stepsize=family == "plain")
        bad = _compare(case, family, O, grads)
        if bad:
            failures[name] = bad
    assert not failures, failures


@functools.lru_cache(maxsize=1)
def _large_mixed_crop():
    """The 64^3 crop at voxel 224 of the 512^3 scene, one view (built once:
    the full scene takes a while)."""
    from diffdvr_gb300 import scenes
    return scenes.crop(scenes.large_mixed_512(seed=4, views=1), (224, 224, 224), 64)


@pytest.mark.parametrize("storage", [torch.bfloat16, torch.float16], ids=["bf16", "f16"])
def test_large_mixed_crop_accuracy(storage, oracle_built, cuda_device):
    O = oracle_built
    c = _large_mixed_crop()
    vol_rounded = torch.from_numpy(c.volume).to(storage).to(torch.float32).numpy()
    case = Case(width=c.width, height=c.height, volume=vol_rounded, tf=c.tf, tf_mode=c.tf_mode,
                filter_mode=c.filter_mode, blend_mode=c.blend_mode, camera_mode=0, step=c.step_size,
                box_min=c.box_min, box_size=c.box_size)
    case.ray_start, case.ray_dir = c.ray_start, c.ray_dir
    sc = case.oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    assert (t64 > 0).sum() > 500  # the view's rays cross the crop
    inp, out = gpu_forward(case, "optimized", volume_dtype=storage, checkpoints=True)
    term = out.terminationIndex.cpu().numpy()
    same = term == t64
    assert np.mean(~same) <= 0.02
    assert symmetric_error(out.color.cpu().numpy()[same], c64[same]) <= 1e-5
    adj = np.where(same[..., None], np.random.default_rng(12).normal(size=c64.shape), 0.0).astype(np.float32)
    req = O.AdjointRequest(volume=True, tf=True, camera=True)
    ref = O.adjoint(sc, c64, t64, adj, req, "port", "f64")
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=True)
    errors = {k: rel_l2(got[k], ref[k]) for k in got}
    assert all(e <= 1e-3 for e in errors.values()), errors
