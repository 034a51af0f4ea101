"""The window adjoint (diffdvr_gb300/csrc/dvr_window.cuh): volume gradients
from the sample record, accumulated per slab in shared memory and added to
global memory once per touched group of four voxels, with the volume staged
in shared memory by bulk copies when camera gradients need the corner
densities.

Every case checks that the call took the window kernel
(dvr_last_adjoint_path), then holds it
* against the FP64 oracle on the same (rounded) inputs, with the tolerances
  of test_gpu_parity.py (relative L2 max(1e-3, 3 r32), <= 1% of entries off
  by more than 1e-3 of the largest), and
* against the general per-ray kernel on the same forward outputs
  (dvr_set_window_adjoint(0)): the same sums in another order, relative L2
  <= 1e-4 for every gradient, step size included.
Cases: all TF modes and both blend modes, per-pixel rays (camera gradients,
staged volume) and the reference-frame camera, FP32 and BF16 storage, a
partial record whose other rays take the general kernel, and a close camera
with a large volume, whose slabs must shrink to fit the shared-memory window.
"""
import numpy as np
import pytest
import torch

from dvr_cases import gpu_adjoint, gpu_forward, make_case, rel_l2

pytestmark = pytest.mark.gpu

PATH_WINDOW = 4


def _grad_errors(got, ref, r32):
    bad = {}
    for k in got:
        if k not in ref:
            continue
        r = rel_l2(got[k], ref[k])
        tol = max(1e-3, 3 * r32[k])
        scale = max(float(np.max(np.abs(ref[k]))), 1e-30)
        frac = float(np.mean(np.abs(np.asarray(got[k], np.float64) - ref[k]) / scale > 1e-3))
        if r > tol or frac > 0.01:
            bad[k] = (r, tol, frac)
    return bad


def _run(case, O, volume_dtype=None, record="full"):
    from diffdvr_gb300 import _abi
    lib = _abi.load()
    cam = case.camera_mode == 0
    inp, out = gpu_forward(case, "optimized", volume_dtype=volume_dtype, checkpoints=True, record=record)
    term = out.terminationIndex.cpu().numpy()
    adj = np.random.default_rng(7).normal(size=out.color.shape).astype(np.float32)
    kw = dict(volume=True, tf=True, camera=cam, stepsize=True)
    prev = lib.dvr_set_window_adjoint(1)
    try:
        got = gpu_adjoint(case, inp, out, adj, **kw)
        path = lib.dvr_last_adjoint_path()
        lib.dvr_set_window_adjoint(0)
        general = gpu_adjoint(case, inp, out, adj, **kw)
        lib.dvr_set_window_adjoint(1)
        # the oracle on the stored (rounded) volume; rays whose sample counts differ get no output adjoint
        sc = case.oracle_scene()
        if volume_dtype is not None:
            sc.volume = torch.from_numpy(case.volume).to(volume_dtype).float().numpy()
        c64, t64 = O.forward(sc, "port", "f64")
        c32, t32 = O.forward(sc, "port", "f32")
        adj_m = np.where((term == t64)[..., None], adj, 0.0).astype(np.float32)
        req = O.AdjointRequest(volume=True, tf=True, camera=cam)
        got_m = gpu_adjoint(case, inp, out, adj_m, volume=True, tf=True, camera=cam)
    finally:
        lib.dvr_set_window_adjoint(prev)
    ref = O.adjoint(sc, c64, t64, adj_m, req, "port", "f64")
    g32 = O.adjoint(sc, c32, t32, np.where((t32 == term)[..., None], adj_m, 0.0), req, "port", "f32")
    r32 = {k: rel_l2(g32[k], ref[k]) for k in g32}
    return path, got, general, got_m, ref, r32


@pytest.mark.parametrize("camera_mode", [0, 2], ids=["per-pixel-rays", "reference-frame"])
def test_window_adjoint_all_tf_and_blend_modes(camera_mode, oracle_built, cuda_device):
    O = oracle_built
    failures = {}
    for i, (tfm, blend) in enumerate([(t, b) for t in (0, 1, 2, 3) for b in (0, 1)]):
        case = make_case(700 + i, tf_mode=tfm, blend_mode=blend, camera_mode=camera_mode, shape=(20, 24, 32), W=40,
                         H=28, B=2, opacity=0.3, pad_faces=True)
        path, got, general, got_m, ref, r32 = _run(case, O)
        bad = {}
        if path != PATH_WINDOW:
            bad["path"] = path
        for k in got:
            r = rel_l2(got[k], general[k])
            if r > 1e-4:
                bad["vs general " + k] = r
        bad.update(_grad_errors(got_m, ref, r32))
        if bad:
            failures[(tfm, blend)] = bad
    assert not failures, failures


@pytest.mark.parametrize("record", ["full", 0.3], ids=["full-record", "partial-record"])
def test_window_adjoint_bf16_storage_and_partial_record(record, oracle_built, cuda_device):
    """BF16 volume (staged rows of 8 voxels), linear TF, per-pixel rays; with a
    pool for about 30% of the samples the rays without a record go through
    the general kernel in the same call."""
    O = oracle_built
    case = make_case(731, tf_mode=2, camera_mode=0, shape=(24, 20, 40), W=48, H=36, B=2, opacity=0.3,
                     pad_faces=True)
    path, got, general, got_m, ref, r32 = _run(case, O, volume_dtype=torch.bfloat16, record=record)
    assert path == PATH_WINDOW
    for k in got:
        assert rel_l2(got[k], general[k]) <= 1e-4, k
    bad = _grad_errors(got_m, ref, r32)
    assert not bad, bad


def test_window_adjoint_close_camera_shrinks_slabs(oracle_built, cuda_device):
    """A 96^3 volume seen from distance 1.2 with a wide field of view: a 16x8
    tile of rays spreads over many voxels, so the slabs shrink (down to one
    step) to fit the window; results stay those of the general kernel and the
    oracle."""
    from diffdvr_gb300 import scenes
    O = oracle_built
    case = make_case(741, tf_mode=1, camera_mode=0, shape=(96, 96, 96), W=64, H=48, B=1, opacity=0.05,
                     pad_faces=True)
    vp = scenes.viewport_from_sphere([0.4], [0.7], 1.2)
    case.ray_start, case.ray_dir = scenes.generate_rays(vp, np.radians(80.0), 64, 48)
    path, got, general, got_m, ref, r32 = _run(case, O)
    assert path == PATH_WINDOW
    for k in got:
        assert rel_l2(got[k], general[k]) <= 1e-4, k
    bad = _grad_errors(got_m, ref, r32)
    assert not bad, bad
