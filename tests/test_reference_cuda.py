"""GPU parity against the reference's own CUDA kernels on the same GPU.

The reference's forward and adjoint kernels are compiled from its headers into
``oracle/_ref/ref_kernels_sm103a.cubin`` (``oracle/ref_device.cu``), with the
options of its runtime compiler, and launched through the CUDA driver API as
its backend launches them (``oracle/ref_cuda.py``).  The cubin is built where
the reference sources are; these tests skip where it is absent, and they run
only when DVR_REFERENCE_CUDA_TESTS=1 is set: their tolerances for the
reference's fast-math build are not yet confirmed over all modes.

The reference's runtime compiler uses --use_fast_math (approximate exp and
division, flush to zero; renderer/kernel_loader.cpp:218-230), so its CUDA
path is itself off the exact FP32 result: against the FP64 oracle it
measured up to 4.6e-5 in the reference's symmetric metric on single pixels
(texture TF, inverse-view-matrix camera).  Hence:
* forward: the scenes of test_gpu_parity.test_forward_all_modes (which hold
  our kernels to max(1e-5, 3 e32) of the FP64 oracle).  The reference's CUDA
  forward is first checked against the FP64 oracle for gross errors (<= 1e-3,
  sample counts agreeing on >= 95% of pixels).  On the pixels where the
  sample counts of ours, the reference's CUDA forward and the FP64 oracle
  agree, ours is within 1e-5 of the reference's CUDA forward on >= 99% of
  pixels (>= 97% with nearest filtering, whose voxel choice is
  rounding-sensitive) and within 1e-4 everywhere.
* gradients: the scenes of test_gpu_parity.test_adjoint_all_modes, one
  output adjoint for all three (zero on rays whose sample counts differ);
  relative L2 between ours and the reference's CUDA adjoint
  <= max(1e-3, 3 r_ref, 3 r_ours), r_* each one's relative L2 error against
  the FP64 oracle.
"""
import os

import numpy as np
import pytest

from dvr_cases import all_mode_combos, gpu_adjoint, gpu_forward, make_case, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_cuda(oracle_built, cuda_device):
    from oracle import ref_cuda as R
    if os.environ.get("DVR_REFERENCE_CUDA_TESTS") != "1":
        pytest.skip("comparison with the reference's CUDA kernels runs with DVR_REFERENCE_CUDA_TESTS=1")
    if not R.available():
        pytest.skip("the reference's CUDA kernels were not built (no reference sources where the repo was built)")
    return R


def _pixel_errors(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(1.0, np.abs(a) + np.abs(b)), axis=-1)


def test_reference_cuda_forward_all_modes(ref_cuda, oracle_built):
    O = oracle_built
    failures = {}
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(200 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam)
        sc = case.oracle_scene()
        rc, rt = ref_cuda.forward(sc)
        c64, t64 = O.forward(sc, "port", "f64")
        bad = []
        ref_ok = rt == t64
        if np.mean(~ref_ok) > 0.05 or not np.all(np.abs(rt - t64) <= 1):
            bad.append(f"reference CUDA: sample counts differ from FP64 on {np.mean(~ref_ok):.3f}")
        e_ref = _pixel_errors(rc[ref_ok], c64[ref_ok])
        if e_ref.size and e_ref.max() > 1e-3:
            bad.append(f"reference CUDA: colour error {e_ref.max():.2e} against FP64")
        share = 0.97 if filt == 0 else 0.99
        stats = [f"mode {(tfm, filt, blend, cam)}: reference CUDA vs FP64 max {e_ref.max() if e_ref.size else 0:.2e}"]
        for family in ("plain", "optimized"):
            _, out = gpu_forward(case, family)
            color, term = out.color.cpu().numpy(), out.terminationIndex.cpu().numpy()
            same = (term == rt) & ref_ok
            if np.mean(term != rt) > 0.05:
                bad.append(f"{family}: sample counts differ on {np.mean(term != rt):.3f}")
            pe = _pixel_errors(color[same], rc[same])
            if pe.size:
                stats.append(f"{family} vs reference CUDA max {pe.max():.2e}, within 1e-5 {np.mean(pe <= 1e-5):.3f}")
            if pe.size and (np.mean(pe <= 1e-5) < share or pe.max() > 1e-4):
                bad.append(f"{family}: {np.mean(pe <= 1e-5):.3f} of pixels within 1e-5, max {pe.max():.2e}")
        print("; ".join(stats))  # shown in full with the failure report
        if bad:
            failures[(tfm, filt, blend, cam)] = bad
    assert not failures, failures


def _three_adjoints(ref_cuda, O, case, inp, out, family, req, adj, gpu_kw, delayed=False):
    """Ours, the reference's CUDA adjoint and the FP64 oracle's, all with one
    output adjoint that is zero where the sample counts differ."""
    sc = case.oracle_scene()
    term = out.terminationIndex.cpu().numpy()
    rc, rt = ref_cuda.forward(sc)
    c64, t64 = O.forward(sc, "port", "f64")
    adj = np.where(((term == rt) & (rt == t64))[..., None], adj, 0.0).astype(np.float32)
    ref = ref_cuda.adjoint(sc, rc, rt, adj, req, delayed=delayed)
    ref64 = O.adjoint(sc, c64, t64, adj, req, "port", "f64")
    got = gpu_adjoint(case, inp, out, adj, family=family, **gpu_kw)
    return got, ref, ref64


@pytest.mark.parametrize("family", ["plain", "optimized"])
def test_reference_cuda_adjoint_all_modes(family, ref_cuda, oracle_built):
    """Volume, TF, step-size and (per-pixel rays) camera gradients.  The
    optimized family returns the full step-size derivative and the reference
    only the last blend term, so the step-size gradient is compared for the
    plain family only."""
    O = oracle_built
    failures = {}
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(300 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam, opacity=0.25,
                         pad_faces=True)
        inp, out = gpu_forward(case, family, checkpoints=(family == "optimized"))
        adj = np.random.default_rng(7).normal(size=out.color.shape).astype(np.float32)
        req = O.AdjointRequest(volume=True, tf=True, camera=cam == 0, stepsize=True)
        got, ref, ref64 = _three_adjoints(ref_cuda, O, case, inp, out, family, req, adj,
                                          dict(volume=True, tf=True, camera=cam == 0, stepsize=True))
        bad = {}
        stats = []
        for k in got:
            if k == "adj_stepsize" and family == "optimized":
                continue
            r = rel_l2(got[k], ref[k])
            tol = max(1e-3, 3 * rel_l2(ref[k], ref64[k]), 3 * rel_l2(got[k], ref64[k]))
            stats.append(f"{k} {r:.2e} (reference CUDA vs FP64 {rel_l2(ref[k], ref64[k]):.2e})")
            if r > tol:
                bad[k] = (r, tol)
        print(f"mode {(tfm, filt, blend, cam)} {family}: " + ", ".join(stats))
        if bad:
            failures[(tfm, filt, blend, cam)] = bad
    assert not failures, failures


def test_reference_cuda_delayed_tf_accumulation(ref_cuda, oracle_built):
    """The reference's default TF adjoint (per-thread shared-memory
    accumulation, one reduction per warp) equals its immediate-atomics
    variant up to summation order, and the optimized family's TF-only adjoint
    from the sample record agrees with it: texture TF (64 entries),
    trilinear, Beer-Lambert, per-pixel rays."""
    O = oracle_built
    case = make_case(77, tf_mode=1, filter_mode=1, blend_mode=0, camera_mode=0, R=64, opacity=0.25, pad_faces=True)
    inp, out = gpu_forward(case, "optimized", checkpoints=True, record="full")
    adj = np.random.default_rng(5).normal(size=out.color.shape).astype(np.float32)
    req = O.AdjointRequest(tf=True)
    got, ref_del, ref64 = _three_adjoints(ref_cuda, O, case, inp, out, "optimized", req, adj, dict(tf=True),
                                          delayed=True)
    _, ref_imm, _ = _three_adjoints(ref_cuda, O, case, inp, out, "optimized", req, adj, dict(tf=True))
    assert rel_l2(ref_del["adj_tf"], ref_imm["adj_tf"]) <= 1e-4
    tol = max(1e-3, 3 * rel_l2(ref_del["adj_tf"], ref64["adj_tf"]), 3 * rel_l2(got["adj_tf"], ref64["adj_tf"]))
    assert rel_l2(got["adj_tf"], ref_del["adj_tf"]) <= tol
