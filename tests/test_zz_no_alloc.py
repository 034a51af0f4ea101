"""dvr_render_adjoint_noalloc (static device scratch, no allocation) against
dvr_render_adjoint, both called through the C ABI on the same forward outputs,
on two calls in a row (the second call reuses the static scratch, so a counter
or TF-gradient slice left dirty by the first would show up there).

Tolerance: the two entry points run the same kernels; gradients differ only
by the order of floating-point atomic additions, so relative L2 <= 1e-5 and
elementwise |a - b| <= 1e-5 * max|b| + 1e-7.
"""
import ctypes

import numpy as np
import pytest
import torch

from dvr_cases import gpu_forward, make_case, rel_l2

pytestmark = pytest.mark.gpu


def _adjoint_through_abi(entry, case, inp, out, adj_color, tf_batch=None):
    from diffdvr_gb300 import _abi
    from diffdvr_gb300 import pyrenderer as pr
    B, H, W = case.batch(), case.height, case.width
    a = pr.AdjointOutputs()
    a.has_volume_derivatives = True
    a.adj_volume = torch.zeros((case.volume.shape[0],) + case.volume.shape[1:], device="cuda")
    a.has_tf_derivatives = True
    a.tf_delayed_accumulation = True
    a.adj_tf = torch.zeros(((tf_batch or case.tf.shape[0]),) + case.tf.shape[1:], device="cuda")
    a.has_camera_derivatives = True
    a.adj_camera_ray_start = torch.zeros((B, H, W, 3), device="cuda")
    a.adj_camera_ray_dir = torch.zeros((B, H, W, 3), device="cuda")
    a.has_stepsize_derivatives = True
    a.adj_stepsize = torch.zeros((B, H, W), device="cuda")
    ci, co = pr._inputs(inp), pr._outputs(out)
    ca, cg = pr._tensor(adj_color, "adj_color"), pr._adjoint_outputs(a)
    stream = torch.cuda.current_stream().cuda_stream
    _abi.check(entry(ctypes.byref(ci), ctypes.byref(co), ctypes.byref(ca), ctypes.byref(cg), stream))
    torch.cuda.synchronize()
    return {"volume": a.adj_volume, "tf": a.adj_tf, "ray_start": a.adj_camera_ray_start,
            "ray_dir": a.adj_camera_ray_dir, "stepsize": a.adj_stepsize}


def _assert_close(got, ref, what):
    g, r = got.double().cpu().numpy(), ref.double().cpu().numpy()
    assert np.isfinite(g).all(), what
    scale = float(np.abs(r).max())
    if scale == 0:   # e.g. camera gradients under nearest filtering
        assert not g.any(), what
        return
    assert rel_l2(g, r) <= 1e-5, (what, rel_l2(g, r))
    assert np.abs(g - r).max() <= 1e-5 * scale + 1e-7, (what, float(np.abs(g - r).max()), scale)


@pytest.mark.parametrize("tf_mode,filter_mode,blend_mode,checkpoints", [
    (1, 1, 0, True),    # texture TF, trilinear, Beer-Lambert, checkpointed adjoint
    (3, 0, 1, False),   # Gaussian TF (5 channels), nearest, alpha blending, blend inversion
])
def test_noalloc_adjoint_matches_dvr_render_adjoint(tf_mode, filter_mode, blend_mode, checkpoints, cuda_device):
    from diffdvr_gb300 import _abi
    lib = _abi.load()
    case = make_case(61 + tf_mode, tf_mode=tf_mode, filter_mode=filter_mode, blend_mode=blend_mode,
                     shape=(24, 28, 32), W=48, H=40, B=2, R=24 if tf_mode == 1 else None, opacity=0.4,
                     pad_faces=True)
    inp, out = gpu_forward(case, checkpoints=checkpoints)
    rng = np.random.default_rng(7)
    adj = torch.from_numpy(rng.standard_normal((case.batch(), case.height, case.width, 4)).astype(np.float32)).cuda()
    for call in range(2):
        ref = _adjoint_through_abi(lib.dvr_render_adjoint, case, inp, out, adj)
        got = _adjoint_through_abi(lib.dvr_render_adjoint_noalloc, case, inp, out, adj)
        for k in ref:
            _assert_close(got[k], ref[k], f"call {call}: adj_{k}")


def test_noalloc_adjoint_rejects_tf_beyond_static_scratch(cuda_device):
    from diffdvr_gb300 import _abi
    lib = _abi.load()
    case = make_case(5, tf_mode=1, shape=(8, 8, 8), W=8, H=8, B=1, R=2048)   # R*C = 8192 > 4 MiB / (4 B * SMs)
    inp, out = gpu_forward(case)
    adj = torch.ones((1, 8, 8, 4), device="cuda")
    with pytest.raises(_abi.DvrError, match="TF too large for the no-allocation adjoint") as e:
        _adjoint_through_abi(lib.dvr_render_adjoint_noalloc, case, inp, out, adj)
    assert e.value.code == _abi.DVR_E_INVALID_ARGUMENT
