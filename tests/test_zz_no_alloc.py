"""dvr_render_adjoint_noalloc — the adjoint for callers that cannot let the
library allocate device memory — against dvr_render_adjoint.

Both are called through the C ABI on the same forward outputs, twice in a row
(the second call reuses the static scratch, so a counter or TF-gradient slice
left dirty by the first would show up there), with and without a sample
record from the forward.  A separate fresh process makes the no-allocation
call the first adjoint call of its life, on a stream no other call used, and
checks that the device's free memory does not change across it: the
dvr_render_adjoint pools are then still empty, so an allocation slipped into
the no-allocation path could not hide in them.

Tolerance: the two entry points run the same kernels; gradients differ only
by the order of floating-point atomic additions, so relative L2 <= 1e-5 and
elementwise |a - b| <= 1e-5 * max|b| + 1e-7.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from dvr_cases import gpu_forward, make_case, rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _adjoint_outputs(case):
    """Zeroed gradient outputs of every kind for case."""
    from diffdvr_gb300 import pyrenderer as pr
    B, H, W = case.batch(), case.height, case.width
    a = pr.AdjointOutputs()
    a.has_volume_derivatives = True
    a.adj_volume = torch.zeros((case.volume.shape[0],) + case.volume.shape[1:], device="cuda")
    a.has_tf_derivatives = True
    a.tf_delayed_accumulation = True
    a.adj_tf = torch.zeros(case.tf.shape, device="cuda")
    a.has_camera_derivatives = True
    a.adj_camera_ray_start = torch.zeros((B, H, W, 3), device="cuda")
    a.adj_camera_ray_dir = torch.zeros((B, H, W, 3), device="cuda")
    a.has_stepsize_derivatives = True
    a.adj_stepsize = torch.zeros((B, H, W), device="cuda")
    torch.cuda.synchronize()
    return a


def _adjoint_through_abi(entry, case, inp, out, adj_color, stream=None, a=None):
    """Calls entry (one of the two adjoint entry points) through ctypes; a:
    the gradient outputs (zeroed), made here when not given."""
    from diffdvr_gb300 import _abi
    from diffdvr_gb300 import pyrenderer as pr
    a = a or _adjoint_outputs(case)
    ci, co = pr._inputs(inp), pr._outputs(out)
    ca, cg = pr._tensor(adj_color, "adj_color"), pr._adjoint_outputs(a)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    _abi.check(entry(ctypes.byref(ci), ctypes.byref(co), ctypes.byref(ca), ctypes.byref(cg), s))
    torch.cuda.synchronize()
    return {"volume": a.adj_volume, "tf": a.adj_tf, "ray_start": a.adj_camera_ray_start,
            "ray_dir": a.adj_camera_ray_dir, "stepsize": a.adj_stepsize}


def _max_error(got, ref):
    """(relative L2, max |a-b| / max|b|) of two gradients; (0, 0) when both are zero."""
    g, r = got.double().cpu().numpy(), ref.double().cpu().numpy()
    if not np.isfinite(g).all():
        return float("inf"), float("inf")
    scale = float(np.abs(r).max())
    if scale == 0:   # e.g. camera gradients under nearest filtering
        return (0.0, 0.0) if not g.any() else (float("inf"), float("inf"))
    return rel_l2(g, r), float(np.abs(g - r).max()) / scale


def _assert_close(got, ref, what):
    rl2, rmax = _max_error(got, ref)
    assert rl2 <= 1e-5, (what, rl2)
    assert rmax <= 1e-5 + 1e-7, (what, rmax)


def _case(tf_mode, filter_mode, blend_mode):
    return make_case(61 + tf_mode, tf_mode=tf_mode, filter_mode=filter_mode, blend_mode=blend_mode,
                     shape=(24, 28, 32), W=48, H=40, B=2, R=24 if tf_mode == 1 else None, opacity=0.4,
                     pad_faces=True)


@pytest.mark.parametrize("tf_mode,filter_mode,blend_mode,checkpoints,record", [
    (1, 1, 0, True, None),     # texture TF, trilinear, Beer-Lambert, checkpointed adjoint
    (1, 1, 0, True, "full"),   # the same forward with a sample record: the general kernel reads it
    (3, 0, 1, False, None),    # Gaussian TF (6 channels), nearest, alpha blending, blend inversion
])
def test_noalloc_adjoint_matches_dvr_render_adjoint(tf_mode, filter_mode, blend_mode, checkpoints, record,
                                                     cuda_device):
    from diffdvr_gb300 import _abi
    lib = _abi.load()
    case = _case(tf_mode, filter_mode, blend_mode)
    inp, out = gpu_forward(case, checkpoints=checkpoints, record=record)
    if record is not None:
        assert (out.sample_offset.cpu().numpy()[out.terminationIndex.cpu().numpy() > 0] >= 0).all()
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
    # the static scratch holds (4 MiB - 256 B) / (4 B x C x SMs) texels of TF gradient per block;
    # one texel more than that is rejected, whatever the SM count
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    R = ((4 << 20) - 256) // (4 * 4 * sms) + 1
    case = make_case(5, tf_mode=1, shape=(8, 8, 8), W=8, H=8, B=1, R=R)
    inp, out = gpu_forward(case)
    adj = torch.ones((1, 8, 8, 4), device="cuda")
    with pytest.raises(_abi.DvrError, match="TF too large for the no-allocation adjoint") as e:
        _adjoint_through_abi(lib.dvr_render_adjoint_noalloc, case, inp, out, adj)
    assert e.value.code == _abi.DVR_E_INVALID_ARGUMENT


_FIRST_CALL = r"""
import json, sys
import numpy as np, torch
sys.path[:0] = [sys.argv[1], sys.argv[2]]
import test_zz_no_alloc as T
from dvr_cases import gpu_forward
from diffdvr_gb300 import _abi
lib = _abi.load()
case = T._case(1, 1, 0)
inp, out = gpu_forward(case, checkpoints=True)
adj = torch.from_numpy(np.random.default_rng(7).standard_normal(
    (case.batch(), case.height, case.width, 4)).astype(np.float32)).cuda()
fresh = torch.cuda.Stream()
# every tensor the calls write is made before the first measurement
a1, a2 = T._adjoint_outputs(case), T._adjoint_outputs(case)
torch.cuda.synchronize()
free_before = torch.cuda.mem_get_info()[0]
got = T._adjoint_through_abi(lib.dvr_render_adjoint_noalloc, case, inp, out, adj, stream=fresh, a=a1)
free_first = torch.cuda.mem_get_info()[0]
got2 = T._adjoint_through_abi(lib.dvr_render_adjoint_noalloc, case, inp, out, adj, stream=fresh, a=a2)
free_second = torch.cuda.mem_get_info()[0]
ref = T._adjoint_through_abi(lib.dvr_render_adjoint, case, inp, out, adj)
err = {k: list(T._max_error(got[k], ref[k])) + list(T._max_error(got2[k], ref[k])) for k in ref}
print(json.dumps({"free_before": free_before, "free_first": free_first, "free_second": free_second,
                  "torch_reserved": torch.cuda.memory_reserved(), "errors": err}))
"""


def test_noalloc_adjoint_first_call_allocates_nothing(cuda_device):
    """In a fresh process, the no-allocation adjoint is the first adjoint call
    (dvr_render_adjoint's pools are still empty) on a stream nothing else
    used; the device's free memory is the same after its first and second
    calls as before them.  Every tensor the calls write exists before the
    first measurement, and modules load eagerly, so that loading the
    kernels' code on first use does not count as an allocation."""
    root = os.path.dirname(HERE)
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    r = subprocess.run([sys.executable, "-c", _FIRST_CALL, HERE, root], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for k, (rl2, rmax, rl2b, rmaxb) in res["errors"].items():
        assert rl2 <= 1e-5 and rmax <= 1e-5 + 1e-7, (k, rl2, rmax)
        assert rl2b <= 1e-5 and rmaxb <= 1e-5 + 1e-7, (k, rl2b, rmaxb)
    assert res["free_first"] == res["free_before"], res
    assert res["free_second"] == res["free_before"], res
