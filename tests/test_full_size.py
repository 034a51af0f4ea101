"""Size-independent properties at the full size of the TF-reconstruction
workload (256^3 BF16 volume, 8 views at 256^2, step 0.25 voxel, 90 M samples
per pass), where the oracle is too slow to run:

* linearity: the adjoint is linear in adj_color, so the gradient of
  adj1 + adj2 equals the sum of the two gradients;
* the TF gradient from the sample record (record adjoint kernel) equals the
  one re-marched from checkpoints (general kernel), and both are independent
  of the checkpoint interval;
* the batched entry point gives the single-instance result;
* every termination index lies within the ray's sample bound.

Tolerances: the kernels differ in summation order only (float atomics,
warp scans), so relative L2 <= 1e-4 for gradients and 1e-5 in the
reference's symmetric metric for images.
"""
import numpy as np
import pytest
import torch

from dvr_cases import rel_l2, symmetric_error

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload(cuda_device):
    from diffdvr_gb300 import pyrenderer as pr, scenes
    w = scenes.tf_reconstruction_256(seed=1)
    dev = torch.device("cuda")
    vol = torch.from_numpy(w.volume).to(dev).to(torch.bfloat16)
    tf = torch.from_numpy(w.tf).to(dev)
    vp = torch.from_numpy(w.viewport.astype(np.float32)).to(dev)
    inp = pr.RendererInputs()
    inp.screen_size = pr.int2(w.width, w.height)
    inp.volume = vol
    inp.box_min = pr.real3(*w.box_min)
    inp.box_size = pr.real3(*w.box_size)
    inp.camera_mode = pr.CameraMode.ReferenceFrame
    inp.camera = pr.CameraReferenceFrame(vp, float(w.fov_y))
    inp.step_size = float(w.step_size)
    inp.tf_mode = pr.TFMode.Texture
    inp.tf = tf
    return w, inp


def _forward(inp, K, record):
    from diffdvr_gb300 import pyrenderer as pr
    B, H, W = inp.camera.viewport.shape[0], inp.screen_size.y, inp.screen_size.x
    out = pr.RendererOutputs(torch.empty(B, H, W, 4, device="cuda"),
                             torch.empty(B, H, W, dtype=torch.int32, device="cuda"),
                             torch.empty(B, H, W, pr.Renderer.checkpoint_slots(inp, K), device="cuda"), K)
    if record:
        out.sample_density = torch.empty(pr.Renderer.sample_density_size(inp, B), device="cuda")
        out.sample_offset = torch.empty(B, H, W, dtype=torch.int32, device="cuda")
    pr.Renderer.render_forward(inp, out)
    torch.cuda.synchronize()
    return out


def _tf_grad(inp, out, adj):
    from diffdvr_gb300 import pyrenderer as pr
    a = pr.AdjointOutputs()
    a.has_tf_derivatives = True
    a.tf_delayed_accumulation = True
    a.adj_tf = torch.zeros_like(inp.tf)
    pr.Renderer.render_adjoint(inp, out, adj, a)
    torch.cuda.synchronize()
    return a.adj_tf.double().cpu().numpy()


def test_full_size_adjoint_properties(workload):
    w, inp = workload
    out16 = _forward(inp, 16, True)
    term = out16.terminationIndex
    S = int(term.to(torch.int64).sum())
    assert S > 80_000_000
    # sample bound: n <= floor(diagonal / step) + 2
    bound = int(np.floor(np.sqrt(3.0) / w.step_size)) + 2
    assert int(term.min()) >= 0 and int(term.max()) <= bound
    assert (out16.sample_offset.cpu().numpy()[term.cpu().numpy() > 0] >= 0).all()

    g = torch.Generator(device="cuda").manual_seed(11)
    adj1 = torch.randn(out16.color.shape, device="cuda", generator=g) * 1e-3
    adj2 = torch.randn(out16.color.shape, device="cuda", generator=g) * 1e-3
    g1, g2, g12 = _tf_grad(inp, out16, adj1), _tf_grad(inp, out16, adj2), _tf_grad(inp, out16, adj1 + adj2)
    assert rel_l2(g12, g1 + g2) <= 1e-4

    # record kernel against the general kernel (no record), intervals 8 and 32
    for K in (8, 32):
        outK = _forward(inp, K, False)
        assert symmetric_error(outK.color.cpu().numpy(), out16.color.cpu().numpy()) <= 1e-5
        assert torch.equal(outK.terminationIndex, term)
        assert rel_l2(_tf_grad(inp, outK, adj1), g1) <= 1e-4


def test_full_size_batched_equals_single(workload):
    from diffdvr_gb300 import pyrenderer as pr
    w, inp = workload
    single = _forward(inp, 16, False)
    B, H, W = single.color.shape[:3]
    out = pr.RendererOutputs(torch.empty_like(single.color), torch.empty_like(single.terminationIndex),
                             torch.empty_like(single.checkpoints), 16)
    pr.Renderer.render_forward_batched([inp], [out])
    torch.cuda.synchronize()
    same = (out.terminationIndex == single.terminationIndex).cpu().numpy()
    assert same.mean() >= 0.999
    assert symmetric_error(out.color.cpu().numpy()[same], single.color.cpu().numpy()[same]) <= 1e-5
    adj = torch.randn(single.color.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    gs = _tf_grad(inp, single, adj)
    a = pr.AdjointOutputs()
    a.has_tf_derivatives = True
    a.tf_delayed_accumulation = True
    a.adj_tf = torch.zeros_like(inp.tf)
    pr.Renderer.render_adjoint_batched([inp], [out], [adj], [a])
    torch.cuda.synchronize()
    assert rel_l2(a.adj_tf.double().cpu().numpy(), gs) <= 1e-4
