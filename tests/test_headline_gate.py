"""The metric's gates at the full TF-reconstruction workload: 256^3 volume
of 32 blobs + 0.02 noise stored in BF16, 64-entry texture TF, 8 Fibonacci
views at 256^2 (reference-frame camera), Beer-Lambert, step 0.25 voxel,
about 90 M samples per pass; TF gradient only.

The GPU kernels (optimized family, BF16 storage, FP32 arithmetic) are held
against the FP64 oracle on the same inputs (the BF16-rounded volume), every
pixel and every view counted (oracle.check.render_errors):

* image: no pixel's symmetric error against FP64 above max(1e-5, 3 e32),
  e32 = the reference FP32 arithmetic's own error on that pixel, except on
  rays whose sample count is decided by the rounding of the box exit
  distance ((tmax - tmin) / step within 2e-3 of an integer, count off by
  one; measured: 15 such pixels of 524,288, the reference's FP32 CPU
  arithmetic has 33 of its own, at other pixels);
* termination: at most 0.1 % of the pixels with a sample count other than
  the FP64 oracle's (each such pixel is also in the image check above);
* TF gradient: relative L2 error <= 1e-3 against the FP64 adjoint for one
  seeded N(0, 1e-3) output adjoint on every pixel, both for the recorded
  path the benchmark times (sample record, record adjoint kernel) and for the
  memory-lean path (transmittance checkpoints every 16 samples, general
  adjoint re-marching each segment).

The oracle takes about 10 s (8 x86 cores) for the forward and the adjoint in
FP64 and FP32.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

IMAGE_FLOOR = 1e-5
TERM_MISMATCH_SHARE = 1e-3
GRAD_GATE = 1e-3


@pytest.fixture(scope="module")
def headline(cuda_device, oracle_built):
    from diffdvr_gb300 import pyrenderer as pr, scenes
    from oracle import oracle as O
    w = scenes.tf_reconstruction_256(seed=1)
    vol = torch.from_numpy(w.volume).to("cuda").to(torch.bfloat16)
    vp = w.viewport.astype(np.float32)
    fov = float(np.float32(w.fov_y))
    inp = pr.RendererInputs()
    inp.screen_size = pr.int2(w.width, w.height)
    inp.volume = vol
    inp.box_min = pr.real3(*w.box_min)
    inp.box_size = pr.real3(*w.box_size)
    inp.camera_mode = pr.CameraMode.ReferenceFrame
    inp.camera = pr.CameraReferenceFrame(torch.from_numpy(vp).cuda(), fov)
    inp.step_size = float(w.step_size)
    inp.tf_mode = pr.TFMode.Texture
    inp.tf = torch.from_numpy(w.tf).cuda()
    sc = O.Scene(width=w.width, height=w.height, volume=vol.float().cpu().numpy(), tf=w.tf,
                 step_size=np.full((1, 1, 1), w.step_size, np.float32),
                 box_min=np.asarray([w.box_min], np.float32), box_size=np.asarray([w.box_size], np.float32),
                 filter_mode=1, camera_mode=2, tf_mode=1, blend_mode=0, camera_matrix=vp, fov_y_radians=fov)
    B = vp.shape[0]
    adj = (np.random.default_rng(5).standard_normal((B, w.height, w.width, 4)) * 1e-3).astype(np.float32)
    return w, inp, sc, adj


def _run(inp, adj_np, record: bool, K: int = 16):
    from diffdvr_gb300 import pyrenderer as pr
    pr.set_kernel_family("optimized")
    B, H, W = adj_np.shape[:3]
    out = pr.RendererOutputs(torch.empty(B, H, W, 4, device="cuda"),
                             torch.empty(B, H, W, dtype=torch.int32, device="cuda"),
                             torch.empty(B, H, W, pr.Renderer.checkpoint_slots(inp, K), device="cuda"), K)
    if record:
        out.sample_density = torch.empty(pr.Renderer.sample_density_size(inp, B), device="cuda")
        out.sample_offset = torch.empty(B, H, W, dtype=torch.int32, device="cuda")
    pr.Renderer.render_forward(inp, out)
    a = pr.AdjointOutputs()
    a.has_tf_derivatives = True
    a.tf_delayed_accumulation = True
    a.adj_tf = torch.zeros_like(inp.tf)
    pr.Renderer.render_adjoint(inp, out, torch.from_numpy(adj_np).cuda(), a)
    torch.cuda.synchronize()
    if record:
        recorded = out.sample_offset.cpu().numpy()[out.terminationIndex.cpu().numpy() > 0]
        assert (recorded >= 0).all(), "the full-size pool must record every ray with samples"
    return out.color.cpu().numpy(), out.terminationIndex.cpu().numpy(), a.adj_tf.double().cpu().numpy()


@pytest.mark.parametrize("record", [True, False], ids=["sample-record", "checkpoints-only"])
def test_headline_against_fp64_oracle(headline, record):
    from oracle import check
    w, inp, sc, adj = headline
    color, term, g = _run(inp, adj, record)
    r = check.render_errors(sc, color, term, adj, {"adj_tf": g}, floor=IMAGE_FLOOR)
    print("headline gate", "record" if record else "checkpoints", r)
    assert r["samples"] > 80_000_000
    assert r["term_mismatch"] <= TERM_MISMATCH_SHARE * r["pixels"], r
    assert r["image_fail_unexplained"] == 0, r
    assert r["grad_rel_err"] <= GRAD_GATE, r
