"""The differentiable camera of diffdvr_gb300.camera on the CPU.

* Camera.generate_rays (the per-pixel rays of a viewport, the formula of the
  reference's generateRaysForwardImpl, renderer/camera_impl.cu:17-36) gives
  the rays the march computes itself for the reference-frame camera
  (renderer/renderer_camera.cuh:13-59, the oracle's restatement, pinned to
  the reference by the golden fixtures); the numpy twin used by the
  workloads gives the same rays.
* Its autograd backward, which stands in for the reference's
  GenerateRayFunction adjoint (renderer/camera.cpp:200-266), matches finite
  differences (torch.autograd.gradcheck, FP64).
* viewport_from_lookat returns (eye, right, up) with right and up orthonormal
  and cross(up, right) the viewing direction, the frame generate_rays expects.
"""
import numpy as np
import pytest
import torch

from diffdvr_gb300 import scenes
from diffdvr_gb300.camera import Camera


def _viewports(n=3, seed=0):
    rng = np.random.default_rng(seed)
    origins = torch.tensor(rng.uniform(-3, 3, (n, 3)), dtype=torch.float64)
    look = torch.tensor(rng.uniform(-0.2, 0.2, (n, 3)), dtype=torch.float64)
    up = torch.tensor([[0.0, 1.0, 0.0]], dtype=torch.float64)
    return origins, look, Camera.viewport_from_lookat(origins, look, up)


@pytest.mark.parametrize("W,H,fov", [(7, 5, 0.7), (4, 9, 1.1), (1, 1, 0.4)])
def test_generate_rays_is_the_reference_frame_camera(oracle_built, W, H, fov):
    O = oracle_built
    _, _, vp = _viewports()
    rs, rd = Camera.generate_rays(vp, fov, W, H)
    sc = O.Scene(width=W, height=H, volume=np.zeros((1, 2, 2, 2)), tf=np.zeros((1, 1, 4)),
                 step_size=np.full((1, 1, 1), 0.1), box_min=np.full((1, 3), -0.5), box_size=np.ones((1, 3)),
                 camera_mode=2, camera_matrix=vp.numpy(), fov_y_radians=fov)
    s_ref, d_ref = O.camera_rays(sc)
    assert np.array_equal(rs.numpy(), s_ref)
    # the field of view's tangents are taken in FP32, as the reference's ray generator does
    assert np.abs(rd.numpy() - d_ref).max() <= 1e-7
    rs_np, rd_np = scenes.generate_rays(vp.numpy(), fov, W, H, dtype=np.float64)
    assert np.array_equal(rs_np, rs.numpy()) and np.abs(rd_np - rd.numpy()).max() <= 1e-7


def test_generate_rays_backward_matches_finite_differences():
    _, _, vp = _viewports(n=2, seed=1)
    vp = vp.clone().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda v: Camera.generate_rays(v, 0.8, 4, 3), (vp,), eps=1e-6, atol=1e-7)


def test_viewport_from_lookat_frame():
    origins, look, vp = _viewports(n=4, seed=2)
    eye, right, up = vp[:, 0], vp[:, 1], vp[:, 2]
    assert torch.equal(eye, origins)
    assert torch.allclose(right.norm(dim=1), torch.ones(4, dtype=torch.float64))
    assert torch.allclose(up.norm(dim=1), torch.ones(4, dtype=torch.float64))
    assert torch.allclose((right * up).sum(1), torch.zeros(4, dtype=torch.float64), atol=1e-12)
    front = torch.nn.functional.normalize(look - origins, dim=1)
    assert torch.allclose(torch.cross(up, right, dim=1), front, atol=1e-12)
