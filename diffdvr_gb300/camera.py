"""Camera helpers of the reference's ``pyrenderer.Camera`` (renderer/camera.cpp).

* ``generate_rays``: per-pixel rays from a B*3*3 viewport (eye, right, up)
  and a vertical field of view, the formula of generateRaysForwardImpl
  (renderer/camera_impl.cu:17-36); written with differentiable torch ops so
  autograd provides the viewport adjoint (the reference's GenerateRayFunction,
  renderer/camera.cpp:200-266).
* ``viewport_from_lookat`` / ``viewport_from_sphere`` (renderer/camera.cpp:127-197).
* ``compute_matrix``: inverse view-projection matrix of a left-handed look-at
  camera with a [0,1]-depth perspective (renderer/camera.cpp:86-125).
"""
from __future__ import annotations

import enum
import math

import numpy as np
import torch


class Orientation(enum.IntEnum):
    Xp = 0
    Xm = 1
    Yp = 2
    Ym = 3
    Zp = 4
    Zm = 5


# up vectors, axis permutations and yaw inversion per orientation (renderer/camera.cpp:70-85)
_UP = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
_PERM = [(2, -1, -3), (-2, 1, 3), (1, 2, 3), (-1, -2, -3), (-3, -1, 2), (3, 1, -2)]
_INVERT_YAW = [True, False, False, True, False, True]


def _normalize(v: torch.Tensor) -> torch.Tensor:
    return torch.nn.functional.normalize(v, dim=1)


class Camera:
    Orientation = Orientation

    @staticmethod
    def generate_rays(viewport: torch.Tensor, fov_y: float, screen_width: int, screen_height: int):
        """Returns (ray_start, ray_dir), each B*H*W*3; differentiable w.r.t. viewport."""
        W, H = int(screen_width), int(screen_height)
        dt, dev = viewport.dtype, viewport.device
        eye, right, up = viewport[:, 0, :], viewport[:, 1, :], viewport[:, 2, :]
        front = torch.cross(up, right, dim=1)
        fov_x = float(np.float32(fov_y) * np.float32(W) / np.float32(H))
        tan_x = float(np.tan(np.float32(fov_x / 2)))
        tan_y = float(np.tan(np.float32(fov_y / 2)))
        fx = (2 * (torch.arange(W, device=dev, dtype=dt) + 0.5) / W - 1) * tan_x
        fy = (2 * (torch.arange(H, device=dev, dtype=dt) + 0.5) / H - 1) * tan_y
        d = (front[:, None, None, :] + fx[None, None, :, None] * right[:, None, None, :]
             + fy[None, :, None, None] * up[:, None, None, :])
        d = d * torch.rsqrt((d * d).sum(-1, keepdim=True))
        start = eye[:, None, None, :].expand(-1, H, W, -1)
        return start.contiguous(), d.contiguous()

    @staticmethod
    def viewport_from_lookat(origin: torch.Tensor, look_at: torch.Tensor, camera_up: torch.Tensor) -> torch.Tensor:
        front = _normalize(look_at - origin)
        right = _normalize(torch.cross(front, camera_up.expand_as(front), dim=1))
        up2 = _normalize(torch.cross(right, front, dim=1))
        return torch.stack([origin.expand_as(front), right, up2], dim=1)

    @staticmethod
    def viewport_from_sphere(center: torch.Tensor, yaw_radians: torch.Tensor, pitch_radians: torch.Tensor,
                             distance: torch.Tensor, orientation: Orientation) -> torch.Tensor:
        o = int(orientation)
        yaw = yaw_radians * (1.0 if _INVERT_YAW[o] else -1.0)
        pitch = pitch_radians * -1.0
        pos = [torch.cos(pitch) * torch.cos(yaw) * distance, torch.sin(pitch) * distance,
               torch.cos(pitch) * torch.sin(yaw) * distance]
        pos2 = [pos[abs(p) - 1] * (1 if p > 0 else -1) for p in _PERM[o]]
        origin = torch.cat(pos2, dim=1)
        B = origin.shape[0]
        up = torch.tensor([_UP[o]], dtype=center.dtype, device=center.device).expand(B, 3)
        return Camera.viewport_from_lookat(origin + center, center.expand_as(origin), up)

    @staticmethod
    def compute_matrix(origin, look_at, up, fov_degrees: float, width: int, height: int, near_clip: float = 0.1,
                       far_clip: float = 10.0) -> np.ndarray:
        """Inverse view-projection matrix (4x4, rows as the renderer reads them)."""
        eye = np.asarray(list(origin), dtype=np.float64)
        ctr = np.asarray(list(look_at), dtype=np.float64)
        upv = np.asarray(list(up), dtype=np.float64)
        upv = upv / np.linalg.norm(upv)
        f = ctr - eye
        f /= np.linalg.norm(f)
        s = np.cross(upv, f)
        s /= np.linalg.norm(s)
        u = np.cross(f, s)
        view = np.array([[s[0], s[1], s[2], -s @ eye], [u[0], u[1], u[2], -u @ eye], [f[0], f[1], f[2], -f @ eye],
                         [0, 0, 0, 1]])
        h = math.cos(0.5 * math.radians(fov_degrees)) / math.sin(0.5 * math.radians(fov_degrees))
        w = h * height / width
        n, fa = near_clip, far_clip
        proj = np.array([[w, 0, 0, 0], [0, h, 0, 0], [0, 0, fa / (fa - n), -(fa * n) / (fa - n)], [0, 0, 1, 0]])
        return np.linalg.inv(proj @ view).astype(np.float32)
