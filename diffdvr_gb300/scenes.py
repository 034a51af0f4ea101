"""Seeded synthetic scenes for the ray marcher (numpy only, no GPU).

Volumes, transfer functions and cameras with the shapes and value
distributions of DiffDVR's workloads.  Cameras follow the reference's
conventions:

* orbit / Fibonacci viewpoints as ``Camera::viewportFromSphere`` builds them
  (renderer/camera.cpp:149-197; up +y, orientation ``Yp``) and
  ``fibonacci_sphere`` (pytests/diffdvr/utils.py:76-88);
* per-pixel rays from a 3x3 viewport (eye, right, up) and a vertical field of
  view, the formula of ``generateRaysForwardImpl`` (renderer/camera_impl.cu:17-36).

The box is [-0.5, 0.5]^3 and a step of ``s`` voxels is ``s / (res - 1)``
world units, as in the reference's consistency tests.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np


# ---------------------------------------------------------------- volumes
def blob_volume(res, n_blobs: int, rng: np.random.Generator, sigma=(4.0, 12.0), amp=(0.3, 1.0),
                noise: float = 0.0, dtype=np.float32) -> np.ndarray:
    """Sum of isotropic Gaussian blobs, clamped to [0, 1]; shape 1*X*Y*Z."""
    X, Y, Z = (res, res, res) if np.isscalar(res) else res
    x = np.arange(X, dtype=np.float32)[:, None, None]
    y = np.arange(Y, dtype=np.float32)[None, :, None]
    z = np.arange(Z, dtype=np.float32)[None, None, :]
    vol = np.zeros((X, Y, Z), dtype=np.float32)
    scale = max(X, Y, Z) / 64.0  # sigma ranges are quoted for 64^3
    for _ in range(n_blobs):
        c = rng.uniform(0, 1, 3) * np.array([X, Y, Z])
        s = rng.uniform(*sigma) * scale
        a = rng.uniform(*amp)
        # separable evaluation keeps 256^3 and 512^3 cheap
        gx = np.exp(-((x - c[0]) ** 2) / (2 * s * s))
        gy = np.exp(-((y - c[1]) ** 2) / (2 * s * s))
        gz = np.exp(-((z - c[2]) ** 2) / (2 * s * s))
        vol += (a * gx) * gy * gz
    if noise > 0:
        vol += noise * rng.uniform(0, 1, vol.shape).astype(np.float32)
    return np.clip(vol, 0, 1).astype(dtype)[None]


def ellipsoid_volume(res: int, n: int, rng: np.random.Generator, dtype=np.float32) -> np.ndarray:
    """Seeded ellipsoids with density U(0.2, 1) on a zero background; shape 1*R*R*R."""
    g = (np.arange(res, dtype=np.float32) + 0.5) / res
    x, y, z = g[:, None, None], g[None, :, None], g[None, None, :]
    vol = np.zeros((res, res, res), dtype=np.float32)
    for _ in range(n):
        c = rng.uniform(0.2, 0.8, 3)
        r = rng.uniform(0.05, 0.2, 3)
        d = rng.uniform(0.2, 1.0)
        inside = ((x - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((z - c[2]) / r[2]) ** 2 <= 1
        vol = np.where(inside, np.maximum(vol, d), vol)
    return vol.astype(dtype)[None]


# ---------------------------------------------------------------- transfer functions
def tf_texture(R: int, rng: np.random.Generator, dtype=np.float32) -> np.ndarray:
    return rng.uniform(0, 1, (1, R, 4)).astype(dtype)


def tf_linear(R: int, rng: np.random.Generator, absorption_scale: float = 10.0, dtype=np.float32) -> np.ndarray:
    tf = np.empty((1, R, 5), dtype=np.float64)
    tf[0, :, :4] = rng.uniform(0, 1, (R, 4))
    tf[0, :, 3] *= absorption_scale
    pos = np.sort(rng.uniform(0, 1, R))
    pos[0], pos[-1] = 0.0, 1.0
    tf[0, :, 4] = pos
    return tf.astype(dtype)


def tf_gaussian(R: int, rng: np.random.Generator, absorption_scale: float = 10.0, dtype=np.float32) -> np.ndarray:
    tf = np.empty((1, R, 6), dtype=np.float64)
    tf[0, :, :4] = rng.uniform(0, 1, (R, 4))
    tf[0, :, 3] *= absorption_scale
    tf[0, :, 4] = rng.uniform(0, 1, R)
    tf[0, :, 5] = rng.uniform(0.02, 0.2, R)
    return tf.astype(dtype)


def tf_identity(absorption: float, color: float = 1.0, dtype=np.float32) -> np.ndarray:
    return np.array([[[absorption, color]]], dtype=dtype)


# ---------------------------------------------------------------- cameras
def fibonacci_sphere(n: int):
    """(latitude, longitude) of n points on a Fibonacci spiral."""
    gr = (np.sqrt(5.0) + 1.0) / 2.0
    ga = (2 - gr) * (2 * np.pi)
    i = np.arange(1, n + 1, dtype=np.float64)
    lat = np.arcsin(-1 + 2 * i / (n + 1))
    lon = np.remainder(ga * i, 2 * np.pi)
    return lat, lon


def _normalize(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def viewport_from_sphere(lat, lon, distance: float, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """B*3*3 viewport (eye, right, up) on a sphere, up +y (orientation Yp)."""
    lat = np.atleast_1d(np.asarray(lat, dtype=np.float64))
    lon = np.atleast_1d(np.asarray(lon, dtype=np.float64))
    yaw, pitch = -lon, -lat  # orientation Yp inverts neither, both are negated
    pos = np.stack([np.cos(pitch) * np.cos(yaw) * distance,
                    np.sin(pitch) * distance,
                    np.cos(pitch) * np.sin(yaw) * distance], axis=1)
    center = np.asarray(center, dtype=np.float64)[None]
    eye = pos + center
    up = np.array([[0.0, 1.0, 0.0]])
    front = _normalize(center - eye)
    right = _normalize(np.cross(front, up))
    up2 = _normalize(np.cross(right, front))
    return np.stack([eye, right, up2], axis=1)


def generate_rays(viewport: np.ndarray, fov_y: float, W: int, H: int, dtype=np.float32):
    """Per-pixel rays (B*H*W*3 start, B*H*W*3 direction) from a B*3*3 viewport."""
    vp = np.asarray(viewport, dtype=np.float64)
    eye, right, up = vp[:, 0], vp[:, 1], vp[:, 2]
    front = np.cross(up, right)
    fov_x = fov_y * W / H
    tx, ty = np.tan(fov_x / 2), np.tan(fov_y / 2)
    fx = 2 * (np.arange(W) + 0.5) / W - 1
    fy = 2 * (np.arange(H) + 0.5) / H - 1
    d = (front[:, None, None, :] + (fx * tx)[None, None, :, None] * right[:, None, None, :]
         + (fy * ty)[None, :, None, None] * up[:, None, None, :])
    d = _normalize(d)
    B = vp.shape[0]
    start = np.broadcast_to(eye[:, None, None, :], (B, H, W, 3))
    return np.ascontiguousarray(start, dtype=dtype), np.ascontiguousarray(d, dtype=dtype)


# ---------------------------------------------------------------- workloads
@dataclass
class Workload:
    """A complete set of renderer inputs in the reference layout."""
    name: str
    volume: np.ndarray          # B*X*Y*Z (pre-shaded: 4*X*Y*Z colour and absorption)
    tf: np.ndarray              # B*R*C
    tf_mode: int                # 0 identity, 1 texture, 2 linear, 3 gaussian, 5 pre-shaded
    blend_mode: int             # 0 Beer-Lambert, 1 alpha
    filter_mode: int            # 0 nearest, 1 trilinear, 3 pre-shaded
    ray_start: np.ndarray       # B*H*W*3
    ray_dir: np.ndarray         # B*H*W*3
    step_size: float
    width: int
    height: int
    viewport: Optional[np.ndarray] = None
    fov_y: float = np.radians(45.0)
    box_min: tuple = (-0.5, -0.5, -0.5)
    box_size: tuple = (1.0, 1.0, 1.0)
    grads: tuple = ("tf",)


def tf_reconstruction_256(seed: int = 1, res: int = 256, views: int = 8, image: int = 256) -> Workload:
    """TF reconstruction: 256^3 volume of 32 blobs + 0.02 noise, 64-entry RGBA
    texture TF, 8 Fibonacci views at 256^2 on radius 3, Beer-Lambert, step
    0.25 voxel, gradient with respect to the TF only."""
    rng = np.random.default_rng(seed)
    vol = blob_volume(res, 32, rng, noise=0.02)
    tf = tf_texture(64, rng)
    lat, lon = fibonacci_sphere(views)
    vp = viewport_from_sphere(lat, lon, 3.0)
    fov = np.radians(45.0)
    rs, rd = generate_rays(vp, fov, image, image)
    return Workload("tf_reconstruction_256", vol, tf, 1, 0, 1, rs, rd, 0.25 / (res - 1), image, image,
                    viewport=vp, fov_y=fov, grads=("tf",))


def preshade_texture(density: np.ndarray, tf: np.ndarray) -> np.ndarray:
    """Colour volume 4*X*Y*Z of a density volume 1*X*Y*Z through a texture TF
    (batch entry 0): texel centres at (i + 0.5) / R, clamped neighbours, as
    the texture TF evaluates a sample (renderer/renderer_tf.cuh:160-171)."""
    R = tf.shape[1]
    d = density[0].astype(np.float32) * np.float32(R) - np.float32(0.5)
    di = np.floor(d).astype(np.int64)
    f = (d - di).astype(np.float32)
    t = tf[0].astype(np.float32)
    a = t[np.clip(di, 0, R - 1)]
    b = t[np.clip(di + 1, 0, R - 1)]
    out = a + f[..., None] * (b - a)
    return np.ascontiguousarray(np.moveaxis(out, -1, 0)).astype(np.float32)


def preshaded_256(seed: int = 1, res: int = 256, views: int = 8, image: int = 256) -> Workload:
    """The TF-reconstruction scene pre-shaded: its density volume through its
    texture TF gives a 4*256^3 colour volume (r, g, b, absorption), rendered
    with the pre-shaded filter and TF modes; 8 views at 256^2, step 0.25
    voxel, gradient with respect to the colour volume."""
    w = tf_reconstruction_256(seed, res, views, image)
    rgba = preshade_texture(w.volume, w.tf)
    return Workload("preshaded_256", rgba, np.zeros((1, 1, 1), np.float32), 5, 0, 3, w.ray_start, w.ray_dir,
                    w.step_size, image, image, viewport=w.viewport, fov_y=w.fov_y, grads=("volume",))


def batched_uneven(seed: int = 3, n: int = 32, n_blobs: int = 16) -> list:
    """n independent instances for one batched call: volume edge drawn from
    {32, 64, 96, 128, 192, 256}, image edge from {64, 128, 256, 512}, a
    volume of n_blobs seeded blobs, a sum of 4 Gaussians TF (means U(0,1),
    sigma U(0.02,0.2), RGBA U(0,1)), trilinear, Beer-Lambert, step 0.5 voxel,
    one orbit view at radius 3 (FOV 45 degrees) as per-pixel rays, gradients
    with respect to the TF and the volume."""
    rng = np.random.default_rng(seed)
    edges = rng.choice([32, 64, 96, 128, 192, 256], size=n)
    images = rng.choice([64, 128, 256, 512], size=n)
    fov = np.radians(45.0)
    out = []
    for i in range(n):
        res, img = int(edges[i]), int(images[i])
        vol = blob_volume(res, n_blobs, rng)
        tf = tf_gaussian(4, rng, absorption_scale=1.0)
        lat = rng.uniform(-np.pi / 2 * 0.9, np.pi / 2 * 0.9)
        lon = rng.uniform(0, 2 * np.pi)
        vp = viewport_from_sphere(lat, lon, 3.0)
        rs, rd = generate_rays(vp, fov, img, img)
        out.append(Workload(f"batched_uneven_{i}", vol, tf, 3, 0, 1, rs, rd, 0.5 / (res - 1), img, img,
                            viewport=vp, fov_y=fov, grads=("tf", "volume")))
    return out


def plain_cpu_64(seed: int = 0) -> Workload:
    """64^3 volume of 8 blobs, trilinear, 8-point linear TF (absorption x10),
    Beer-Lambert, step 0.5 voxel, one 128^2 orbit view at radius 3."""
    rng = np.random.default_rng(seed)
    vol = blob_volume(64, 8, rng)
    tf = tf_linear(8, rng, 10.0)
    lat = rng.uniform(-np.pi / 2 * 0.9, np.pi / 2 * 0.9)
    lon = rng.uniform(0, 2 * np.pi)
    vp = viewport_from_sphere(lat, lon, 3.0)
    fov = np.radians(45.0)
    rs, rd = generate_rays(vp, fov, 128, 128)
    return Workload("plain_cpu_64", vol, tf, 2, 0, 1, rs, rd, 0.5 / 63, 128, 128, viewport=vp, fov_y=fov,
                    grads=("tf", "volume"))


def absorption_recon_128(seed: int = 2, views: int = 64, image: int = 256) -> Workload:
    """Absorption-only reconstruction: 128^3 ellipsoids target, identity TF
    (absorption 20), 64 Fibonacci views at 256^2, step 0.5 voxel, volume gradient."""
    rng = np.random.default_rng(seed)
    vol = ellipsoid_volume(128, 16, rng)
    tf = tf_identity(20.0, 1.0)
    lat, lon = fibonacci_sphere(views)
    vp = viewport_from_sphere(lat, lon, 3.0)
    fov = np.radians(45.0)
    rs, rd = generate_rays(vp, fov, image, image)
    return Workload("absorption_recon_128", vol, tf, 0, 0, 1, rs, rd, 0.5 / 127, image, image,
                    viewport=vp, fov_y=fov, grads=("volume",))


def band_limited_noise(res: int, rng: np.random.Generator, cells: int = 64, dtype=np.float32) -> np.ndarray:
    """Low-pass filtered white noise in [0, 1): U(0,1) on a cells^3 lattice,
    trilinearly interpolated to res^3 (cell-centred); shape res*res*res."""
    from scipy import ndimage
    lattice = rng.uniform(0, 1, (cells, cells, cells)).astype(np.float32)
    coords = (np.arange(res, dtype=np.float32) + 0.5) * (cells / res) - 0.5
    out = np.empty((res, res, res), dtype=np.float32)
    gy, gz = np.meshgrid(coords, coords, indexing="ij")
    for i, cx in enumerate(coords):  # one x slice at a time keeps memory small
        pts = np.stack([np.full_like(gy, cx), gy, gz])
        out[i] = ndimage.map_coordinates(lattice, pts, order=1, mode="nearest")
    return out.astype(dtype)


def large_mixed_512(seed: int = 4, res: int = 512, views: int = 16, image: int = 1024,
                    noise: float = 0.1) -> Workload:
    """Large mixed-precision case: res^3 volume of 64 blobs plus band-limited
    noise (stored BF16/FP16 by the caller), 16-point linear TF (absorption x10),
    `views` Fibonacci views at image^2 on radius 3 as per-pixel rays, Beer-Lambert,
    step 0.5 voxel; gradients with respect to the rays, the volume and the TF."""
    rng = np.random.default_rng(seed)
    vol = blob_volume(res, 64, rng)[0]
    vol = np.clip(vol + noise * band_limited_noise(res, rng), 0, 1).astype(np.float32)[None]
    tf = tf_linear(16, rng, 10.0)
    lat, lon = fibonacci_sphere(views)
    vp = viewport_from_sphere(lat, lon, 3.0)
    fov = np.radians(45.0)
    rs, rd = generate_rays(vp, fov, image, image)
    return Workload("large_mixed_512", vol, tf, 2, 0, 1, rs, rd, 0.5 / (res - 1), image, image,
                    viewport=vp, fov_y=fov, grads=("camera", "volume", "tf"))


def crop(w: Workload, origin, size: int, views=None) -> Workload:
    """The sub-volume of `size`^3 voxels starting at voxel `origin` of a
    workload whose volume fills its box, with the box shrunk to that
    sub-volume (same voxel size, same world positions, same step size) and
    the rays of the chosen views (all by default), which keep their pixels;
    rays that miss the sub-box take no samples."""
    o = np.asarray(origin, dtype=np.int64)
    X = np.array(w.volume.shape[1:], dtype=np.int64)
    if np.any(o < 0) or np.any(o + size > X) or size < 2:
        raise ValueError("the crop must lie inside the volume and hold at least 2 voxels per axis")
    voxel = np.asarray(w.box_size, np.float64) / (X - 1)
    bmin = np.asarray(w.box_min, np.float64) + o * voxel
    vol = np.ascontiguousarray(w.volume[:, o[0]:o[0] + size, o[1]:o[1] + size, o[2]:o[2] + size])
    sel = slice(None) if views is None else list(views)
    return Workload(f"{w.name}_crop{size}", vol, w.tf, w.tf_mode, w.blend_mode, w.filter_mode,
                    np.ascontiguousarray(w.ray_start[sel]), np.ascontiguousarray(w.ray_dir[sel]), w.step_size,
                    w.width, w.height, viewport=None if w.viewport is None else w.viewport[sel], fov_y=w.fov_y,
                    box_min=tuple(float(v) for v in bmin), box_size=tuple(float(v) for v in voxel * (size - 1)),
                    grads=w.grads)


def small_scene(seed: int, shape=(9, 10, 11), W: int = 12, H: int = 10, B: int = 2,
                tf_mode: int = 1, R: Optional[int] = None, opacity: float = 1.0, pad_faces: bool = False,
                dtype=np.float32) -> Workload:
    """Tiny non-cubic scene with random rays aimed at the box (test sizes);
    `opacity` scales the TF's absorption."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    vol = np.concatenate([blob_volume((X, Y, Z), 3, rng, sigma=(6, 14)) for _ in range(B)], 0)
    vol = np.clip(vol + 0.05 * rng.uniform(0, 1, vol.shape), 0, 1)
    if pad_faces:
        # densities strictly inside (0, 1), and the outermost two layers of each
        # face equal, so the trilinear position derivative is continuous where
        # rays enter the box
        vol = 0.02 + 0.9 * vol
        vol[:, 0], vol[:, -1] = vol[:, 1], vol[:, -2]
        vol[:, :, 0], vol[:, :, -1] = vol[:, :, 1], vol[:, :, -2]
        vol[:, :, :, 0], vol[:, :, :, -1] = vol[:, :, :, 1], vol[:, :, :, -2]
    vol = vol.astype(dtype)
    if tf_mode == 0:
        tf = np.concatenate([tf_identity(rng.uniform(5, 15), rng.uniform(0.5, 1.5)) for _ in range(B)], 0)
    elif tf_mode == 1:
        tf = np.concatenate([tf_texture(R or 8, rng) for _ in range(B)], 0)
        tf[..., 3] *= 10
    elif tf_mode == 2:
        tf = np.concatenate([tf_linear(R or 5, rng, 10.0) for _ in range(B)], 0)
    else:
        tf = np.concatenate([tf_gaussian(R or 4, rng, 10.0) for _ in range(B)], 0)
    if opacity != 1.0:
        if tf_mode == 0:
            tf[..., 0] *= opacity
        else:
            tf[..., 3] *= opacity
    lat = rng.uniform(-1.2, 1.2, B)
    lon = rng.uniform(0, 2 * np.pi, B)
    vp = viewport_from_sphere(lat, lon, 2.0)
    fov = np.radians(40.0)
    rs, rd = generate_rays(vp, fov, W, H)
    res = max(shape)
    return Workload(f"small_{seed}", vol.astype(dtype), tf.astype(dtype), tf_mode, 0, 1, rs, rd,
                    0.5 / (res - 1), W, H, viewport=vp, fov_y=fov, grads=("tf", "volume", "camera"))
