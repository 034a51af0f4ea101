"""Drop-in for the reference's ``diffdvr.Renderer`` module and its autograd
function (pytests/diffdvr/renderer.py:61-359), adjoint method.

``forward`` renders with ``pyrenderer.Renderer.render_forward`` and saves the
outputs; ``backward`` zero-initialises the enabled gradients and calls
``render_adjoint``.  When gradients are required, the forward pass also
fills a transmittance-checkpoint buffer (the adjoint re-marches segments
instead of inverting the blend) and, by default, a sample record: every
sample's density and incoming opacity, which the adjoint reads instead of
re-sampling the volume.  The record takes 8 bytes per sample; with
``sample_record="auto"`` the pool is sized for every ray when that fits in a
quarter of the free device memory, else as large as that allows (rays that
find it full are re-sampled).

With ``gradient_method="forward"`` (pytests/diffdvr/renderer.py:63-80,
:136-158, :218-253) the forward pass traces forward-mode derivatives of the
colour with respect to the camera rays (6 variables) and every TF entry
(``render_forward_gradients``), and ``backward`` contracts them with the
colour gradient (``forward_variables_to_gradients``); with
``forward_delayed_gradients=True`` the traced pass runs in ``backward``
instead.  Camera optimisation in forward mode renders per-pixel rays
generated by the differentiable ``Camera.generate_rays``.  Volume gradients
need the adjoint method, as in the reference.
"""
from __future__ import annotations

import time
from typing import Optional

import torch
import torch.nn as nn

from . import pyrenderer
from .camera import Camera


class ProfileRenderer:
    def __init__(self):
        self.forward_ms = 0.0
        self.forward_bytes = 0
        self.backward_ms = 0.0


class _Timer:
    def __init__(self, enable: bool):
        self._enable = enable
        self._elapsed_ms = None

    def elapsed_ms(self):
        return self._elapsed_ms

    def __enter__(self):
        if self._enable:
            self._t = pyrenderer.GpuTimer()
            torch.cuda.synchronize()
            self._t.start()
        return self

    def __exit__(self, *exc):
        if self._enable:
            self._t.stop()
            self._elapsed_ms = self._t.elapsed_ms()


def _size_of(*ts) -> int:
    return sum(t.element_size() * t.numel() for t in ts if t is not None)


def _implies(a, b) -> bool:
    return (not a) or b


def _record_floats(inputs, batch: int, sample_record, device) -> int:
    """Floats of the sample-record pool for a forward pass (0: none).
    sample_record: False / 0 (none), True (every ray), "auto" (every ray if
    that fits in a quarter of the free device memory, else as much as fits),
    or an int number of bytes."""
    if sample_record is False or sample_record is None or sample_record == 0:
        return 0
    full = pyrenderer.Renderer.sample_density_size(inputs, batch)
    if sample_record is True:
        n = full
    elif sample_record == "auto":
        free, _ = torch.cuda.mem_get_info(device)
        n = min(full, free // 4 // 4)
    else:
        n = min(full, int(sample_record) // 4)
    n = n // 4 * 4
    return n if n >= 4 else 0


class _RendererFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, camera_matrix, camera_ray_start, camera_ray_dir, tf, volume,
                inputs: pyrenderer.RendererInputs, fov_y_radians,
                optimize_camera, optimize_tf, optimize_volume, tf_delayed_accumulation,
                checkpoint_interval, sample_record, profiling: Optional[ProfileRenderer]):
        ctx.inputs = inputs
        ctx.fov_y_radians = fov_y_radians
        ctx.optimize = (optimize_camera, optimize_tf, optimize_volume)
        ctx.tf_delayed_accumulation = tf_delayed_accumulation
        ctx.profiling = profiling
        assert _implies(optimize_camera, inputs.camera_mode in (pyrenderer.CameraMode.RayStartDir,
                                                                pyrenderer.CameraMode.ReferenceFrame))
        if inputs.camera_mode == pyrenderer.CameraMode.RayStartDir:
            inputs.camera = pyrenderer.CameraPerPixelRays(camera_ray_start, camera_ray_dir)
        else:
            inputs.camera = pyrenderer.CameraReferenceFrame(camera_matrix, fov_y_radians)
        inputs.tf = tf
        inputs.volume = volume

        # a pre-shaded volume holds its four channels in the first dimension
        # (pytests/diffdvr/renderer.py:110-112)
        batched = [camera_matrix, camera_ray_start, camera_ray_dir, tf]
        if inputs.volume_filter_mode != pyrenderer.VolumeFilterMode.Preshaded:
            batched.append(volume)
        B = max([(1 if t is None else t.shape[0]) for t in batched])
        W, H = inputs.screen_size.x, inputs.screen_size.y
        color = torch.empty(B, H, W, 4, dtype=torch.float32, device=volume.device)
        term = torch.empty(B, H, W, dtype=torch.int32, device=volume.device)
        needs_grad = any(ctx.needs_input_grad[:5])
        ckpt = None
        # pre-shaded volumes need no checkpoints: rays without a record invert the blend
        preshaded = inputs.volume_filter_mode == pyrenderer.VolumeFilterMode.Preshaded
        if needs_grad and checkpoint_interval > 0 and not preshaded:
            slots = pyrenderer.Renderer.checkpoint_slots(inputs, checkpoint_interval)
            ckpt = torch.empty(B, H, W, slots, dtype=torch.float32, device=volume.device)
        outputs = pyrenderer.RendererOutputs(color, term, ckpt, checkpoint_interval)
        # pre-shaded rays use the record only when they are too few to fill the GPU one per lane
        recordable = ckpt is not None or (preshaded and needs_grad and checkpoint_interval > 0 and B * H * W <= 1 << 17)
        pool = _record_floats(inputs, B, sample_record, volume.device) if recordable else 0
        if pool > 0:
            outputs.sample_density = torch.empty(pool, dtype=torch.float32, device=volume.device)
            outputs.sample_offset = torch.empty(B, H, W, dtype=torch.int32, device=volume.device)
        with _Timer(profiling is not None) as timer:
            pyrenderer.Renderer.render_forward(inputs, outputs)
        if profiling is not None:
            profiling.forward_ms += timer.elapsed_ms()
            profiling.forward_bytes += _size_of(camera_matrix, camera_ray_start, camera_ray_dir, tf, volume, color,
                                                term, ckpt, outputs.sample_density, outputs.sample_offset)
        ctx.save_for_backward(camera_matrix, camera_ray_start, camera_ray_dir, tf, volume, color, term, ckpt,
                              outputs.sample_density, outputs.sample_offset)
        ctx.checkpoint_interval = checkpoint_interval
        return color

    @staticmethod
    def backward(ctx, grad_color):
        camera_matrix, ray_start, ray_dir, tf, volume, color, term, ckpt, rec, rec_off = ctx.saved_tensors
        optimize_camera, optimize_tf, optimize_volume = ctx.optimize
        inputs = ctx.inputs
        if inputs.camera_mode == pyrenderer.CameraMode.RayStartDir:
            inputs.camera = pyrenderer.CameraPerPixelRays(ray_start, ray_dir)
        else:
            inputs.camera = pyrenderer.CameraReferenceFrame(camera_matrix, ctx.fov_y_radians)
        inputs.tf = tf
        inputs.volume = volume
        g_cam = g_start = g_dir = g_tf = g_volume = None
        adj = pyrenderer.AdjointOutputs()
        if optimize_camera and inputs.camera_mode == pyrenderer.CameraMode.ReferenceFrame:
            # rays generated in the kernel: the viewport gradient directly
            g_cam = torch.zeros(camera_matrix.shape, dtype=torch.float32, device=camera_matrix.device)
            adj.has_viewport_derivatives = True
            adj.adj_viewport = g_cam
        elif optimize_camera:
            g_start = torch.zeros_like(ray_start)
            g_dir = torch.zeros_like(ray_dir)
            adj.has_camera_derivatives = True
            adj.adj_camera_ray_start = g_start
            adj.adj_camera_ray_dir = g_dir
        if optimize_tf:
            g_tf = torch.zeros(tf.shape, dtype=torch.float32, device=tf.device)
            adj.has_tf_derivatives = True
            adj.tf_delayed_accumulation = ctx.tf_delayed_accumulation
            adj.adj_tf = g_tf
        if optimize_volume:
            g_volume = torch.zeros(volume.shape, dtype=torch.float32, device=volume.device)
            adj.has_volume_derivatives = True
            adj.adj_volume = g_volume
        fwd = pyrenderer.RendererOutputs(color, term, ckpt, ctx.checkpoint_interval, rec, rec_off)
        with _Timer(ctx.profiling is not None) as timer:
            pyrenderer.Renderer.render_adjoint(inputs, fwd, grad_color.contiguous().float(), adj)
        if ctx.profiling is not None:
            ctx.profiling.backward_ms += timer.elapsed_ms()
        if g_tf is not None and tf.dtype != torch.float32:
            g_tf = g_tf.to(tf.dtype)
        if g_volume is not None and volume.dtype != torch.float32:
            g_volume = g_volume.to(volume.dtype)
        if g_cam is not None and camera_matrix.dtype != torch.float32:
            g_cam = g_cam.to(camera_matrix.dtype)
        return g_cam, g_start, g_dir, g_tf, g_volume, None, None, None, None, None, None, None, None, None


def _forward_settings(optimize_camera, optimize_tf, tf) -> pyrenderer.ForwardDifferencesSettings:
    """Derivative indices of the forward method: the six ray components
    first, then the TF entries in row-major order
    (pytests/diffdvr/renderer.py:63-80)."""
    s = pyrenderer.ForwardDifferencesSettings()
    D = 0
    if optimize_camera:
        s.d_rayStart = pyrenderer.int3(D, D + 1, D + 2)
        s.d_rayDir = pyrenderer.int3(D + 3, D + 4, D + 5)
        D += 6
    if optimize_tf:
        B, R, C = tf.shape
        idx = torch.arange(D, D + R * C, dtype=torch.int32, device=tf.device).reshape(1, R, C)
        s.d_tf = idx.expand(B, R, C).contiguous()
        s.has_tf_derivatives = True
        D += R * C
    s.D = D
    return s


class _ForwardModeFunction(torch.autograd.Function):
    """The forward method: forward-mode derivatives traced by the renderer,
    contracted with the colour gradient in backward."""

    @staticmethod
    def forward(ctx, ray_start, ray_dir, tf, volume, inputs: pyrenderer.RendererInputs, optimize_camera,
                optimize_tf, delayed, profiling: Optional[ProfileRenderer]):
        ctx.inputs = inputs
        ctx.optimize = (optimize_camera, optimize_tf)
        ctx.delayed = delayed
        ctx.profiling = profiling
        if inputs.camera_mode == pyrenderer.CameraMode.RayStartDir:
            inputs.camera = pyrenderer.CameraPerPixelRays(ray_start, ray_dir)
        inputs.tf = tf
        inputs.volume = volume
        B = max([(1 if t is None else t.shape[0]) for t in (ray_start, ray_dir, tf, volume)])
        W, H = inputs.screen_size.x, inputs.screen_size.y
        color = torch.empty(B, H, W, 4, dtype=torch.float32, device=volume.device)
        term = torch.empty(B, H, W, dtype=torch.int32, device=volume.device)
        outputs = pyrenderer.RendererOutputs(color, term)
        settings = _forward_settings(optimize_camera, optimize_tf, tf)
        ctx.settings = settings
        grads = None
        with _Timer(profiling is not None) as timer:
            if delayed or settings.D == 0:
                pyrenderer.Renderer.render_forward(inputs, outputs)
            else:
                grads = torch.empty(B, H, W, settings.D, 4, dtype=torch.float32, device=volume.device)
                pyrenderer.Renderer.render_forward_gradients(inputs, settings, outputs, grads)
        if profiling is not None:
            profiling.forward_ms += timer.elapsed_ms()
            profiling.forward_bytes += _size_of(ray_start, ray_dir, tf, volume, color, term, grads)
        ctx.save_for_backward(ray_start, ray_dir, tf, volume, grads)
        return color

    @staticmethod
    def backward(ctx, grad_color):
        ray_start, ray_dir, tf, volume, grads = ctx.saved_tensors
        optimize_camera, optimize_tf = ctx.optimize
        settings = ctx.settings
        inputs = ctx.inputs
        if settings.D == 0:
            return None, None, None, None, None, None, None, None, None
        with _Timer(ctx.profiling is not None) as timer:
            if grads is None:
                if inputs.camera_mode == pyrenderer.CameraMode.RayStartDir:
                    inputs.camera = pyrenderer.CameraPerPixelRays(ray_start, ray_dir)
                inputs.tf = tf
                inputs.volume = volume
                B, H, W = grad_color.shape[:3]
                color = torch.empty(B, H, W, 4, dtype=torch.float32, device=volume.device)
                term = torch.empty(B, H, W, dtype=torch.int32, device=volume.device)
                grads = torch.empty(B, H, W, settings.D, 4, dtype=torch.float32, device=volume.device)
                pyrenderer.Renderer.render_forward_gradients(inputs, settings, pyrenderer.RendererOutputs(color, term),
                                                             grads)
            adj = pyrenderer.AdjointOutputs()
            g_start = g_dir = g_tf = None
            if optimize_camera:
                g_start = torch.zeros(ray_start.shape, dtype=torch.float32, device=ray_start.device)
                g_dir = torch.zeros(ray_dir.shape, dtype=torch.float32, device=ray_dir.device)
                adj.has_camera_derivatives = True
                adj.adj_camera_ray_start = g_start
                adj.adj_camera_ray_dir = g_dir
            if optimize_tf:
                g_tf = torch.zeros(tf.shape, dtype=torch.float32, device=tf.device)
                adj.has_tf_derivatives = True
                adj.adj_tf = g_tf
            pyrenderer.Renderer.forward_variables_to_gradients(grads, grad_color.contiguous().float(), settings, adj)
        if ctx.profiling is not None:
            ctx.profiling.backward_ms += timer.elapsed_ms()
        if g_tf is not None and tf.dtype != torch.float32:
            g_tf = g_tf.to(tf.dtype)
        return g_start, g_dir, g_tf, None, None, None, None, None, None


class Renderer(nn.Module):
    """Mirrors diffdvr.Renderer (pytests/diffdvr/renderer.py:264-359)."""

    def __init__(self, settings: Optional[pyrenderer.RendererInputs] = None, optimize_camera=False,
                 optimize_tf=False, optimize_volume=False, gradient_method="adjoint",
                 forward_delayed_gradients=False, tf_delayed_accumulation=True, checkpoint_interval: int = 16,
                 sample_record="auto", fused_camera: bool = True):
        super().__init__()
        self._settings = settings if settings is not None else pyrenderer.RendererInputs()
        self._optimize_camera = optimize_camera
        self._optimize_tf = optimize_tf
        self._optimize_volume = optimize_volume
        self._has_parameters_to_optimize = optimize_camera or optimize_tf or optimize_volume
        assert gradient_method in ["adjoint", "forward"]
        assert _implies(optimize_volume, gradient_method == "adjoint"), \
            "if volume densities should be optimized, the gradient method must be 'adjoint'"
        self._use_adjoint_method = gradient_method == "adjoint"
        self._forward_delayed_gradients = bool(forward_delayed_gradients)
        self._tf_delayed_accumulation = tf_delayed_accumulation
        self._checkpoint_interval = int(checkpoint_interval)
        self._sample_record = sample_record
        self._fused_camera = bool(fused_camera)
        self._renderer_function = _RendererFunction.apply

    def get_settings(self):
        return self._settings

    def set_settings(self, settings: pyrenderer.RendererInputs):
        assert settings is not None
        self._settings = settings

    settings = property(get_settings, set_settings)

    def train(self, mode: bool = True):
        if mode is True and not self._has_parameters_to_optimize:
            raise ValueError("requested training mode, but no parameters were specified to be optimized")
        return super().train(mode)

    def forward(self, *, camera: torch.Tensor = None, fov_y_radians: float = None, tf: torch.Tensor = None,
                volume: torch.Tensor = None, profiling: ProfileRenderer = None):
        """Renders the volume; returns the B*H*W*4 colour image."""
        assert _implies(self._optimize_camera, camera is not None)
        assert _implies(self._optimize_camera, fov_y_radians is not None)
        assert _implies(self._optimize_tf, tf is not None)
        assert _implies(self._optimize_volume, volume is not None)
        inputs = self._settings.clone()
        camera_matrix = ray_start = ray_dir = None
        if not self._use_adjoint_method:
            return self._forward_method(inputs, camera, fov_y_radians, tf, volume, profiling)
        if camera is not None:
            if self._optimize_camera and not self._fused_camera:
                ray_start, ray_dir = Camera.generate_rays(camera, fov_y_radians, self._settings.screen_size.x,
                                                          self._settings.screen_size.y)
                inputs.camera_mode = pyrenderer.CameraMode.RayStartDir
            else:
                camera_matrix = camera
                inputs.camera_mode = pyrenderer.CameraMode.ReferenceFrame
        elif isinstance(inputs.camera, pyrenderer.CameraPerPixelRays):
            ray_start, ray_dir = inputs.camera.ray_start, inputs.camera.ray_dir
        elif isinstance(inputs.camera, pyrenderer.CameraReferenceFrame):
            camera_matrix, fov_y_radians = inputs.camera.viewport, inputs.camera.fov_y_radians
        if tf is None:
            tf = inputs.tf
        if volume is None:
            volume = inputs.volume
        return self._renderer_function(camera_matrix, ray_start, ray_dir, tf, volume, inputs, fov_y_radians,
                                       self._optimize_camera, self._optimize_tf, self._optimize_volume,
                                       self._tf_delayed_accumulation, self._checkpoint_interval,
                                       self._sample_record, profiling)

    def _forward_method(self, inputs, camera, fov_y_radians, tf, volume, profiling):
        ray_start = ray_dir = None
        if camera is not None:
            # forward variables are taken with respect to per-pixel rays
            ray_start, ray_dir = Camera.generate_rays(camera, fov_y_radians, self._settings.screen_size.x,
                                                      self._settings.screen_size.y)
            inputs.camera_mode = pyrenderer.CameraMode.RayStartDir
        elif isinstance(inputs.camera, pyrenderer.CameraPerPixelRays):
            ray_start, ray_dir = inputs.camera.ray_start, inputs.camera.ray_dir
        assert _implies(self._optimize_camera, inputs.camera_mode == pyrenderer.CameraMode.RayStartDir)
        if tf is None:
            tf = inputs.tf
        if volume is None:
            volume = inputs.volume
        return _ForwardModeFunction.apply(ray_start, ray_dir, tf, volume, inputs, self._optimize_camera,
                                          self._optimize_tf, self._forward_delayed_gradients, profiling)
