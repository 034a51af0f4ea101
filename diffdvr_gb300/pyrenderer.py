"""Drop-in for the reference's ``pyrenderer`` module (the forward/adjoint path).

Same names, fields and argument meaning as the pybind11 module of the
reference (bindings/bindings.cpp:143-511): the settings structs
``RendererInputs`` / ``RendererOutputs`` / ``AdjointOutputs``, the enums, the
small vector types, and ``Renderer.render_forward`` / ``render_adjoint``.
Each call hands plain pointers, sizes and strides to the C ABI of
libdvr_gb300.so (include/diffdvr_gb300.h) together with the PyTorch current
CUDA stream; validation and kernel launches happen in the library.  Invalid
arguments raise ``RuntimeError`` with the reference's check messages.

Differences from the reference:
* tensors must be CUDA tensors (there is no CPU renderer);
* the volume and the TF may be float16/bfloat16 (sampled in FP32);
* ``RendererOutputs`` may carry a ``checkpoints`` buffer that lets the
  optimized adjoint re-march from transmittance checkpoints instead of
  inverting the blend;
* ``Renderer.render_forward_batched`` / ``render_adjoint_batched`` render
  instances of different volume and image sizes in one launch.
"""
from __future__ import annotations

import ctypes
import enum
import math
from typing import Optional, Sequence, Union

import numpy as np
import torch

from . import _abi

# --------------------------------------------------------------------- enums
class VolumeFilterMode(enum.IntEnum):
    Nearest = 0
    Trilinear = 1
    Preshaded = 3


class CameraMode(enum.IntEnum):
    RayStartDir = 0
    InverseViewMatrix = 1
    ReferenceFrame = 2


class TFMode(enum.IntEnum):
    Identity = 0
    Texture = 1
    Linear = 2
    Gaussian = 3
    Preshaded = 5
    GaussianLog = 6


class BlendMode(enum.IntEnum):
    BeerLambert = 0
    Alpha = 1


# --------------------------------------------------------------------- small types
class _Vec:
    _names = ()

    def __init__(self, *values):
        if values and len(values) != len(self._names):
            raise TypeError(f"{type(self).__name__} takes {len(self._names)} values")
        for n, v in zip(self._names, values or (0,) * len(self._names)):
            setattr(self, n, v)

    def __iter__(self):
        return iter(getattr(self, n) for n in self._names)

    def __str__(self):
        return "(" + ", ".join(str(v) for v in self) + ")"

    __repr__ = __str__


class real3(_Vec):
    _names = ("x", "y", "z")


class real4(_Vec):
    _names = ("x", "y", "z", "w")


class int2(_Vec):
    _names = ("x", "y")


class int3(_Vec):
    _names = ("x", "y", "z")


class mat4:
    """A 4x4 matrix given by value (the reference wraps glm::mat4)."""

    def __init__(self, m=None):
        a = np.eye(4, dtype=np.float32) if m is None else np.asarray(m, dtype=np.float32)
        if a.shape != (4, 4):
            raise RuntimeError("Incompatible buffer sizes! Expected a shape of 4x4")
        self.m = a.copy()

    def to_torch(self) -> torch.Tensor:
        return torch.from_numpy(self.m.copy()).reshape(1, 4, 4)

    def __str__(self):
        return str(self.m)


class CameraPerPixelRays:
    def __init__(self, ray_start: Optional[torch.Tensor] = None, ray_dir: Optional[torch.Tensor] = None):
        self.ray_start = ray_start
        self.ray_dir = ray_dir


class CameraReferenceFrame:
    def __init__(self, viewport: Optional[torch.Tensor] = None, fov_y_radians: float = 0.0):
        self.viewport = viewport
        self.fov_y_radians = float(fov_y_radians)


# --------------------------------------------------------------------- settings structs
class RendererInputs:
    """Mirrors RendererInputsHost (renderer/renderer.h:20-64)."""

    def __init__(self):
        self.screen_size = int2(0, 0)
        self.volume: Optional[torch.Tensor] = None
        self.volume_filter_mode = VolumeFilterMode.Trilinear
        self.box_min: Union[torch.Tensor, real3] = real3(0, 0, 0)
        self.box_size: Union[torch.Tensor, real3] = real3(1, 1, 1)
        self.camera_mode = CameraMode.RayStartDir
        self.camera = CameraPerPixelRays()
        self.step_size: Union[torch.Tensor, float] = 0.1
        self.tf_mode = TFMode.Texture
        self.tf: Optional[torch.Tensor] = None
        self.blend_mode = BlendMode.BeerLambert
        self.blending_early_out = 1.0 - 1e-5

    def clone(self) -> "RendererInputs":
        """performs a shallow clone"""
        c = RendererInputs()
        c.__dict__.update(self.__dict__)
        return c


class RendererOutputs:
    """Mirrors RendererOutputsHost (renderer/renderer.h:67-71).

    ``checkpoints`` (optional, B*H*W*C float32) receives the accumulated opacity
    every ``checkpoint_interval`` samples during the forward pass; see
    ``Renderer.checkpoint_slots``.

    ``sample_density`` (optional, 1-D float32 pool, with ``sample_offset``, a
    B*H*W int32 tensor, and checkpoints) receives, for every sample of each
    ray, its density and the opacity accumulated in front of it; the adjoint
    then reads these instead of re-sampling the volume.  Rays that find the
    pool full are re-sampled; ``Renderer.sample_density_size`` gives a size
    that holds every ray."""

    def __init__(self, color: Optional[torch.Tensor] = None, terminationIndex: Optional[torch.Tensor] = None,
                 checkpoints: Optional[torch.Tensor] = None, checkpoint_interval: int = 16,
                 sample_density: Optional[torch.Tensor] = None, sample_offset: Optional[torch.Tensor] = None):
        self.color = color
        self.terminationIndex = terminationIndex
        self.checkpoints = checkpoints
        self.checkpoint_interval = checkpoint_interval
        self.sample_density = sample_density
        self.sample_offset = sample_offset


class AdjointOutputs:
    """Mirrors AdjointOutputsHost (renderer/renderer.h:95-111)."""

    def __init__(self):
        self.has_volume_derivatives = False
        self.adj_volume: Optional[torch.Tensor] = None
        self.has_stepsize_derivatives = False
        self.adj_stepsize: Optional[torch.Tensor] = None
        self.has_camera_derivatives = False
        self.adj_camera_ray_start: Optional[torch.Tensor] = None
        self.adj_camera_ray_dir: Optional[torch.Tensor] = None
        self.has_tf_derivatives = False
        self.tf_delayed_accumulation = False
        self.adj_tf: Optional[torch.Tensor] = None
        # extension: gradient of a CameraReferenceFrame viewport ((B) 3 3), the
        # rays being generated inside the kernel
        self.has_viewport_derivatives = False
        self.adj_viewport: Optional[torch.Tensor] = None


class ForwardDifferencesSettings:
    """Mirrors ForwardDifferencesSettingsHost (renderer/renderer.h:73-93,
    bindings/bindings.cpp:423-436): the derivative index of each traced
    variable, NOT_ENABLED (-1) for the others."""
    NOT_ENABLED = -1

    def __init__(self):
        self.D = 0
        self.d_stepsize = -1
        self.d_rayStart = int3(-1, -1, -1)
        self.d_rayDir = int3(-1, -1, -1)
        self.d_tf: Optional[torch.Tensor] = None
        self.has_tf_derivatives = False


# --------------------------------------------------------------------- marshalling
_DTYPES = {
    torch.float32: _abi.DVR_FLOAT32,
    torch.float64: _abi.DVR_FLOAT64,
    torch.float16: _abi.DVR_FLOAT16,
    torch.bfloat16: _abi.DVR_BFLOAT16,
    torch.int32: _abi.DVR_INT32,
}


def _tensor(t: Optional[torch.Tensor], name: str = "tensor") -> _abi.DvrTensor:
    d = _abi.DvrTensor()
    if t is None:
        d.ndim = -1
        return d
    if not isinstance(t, torch.Tensor):
        raise RuntimeError(f"{name} must be a torch.Tensor, got {type(t).__name__}")
    if t.dim() > 5:
        raise RuntimeError(f"{name} has more than 5 dimensions")
    d.data = t.data_ptr() if t.numel() > 0 else 0
    d.ndim = t.dim()
    d.dtype = _DTYPES.get(t.dtype, 99)
    d.device_type = _abi.DVR_DEVICE_CUDA if t.is_cuda else _abi.DVR_DEVICE_CPU
    d.device_index = t.device.index if t.is_cuda else -1
    for i in range(t.dim()):
        d.sizes[i] = t.shape[i]
        d.strides[i] = t.stride(i)
    return d


def _inputs(inp: RendererInputs) -> _abi.DvrRendererInputs:
    c = _abi.DvrRendererInputs()
    c.screen_width, c.screen_height = int(inp.screen_size.x), int(inp.screen_size.y)
    c.volume_filter_mode = int(inp.volume_filter_mode)
    c.camera_mode = int(inp.camera_mode)
    c.tf_mode = int(inp.tf_mode)
    c.blend_mode = int(inp.blend_mode)
    c.volume = _tensor(inp.volume, "volume")
    for name in ("box_min", "box_size"):
        v = getattr(inp, name)
        if isinstance(v, torch.Tensor):
            setattr(c, name + "_kind", _abi.DVR_KIND_TENSOR)
            setattr(c, name, _tensor(v, name))
        else:
            setattr(c, name + "_kind", _abi.DVR_KIND_VALUE)
            setattr(c, name, _tensor(None))
            arr = getattr(c, name + "_value")
            for i, x in enumerate(v):
                arr[i] = float(x)
    cam = inp.camera
    c.camera_ray_start = _tensor(None)
    c.camera_ray_dir = _tensor(None)
    c.camera_matrix = _tensor(None)
    if isinstance(cam, CameraPerPixelRays):
        c.camera_kind = _abi.DVR_CAMERA_PER_PIXEL_RAYS
        c.camera_ray_start = _tensor(cam.ray_start, "cameraRayStart")
        c.camera_ray_dir = _tensor(cam.ray_dir, "cameraRayDir")
    elif isinstance(cam, CameraReferenceFrame):
        c.camera_kind = _abi.DVR_CAMERA_REFERENCE_FRAME_KIND
        c.camera_matrix = _tensor(cam.viewport, "cameraMatrix")
        c.camera_fov_y_radians = float(cam.fov_y_radians)
    elif isinstance(cam, mat4):
        c.camera_kind = _abi.DVR_CAMERA_INVERSE_VIEW_VALUE
        for i, x in enumerate(cam.m.reshape(-1)):
            c.camera_matrix_value[i] = float(x)
    elif isinstance(cam, torch.Tensor):
        c.camera_kind = _abi.DVR_CAMERA_INVERSE_VIEW_TENSOR
        c.camera_matrix = _tensor(cam, "cameraMatrix")
    else:
        raise RuntimeError("unknown camera type")
    if isinstance(inp.step_size, torch.Tensor):
        c.step_size_kind = _abi.DVR_KIND_TENSOR
        c.step_size = _tensor(inp.step_size, "stepSize")
    else:
        c.step_size_kind = _abi.DVR_KIND_VALUE
        c.step_size = _tensor(None)
        c.step_size_value = float(inp.step_size)
    c.tf = _tensor(inp.tf, "tf")
    c.blending_early_out = float(inp.blending_early_out)
    return c


def _outputs(out: RendererOutputs) -> _abi.DvrRendererOutputs:
    c = _abi.DvrRendererOutputs()
    c.color = _tensor(out.color, "color")
    c.termination_index = _tensor(out.terminationIndex, "terminationIndex")
    c.checkpoints = _tensor(getattr(out, "checkpoints", None), "checkpoints")
    c.checkpoint_interval = int(getattr(out, "checkpoint_interval", 16) or 16)
    c.sample_density = _tensor(getattr(out, "sample_density", None), "sample_density")
    c.sample_offset = _tensor(getattr(out, "sample_offset", None), "sample_offset")
    return c


def _adjoint_outputs(a: AdjointOutputs) -> _abi.DvrAdjointOutputs:
    c = _abi.DvrAdjointOutputs()
    c.has_volume_derivatives = int(bool(a.has_volume_derivatives))
    c.has_stepsize_derivatives = int(bool(a.has_stepsize_derivatives))
    c.has_camera_derivatives = int(bool(a.has_camera_derivatives))
    c.has_tf_derivatives = int(bool(a.has_tf_derivatives))
    c.tf_delayed_accumulation = int(bool(a.tf_delayed_accumulation))
    c.adj_volume = _tensor(a.adj_volume if a.has_volume_derivatives else None, "adj_volume")
    c.adj_stepsize = _tensor(a.adj_stepsize if a.has_stepsize_derivatives else None, "adj_stepsize")
    c.adj_camera_ray_start = _tensor(a.adj_camera_ray_start if a.has_camera_derivatives else None,
                                     "adj_camera_ray_start")
    c.adj_camera_ray_dir = _tensor(a.adj_camera_ray_dir if a.has_camera_derivatives else None, "adj_camera_ray_dir")
    c.adj_tf = _tensor(a.adj_tf if a.has_tf_derivatives else None, "adj_tf")
    c.has_viewport_derivatives = int(bool(getattr(a, "has_viewport_derivatives", False)))
    c.adj_viewport = _tensor(a.adj_viewport if c.has_viewport_derivatives else None, "adj_viewport")
    return c


def _forward_settings(fs: ForwardDifferencesSettings) -> _abi.DvrForwardDifferencesSettings:
    c = _abi.DvrForwardDifferencesSettings()
    c.D = int(fs.D)
    c.d_stepsize = int(fs.d_stepsize)
    start, direction = list(fs.d_rayStart), list(fs.d_rayDir)
    for i in range(3):
        c.d_ray_start[i] = int(start[i])
        c.d_ray_dir[i] = int(direction[i])
    c.has_tf_derivatives = int(bool(fs.has_tf_derivatives))
    c.d_tf = _tensor(fs.d_tf, "d_tf")
    return c


def _stream_of(t: Optional[torch.Tensor]) -> int:
    if t is not None and t.is_cuda:
        return torch.cuda.current_stream(t.device).cuda_stream
    return 0


# --------------------------------------------------------------------- renderer
class Renderer:
    """The reference's static renderer entry points (renderer/renderer.h:113-269)."""

    @staticmethod
    def render_forward(inputs: RendererInputs, outputs: RendererOutputs) -> None:
        """Performs a simple forward rendering without gradients."""
        lib = _abi.load()
        ci, co = _inputs(inputs), _outputs(outputs)
        _abi.check(lib.dvr_render_forward(ctypes.byref(ci), ctypes.byref(co), _stream_of(inputs.volume)))

    @staticmethod
    def render_adjoint(inputs: RendererInputs, outputs_from_forward: RendererOutputs, adj_color: torch.Tensor,
                       adj_outputs: AdjointOutputs) -> None:
        """Performs adjoint/backward rendering; gradients are accumulated
        into the (zero-initialised) tensors of adj_outputs."""
        lib = _abi.load()
        ci, co = _inputs(inputs), _outputs(outputs_from_forward)
        ca, cg = _tensor(adj_color, "adj_color"), _adjoint_outputs(adj_outputs)
        _abi.check(lib.dvr_render_adjoint(ctypes.byref(ci), ctypes.byref(co), ctypes.byref(ca), ctypes.byref(cg),
                                          _stream_of(inputs.volume)))

    @staticmethod
    def render_forward_gradients(inputs: RendererInputs, differences_settings: ForwardDifferencesSettings,
                                 outputs: RendererOutputs, gradients_out: torch.Tensor) -> None:
        """Forward rendering with forward-mode derivatives: fills outputs and
        gradients_out (B*H*W*D*4, d color / d variable) for the variables
        selected by differences_settings."""
        lib = _abi.load()
        ci, co = _inputs(inputs), _outputs(outputs)
        cs, cg = _forward_settings(differences_settings), _tensor(gradients_out, "gradients_out")
        _abi.check(lib.dvr_render_forward_gradients(ctypes.byref(ci), ctypes.byref(cs), ctypes.byref(co),
                                                    ctypes.byref(cg), _stream_of(inputs.volume)))

    @staticmethod
    def forward_variables_to_gradients(forward_variables: torch.Tensor, adj_color: torch.Tensor,
                                       differences_settings: ForwardDifferencesSettings,
                                       adj_outputs: AdjointOutputs) -> None:
        """Converts forward variables (B*H*W*D*4) to the gradients of the
        step size, camera rays and TF for the colour adjoint adj_color."""
        lib = _abi.load()
        cf, ca = _tensor(forward_variables, "forward_variables"), _tensor(adj_color, "adj_color")
        cs, cg = _forward_settings(differences_settings), _adjoint_outputs(adj_outputs)
        _abi.check(lib.dvr_forward_variables_to_gradients(ctypes.byref(cf), ctypes.byref(ca), ctypes.byref(cs),
                                                          ctypes.byref(cg), _stream_of(forward_variables)))

    @staticmethod
    def render_forward_batched(inputs: Sequence[RendererInputs], outputs: Sequence[RendererOutputs],
                               tile_shapes: Optional[Sequence[int]] = None) -> None:
        """Renders instances of different volume/image sizes in one launch.
        tile_shapes: a DvrTileShape per instance (0 = 16x8, 1 = 32x4, 2 =
        8x16), e.g. from diffdvr_gb300.autotune; None = 16x8 for all."""
        lib = _abi.load()
        n = len(inputs)
        if len(outputs) != n:
            raise RuntimeError("inputs and outputs must have the same length")
        ci = (_abi.DvrRendererInputs * max(n, 1))(*[_inputs(i) for i in inputs])
        co = (_abi.DvrRendererOutputs * max(n, 1))(*[_outputs(o) for o in outputs])
        stream = _stream_of(inputs[0].volume) if n else 0
        _abi.check(lib.dvr_render_forward_batched_tiled(ci, co, _shapes(tile_shapes, n), n, stream))

    @staticmethod
    def render_adjoint_batched(inputs: Sequence[RendererInputs], outputs_from_forward: Sequence[RendererOutputs],
                               adj_colors: Sequence[torch.Tensor], adj_outputs: Sequence[AdjointOutputs],
                               tile_shapes: Optional[Sequence[int]] = None) -> None:
        lib = _abi.load()
        n = len(inputs)
        if not (len(outputs_from_forward) == len(adj_colors) == len(adj_outputs) == n):
            raise RuntimeError("all instance lists must have the same length")
        ci = (_abi.DvrRendererInputs * max(n, 1))(*[_inputs(i) for i in inputs])
        co = (_abi.DvrRendererOutputs * max(n, 1))(*[_outputs(o) for o in outputs_from_forward])
        ca = (_abi.DvrTensor * max(n, 1))(*[_tensor(a, "adj_color") for a in adj_colors])
        cg = (_abi.DvrAdjointOutputs * max(n, 1))(*[_adjoint_outputs(a) for a in adj_outputs])
        stream = _stream_of(inputs[0].volume) if n else 0
        _abi.check(lib.dvr_render_adjoint_batched_tiled(ci, co, ca, cg, _shapes(tile_shapes, n), n, stream))

    @staticmethod
    def checkpoint_slots(inputs: RendererInputs, interval: int = 16) -> int:
        """Checkpoint slots per ray for RendererOutputs.checkpoints: from the
        box diagonal and the smallest step size."""
        bs = inputs.box_size
        bs = bs.detach().abs().amax(0).tolist() if isinstance(bs, torch.Tensor) else list(bs)
        length = math.sqrt(sum(float(v) * float(v) for v in bs))
        st = inputs.step_size
        min_step = float(st.detach().amin()) if isinstance(st, torch.Tensor) else float(st)
        n = _abi.load().dvr_checkpoint_slots(length, min_step, int(interval))
        if n < 0:
            _abi.check(int(n))
        return int(n)

    @staticmethod
    def sample_density_size(inputs: RendererInputs, batch: int) -> int:
        """Floats of a RendererOutputs.sample_density pool that holds every
        ray of a batch-``batch`` image: B*H*W rays of 2 floats per sample,
        4*ceil(n/2) floats each, n the sample bound from the box diagonal and
        the smallest step size."""
        W, H = int(inputs.screen_size.x), int(inputs.screen_size.y)
        return int(batch) * H * W * 4 * Renderer.checkpoint_slots(inputs, 2)


# --------------------------------------------------------------------- module functions
class _PreshadeFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, density, tf, tf_mode):
        lib = _abi.load()
        out = torch.empty((4,) + tuple(density.shape[1:]), dtype=torch.float32, device=density.device)
        cd, ct, co = _tensor(density, "density"), _tensor(tf, "tf"), _tensor(out, "color")
        _abi.check(lib.dvr_preshade_volume(ctypes.byref(cd), ctypes.byref(ct), int(tf_mode), ctypes.byref(co),
                                           _stream_of(density)))
        ctx.save_for_backward(density, tf)
        ctx.tf_mode = int(tf_mode)
        return out

    @staticmethod
    def backward(ctx, grad_color):
        density, tf = ctx.saved_tensors
        lib = _abi.load()
        adj = torch.empty_like(density)
        cd, ct = _tensor(density, "density"), _tensor(tf, "tf")
        ca, co = _tensor(grad_color.contiguous().float(), "adj_color"), _tensor(adj, "adj_density")
        _abi.check(lib.dvr_preshade_volume_adjoint(ctypes.byref(cd), ctypes.byref(ct), ctx.tf_mode, ctypes.byref(ca),
                                                   ctypes.byref(co), _stream_of(density)))
        return adj, None, None


class TFUtils:
    """The pre-shading entry of the reference's TFUtils (renderer/tf_utils.h:125-140,
    bindings/bindings.cpp:570-581)."""

    @staticmethod
    def preshade_volume(density: torch.Tensor, tf: torch.Tensor, tfMode) -> torch.Tensor:
        """Pre-shades a density volume of shape 1*X*Y*Z with the transfer
        function into a colour volume of shape 4*X*Y*Z (r, g, b, opacity),
        differentiable with respect to the density."""
        return _PreshadeFunction.apply(density, tf, int(tfMode))


def set_kernel_family(family: str) -> str:
    """'optimized' (default) or 'plain' (one thread per ray, reference semantics)."""
    code = {"plain": _abi.DVR_KERNELS_PLAIN, "optimized": _abi.DVR_KERNELS_OPTIMIZED}[family]
    prev = _abi.load().dvr_set_kernel_family(code)
    _abi.check(min(prev, 0))
    return "plain" if prev == _abi.DVR_KERNELS_PLAIN else "optimized"


def get_kernel_family() -> str:
    return "plain" if _abi.load().dvr_get_kernel_family() == _abi.DVR_KERNELS_PLAIN else "optimized"


def set_cuda_sync_mode(sync: bool) -> None:
    _abi.load().dvr_set_sync_mode(int(bool(sync)))


def get_cuda_sync_mode() -> bool:
    return bool(_abi.load().dvr_get_sync_mode())


def use_double_precision() -> int:
    """0: the renderer computes in single precision."""
    return 0


# Kernel-cache controls of the reference's NVRTC loader.  The kernels here are
# compiled ahead of time, so these have nothing to do and are accepted as no-ops.
def reload_kernels() -> None:
    pass


def set_cuda_cache_dir(path: str) -> None:
    pass


def disable_cuda_cache() -> None:
    pass


def set_kernel_cache_file(filename: str) -> None:
    pass


def set_cuda_debug_mode(debug: bool) -> None:
    pass


def _shapes(tile_shapes, n: int):
    """ctypes int32 array of n tile shapes, or None."""
    if tile_shapes is None:
        return None
    if len(tile_shapes) != n:
        raise RuntimeError("tile_shapes must hold one shape per instance")
    return (ctypes.c_int32 * max(n, 1))(*[int(t) for t in tile_shapes])


def set_window_adjoint(enable: bool) -> bool:
    """Volume gradients from the sample record through the window adjoint
    or the general per-ray adjoint (the default, measured faster); returns
    the previous setting."""
    return bool(_abi.load().dvr_set_window_adjoint(int(bool(enable))))


def set_forward_gather(mode: str) -> str:
    """How the forward reads a trilinear sample's eight corners: "auto"
    (default), "direct" (eight loads), "cells" (one cell record per sample)
    or "texture" (two gathers from the slab texture); returns the previous
    mode."""
    if mode not in _abi.FORWARD_GATHERS:
        raise RuntimeError(f"unknown forward gather mode {mode!r}")
    prev = _abi.load().dvr_set_forward_gather(_abi.FORWARD_GATHERS[mode])
    return {v: k for k, v in _abi.FORWARD_GATHERS.items()}[prev]


def last_adjoint_path() -> str:
    """The kernels the last render_adjoint call on this thread ran: "plain",
    "general", "record", "window", "preshaded" or "none"."""
    return _abi.ADJOINT_PATHS.get(_abi.load().dvr_last_adjoint_path(), "none")


def cleanup() -> None:
    pass


def sync() -> None:
    torch.cuda.synchronize()


class GpuTimer:
    """CUDA-event timer on the current stream (bindings/bindings.cpp:99-129)."""

    def __init__(self):
        self._start = torch.cuda.Event(enable_timing=True)
        self._stop = torch.cuda.Event(enable_timing=True)

    def start(self):
        self._start.record()

    def stop(self):
        self._stop.record()

    def elapsed_ms(self) -> float:
        self._stop.synchronize()
        return self._start.elapsed_time(self._stop)


# pyrenderer.Camera and pyrenderer.Orientation (bindings/bindings.cpp:514-552):
# the reference's diffdvr.Renderer generates per-pixel rays through
# pyrenderer.Camera.generate_rays when it optimises the camera
from .camera import Camera, Orientation  # noqa: E402
