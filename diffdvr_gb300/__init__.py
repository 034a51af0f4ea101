"""diffdvr_gb300 — DiffDVR's differentiable volume ray marcher on GB300 (sm_103a).

* ``diffdvr_gb300.pyrenderer``: drop-in for the reference's ``pyrenderer``
  forward/adjoint entry points and settings structs;
* ``diffdvr_gb300.Renderer``: drop-in for ``diffdvr.Renderer`` (autograd);
* ``diffdvr_gb300.Camera``: ray generation and viewport helpers;
* ``diffdvr_gb300.scenes``: seeded synthetic volumes, TFs and cameras.

The kernels and the C ABI live in ``lib/libdvr_gb300.so`` (built by
``diffdvr_gb300.build``); see include/diffdvr_gb300.h.
"""
from . import pyrenderer
from .camera import Camera, Orientation
from .renderer import ProfileRenderer, Renderer

__all__ = ["pyrenderer", "Camera", "Orientation", "Renderer", "ProfileRenderer"]
