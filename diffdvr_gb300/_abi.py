"""ctypes mirror of include/diffdvr_gb300.h and the loader of libdvr_gb300.so.

The library is built in-tree by ``diffdvr_gb300.build`` (``__graft_entry__.build()``
does it).  There is no fallback: when the library is missing every renderer
call raises, so a run can never silently render on the CPU.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

# ---- status codes and enums (values of the C header) ----
DVR_OK = 0
DVR_E_INVALID_ARGUMENT = -1
DVR_E_NO_GRADIENT = -2
DVR_E_UNSUPPORTED = -3
DVR_E_CUDA = -4

DVR_FLOAT32, DVR_FLOAT64, DVR_FLOAT16, DVR_BFLOAT16, DVR_INT32 = 0, 1, 2, 3, 4
DVR_DEVICE_CPU, DVR_DEVICE_CUDA = 0, 1
DVR_KIND_TENSOR, DVR_KIND_VALUE = 0, 1
DVR_CAMERA_PER_PIXEL_RAYS = 0
DVR_CAMERA_INVERSE_VIEW_TENSOR = 1
DVR_CAMERA_INVERSE_VIEW_VALUE = 2
DVR_CAMERA_REFERENCE_FRAME_KIND = 3
DVR_KERNELS_PLAIN, DVR_KERNELS_OPTIMIZED = 0, 1


class DvrTensor(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("ndim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("device_type", ctypes.c_int32),
        ("device_index", ctypes.c_int32),
        ("sizes", ctypes.c_int64 * 5),
        ("strides", ctypes.c_int64 * 5),
    ]


class DvrRendererInputs(ctypes.Structure):
    _fields_ = [
        ("screen_width", ctypes.c_int32),
        ("screen_height", ctypes.c_int32),
        ("volume_filter_mode", ctypes.c_int32),
        ("camera_mode", ctypes.c_int32),
        ("tf_mode", ctypes.c_int32),
        ("blend_mode", ctypes.c_int32),
        ("volume", DvrTensor),
        ("box_min_kind", ctypes.c_int32),
        ("box_size_kind", ctypes.c_int32),
        ("box_min", DvrTensor),
        ("box_size", DvrTensor),
        ("box_min_value", ctypes.c_double * 3),
        ("box_size_value", ctypes.c_double * 3),
        ("camera_kind", ctypes.c_int32),
        ("step_size_kind", ctypes.c_int32),
        ("camera_ray_start", DvrTensor),
        ("camera_ray_dir", DvrTensor),
        ("camera_matrix", DvrTensor),
        ("camera_matrix_value", ctypes.c_float * 16),
        ("camera_fov_y_radians", ctypes.c_double),
        ("step_size", DvrTensor),
        ("step_size_value", ctypes.c_double),
        ("tf", DvrTensor),
        ("blending_early_out", ctypes.c_double),
    ]


class DvrRendererOutputs(ctypes.Structure):
    _fields_ = [
        ("color", DvrTensor),
        ("termination_index", DvrTensor),
        ("checkpoints", DvrTensor),
        ("checkpoint_interval", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("sample_density", DvrTensor),
        ("sample_offset", DvrTensor),
    ]


class DvrAdjointOutputs(ctypes.Structure):
    _fields_ = [
        ("has_volume_derivatives", ctypes.c_int32),
        ("has_stepsize_derivatives", ctypes.c_int32),
        ("has_camera_derivatives", ctypes.c_int32),
        ("has_tf_derivatives", ctypes.c_int32),
        ("tf_delayed_accumulation", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("adj_volume", DvrTensor),
        ("adj_stepsize", DvrTensor),
        ("adj_camera_ray_start", DvrTensor),
        ("adj_camera_ray_dir", DvrTensor),
        ("adj_tf", DvrTensor),
        ("has_viewport_derivatives", ctypes.c_int32),
        ("pad2_", ctypes.c_int32),
        ("adj_viewport", DvrTensor),
    ]


class DvrForwardDifferencesSettings(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int32),
        ("d_stepsize", ctypes.c_int32),
        ("d_ray_start", ctypes.c_int32 * 3),
        ("d_ray_dir", ctypes.c_int32 * 3),
        ("has_tf_derivatives", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("d_tf", DvrTensor),
    ]


# every exported symbol of the header, with its signature
_P = ctypes.POINTER
SIGNATURES = {
    "dvr_render_forward": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), ctypes.c_void_p]),
    "dvr_render_adjoint": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), _P(DvrTensor),
                                          _P(DvrAdjointOutputs), ctypes.c_void_p]),
    "dvr_render_adjoint_noalloc": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), _P(DvrTensor),
                                                  _P(DvrAdjointOutputs), ctypes.c_void_p]),
    "dvr_render_forward_batched": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), ctypes.c_int32,
                                                  ctypes.c_void_p]),
    "dvr_render_adjoint_batched": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), _P(DvrTensor),
                                                  _P(DvrAdjointOutputs), ctypes.c_int32, ctypes.c_void_p]),
    "dvr_render_forward_gradients": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrForwardDifferencesSettings),
                                                    _P(DvrRendererOutputs), _P(DvrTensor), ctypes.c_void_p]),
    "dvr_forward_variables_to_gradients": (ctypes.c_int, [_P(DvrTensor), _P(DvrTensor),
                                                          _P(DvrForwardDifferencesSettings), _P(DvrAdjointOutputs),
                                                          ctypes.c_void_p]),
    "dvr_preshade_volume": (ctypes.c_int, [_P(DvrTensor), _P(DvrTensor), ctypes.c_int32, _P(DvrTensor),
                                           ctypes.c_void_p]),
    "dvr_preshade_volume_adjoint": (ctypes.c_int, [_P(DvrTensor), _P(DvrTensor), ctypes.c_int32, _P(DvrTensor),
                                                   _P(DvrTensor), ctypes.c_void_p]),
    "dvr_checkpoint_slots": (ctypes.c_int64, [ctypes.c_double, ctypes.c_double, ctypes.c_int32]),
    "dvr_last_error": (ctypes.c_char_p, []),
    "dvr_set_kernel_family": (ctypes.c_int, [ctypes.c_int32]),
    "dvr_get_kernel_family": (ctypes.c_int, []),
    "dvr_set_sync_mode": (ctypes.c_int, [ctypes.c_int32]),
    "dvr_get_sync_mode": (ctypes.c_int, []),
    "dvr_abi_version": (ctypes.c_int, []),
    "dvr_set_window_adjoint": (ctypes.c_int, [ctypes.c_int32]),
    "dvr_get_window_adjoint": (ctypes.c_int, []),
    "dvr_set_forward_gather": (ctypes.c_int, [ctypes.c_int32]),
    "dvr_get_forward_gather": (ctypes.c_int, []),
    "dvr_last_adjoint_path": (ctypes.c_int, []),
    "dvr_render_forward_batched_tiled": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs),
                                                        _P(ctypes.c_int32), ctypes.c_int32, ctypes.c_void_p]),
    "dvr_render_adjoint_batched_tiled": (ctypes.c_int, [_P(DvrRendererInputs), _P(DvrRendererOutputs), _P(DvrTensor),
                                                        _P(DvrAdjointOutputs), _P(ctypes.c_int32), ctypes.c_int32,
                                                        ctypes.c_void_p]),
}

# DvrAdjointPath
FORWARD_GATHERS = {"auto": 0, "direct": 1, "cells": 2, "texture": 3}
ADJOINT_PATHS = {0: "none", 1: "plain", 2: "general", 3: "record", 4: "window", 5: "preshaded", 6: "remarch"}

_LIB = None
ABI_VERSION = 6


def library_path() -> str:
    return _build.LIB_PATH


def load() -> ctypes.CDLL:
    """Loads libdvr_gb300.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"diffdvr_gb300 CUDA library not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (or diffdvr_gb300.build.build())")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.dvr_abi_version() != ABI_VERSION:
            raise RuntimeError("libdvr_gb300.so has an unexpected ABI version")
        _LIB = lib
    return _LIB


class DvrError(RuntimeError):
    """An error reported by the C ABI (the reference raises RuntimeError too)."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def check(code: int) -> None:
    if code != DVR_OK:
        msg = load().dvr_last_error().decode("utf-8", "replace")
        raise DvrError(code, msg or f"diffdvr_gb300 call failed with code {code}")
