"""C ABI and host logic without a GPU: the library loads and exports every
symbol of include/diffdvr_gb300.h; argument validation mirrors the reference's
checks (renderer/renderer.cpp:49-391, :660-742) and fails before any CUDA call."""
import ctypes
import os
import re

import numpy as np
import pytest

from diffdvr_gb300 import _abi
from diffdvr_gb300 import pyrenderer as pr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "diffdvr_gb300.h")


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(dvr_\w+)\(", text, re.M)))


def test_library_exports_every_header_symbol(dvr_lib):
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(dvr_lib, n), n
    assert set(names) == set(_abi.SIGNATURES)
    assert dvr_lib.dvr_abi_version() == 6


def _fake(shape, dtype=_abi.DVR_FLOAT32, cuda=True, ptr=0x100000):
    t = _abi.DvrTensor()
    t.data = ptr
    t.ndim = len(shape)
    t.dtype = dtype
    t.device_type = _abi.DVR_DEVICE_CUDA if cuda else _abi.DVR_DEVICE_CPU
    t.device_index = 0 if cuda else -1
    st = 1
    for i in reversed(range(len(shape))):
        t.sizes[i] = shape[i]
        t.strides[i] = st
        st *= shape[i]
    return t


def _inputs(B=1, X=4, Y=5, Z=6, W=8, H=7, tf_mode=1, R=8):
    c = _abi.DvrRendererInputs()
    c.screen_width, c.screen_height = W, H
    c.volume_filter_mode, c.camera_mode, c.tf_mode, c.blend_mode = 1, 0, tf_mode, 0
    c.volume = _fake((B, X, Y, Z))
    c.box_min_kind = c.box_size_kind = _abi.DVR_KIND_VALUE
    c.box_min = _fake(())
    c.box_min.ndim = -1
    c.box_size = _fake(())
    c.box_size.ndim = -1
    for i in range(3):
        c.box_min_value[i], c.box_size_value[i] = -0.5, 1.0
    c.camera_kind = _abi.DVR_CAMERA_PER_PIXEL_RAYS
    c.camera_ray_start = _fake((B, H, W, 3))
    c.camera_ray_dir = _fake((B, H, W, 3))
    c.camera_matrix = _fake(())
    c.camera_matrix.ndim = -1
    c.step_size_kind = _abi.DVR_KIND_VALUE
    c.step_size = _fake(())
    c.step_size.ndim = -1
    c.step_size_value = 0.01
    C = {0: 2, 1: 4, 2: 5, 3: 6}[tf_mode]
    c.tf = _fake((B, 1 if tf_mode == 0 else R, C))
    c.blending_early_out = 1 - 1e-5
    return c


def _outputs(B=1, W=8, H=7):
    o = _abi.DvrRendererOutputs()
    o.color = _fake((B, H, W, 4))
    o.termination_index = _fake((B, H, W), _abi.DVR_INT32)
    o.checkpoints = _fake(())
    o.checkpoints.ndim = -1
    o.checkpoint_interval = 32
    return o


def _forward(lib, i, o):
    code = lib.dvr_render_forward(ctypes.byref(i), ctypes.byref(o), None)
    return code, lib.dvr_last_error().decode()


@pytest.mark.parametrize("mutate,expect", [
    (lambda i, o: setattr(i, "volume", _fake((4, 5, 6))), "volume must be a tensor with 4 dimensions"),
    (lambda i, o: setattr(i, "volume", _fake((1, 4, 5, 6), cuda=False)), "CPU tensor"),
    (lambda i, o: setattr(i, "volume", _fake((1, 4, 5, 6), _abi.DVR_FLOAT64)), "volume must be of type float32"),
    (lambda i, o: setattr(i, "tf", _fake((1, 8, 3))), "tf must have 4 entries at dimension 2"),
    (lambda i, o: setattr(i, "tf_mode", 6), "TFGaussianLog is not supported"),
    (lambda i, o: setattr(i, "volume_filter_mode", 3),
     "if pre-shading is selected, both the filter mode and TF mode must be set to preshaded"),
    (lambda i, o: (setattr(i, "volume_filter_mode", 3), setattr(i, "tf_mode", 5)),
     "the volume colors are encoded in the batch dimension of the volume. It must be 4, but is 1"),
    (lambda i, o: setattr(i, "camera_ray_start", _fake((1, 7, 9, 3))), "cameraRayStart must have 8 entries at dimension 2"),
    (lambda i, o: setattr(i, "camera_ray_dir", _fake((3, 7, 8, 3))), None),  # batch 3 vs 1 broadcasts; passes checks
    (lambda i, o: setattr(i, "camera_mode", 2), "'CameraReferenceFrame' specified in 'cameraMode'"),
    (lambda i, o: setattr(o, "color", _fake((1, 7, 8, 3))), "color must have 4 entries at dimension 3"),
    (lambda i, o: setattr(o, "termination_index", _fake((1, 7, 8))), "terminationIndex must be of type int32"),
])
def test_forward_validation_messages(dvr_lib, mutate, expect):
    i, o = _inputs(), _outputs()
    mutate(i, o)
    code, msg = _forward(dvr_lib, i, o)
    if expect is None:
        # all checks pass for broadcasting, the output batch (1) is then wrong
        assert code == _abi.DVR_E_INVALID_ARGUMENT and "color must have 3 entries at dimension 0" in msg
    else:
        assert code in (_abi.DVR_E_INVALID_ARGUMENT, _abi.DVR_E_UNSUPPORTED)
        assert expect in msg, msg


def test_linear_tf_needs_two_points(dvr_lib):
    i, o = _inputs(tf_mode=2, R=1), _outputs()
    code, msg = _forward(dvr_lib, i, o)
    assert code == _abi.DVR_E_INVALID_ARGUMENT and "at least two control points" in msg


def test_batch_mismatch(dvr_lib):
    i, o = _inputs(B=2), _outputs(B=2)
    i.tf = _fake((3, 8, 4))
    code, msg = _forward(dvr_lib, i, o)
    assert "tf must be have the same batch size as other tensors" in msg


def test_adjoint_without_gradients_is_rejected(dvr_lib):
    i, o = _inputs(), _outputs()
    a = _abi.DvrAdjointOutputs()
    for n in ("adj_volume", "adj_stepsize", "adj_camera_ray_start", "adj_camera_ray_dir", "adj_tf"):
        getattr(a, n).ndim = -1
    adj = _fake((1, 7, 8, 4))
    code = dvr_lib.dvr_render_adjoint(ctypes.byref(i), ctypes.byref(o), ctypes.byref(adj), ctypes.byref(a), None)
    assert code == _abi.DVR_E_NO_GRADIENT
    assert "At least one adjoint variable must be activated" in dvr_lib.dvr_last_error().decode()


def test_adjoint_output_shape_checks(dvr_lib):
    i, o = _inputs(), _outputs()
    a = _abi.DvrAdjointOutputs()
    a.has_tf_derivatives = 1
    a.adj_tf = _fake((1, 7, 4))
    adj = _fake((1, 7, 8, 4))
    code = dvr_lib.dvr_render_adjoint(ctypes.byref(i), ctypes.byref(o), ctypes.byref(adj), ctypes.byref(a), None)
    assert code == _abi.DVR_E_INVALID_ARGUMENT
    assert "adj_tf must have 8 entries at dimension 1" in dvr_lib.dvr_last_error().decode()


@pytest.mark.parametrize("frame,shape,expect", [
    (False, (1, 3, 3), "viewport derivatives require cameraMode == ReferenceFrame"),
    (True, (1, 3, 4), "adj_viewport must have 3 entries at dimension 2"),
])
def test_viewport_derivative_checks(dvr_lib, frame, shape, expect):
    i, o = _inputs(), _outputs()
    if frame:
        i.camera_mode = 2
        i.camera_kind = _abi.DVR_CAMERA_REFERENCE_FRAME_KIND
        i.camera_matrix = _fake((1, 3, 3))
        i.camera_fov_y_radians = 0.7
    a = _abi.DvrAdjointOutputs()
    a.has_viewport_derivatives = 1
    a.adj_viewport = _fake(shape)
    adj = _fake((1, 7, 8, 4))
    code = dvr_lib.dvr_render_adjoint(ctypes.byref(i), ctypes.byref(o), ctypes.byref(adj), ctypes.byref(a), None)
    assert code == _abi.DVR_E_INVALID_ARGUMENT
    assert expect in dvr_lib.dvr_last_error().decode()


def test_checkpoint_slots(dvr_lib):
    # 256^3 box diagonal sqrt(3), step 0.25 voxel: at most 1768 samples -> 56 slots of 32
    n = dvr_lib.dvr_checkpoint_slots(np.sqrt(3.0), 0.25 / 255, 32)
    assert n == int(np.ceil((np.floor(np.sqrt(3.0) / (0.25 / 255)) + 2) / 32))
    assert dvr_lib.dvr_checkpoint_slots(1.0, 0.0, 32) < 0
    assert dvr_lib.dvr_checkpoint_slots(1.0, 0.1, 100) < 0


def test_kernel_family_and_sync_mode(dvr_lib):
    prev = pr.set_kernel_family("plain")
    assert pr.get_kernel_family() == "plain"
    pr.set_kernel_family(prev)
    pr.set_cuda_sync_mode(True)
    assert pr.get_cuda_sync_mode()
    pr.set_cuda_sync_mode(False)
    assert dvr_lib.dvr_set_kernel_family(7) == _abi.DVR_E_INVALID_ARGUMENT


def test_python_api_mirrors_reference_names():
    inp = pr.RendererInputs()
    for f in ("screen_size", "volume", "volume_filter_mode", "box_min", "box_size", "camera_mode", "camera",
              "step_size", "tf_mode", "tf", "blend_mode", "blending_early_out"):
        assert hasattr(inp, f), f
    c = inp.clone()
    assert c is not inp and c.camera is inp.camera  # shallow
    a = pr.AdjointOutputs()
    for f in ("has_volume_derivatives", "adj_volume", "has_stepsize_derivatives", "adj_stepsize",
              "has_camera_derivatives", "adj_camera_ray_start", "adj_camera_ray_dir", "has_tf_derivatives",
              "tf_delayed_accumulation", "adj_tf"):
        assert hasattr(a, f), f
    assert pr.TFMode.Gaussian == 3 and pr.BlendMode.Alpha == 1 and pr.CameraMode.ReferenceFrame == 2
    assert pr.VolumeFilterMode.Trilinear == 1
    assert abs(inp.blending_early_out - (1 - 1e-5)) < 1e-12


def test_forward_mode_interface():
    """The forward method's names (bindings/bindings.cpp:423-436, :455, :496;
    pytests/diffdvr/renderer.py:271-311)."""
    from diffdvr_gb300 import Renderer
    s = pr.ForwardDifferencesSettings()
    for f in ("D", "d_stepsize", "d_rayStart", "d_rayDir", "d_tf", "has_tf_derivatives"):
        assert hasattr(s, f), f
    assert s.NOT_ENABLED == -1 and s.d_stepsize == -1 and tuple(s.d_rayStart) == (-1, -1, -1)
    assert callable(pr.Renderer.render_forward_gradients)
    assert callable(pr.Renderer.forward_variables_to_gradients)
    Renderer(optimize_tf=True, gradient_method="forward")
    Renderer(optimize_camera=True, gradient_method="forward", forward_delayed_gradients=True)
    with pytest.raises(AssertionError):
        Renderer(optimize_volume=True, gradient_method="forward")


# ---------------------------------------------------------------- forward mode and pre-shading
def _settings(D=3, step=0, start=(-1, -1, -1), dirs=(-1, -1, -1), d_tf=None, has_tf=None):
    s = _abi.DvrForwardDifferencesSettings()
    s.D, s.d_stepsize = D, step
    for k in range(3):
        s.d_ray_start[k], s.d_ray_dir[k] = start[k], dirs[k]
    if d_tf is None:
        s.d_tf = _fake(())
        s.d_tf.ndim = -1
    else:
        s.d_tf = d_tf
    s.has_tf_derivatives = int(d_tf is not None if has_tf is None else has_tf)
    return s


def _no_gpu():
    """Descriptors that pass every check reach the launch; their pointers are
    fake, so such cases run only where there is no GPU to launch on."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("fake device pointers: validation pass-through is checked without a GPU only")


def _preshaded_inputs():
    i = _inputs()
    i.volume_filter_mode, i.tf_mode = 3, 5
    i.volume = _fake((4, 4, 5, 6))
    i.tf = _fake((1, 1, 1))
    return i


# renderer/renderer.cpp:419-498
@pytest.mark.parametrize("make,expect", [
    (lambda: (_inputs(), _settings(D=0), _fake((1, 7, 8, 1, 4))), "number of derivatives must be positive"),
    (lambda: (_inputs(), _settings(step=-1), _fake((1, 7, 8, 3, 4))), "at least one derivative must be activated"),
    (lambda: (_inputs(), _settings(step=5), _fake((1, 7, 8, 3, 4))), "d_stepsize = 5 is not a derivative index"),
    (lambda: (_inputs(), _settings(start=(0, 1, 7)), _fake((1, 7, 8, 3, 4))), "d_rayStart = 7"),
    (lambda: (_inputs(), _settings(has_tf=True), _fake((1, 7, 8, 3, 4))), "d_tf not defined"),
    (lambda: (_inputs(), _settings(d_tf=_fake((1, 8, 4))), _fake((1, 7, 8, 3, 4))), "d_tf must be of type int32"),
    (lambda: (_inputs(), _settings(d_tf=_fake((1, 2, 4), _abi.DVR_INT32)), _fake((1, 7, 8, 3, 4))),
     "d_tf must have 8 entries at dimension 1"),
    (lambda: (_inputs(), _settings(), _fake((1, 7, 8, 2, 4))), "gradientsOut must have 3 entries at dimension 3"),
    (lambda: (_inputs(), _settings(), _fake((1, 7, 8, 3, 4), _abi.DVR_FLOAT64)), "gradientsOut must be of type float32"),
    (lambda: (_preshaded_inputs(), _settings(), _fake((1, 7, 8, 3, 4))),
     "forward derivatives are not available for pre-shaded volumes"),
    (lambda: (_inputs(), _settings(d_tf=_fake((1, 8, 4), _abi.DVR_INT32)), _fake((1, 7, 8, 3, 4))), None),
])
def test_forward_gradients_validation(dvr_lib, make, expect):
    if expect is None:
        _no_gpu()
    i, s, g = make()
    o = _outputs()
    code = dvr_lib.dvr_render_forward_gradients(ctypes.byref(i), ctypes.byref(s), ctypes.byref(o), ctypes.byref(g),
                                                None)
    msg = dvr_lib.dvr_last_error().decode()
    if expect is None:
        assert code == _abi.DVR_E_CUDA, msg  # every check passed; no GPU here
    else:
        assert code in (_abi.DVR_E_INVALID_ARGUMENT, _abi.DVR_E_UNSUPPORTED)
        assert expect in msg, msg


def _adj_outputs(**kw):
    a = _abi.DvrAdjointOutputs()
    for name in ("adj_volume", "adj_stepsize", "adj_camera_ray_start", "adj_camera_ray_dir", "adj_tf", "adj_viewport"):
        t = _fake(())
        t.ndim = -1
        setattr(a, name, t)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


# renderer/renderer.cpp:500-558
@pytest.mark.parametrize("make,expect", [
    (lambda: (_fake((1, 7, 8, 3, 4), cuda=False), _fake((1, 7, 8, 4)), _settings(), _adj_outputs()), "is a CPU tensor"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 6, 8, 4)), _settings(), _adj_outputs()),
     "gradientOutputColor must have 7 entries at dimension 1"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 7, 8, 4)), _settings(),
              _adj_outputs(has_volume_derivatives=1, adj_volume=_fake((1, 4, 5, 6)))),
     "volume derivatives are not supported with forward variables"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 7, 8, 4)), _settings(dirs=(9, -1, -1)), _adj_outputs()),
     "d_rayDir = 9 is not a derivative index"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 7, 8, 4)), _settings(),
              _adj_outputs(has_tf_derivatives=1, adj_tf=_fake((1, 8, 4)))),
     "TF derivatives need the TF derivative indices"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 7, 8, 4)), _settings(d_tf=_fake((1, 8, 4), _abi.DVR_INT32)),
              _adj_outputs(has_tf_derivatives=1, adj_tf=_fake((1, 8, 5)))), "adj_tf must have 4 entries at dimension 2"),
    (lambda: (_fake((1, 7, 8, 3, 4)), _fake((1, 7, 8, 4)), _settings(),
              _adj_outputs(has_stepsize_derivatives=1, adj_stepsize=_fake((1, 7, 8)))), None),
])
def test_forward_variables_to_gradients_validation(dvr_lib, make, expect):
    if expect is None:
        _no_gpu()
    fv, ac, s, a = make()
    code = dvr_lib.dvr_forward_variables_to_gradients(ctypes.byref(fv), ctypes.byref(ac), ctypes.byref(s),
                                                      ctypes.byref(a), None)
    msg = dvr_lib.dvr_last_error().decode()
    if expect is None:
        assert code == _abi.DVR_E_CUDA, msg
    else:
        assert code == _abi.DVR_E_INVALID_ARGUMENT and expect in msg, msg


# renderer/tf_utils.cpp:173-249
@pytest.mark.parametrize("make,expect", [
    (lambda: (_fake((2, 4, 5, 6)), _fake((1, 8, 4)), 1, _fake((4, 4, 5, 6))),
     "densityVolume must have 1 entries at dimension 0"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((2, 8, 4)), 1, _fake((4, 4, 5, 6))), "tf must have 1 entries at dimension 0"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((1, 8, 5)), 1, _fake((4, 4, 5, 6))), "tf must have 4 entries at dimension 2"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((1, 8, 6)), 6, _fake((4, 4, 5, 6))), "TFGaussianLog is not supported"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((1, 8, 4)), 1, _fake((3, 4, 5, 6))), "color must have 4 entries at dimension 0"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((1, 8, 4)), 1, _fake((4, 4, 5, 7))), "color must have 6 entries at dimension 3"),
    (lambda: (_fake((1, 4, 5, 6)), _fake((1, 8, 4)), 1, _fake((4, 4, 5, 6))), None),
])
def test_preshade_volume_validation(dvr_lib, make, expect):
    if expect is None:
        _no_gpu()
    d, tf, mode, out = make()
    code = dvr_lib.dvr_preshade_volume(ctypes.byref(d), ctypes.byref(tf), mode, ctypes.byref(out), None)
    msg = dvr_lib.dvr_last_error().decode()
    if expect is None:
        assert code == _abi.DVR_E_CUDA, msg
    else:
        assert code in (_abi.DVR_E_INVALID_ARGUMENT, _abi.DVR_E_UNSUPPORTED) and expect in msg, msg


def test_preshade_volume_adjoint_validation(dvr_lib):
    d, tf = _fake((1, 4, 5, 6)), _fake((1, 8, 4))
    code = dvr_lib.dvr_preshade_volume_adjoint(ctypes.byref(d), ctypes.byref(tf), 1, ctypes.byref(_fake((4, 4, 5, 6))),
                                               ctypes.byref(_fake((2, 4, 5, 6))), None)
    msg = dvr_lib.dvr_last_error().decode()
    assert code == _abi.DVR_E_INVALID_ARGUMENT and "adj_density must have 1 entries at dimension 0" in msg


def test_preshaded_inputs_validation(dvr_lib):
    _no_gpu()
    i, o = _preshaded_inputs(), _outputs()
    code, msg = _forward(dvr_lib, i, o)
    assert code == _abi.DVR_E_CUDA, msg  # valid pre-shaded inputs: every check passes
    o.sample_density = _fake((64,))
    o.sample_offset = _fake((1, 7, 8), _abi.DVR_INT32)
    code, msg = _forward(dvr_lib, i, o)
    assert code == _abi.DVR_E_CUDA, msg  # a record without checkpoints is fine for pre-shaded volumes


def test_forward_method_derivative_layout():
    """The forward method's derivative indices: the six ray components first,
    then the TF entries row-major, one index per entry and batch entry
    (pytests/diffdvr/renderer.py:63-80)."""
    import torch
    from diffdvr_gb300.renderer import _forward_settings
    tf = torch.zeros(2, 3, 4)
    s = _forward_settings(True, True, tf)
    assert s.D == 6 + 12
    assert tuple(s.d_rayStart) == (0, 1, 2) and tuple(s.d_rayDir) == (3, 4, 5)
    assert s.has_tf_derivatives and s.d_tf.dtype == torch.int32 and tuple(s.d_tf.shape) == (2, 3, 4)
    assert torch.equal(s.d_tf[0], torch.arange(6, 18, dtype=torch.int32).reshape(3, 4))
    assert torch.equal(s.d_tf[1], s.d_tf[0])
    s = _forward_settings(False, True, tf)
    assert s.D == 12 and tuple(s.d_rayStart) == (-1, -1, -1) and int(s.d_tf.min()) == 0
    s = _forward_settings(True, False, tf)
    assert s.D == 6 and not s.has_tf_derivatives and s.d_tf is None


def test_header_is_plain_c_and_links(dvr_lib, tmp_path):
    """The boundary is plain C: a C99 program includes the header, links the
    library and calls it (version, checkpoint sizing, a validation failure
    with its message) without a GPU."""
    import shutil
    import subprocess
    from diffdvr_gb300 import _abi as abi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    src = tmp_path / "probe.c"
    src.write_text(r"""
#include <stdio.h>
#include <string.h>
#include "diffdvr_gb300.h"
int main(void) {
  if (dvr_abi_version() != DVR_ABI_VERSION) return 1;
  if (dvr_checkpoint_slots(1.7320508, 0.001, 16) <= 0) return 2;
  if (dvr_checkpoint_slots(1.0, -1.0, 16) >= 0) return 3;
  DvrRendererInputs in;
  DvrRendererOutputs out;
  memset(&in, 0, sizeof in);
  memset(&out, 0, sizeof out);
  in.volume.ndim = 3;  /* must be 4 */
  int code = dvr_render_forward(&in, &out, NULL);
  if (code != DVR_E_INVALID_ARGUMENT) return 4;
  if (strstr(dvr_last_error(), "volume must be a tensor with 4 dimensions") == NULL) return 5;
  printf("ok %d\n", dvr_abi_version());
  return 0;
}
""")
    lib_dir = os.path.dirname(abi.library_path())
    exe = tmp_path / "probe"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", lib_dir, "-ldvr_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok 6", (r.returncode, r.stdout, r.stderr)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without libdvr_gb300.so every entry point raises: there is no CPU
    fallback, in the direct binding or the autograd module."""
    from diffdvr_gb300 import _abi as abi, pyrenderer as pr
    monkeypatch.setattr(abi, "_LIB", None)
    monkeypatch.setattr(abi, "library_path", lambda: str(tmp_path / "libdvr_gb300.so"))
    with pytest.raises(RuntimeError, match="CUDA library not found"):
        pr.Renderer.render_forward(pr.RendererInputs(), pr.RendererOutputs(None, None))
    with pytest.raises(RuntimeError, match="CUDA library not found"):
        pr.set_kernel_family("plain")
    with pytest.raises(RuntimeError, match="CUDA library not found"):
        abi.load()


def _batched_forward(lib, ins, outs, n=None):
    ci = (_abi.DvrRendererInputs * max(len(ins), 1))(*ins)
    co = (_abi.DvrRendererOutputs * max(len(outs), 1))(*outs)
    code = lib.dvr_render_forward_batched(ci, co, len(ins) if n is None else n, None)
    return code, lib.dvr_last_error().decode()


def _with(obj, **kw):
    for k, v in kw.items():
        setattr(obj, k, v)
    return obj


# batched calls: each instance is checked as a single call, and all must share
# their modes, storage types and device (diffdvr_gb300/csrc/dvr_host.cpp)
@pytest.mark.parametrize("make,expect", [
    (lambda: ([_inputs()], [_outputs()], -1), "invalid instance list"),
    (lambda: ([_inputs(), _inputs(tf_mode=3)], [_outputs(), _outputs()], None),
     "must share filter, TF and blend modes, storage types and device"),
    (lambda: ([_inputs(), _with(_inputs(), blend_mode=1)], [_outputs(), _outputs()], None),
     "must share filter, TF and blend modes"),
    (lambda: ([_inputs(), _with(_inputs(), volume=_fake((1, 4, 5, 6), _abi.DVR_BFLOAT16))],
              [_outputs(), _outputs()], None), "storage types"),
    (lambda: ([_preshaded_inputs()], [_outputs()], None), "pre-shaded volumes are rendered by the single-instance"),
    (lambda: ([_inputs(), _inputs(W=9)], [_outputs(), _outputs()], None), "must have 9 entries at dimension 2"),
    (lambda: ([_inputs(X=9, Y=3, Z=17), _inputs(W=16, H=4)], [_outputs(), _outputs(W=16, H=4)], None), None),
])
def test_batched_forward_validation(dvr_lib, make, expect):
    if expect is None:
        _no_gpu()
    ins, outs, n = make()
    code, msg = _batched_forward(dvr_lib, ins, outs, n)
    if expect is None:
        assert code == _abi.DVR_E_CUDA, msg  # instances of different sizes pass every check; no GPU here
    else:
        assert code in (_abi.DVR_E_INVALID_ARGUMENT, _abi.DVR_E_UNSUPPORTED)
        assert expect in msg, msg


def test_batched_calls_without_instances_do_nothing(dvr_lib):
    assert dvr_lib.dvr_render_forward_batched(None, None, 0, None) == _abi.DVR_OK
    assert dvr_lib.dvr_render_adjoint_batched(None, None, None, None, 0, None) == _abi.DVR_OK


def _batched_adjoint(lib, ins, outs, adjs, grads):
    n = len(ins)
    code = lib.dvr_render_adjoint_batched((_abi.DvrRendererInputs * n)(*ins), (_abi.DvrRendererOutputs * n)(*outs),
                                          (_abi.DvrTensor * n)(*adjs), (_abi.DvrAdjointOutputs * n)(*grads), n, None)
    return code, lib.dvr_last_error().decode()


def _tf_grad(B=1, R=8):
    return _adj_outputs(has_tf_derivatives=1, adj_tf=_fake((B, R, 4)))


@pytest.mark.parametrize("make,expect", [
    (lambda: ([_inputs(), _inputs()], [_outputs(), _outputs()],
              [_tf_grad(), _adj_outputs(has_volume_derivatives=1, adj_volume=_fake((1, 4, 5, 6)))]),
     "must share modes, storage types, device and gradient selection"),
    (lambda: ([_inputs(), _inputs()], [_outputs(), _outputs()],
              [_tf_grad(), _with(_tf_grad(), has_volume_derivatives=1, adj_volume=_fake((1, 4, 5, 6)))]),
     "gradient selection"),
    (lambda: ([_with(_inputs(), camera_mode=2, camera_kind=_abi.DVR_CAMERA_REFERENCE_FRAME_KIND,
                     camera_matrix=_fake((1, 3, 3)), camera_fov_y_radians=0.7)], [_outputs()],
              [_adj_outputs(has_viewport_derivatives=1, adj_viewport=_fake((1, 3, 3)))]),
     "do not compute viewport derivatives"),
    (lambda: ([_inputs(), _inputs(W=16, H=4)], [_outputs(), _outputs(W=16, H=4)], [_tf_grad(), _tf_grad()]), None),
])
def test_batched_adjoint_validation(dvr_lib, make, expect):
    if expect is None:
        _no_gpu()
    ins, outs, grads = make()
    adjs = [_fake((1, o.color.sizes[1], o.color.sizes[2], 4)) for o in outs]
    code, msg = _batched_adjoint(dvr_lib, ins, outs, adjs, grads)
    if expect is None:
        assert code == _abi.DVR_E_CUDA, msg
    else:
        assert code in (_abi.DVR_E_INVALID_ARGUMENT, _abi.DVR_E_UNSUPPORTED)
        assert expect in msg, msg


@pytest.mark.parametrize("make,expect", [
    (lambda: (_preshaded_inputs(), _tf_grad(1, 1)), "pre-shaded volumes take dvr_render_adjoint"),
    (lambda: (_inputs(), _adj_outputs()), None),  # no gradient requested
    (lambda: (_inputs(), _tf_grad()), "pass"),
])
def test_noalloc_adjoint_validation(dvr_lib, make, expect):
    """dvr_render_adjoint_noalloc checks its arguments as dvr_render_adjoint
    does, and rejects pre-shaded volumes, before any CUDA call."""
    if expect == "pass":
        _no_gpu()
    i, g = make()
    o = _outputs()
    code = dvr_lib.dvr_render_adjoint_noalloc(ctypes.byref(i), ctypes.byref(o), ctypes.byref(_fake((1, 7, 8, 4))),
                                              ctypes.byref(g), None)
    msg = dvr_lib.dvr_last_error().decode()
    if expect == "pass":
        assert code == _abi.DVR_E_CUDA, msg  # every check passed; no GPU here
    elif expect is None:
        assert code == _abi.DVR_E_NO_GRADIENT, msg
    else:
        assert code == _abi.DVR_E_UNSUPPORTED and expect in msg, msg


def test_python_mirror_descriptors():
    """pyrenderer turns the reference's settings variants into the C ABI's
    tagged descriptors (renderer/renderer.h:20-71): value or tensor boxes and
    step sizes, the four camera types, element strides as the tensors have
    them (non-contiguous views included), dtype codes, no pointer for an
    empty tensor."""
    import torch
    inp = pr.RendererInputs()
    inp.screen_size = pr.int2(6, 5)
    inp.volume = torch.zeros(1, 4, 5, 6, dtype=torch.bfloat16)
    inp.box_min = pr.real3(-0.5, -0.25, -0.125)
    rays = torch.zeros(2, 6, 5, 3).transpose(1, 2)  # B H W 3 with non-contiguous strides
    inp.camera = pr.CameraPerPixelRays(rays, rays)
    inp.step_size = 0.01
    inp.tf = torch.zeros(1, 8, 4)
    c = pr._inputs(inp)
    assert (c.screen_width, c.screen_height) == (6, 5)
    assert c.volume.dtype == _abi.DVR_BFLOAT16 and tuple(c.volume.sizes[:4]) == (1, 4, 5, 6)
    assert c.box_min_kind == _abi.DVR_KIND_VALUE and tuple(c.box_min_value) == (-0.5, -0.25, -0.125)
    assert c.box_min.ndim == -1 and c.box_size_kind == _abi.DVR_KIND_VALUE
    assert c.camera_kind == _abi.DVR_CAMERA_PER_PIXEL_RAYS and c.camera_matrix.ndim == -1
    assert tuple(c.camera_ray_start.sizes[:4]) == (2, 5, 6, 3)
    assert tuple(c.camera_ray_start.strides[:4]) == tuple(rays.stride())
    assert c.camera_ray_start.device_type == _abi.DVR_DEVICE_CPU and c.camera_ray_start.device_index == -1
    assert c.step_size_kind == _abi.DVR_KIND_VALUE and c.step_size_value == pytest.approx(0.01)

    inp.box_min = torch.zeros(1, 3)
    inp.box_size = torch.ones(2, 3)
    inp.step_size = torch.full((1, 5, 6), 0.02)
    inp.camera = pr.CameraReferenceFrame(torch.zeros(2, 3, 3), 0.7)
    c = pr._inputs(inp)
    assert c.box_min_kind == c.box_size_kind == c.step_size_kind == _abi.DVR_KIND_TENSOR
    assert tuple(c.box_size.sizes[:2]) == (2, 3) and tuple(c.step_size.sizes[:3]) == (1, 5, 6)
    assert c.camera_kind == _abi.DVR_CAMERA_REFERENCE_FRAME_KIND and c.camera_fov_y_radians == pytest.approx(0.7)
    assert tuple(c.camera_matrix.sizes[:3]) == (2, 3, 3) and c.camera_ray_start.ndim == -1

    m = np.arange(16, dtype=np.float32).reshape(4, 4)
    inp.camera = pr.mat4(m)
    c = pr._inputs(inp)
    assert c.camera_kind == _abi.DVR_CAMERA_INVERSE_VIEW_VALUE and list(c.camera_matrix_value) == list(range(16))
    inp.camera = torch.zeros(1, 4, 4)
    c = pr._inputs(inp)
    assert c.camera_kind == _abi.DVR_CAMERA_INVERSE_VIEW_TENSOR and tuple(c.camera_matrix.sizes[:3]) == (1, 4, 4)
    inp.camera = "eye"
    with pytest.raises(RuntimeError, match="unknown camera type"):
        pr._inputs(inp)

    out = pr.RendererOutputs(torch.zeros(2, 0, 6, 4), torch.zeros(2, 0, 6, dtype=torch.int32))
    o = pr._outputs(out)
    assert o.color.data is None and o.color.ndim == 4  # an empty tensor passes no pointer
    assert o.termination_index.dtype == _abi.DVR_INT32 and o.checkpoints.ndim == -1 and o.sample_density.ndim == -1
    assert pr._tensor(torch.zeros(3, dtype=torch.int64)).dtype not in (_abi.DVR_FLOAT32, _abi.DVR_INT32)


def test_autograd_module_argument_checks():
    """diffdvr_gb300.Renderer checks its arguments as the reference's module
    does (pytests/diffdvr/renderer.py:264-335): assertion errors for an
    unknown gradient method, a volume optimised by the forward method, or a
    missing input of an optimised quantity; a ValueError for training
    without parameters."""
    import torch
    from diffdvr_gb300 import Renderer
    with pytest.raises(AssertionError):
        Renderer(gradient_method="backward")
    with pytest.raises(AssertionError, match="gradient method must be 'adjoint'"):
        Renderer(optimize_volume=True, gradient_method="forward")
    r = Renderer(optimize_tf=True)
    with pytest.raises(AssertionError):
        r(tf=None, volume=torch.zeros(1, 2, 2, 2))
    with pytest.raises(ValueError, match="no parameters were specified"):
        Renderer().train()
    with pytest.raises(AssertionError):
        r.settings = None
    assert Renderer(optimize_camera=True).train() is not None
