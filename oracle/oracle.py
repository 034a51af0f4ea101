"""Oracle wrapper — TEST INFRASTRUCTURE ONLY.

ctypes front end for the CPU ray-marcher oracle libraries declared in
``oracle/dvr_oracle.h``:

* ``kind="port"``: our plain-C restatement (``oracle/_build/libdvr_oracle_*.so``),
  built on any machine by ``build()`` below;
* ``kind="reference"``: the reference's own CPU templates
  (``oracle/_ref/libdvr_ref_*.so``), built only where the reference sources are
  present.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module; the ``diffdvr_gb300`` package never imports it.

Inputs are numpy arrays in the reference layout (renderer/renderer_settings.cuh:8-45):
volume (B)XYZ, box_min/box_size (B)3, ray_start/ray_dir (B)HW3, camera_matrix
(B)44 or (B)33, step_size (B)(H)(W), tf (B)RC.  Size-1 leading dimensions
broadcast, as in the reference.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: DIFFDVR_REFERENCE, else its path in the build container
REFERENCE_ROOT = os.environ.get("DIFFDVR_REFERENCE", "/root/reference")
REFERENCE_SOURCES = os.path.join(REFERENCE_ROOT, "renderer")


class OracleTensor(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("ndim", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("sizes", ctypes.c_int64 * 5),
        ("strides", ctypes.c_int64 * 5),
    ]


class OracleInputs(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32), ("height", ctypes.c_int32),
        ("filter_mode", ctypes.c_int32), ("camera_mode", ctypes.c_int32),
        ("tf_mode", ctypes.c_int32), ("blend_mode", ctypes.c_int32),
        ("volume", OracleTensor), ("box_min", OracleTensor), ("box_size", OracleTensor),
        ("ray_start", OracleTensor), ("ray_dir", OracleTensor), ("camera_matrix", OracleTensor),
        ("fov_y_radians", ctypes.c_double), ("step_size", OracleTensor), ("tf", OracleTensor),
        ("blending_early_out", ctypes.c_double), ("batch", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


class OracleAdjointOutputs(ctypes.Structure):
    _fields_ = [
        ("has_volume", ctypes.c_int32), ("has_stepsize", ctypes.c_int32),
        ("has_camera", ctypes.c_int32), ("has_tf", ctypes.c_int32),
        ("stepsize_broadcast", ctypes.c_int32), ("camera_broadcast", ctypes.c_int32),
        ("adj_volume", OracleTensor), ("adj_stepsize", OracleTensor),
        ("adj_ray_start", OracleTensor), ("adj_ray_dir", OracleTensor), ("adj_tf", OracleTensor),
    ]


class OracleForwardSettings(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int32), ("d_stepsize", ctypes.c_int32),
        ("d_ray_start", ctypes.c_int32 * 3), ("d_ray_dir", ctypes.c_int32 * 3),
        ("has_tf", ctypes.c_int32), ("pad_", ctypes.c_int32),
        ("d_tf", OracleTensor),
    ]


def build(reference: bool = True, quiet: bool = True) -> None:
    """Builds the port libraries (and the reference harness when its sources exist)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "-j2", "all"], check=True, stdout=out)
    if reference and os.path.isdir(REFERENCE_SOURCES):
        subprocess.run(["make", "-C", HERE, "-j3", "ref", f"REF_DIR={REFERENCE_SOURCES}"],
                       check=True, stdout=out)


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libdvr_ref_f32.so"))


_LIBS: dict = {}


def load(kind: str = "port", precision: str = "f64") -> ctypes.CDLL:
    key = (kind, precision)
    if key not in _LIBS:
        if kind == "port":
            path = os.path.join(BUILD_DIR, f"libdvr_oracle_{precision}.so")
        elif kind == "reference":
            path = os.path.join(REF_DIR, f"libdvr_ref_{precision}.so")
        else:
            raise ValueError(kind)
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built (run oracle.oracle.build())")
        lib = ctypes.CDLL(path)
        lib.oracle_forward.argtypes = [ctypes.POINTER(OracleInputs), ctypes.POINTER(OracleTensor),
                                       ctypes.POINTER(OracleTensor)]
        lib.oracle_adjoint.argtypes = [ctypes.POINTER(OracleInputs), ctypes.POINTER(OracleTensor),
                                       ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleTensor),
                                       ctypes.POINTER(OracleAdjointOutputs)]
        lib.oracle_forward.restype = ctypes.c_int
        lib.oracle_adjoint.restype = ctypes.c_int
        lib.oracle_real_size.restype = ctypes.c_int
        if hasattr(lib, "oracle_preshade_volume"):
            lib.oracle_preshade_volume.argtypes = [ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleTensor),
                                                   ctypes.c_int, ctypes.POINTER(OracleTensor)]
            lib.oracle_preshade_volume.restype = ctypes.c_int
            lib.oracle_preshade_volume_adjoint.argtypes = [ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleTensor),
                                                           ctypes.c_int, ctypes.POINTER(OracleTensor),
                                                           ctypes.POINTER(OracleTensor)]
            lib.oracle_preshade_volume_adjoint.restype = ctypes.c_int
        if hasattr(lib, "oracle_set_exact_preshaded"):
            lib.oracle_set_exact_preshaded.argtypes = [ctypes.c_int]
            lib.oracle_set_exact_preshaded.restype = None
        if hasattr(lib, "oracle_forward_gradients"):  # the port only: the reference's needs cudAD
            lib.oracle_forward_gradients.argtypes = [
                ctypes.POINTER(OracleInputs), ctypes.POINTER(OracleForwardSettings), ctypes.POINTER(OracleTensor),
                ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleTensor)]
            lib.oracle_forward_gradients.restype = ctypes.c_int
            lib.oracle_forward_variables_to_gradients.argtypes = [
                ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleTensor), ctypes.POINTER(OracleForwardSettings),
                ctypes.POINTER(OracleAdjointOutputs)]
            lib.oracle_forward_variables_to_gradients.restype = ctypes.c_int
        _LIBS[key] = lib
    return _LIBS[key]


def _tensor(arr: Optional[np.ndarray], keep: list) -> OracleTensor:
    t = OracleTensor()
    if arr is None:
        t.data = None
        t.ndim = 0
        return t
    arr = np.ascontiguousarray(arr)
    keep.append(arr)
    t.data = arr.ctypes.data
    t.ndim = arr.ndim
    for d in range(arr.ndim):
        t.sizes[d] = arr.shape[d]
        t.strides[d] = arr.strides[d] // arr.itemsize
    return t


@dataclass
class Scene:
    """Renderer inputs in the reference layout (numpy, any float dtype)."""
    width: int
    height: int
    volume: np.ndarray
    tf: np.ndarray
    step_size: np.ndarray            # (B)(H)(W)
    box_min: np.ndarray              # (B)3
    box_size: np.ndarray             # (B)3
    filter_mode: int = 1
    camera_mode: int = 0
    tf_mode: int = 1
    blend_mode: int = 0
    ray_start: Optional[np.ndarray] = None
    ray_dir: Optional[np.ndarray] = None
    camera_matrix: Optional[np.ndarray] = None
    fov_y_radians: float = 0.0
    blending_early_out: float = 1.0 - 1e-5

    def batch(self) -> int:
        # a pre-shaded volume (filter 3) holds its 4 channels in the first dimension
        arrs = [self.tf, self.step_size, self.box_min, self.box_size]
        if self.filter_mode != 3:
            arrs.append(self.volume)
        if self.camera_mode == 0:
            arrs += [self.ray_start, self.ray_dir]
        else:
            arrs += [self.camera_matrix]
        return max(int(a.shape[0]) for a in arrs)


def _inputs(scene: Scene, dtype, keep: list) -> OracleInputs:
    cast = lambda a: None if a is None else np.asarray(a, dtype=dtype)
    i = OracleInputs()
    i.width, i.height = scene.width, scene.height
    i.filter_mode, i.camera_mode = scene.filter_mode, scene.camera_mode
    i.tf_mode, i.blend_mode = scene.tf_mode, scene.blend_mode
    i.volume = _tensor(cast(scene.volume), keep)
    i.box_min = _tensor(cast(scene.box_min), keep)
    i.box_size = _tensor(cast(scene.box_size), keep)
    empty4 = np.zeros((1, 1, 1, 3), dtype=dtype)
    i.ray_start = _tensor(cast(scene.ray_start) if scene.ray_start is not None else empty4, keep)
    i.ray_dir = _tensor(cast(scene.ray_dir) if scene.ray_dir is not None else empty4, keep)
    empty3 = np.zeros((1, 4, 4), dtype=dtype)
    i.camera_matrix = _tensor(cast(scene.camera_matrix) if scene.camera_matrix is not None else empty3, keep)
    i.fov_y_radians = float(scene.fov_y_radians)
    i.step_size = _tensor(cast(scene.step_size), keep)
    i.tf = _tensor(cast(scene.tf), keep)
    i.blending_early_out = float(scene.blending_early_out)
    i.batch = scene.batch()
    return i


def _dtype(lib) -> type:
    return np.float64 if lib.oracle_real_size() == 8 else np.float32


def set_threads(n: int) -> int:
    """Threads of the oracle's (and the reference templates') parallel loops
    from now on; returns the previous number.  One thread makes the adjoint's
    atomic sums deterministic."""
    lib = load("port", "f64")
    lib.oracle_set_threads.argtypes = [ctypes.c_int]
    lib.oracle_set_threads.restype = ctypes.c_int
    return int(lib.oracle_set_threads(int(n)))


def forward(scene: Scene, kind: str = "port", precision: str = "f64"):
    """Returns (color B*H*W*4, termination_index B*H*W int32)."""
    lib = load(kind, precision)
    dt = _dtype(lib)
    keep: list = []
    inp = _inputs(scene, dt, keep)
    B = inp.batch
    color = np.zeros((B, scene.height, scene.width, 4), dtype=dt)
    term = np.zeros((B, scene.height, scene.width), dtype=np.int32)
    tc, tt = _tensor(color, keep), _tensor(term, keep)
    rc = lib.oracle_forward(ctypes.byref(inp), ctypes.byref(tc), ctypes.byref(tt))
    if rc != 0:
        raise RuntimeError(f"oracle_forward failed with code {rc}")
    return color, term


@dataclass
class AdjointRequest:
    volume: bool = False
    tf: bool = False
    camera: bool = False
    stepsize: bool = False
    # shapes of the gradient outputs (broadcast dims allowed); None = full shape
    stepsize_shape: Optional[tuple] = None
    camera_batch: Optional[int] = None
    volume_batch: Optional[int] = None
    tf_batch: Optional[int] = None
    results: dict = field(default_factory=dict)


def adjoint(scene: Scene, color: np.ndarray, term: np.ndarray, adj_color: np.ndarray,
            req: AdjointRequest, kind: str = "port", precision: str = "f64",
            exact_preshaded: bool = False) -> dict:
    """Runs the adjoint march; returns a dict of gradient arrays (zero-initialised).
    exact_preshaded (port only): the exact position derivative of pre-shaded
    volumes instead of the reference's."""
    lib = load(kind, precision)
    if kind == "port":
        lib.oracle_set_exact_preshaded(int(exact_preshaded))
    dt = _dtype(lib)
    keep: list = []
    inp = _inputs(scene, dt, keep)
    out, res = _adjoint_outputs(scene, req, inp.batch, dt, keep)
    tc =_tensor(np.asarray(color, dtype=dt), keep)
    tt = _tensor(np.asarray(term, dtype=np.int32), keep)
    ta = _tensor(np.asarray(adj_color, dtype=dt), keep)
    rc = lib.oracle_adjoint(ctypes.byref(inp), ctypes.byref(tc), ctypes.byref(tt), ctypes.byref(ta),
                            ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle_adjoint failed with code {rc}")
    return res


def _adjoint_outputs(scene: Scene, req: AdjointRequest, B: int, dt, keep: list):
    """Zeroed gradient arrays for the request and the OracleAdjointOutputs over them."""
    H, W = scene.height, scene.width
    out = OracleAdjointOutputs()
    res = {}
    if req.volume:
        vb = req.volume_batch or int(scene.volume.shape[0])
        res["adj_volume"] = np.zeros((vb,) + tuple(scene.volume.shape[1:]), dtype=dt)
        out.has_volume = 1
        out.adj_volume = _tensor(res["adj_volume"], keep)
    if req.tf:
        tb = req.tf_batch or int(scene.tf.shape[0])
        res["adj_tf"] = np.zeros((tb,) + tuple(scene.tf.shape[1:]), dtype=dt)
        out.has_tf = 1
        out.adj_tf = _tensor(res["adj_tf"], keep)
    if req.camera:
        cb = req.camera_batch or B
        res["adj_ray_start"] = np.zeros((cb, H, W, 3), dtype=dt)
        res["adj_ray_dir"] = np.zeros((cb, H, W, 3), dtype=dt)
        out.has_camera = 1
        out.camera_broadcast = int(cb != B)
        out.adj_ray_start = _tensor(res["adj_ray_start"], keep)
        out.adj_ray_dir = _tensor(res["adj_ray_dir"], keep)
    if req.stepsize:
        shp = req.stepsize_shape or (B, H, W)
        res["adj_stepsize"] = np.zeros(shp, dtype=dt)
        out.has_stepsize = 1
        out.stepsize_broadcast = int(tuple(shp) != (B, H, W))
        out.adj_stepsize = _tensor(res["adj_stepsize"], keep)
    return out, res


def reference_image_check(scene: Scene, req: AdjointRequest, precision: str = "f32") -> int:
    """0 when the parameter-block images of oracle/ref_image.h (which the GPU
    harness oracle/ref_device.cu builds) equal what the reference's own
    accessor constructors make of the same inputs and gradient outputs, else
    the number of the failing check (oracle_ref_image_check)."""
    lib = load("reference", precision)
    lib.oracle_ref_image_check.argtypes = [ctypes.POINTER(OracleInputs), ctypes.POINTER(OracleAdjointOutputs)]
    lib.oracle_ref_image_check.restype = ctypes.c_int
    dt = _dtype(lib)
    keep: list = []
    inp = _inputs(scene, dt, keep)
    out, _ = _adjoint_outputs(scene, req, inp.batch, dt, keep)
    return int(lib.oracle_ref_image_check(ctypes.byref(inp), ctypes.byref(out)))


@dataclass
class ForwardSettings:
    """Forward-mode derivative indices (-1 = not traced); d_tf is an int array
    of the TF's shape ((B) R C) or None."""
    D: int
    d_stepsize: int = -1
    d_ray_start: tuple = (-1, -1, -1)
    d_ray_dir: tuple = (-1, -1, -1)
    d_tf: Optional[np.ndarray] = None


def _forward_settings(fs: ForwardSettings, keep: list) -> OracleForwardSettings:
    o = OracleForwardSettings()
    o.D = int(fs.D)
    o.d_stepsize = int(fs.d_stepsize)
    for c in range(3):
        o.d_ray_start[c] = int(fs.d_ray_start[c])
        o.d_ray_dir[c] = int(fs.d_ray_dir[c])
    o.has_tf = int(fs.d_tf is not None)
    o.d_tf = _tensor(None if fs.d_tf is None else np.asarray(fs.d_tf, dtype=np.int32), keep)
    return o


def forward_gradients(scene: Scene, fs: ForwardSettings, precision: str = "f64"):
    """Forward march with forward-mode derivatives; returns (color B*H*W*4,
    termination B*H*W, gradients B*H*W*D*4)."""
    lib = load("port", precision)
    dt = _dtype(lib)
    keep: list = []
    inp = _inputs(scene, dt, keep)
    B, H, W = inp.batch, scene.height, scene.width
    color = np.zeros((B, H, W, 4), dtype=dt)
    term = np.zeros((B, H, W), dtype=np.int32)
    grads = np.zeros((B, H, W, fs.D, 4), dtype=dt)
    tc, tt, tg = _tensor(color, keep), _tensor(term, keep), _tensor(grads, keep)
    ofs = _forward_settings(fs, keep)
    rc = lib.oracle_forward_gradients(ctypes.byref(inp), ctypes.byref(ofs), ctypes.byref(tc), ctypes.byref(tt),
                                      ctypes.byref(tg))
    if rc != 0:
        raise RuntimeError(f"oracle_forward_gradients failed with code {rc}")
    return color, term, grads


def forward_variables_to_gradients(forward_variables: np.ndarray, adj_color: np.ndarray, fs: ForwardSettings,
                                   req: AdjointRequest, tf_shape: Optional[tuple] = None,
                                   precision: str = "f64") -> dict:
    """Contracts forward variables with adj_color into the requested
    stepsize / camera / TF gradients (zero-initialised)."""
    lib = load("port", precision)
    dt = _dtype(lib)
    keep: list = []
    fv = np.asarray(forward_variables, dtype=dt)
    B, H, W = fv.shape[:3]
    out = OracleAdjointOutputs()
    res = {}
    if req.tf:
        shp = tf_shape if tf_shape is not None else fs.d_tf.shape
        res["adj_tf"] = np.zeros(shp, dtype=dt)
        out.has_tf = 1
        out.adj_tf = _tensor(res["adj_tf"], keep)
    if req.camera:
        cb = req.camera_batch or B
        res["adj_ray_start"] = np.zeros((cb, H, W, 3), dtype=dt)
        res["adj_ray_dir"] = np.zeros((cb, H, W, 3), dtype=dt)
        out.has_camera = 1
        out.camera_broadcast = int(cb != B)
        out.adj_ray_start = _tensor(res["adj_ray_start"], keep)
        out.adj_ray_dir = _tensor(res["adj_ray_dir"], keep)
    if req.stepsize:
        shp = req.stepsize_shape or (B, H, W)
        res["adj_stepsize"] = np.zeros(shp, dtype=dt)
        out.has_stepsize = 1
        out.stepsize_broadcast = int(tuple(shp) != (B, H, W))
        out.adj_stepsize = _tensor(res["adj_stepsize"], keep)
    ofs = _forward_settings(fs, keep)
    tf_ = _tensor(fv, keep)
    ta = _tensor(np.asarray(adj_color, dtype=dt), keep)
    rc = lib.oracle_forward_variables_to_gradients(ctypes.byref(tf_), ctypes.byref(ta), ctypes.byref(ofs),
                                                   ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle_forward_variables_to_gradients failed with code {rc}")
    return res


def preshade_volume(density: np.ndarray, tf: np.ndarray, tf_mode: int, precision: str = "f64") -> np.ndarray:
    """Colour volume 4*X*Y*Z of a density volume 1*X*Y*Z (TF batch entry 0)."""
    lib = load("port", precision)
    dt = _dtype(lib)
    keep: list = []
    d = np.asarray(density, dtype=dt)
    out = np.zeros((4,) + d.shape[1:], dtype=dt)
    to = _tensor(out, keep)
    rc = lib.oracle_preshade_volume(ctypes.byref(_tensor(d, keep)), ctypes.byref(_tensor(np.asarray(tf, dt), keep)),
                                    int(tf_mode), ctypes.byref(to))
    if rc != 0:
        raise RuntimeError(f"oracle_preshade_volume failed with code {rc}")
    return out


def preshade_volume_adjoint(density: np.ndarray, tf: np.ndarray, tf_mode: int, adj_color: np.ndarray,
                            precision: str = "f64") -> np.ndarray:
    """d loss / d density (1*X*Y*Z) for the colour-volume adjoint adj_color (4*X*Y*Z)."""
    lib = load("port", precision)
    dt = _dtype(lib)
    keep: list = []
    d = np.asarray(density, dtype=dt)
    out = np.zeros(d.shape, dtype=dt)
    to = _tensor(out, keep)
    rc = lib.oracle_preshade_volume_adjoint(ctypes.byref(_tensor(d, keep)),
                                            ctypes.byref(_tensor(np.asarray(tf, dt), keep)), int(tf_mode),
                                            ctypes.byref(_tensor(np.asarray(adj_color, dt), keep)), ctypes.byref(to))
    if rc != 0:
        raise RuntimeError(f"oracle_preshade_volume_adjoint failed with code {rc}")
    return out


# ---------------------------------------------------------------- per-step components
def _component_lib(precision: str):
    """The port library with the per-step component entry points typed for its real_t."""
    lib = load("port", precision)
    if not getattr(lib, "_components_typed", False):
        R = ctypes.c_double if lib.oracle_real_size() == 8 else ctypes.c_float
        P = ctypes.POINTER(R)
        T = ctypes.POINTER(OracleTensor)
        i = ctypes.c_int
        lib.oracle_blend_step.argtypes = [i, P, P, R, P]
        lib.oracle_blend_step_adjoint.argtypes = [i, P, P, R, P, P, P, P, P]
        lib.oracle_tf_step.argtypes = [T, i, R, P]
        lib.oracle_tf_step_adjoint.argtypes = [T, i, R, P, T, P]
        lib.oracle_sample_step.argtypes = [T, i, P, P]
        lib.oracle_sample_step_adjoint.argtypes = [T, i, P, R, P, T]
        lib.oracle_ray_steps.argtypes = [P, P, P, P, R, R, i, P]
        lib.oracle_ray_steps_adjoint.argtypes = [P, P, P, P, R, R, i, P, P, P, P]
        lib.oracle_camera_rays.argtypes = [ctypes.POINTER(OracleInputs), T, T]
        lib._components_typed = True
        lib._real = R
    return lib


def _vec(v, lib, keep: list, n: Optional[int] = None):
    a = np.ascontiguousarray(v if n is None else np.zeros(n), dtype=np.float64 if lib._real is ctypes.c_double
                             else np.float32)
    keep.append(a)
    return a, a.ctypes.data_as(ctypes.POINTER(lib._real))


def _ok(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed with code {rc}")


def blend_step(mode: int, acc, cur, step: float, precision: str = "f64") -> np.ndarray:
    """The accumulator after compositing cur (r, g, b, absorption) over acc."""
    lib, keep = _component_lib(precision), []
    out, po = _vec(None, lib, keep, 4)
    _ok(lib.oracle_blend_step(mode, _vec(acc, lib, keep)[1], _vec(cur, lib, keep)[1], step, po), "blend_step")
    return out


def blend_step_adjoint(mode: int, acc_out, cur, step: float, adj_out, precision: str = "f64"):
    """(acc_in recovered by inverting the blend, adj_acc_in, adj_cur, adj_step)."""
    lib, keep = _component_lib(precision), []
    acc_in, p1 = _vec(None, lib, keep, 4)
    adj_acc, p2 = _vec(None, lib, keep, 4)
    adj_cur, p3 = _vec(None, lib, keep, 4)
    adj_step, p4 = _vec(None, lib, keep, 1)
    _ok(lib.oracle_blend_step_adjoint(mode, _vec(acc_out, lib, keep)[1], _vec(cur, lib, keep)[1], step,
                                      _vec(adj_out, lib, keep)[1], p1, p2, p3, p4), "blend_step_adjoint")
    return acc_in, adj_acc, adj_cur, float(adj_step[0])


def tf_step(tf: np.ndarray, tf_mode: int, density: float, precision: str = "f64") -> np.ndarray:
    """TF (1 R C) evaluated at one density: (r, g, b, absorption)."""
    lib, keep = _component_lib(precision), []
    t = _tensor(_vec(tf, lib, keep)[0], keep)
    out, po = _vec(None, lib, keep, 4)
    _ok(lib.oracle_tf_step(ctypes.byref(t), tf_mode, density, po), "tf_step")
    return out


def tf_step_adjoint(tf: np.ndarray, tf_mode: int, density: float, adj, precision: str = "f64"):
    """(d/d density, TF gradient 1 R C) of adj . tf(density)."""
    lib, keep = _component_lib(precision), []
    t = _tensor(_vec(tf, lib, keep)[0], keep)
    g, _ = _vec(np.zeros_like(tf), lib, keep)
    tg = _tensor(g, keep)
    ad, pd = _vec(None, lib, keep, 1)
    _ok(lib.oracle_tf_step_adjoint(ctypes.byref(t), tf_mode, density, _vec(adj, lib, keep)[1], ctypes.byref(tg), pd),
        "tf_step_adjoint")
    return float(ad[0]), g


def sample_step(volume: np.ndarray, filter_mode: int, pos, precision: str = "f64") -> float:
    """Volume (1 X Y Z) sampled at a position in voxel coordinates."""
    lib, keep = _component_lib(precision), []
    v = _tensor(_vec(volume, lib, keep)[0], keep)
    d, pd = _vec(None, lib, keep, 1)
    _ok(lib.oracle_sample_step(ctypes.byref(v), filter_mode, _vec(pos, lib, keep)[1], pd), "sample_step")
    return float(d[0])


def sample_step_adjoint(volume: np.ndarray, filter_mode: int, pos, adj_density: float, precision: str = "f64"):
    """(d/d position, volume gradient 1 X Y Z) of adj_density * sample(pos)."""
    lib, keep = _component_lib(precision), []
    v = _tensor(_vec(volume, lib, keep)[0], keep)
    g, _ = _vec(np.zeros_like(volume), lib, keep)
    tg = _tensor(g, keep)
    ap, pp = _vec(None, lib, keep, 3)
    _ok(lib.oracle_sample_step_adjoint(ctypes.byref(v), filter_mode, _vec(pos, lib, keep)[1], adj_density, pp,
                                       ctypes.byref(tg)), "sample_step_adjoint")
    return ap, g


def ray_steps(start, direction, box_min, voxel, tmin: float, step: float, n: int, precision: str = "f64"):
    """The n sample positions of one ray in voxel coordinates (n x 3)."""
    lib, keep = _component_lib(precision), []
    pos, pp = _vec(None, lib, keep, 3 * n)
    _ok(lib.oracle_ray_steps(_vec(start, lib, keep)[1], _vec(direction, lib, keep)[1], _vec(box_min, lib, keep)[1],
                             _vec(voxel, lib, keep)[1], tmin, step, n, pp), "ray_steps")
    return pos.reshape(n, 3)


def ray_steps_adjoint(start, direction, box_min, voxel, tmin: float, step: float, adj_pos, precision: str = "f64"):
    """(adj_start, adj_dir, adj_step) of sum(adj_pos * positions)."""
    lib, keep = _component_lib(precision), []
    n = int(np.asarray(adj_pos).shape[0])
    a1, p1 = _vec(None, lib, keep, 3)
    a2, p2 = _vec(None, lib, keep, 3)
    a3, p3 = _vec(None, lib, keep, 1)
    _ok(lib.oracle_ray_steps_adjoint(_vec(start, lib, keep)[1], _vec(direction, lib, keep)[1],
                                     _vec(box_min, lib, keep)[1], _vec(voxel, lib, keep)[1], tmin, step, n,
                                     _vec(np.asarray(adj_pos).reshape(-1), lib, keep)[1], p1, p2, p3),
        "ray_steps_adjoint")
    return a1, a2, float(a3[0])


def camera_rays(scene: Scene, precision: str = "f64"):
    """(ray start, ray direction), each B*H*W*3, as the march computes them
    for the scene's camera mode."""
    lib, keep = _component_lib(precision), []
    dt = np.float64 if lib._real is ctypes.c_double else np.float32
    inp = _inputs(scene, dt, keep)
    B = inp.batch
    start = np.zeros((B, scene.height, scene.width, 3), dtype=dt)
    direction = np.zeros_like(start)
    ts, td = _tensor(start, keep), _tensor(direction, keep)
    _ok(lib.oracle_camera_rays(ctypes.byref(inp), ctypes.byref(ts), ctypes.byref(td)), "camera_rays")
    return start, direction
