"""Shared test cases: one scene description rendered by the oracle (numpy)
and by diffdvr_gb300 (torch CUDA tensors through the C ABI)."""
from __future__ import annotations

import itertools
import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from diffdvr_gb300 import scenes
from diffdvr_gb300.camera import Camera
from oracle import oracle as O

TF_MODES = (0, 1, 2, 3)
FILTERS = (0, 1)
BLENDS = (0, 1)
CAMERAS = (0, 1, 2)


def symmetric_error(a, b) -> float:
    """max |a-b| / max(1, |a|+|b|), the reference's consistency metric
    (unittests/testConsistencyTF.cpp:16-41)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(a) + np.abs(b))))


def rel_l2(a, b) -> float:
    """||a-b|| / ||b|| (b is the reference value)."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


@dataclass
class Case:
    """Renderer inputs in numpy; all real arrays float32."""
    width: int
    height: int
    volume: np.ndarray
    tf: np.ndarray
    tf_mode: int
    filter_mode: int
    blend_mode: int
    camera_mode: int
    step: object                      # float or (B)(H)(W) array
    box_min: object = (-0.5, -0.5, -0.5)   # tuple or (B)3 array
    box_size: object = (1.0, 1.0, 1.0)
    ray_start: Optional[np.ndarray] = None
    ray_dir: Optional[np.ndarray] = None
    camera_matrix: Optional[np.ndarray] = None
    fov_y: float = 0.0
    early_out: float = 1.0 - 1e-5
    meta: dict = field(default_factory=dict)

    # ---- oracle view
    def oracle_scene(self) -> O.Scene:
        step = self.step
        step_arr = np.full((1, 1, 1), step, np.float32) if np.isscalar(step) else np.asarray(step, np.float32)
        bmin = np.asarray([self.box_min], np.float32) if not isinstance(self.box_min, np.ndarray) else self.box_min
        bsize = np.asarray([self.box_size], np.float32) if not isinstance(self.box_size, np.ndarray) else self.box_size
        return O.Scene(width=self.width, height=self.height, volume=self.volume, tf=self.tf, step_size=step_arr,
                       box_min=bmin, box_size=bsize, filter_mode=self.filter_mode, camera_mode=self.camera_mode,
                       tf_mode=self.tf_mode, blend_mode=self.blend_mode, ray_start=self.ray_start,
                       ray_dir=self.ray_dir, camera_matrix=self.camera_matrix, fov_y_radians=self.fov_y,
                       blending_early_out=self.early_out)

    def batch(self) -> int:
        return self.oracle_scene().batch()

    # ---- GPU view
    def inputs(self, device="cuda", volume_dtype=None, tf_dtype=None):
        import torch
        from diffdvr_gb300 import pyrenderer as pr
        t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dt)
        inp = pr.RendererInputs()
        inp.screen_size = pr.int2(self.width, self.height)
        inp.volume = t(self.volume, volume_dtype or torch.float32)
        inp.volume_filter_mode = pr.VolumeFilterMode(self.filter_mode)
        inp.box_min = t(self.box_min) if isinstance(self.box_min, np.ndarray) else pr.real3(*self.box_min)
        inp.box_size = t(self.box_size) if isinstance(self.box_size, np.ndarray) else pr.real3(*self.box_size)
        inp.camera_mode = pr.CameraMode(self.camera_mode)
        if self.camera_mode == 0:
            inp.camera = pr.CameraPerPixelRays(t(self.ray_start), t(self.ray_dir))
        elif self.camera_mode == 1:
            if self.meta.get("mat4_value"):
                inp.camera = pr.mat4(self.camera_matrix[0])
            else:
                inp.camera = t(self.camera_matrix)
        else:
            inp.camera = pr.CameraReferenceFrame(t(self.camera_matrix), self.fov_y)
        inp.step_size = float(self.step) if np.isscalar(self.step) else t(self.step)
        inp.tf_mode = pr.TFMode(self.tf_mode)
        inp.tf = t(self.tf, tf_dtype or torch.float32)
        inp.blend_mode = pr.BlendMode(self.blend_mode)
        inp.blending_early_out = self.early_out
        return inp


def make_case(seed: int, tf_mode: int = 1, filter_mode: int = 1, blend_mode: int = 0, camera_mode: int = 0,
              shape=(9, 10, 11), W: int = 12, H: int = 10, B: int = 2, R: Optional[int] = None,
              step_voxels: float = 0.5, opacity: float = 1.0, pad_faces: bool = False) -> Case:
    """A small random scene; rays aimed at the box from a sphere of radius 2."""
    w = scenes.small_scene(seed, shape=shape, W=W, H=H, B=B, tf_mode=tf_mode, R=R, opacity=opacity,
                           pad_faces=pad_faces)
    res = max(shape)
    case = Case(width=W, height=H, volume=w.volume, tf=w.tf, tf_mode=tf_mode, filter_mode=filter_mode,
                blend_mode=blend_mode, camera_mode=camera_mode, step=step_voxels / (res - 1))
    if camera_mode == 0:
        case.ray_start, case.ray_dir = w.ray_start, w.ray_dir
    elif camera_mode == 2:
        case.camera_matrix = w.viewport.astype(np.float32)
        case.fov_y = float(np.float32(w.fov_y))
    else:
        mats = [Camera.compute_matrix(vp[0], (0, 0, 0), vp[2], np.degrees(w.fov_y), W, H) for vp in w.viewport]
        case.camera_matrix = np.stack(mats).astype(np.float32)
    return case


def pad_faces(volume: np.ndarray) -> np.ndarray:
    """A copy of a (B)XYZ volume whose outermost two layers are equal on
    every face, so that the trilinear position derivative is continuous
    where rays enter the box."""
    v = np.array(volume, copy=True)
    v[:, 0], v[:, -1] = v[:, 1], v[:, -2]
    v[:, :, 0], v[:, :, -1] = v[:, :, 1], v[:, :, -2]
    v[:, :, :, 0], v[:, :, :, -1] = v[:, :, :, 1], v[:, :, :, -2]
    return v


def edge_cases():
    """Degenerate inputs the marcher must handle: (name, case)."""
    cases = []
    c = make_case(61, shape=(1, 2, 3), W=1, H=1, B=1)
    cases.append(("1x1 image, one-voxel x axis", c))
    c = make_case(62, shape=(2, 1, 1), W=3, H=2, B=2)
    cases.append(("one-voxel y and z axes", c))
    c = make_case(63, W=5, H=4, B=2)
    c.ray_dir = -c.ray_dir  # every ray points away from the box
    cases.append(("all rays miss the box", c))
    c = make_case(64, W=5, H=4, B=1)
    c.step = 4.0  # longer than the box diagonal: at most one sample per ray
    cases.append(("one sample per ray", c))
    c = make_case(65, W=5, H=4, B=1)
    c.early_out = 0.0  # stop after the first sample with any opacity
    cases.append(("early out at zero opacity", c))
    c = make_case(66, W=6, H=5, B=1)
    c.width, c.height = 0, 0
    c.ray_start, c.ray_dir = c.ray_start[:, :0, :0], c.ray_dir[:, :0, :0]
    cases.append(("empty image", c))
    return cases


def all_mode_combos():
    return list(itertools.product(TF_MODES, FILTERS, BLENDS, CAMERAS))


GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN_DIR, name)) as z:
        return {k: z[k] for k in z.files}


def golden_case(g: dict, prefix: str) -> Case:
    tfm, filt, blend, cam, W, H = (int(v) for v in g[prefix + "modes"])
    box = g[prefix + "box"]
    step = g[prefix + "step"]
    case = Case(width=W, height=H, volume=g[prefix + "volume"], tf=g[prefix + "tf"], tf_mode=tfm,
                filter_mode=filt, blend_mode=blend, camera_mode=cam,
                step=float(step) if step.ndim == 0 else step,
                box_min=tuple(float(v) for v in box[0]) if box.ndim == 2 else box[0],
                box_size=tuple(float(v) for v in box[1]) if box.ndim == 2 else box[1],
                fov_y=float(g[prefix + "fov_y"]))
    if cam == 0:
        case.ray_start, case.ray_dir = g[prefix + "ray_start"], g[prefix + "ray_dir"]
    else:
        case.camera_matrix = g[prefix + "camera_matrix"]
    return case


def golden_prefixes(g: dict) -> list:
    return sorted({k.split("_")[0] + "_" for k in g if k.endswith("modes")})


# ---------------------------------------------------------------- GPU runs
def gpu_forward(case: Case, family: str = "optimized", volume_dtype=None, tf_dtype=None, checkpoints: bool = False,
                interval: int = 16, record=None):
    """Renders case on cuda:0; returns (inputs, outputs) with torch tensors.
    record: None, "full" (a sample-density pool that holds every ray), a
    float fraction of that size or an int number of floats (rays that find
    the pool full are re-sampled)."""
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    pr.set_kernel_family(family)
    inp = case.inputs("cuda", volume_dtype, tf_dtype)
    B = case.batch()
    color = torch.full((B, case.height, case.width, 4), float("nan"), device="cuda")
    term = torch.full((B, case.height, case.width), -7, dtype=torch.int32, device="cuda")
    ck = None
    if checkpoints:
        ck = torch.full((B, case.height, case.width, pr.Renderer.checkpoint_slots(inp, interval)), float("nan"),
                        device="cuda")
    out = pr.RendererOutputs(color, term, ck, interval)
    if record is not None:
        full = pr.Renderer.sample_density_size(inp, B)
        if record == "full":
            n = full
        elif isinstance(record, int):
            n = max(4, record // 4 * 4)
        else:
            n = max(4, int(full * float(record)) // 4 * 4)
        out.sample_density = torch.full((n,), float("nan"), device="cuda")
        out.sample_offset = torch.full((B, case.height, case.width), -7, dtype=torch.int32, device="cuda")
    pr.Renderer.render_forward(inp, out)
    torch.cuda.synchronize()
    return inp, out


def gpu_adjoint(case: Case, inp, out, adj_color: np.ndarray, volume=False, tf=False, camera=False, stepsize=False,
                family: str = "optimized", delayed: bool = True, stepsize_shape=None, camera_batch=None,
                volume_batch=None):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    pr.set_kernel_family(family)
    B, H, W = case.batch(), case.height, case.width
    a = pr.AdjointOutputs()
    res = {}
    if volume:
        vb = volume_batch or case.volume.shape[0]
        a.has_volume_derivatives = True
        a.adj_volume = res["adj_volume"] = torch.zeros((vb,) + case.volume.shape[1:], device="cuda")
    if tf:
        a.has_tf_derivatives = True
        a.tf_delayed_accumulation = delayed
        a.adj_tf = res["adj_tf"] = torch.zeros(case.tf.shape, device="cuda")
    if camera:
        cb = camera_batch or B
        a.has_camera_derivatives = True
        a.adj_camera_ray_start = res["adj_ray_start"] = torch.zeros((cb, H, W, 3), device="cuda")
        a.adj_camera_ray_dir = res["adj_ray_dir"] = torch.zeros((cb, H, W, 3), device="cuda")
    if stepsize:
        a.has_stepsize_derivatives = True
        a.adj_stepsize = res["adj_stepsize"] = torch.zeros(stepsize_shape or (B, H, W), device="cuda")
    adj = torch.from_numpy(np.ascontiguousarray(adj_color, np.float32)).cuda()
    pr.Renderer.render_adjoint(inp, out, adj, a)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in res.items()}
