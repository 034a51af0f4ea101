"""The reference's own CUDA kernels on the GPU — TEST INFRASTRUCTURE ONLY.

Runs the cubin that ``oracle/Makefile`` (target ``ref``) compiles from the
reference's headers (``oracle/ref_device.cu``) through the CUDA driver API,
the way the reference's CUDA backend does: the forward and adjoint kernels
take their parameter blocks by value, with the block size and grid that
``cuOccupancyMaxPotentialBlockSize`` gives (renderer/kernel_loader.cpp:514-515,
renderer/renderer_cuda.cpp:85-118).

The reference's delayed TF accumulation (per-thread shared-memory TF
gradients reduced over each warp, renderer/renderer_tf.cuh:173-253 and its
siblings) is never launched: its warp reduction
(renderer/cooperative_groups.cuh:161-212) passes the shuffle's value where
the member mask belongs (:206) whenever a warp's active threads are not a
power of two in number, and kernels built with it raised "an illegal
instruction was encountered" on the GB300.  The TF gradients come from the
reference's immediate-atomics variant.

The parameter blocks are filled on the GPU by ``ref_build_params`` from the
plain-C structs of ``dvr_oracle.h``; every block is read back through the
reference's own accessor getters and checked before the first launch.

``forward`` / ``adjoint`` take and return numpy arrays like ``oracle.forward``
/ ``oracle.adjoint`` (FP32 only: the reference's CUDA build is single
precision).  Only ``tests/`` use this module, as the reference CUDA path the
kernels of ``diffdvr_gb300`` are compared with.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import oracle as O

CUBIN = os.path.join(O.REF_DIR, "ref_kernels_sm103a.cubin")
SLOT = 1024  # bytes per parameter block in ref_build_params' output

FILTERS = {0: "FilterNearest", 1: "FilterTrilinear"}
CAMERAS = {0: "CameraRayStartDir", 1: "CameraInverseViewMatrix", 2: "CameraReferenceFrame"}
TFS = {0: "TFIdentity", 1: "TFTexture", 2: "TFLinear", 3: "TFGaussian"}
BLENDS = {0: "BlendBeerLambert", 1: "BlendAlpha"}


def available() -> bool:
    return os.path.exists(CUBIN)


def forward_kernel_name(scene: O.Scene) -> str:
    return (f"ref_fwd_{FILTERS[scene.filter_mode]}_{CAMERAS[scene.camera_mode]}_"
            f"{TFS[scene.tf_mode]}_{BLENDS[scene.blend_mode]}")


def adjoint_kernel_name(scene: O.Scene, stepsize: bool, camera: bool, tf: bool, delayed: bool,
                        volume: bool) -> str:
    flags = "".join(str(int(v)) for v in (stepsize, camera, tf, delayed, volume))
    return (f"ref_adj_{FILTERS[scene.filter_mode]}_{CAMERAS[scene.camera_mode]}_"
            f"{TFS[scene.tf_mode]}_{BLENDS[scene.blend_mode]}_{flags}")


class _Driver:
    """The few CUDA driver calls the reference's backend makes, via ctypes."""

    def __init__(self):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("the reference's CUDA kernels need a GPU")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # the runtime's primary context is current from here on
        lib = ctypes.CDLL("libcuda.so.1")
        vp, ip, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint
        lib.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        lib.cuOccupancyMaxPotentialBlockSize.argtypes = [ctypes.POINTER(ip), ctypes.POINTER(ip), vp, vp,
                                                         ctypes.c_size_t, ip]
        lib.cuLaunchKernel.argtypes = [vp, u, u, u, u, u, u, u, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        lib.cuGetErrorString.argtypes = [ip, ctypes.POINTER(ctypes.c_char_p)]
        self.lib = lib
        ctx = vp()
        self._check(lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.module = vp()
        self._check(lib.cuModuleLoad(ctypes.byref(self.module), CUBIN.encode()), "cuModuleLoad")
        self.functions: dict = {}

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = ctypes.c_char_p()
            self.lib.cuGetErrorString(rc, ctypes.byref(msg))
            raise RuntimeError(f"{what} failed: {rc} ({(msg.value or b'').decode()})")

    def function(self, name: str):
        """(handle, best block size, min grid size) of a kernel without dynamic shared memory."""
        if name not in self.functions:
            f = ctypes.c_void_p()
            self._check(self.lib.cuModuleGetFunction(ctypes.byref(f), self.module, name.encode()),
                        f"cuModuleGetFunction({name})")
            grid, block = ctypes.c_int(), ctypes.c_int()
            self._check(self.lib.cuOccupancyMaxPotentialBlockSize(ctypes.byref(grid), ctypes.byref(block), f,
                                                                  None, 0, 0), "cuOccupancyMaxPotentialBlockSize")
            self.functions[name] = (f, block.value, grid.value)
        return self.functions[name]

    def launch(self, f, grid: int, block: int, smem: int, stream: int, args: list) -> None:
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self._check(self.lib.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, ctypes.c_void_p(stream), params, None),
                    "cuLaunchKernel")


_DRIVER: Optional[_Driver] = None


def driver() -> _Driver:
    global _DRIVER
    if _DRIVER is None:
        if not available():
            raise FileNotFoundError(f"{CUBIN} not built (oracle.oracle.build(reference=True) where the "
                                    "reference sources exist)")
        _DRIVER = _Driver()
    return _DRIVER


def _dev_tensor(t, keep: list) -> O.OracleTensor:
    """OracleTensor view of a CUDA torch tensor (element strides)."""
    keep.append(t)
    o = O.OracleTensor()
    o.data = t.data_ptr()
    o.ndim = t.dim()
    for d in range(t.dim()):
        o.sizes[d] = t.shape[d]
        o.strides[d] = t.stride(d)
    return o


class Call:
    """One scene on the GPU with its parameter blocks built and checked.

    ``run_forward()`` / ``run_adjoint()`` launch the reference's kernels on
    the current stream and nothing else (the gradient buffers are zeroed by
    the caller, as the reference requires)."""

    def __init__(self, scene: O.Scene, adjoint: Optional[O.AdjointRequest] = None,
                 color=None, term=None, adj_color=None):
        import torch
        self.drv = driver()
        self.scene = scene
        dev = torch.device("cuda")
        f32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=dev)
        keep: list = []
        self.keep = keep
        i = O.OracleInputs()
        i.width, i.height = scene.width, scene.height
        i.filter_mode, i.camera_mode = scene.filter_mode, scene.camera_mode
        i.tf_mode, i.blend_mode = scene.tf_mode, scene.blend_mode
        i.volume = _dev_tensor(f32(scene.volume), keep)
        i.box_min = _dev_tensor(f32(scene.box_min), keep)
        i.box_size = _dev_tensor(f32(scene.box_size), keep)
        i.ray_start = _dev_tensor(f32(scene.ray_start if scene.ray_start is not None else np.zeros((1, 1, 1, 3))), keep)
        i.ray_dir = _dev_tensor(f32(scene.ray_dir if scene.ray_dir is not None else np.zeros((1, 1, 1, 3))), keep)
        i.camera_matrix = _dev_tensor(
            f32(scene.camera_matrix if scene.camera_matrix is not None else np.zeros((1, 4, 4))), keep)
        i.fov_y_radians = float(scene.fov_y_radians)
        i.step_size = _dev_tensor(f32(scene.step_size), keep)
        i.tf = _dev_tensor(f32(scene.tf), keep)
        i.blending_early_out = float(scene.blending_early_out)
        i.batch = scene.batch()
        self.inputs = i
        B, H, W = i.batch, scene.height, scene.width
        self.B = B
        self.color = f32(color) if color is not None else torch.zeros(B, H, W, 4, device=dev)
        self.term = (torch.as_tensor(np.ascontiguousarray(term, dtype=np.int32), device=dev) if term is not None
                     else torch.zeros(B, H, W, dtype=torch.int32, device=dev))
        self.adj_color = f32(adj_color) if adj_color is not None else None
        out = O.OracleAdjointOutputs()
        self.grads: dict = {}
        self.adjoint_name = None
        if adjoint is not None:
            req = adjoint
            if req.camera and scene.camera_mode != 0:
                raise ValueError("camera derivatives need per-pixel rays (camera mode 0)")
            if req.volume:
                self.grads["adj_volume"] = torch.zeros(
                    ((req.volume_batch or int(scene.volume.shape[0])),) + tuple(scene.volume.shape[1:]), device=dev)
                out.has_volume = 1
                out.adj_volume = _dev_tensor(self.grads["adj_volume"], keep)
            if req.tf:
                self.grads["adj_tf"] = torch.zeros(
                    ((req.tf_batch or int(scene.tf.shape[0])),) + tuple(scene.tf.shape[1:]), device=dev)
                out.has_tf = 1
                out.adj_tf = _dev_tensor(self.grads["adj_tf"], keep)
            if req.camera:
                cb = req.camera_batch or B
                self.grads["adj_ray_start"] = torch.zeros(cb, H, W, 3, device=dev)
                self.grads["adj_ray_dir"] = torch.zeros(cb, H, W, 3, device=dev)
                out.has_camera = 1
                out.camera_broadcast = int(cb != B)
                out.adj_ray_start = _dev_tensor(self.grads["adj_ray_start"], keep)
                out.adj_ray_dir = _dev_tensor(self.grads["adj_ray_dir"], keep)
            if req.stepsize:
                shp = req.stepsize_shape or (B, H, W)
                self.grads["adj_stepsize"] = torch.zeros(shp, device=dev)
                out.has_stepsize = 1
                out.stepsize_broadcast = int(tuple(shp) != (B, H, W))
                out.adj_stepsize = _dev_tensor(self.grads["adj_stepsize"], keep)
            if self.adj_color is None:
                raise ValueError("the adjoint needs adj_color")
            self.adjoint_name = adjoint_kernel_name(scene, req.stepsize, req.camera, req.tf, False, req.volume)
        self.adj_out = out
        tc = _dev_tensor(self.color, keep)
        tt = _dev_tensor(self.term, keep)
        ta = _dev_tensor(self.adj_color, keep) if self.adj_color is not None else O.OracleTensor()
        blobs = torch.zeros(5 * SLOT, dtype=torch.uint8, device=dev)
        info = torch.zeros(8, dtype=torch.int64, device=dev)
        bp, ip = ctypes.c_void_p(blobs.data_ptr()), ctypes.c_void_p(info.data_ptr())
        build, _, _ = self.drv.function("ref_build_params")
        stream = torch.cuda.current_stream().cuda_stream
        self.drv.launch(build, 1, 1, 0, stream, [i, tc, tt, ta, out, bp, ip])
        torch.cuda.synchronize()
        inf = info.cpu().numpy()
        if inf[5] != 1 or inf[6] != 4:
            raise RuntimeError(f"reference parameter blocks do not read back as built: {inf.tolist()}")
        raw = blobs.cpu().numpy().tobytes()
        block = lambda k: (ctypes.c_char * int(inf[k])).from_buffer_copy(raw[k * SLOT:k * SLOT + int(inf[k])])
        self.p_inputs, self.p_outputs, self.p_fwd = block(0), block(1), block(2)
        self.p_adj_color, self.p_adj_out = block(3), block(4)
        self.vs = (ctypes.c_uint * 3)(scene.width, scene.height, B)
        # launch configuration, as the reference's backend computes it
        self.fwd_fn, bs, mg = self.drv.function(forward_kernel_name(scene))
        n = scene.width * scene.height * B
        self.fwd_cfg = (max(1, min(-(-n // bs), mg)), bs, 0)
        if self.adjoint_name is not None:
            f, bs, mg = self.drv.function(self.adjoint_name)
            self.adj_fn = f
            self.adj_cfg = (max(1, min(-(-n // bs), mg)), bs, 0)

    def run_forward(self) -> None:
        import torch
        g, b, s = self.fwd_cfg
        self.drv.launch(self.fwd_fn, g, b, s, torch.cuda.current_stream().cuda_stream,
                        [self.vs, self.p_inputs, self.p_outputs])

    def run_adjoint(self) -> None:
        import torch
        g, b, s = self.adj_cfg
        self.drv.launch(self.adj_fn, g, b, s, torch.cuda.current_stream().cuda_stream,
                        [self.vs, self.p_inputs, self.p_fwd, self.p_adj_color, self.p_adj_out])


def forward(scene: O.Scene):
    """The reference's CUDA forward: (color B*H*W*4 float32, termination B*H*W int32)."""
    import torch
    c = Call(scene)
    c.run_forward()
    torch.cuda.synchronize()
    return c.color.cpu().numpy(), c.term.cpu().numpy()


def adjoint(scene: O.Scene, color: np.ndarray, term: np.ndarray, adj_color: np.ndarray,
            req: O.AdjointRequest) -> dict:
    """The reference's CUDA adjoint (TF gradients by immediate atomics): a
    dict of gradient arrays like oracle.adjoint's."""
    import torch
    c = Call(scene, adjoint=req, color=color, term=term, adj_color=adj_color)
    c.run_adjoint()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in c.grads.items()}


# The adjoints the timing below launches, per workload: (TF mode, camera,
# TF, delayed TF accumulation, volume derivatives), all with trilinear
# filtering, per-pixel rays and Beer-Lambert blending, no step-size
# derivatives: the reference's kernel for exactly the gradients each
# workload asks for, TF gradients by immediate atomics.
# oracle/ref_device.cu instantiates each one.
TIMED_ADJOINTS = {
    "tf_reconstruction_256": (1, False, True, False, False),
    "absorption_recon_128": (0, False, False, False, True),
    "large_mixed_512": (2, True, True, False, True),
    "plain_cpu_64": (2, False, True, False, True),
}


def timed_adjoint_name(tf_mode: int, camera: bool, tf: bool, delayed: bool, volume: bool) -> str:
    sc = O.Scene(width=1, height=1, volume=None, tf=None, step_size=None, box_min=None, box_size=None,
                 filter_mode=1, camera_mode=0, tf_mode=tf_mode, blend_mode=0)
    return adjoint_kernel_name(sc, False, camera, tf, delayed, volume)


def time_workload(w, volume: Optional[np.ndarray] = None, steps: int = 5, warmup: int = 3) -> dict:
    """The reference's CUDA forward + adjoint on a workload of
    ``diffdvr_gb300.scenes`` (a Workload with per-pixel rays), with the
    gradients the workload asks for (``TIMED_ADJOINTS``), timed with CUDA
    events on the launching stream after `warmup` steps; a 256 MB buffer is
    written before every step so the volume is not left in L2.  volume: the
    FP32 volume each step renders (the workload's own when None; the
    reference stores volumes in FP32 only)."""
    import torch
    tf_mode, cam, tfg, dl, volg = TIMED_ADJOINTS[w.name]
    assert tf_mode == w.tf_mode and w.filter_mode == 1 and w.blend_mode == 0, w.name
    vol = np.asarray(w.volume if volume is None else volume, dtype=np.float32)
    vol = vol if vol.ndim == 4 else vol[None]
    sc = O.Scene(width=w.width, height=w.height, volume=vol, tf=w.tf,
                 step_size=np.full((1, 1, 1), w.step_size, np.float32),
                 box_min=np.asarray([w.box_min], np.float32), box_size=np.asarray([w.box_size], np.float32),
                 filter_mode=w.filter_mode, camera_mode=0, tf_mode=w.tf_mode, blend_mode=w.blend_mode,
                 ray_start=w.ray_start, ray_dir=w.ray_dir)
    B = sc.batch()
    adj = np.random.default_rng(0).normal(size=(B, w.height, w.width, 4)).astype(np.float32)
    call = Call(sc, adjoint=O.AdjointRequest(tf=tfg, volume=volg, camera=cam), adj_color=adj)
    assert call.adjoint_name == timed_adjoint_name(tf_mode, cam, tfg, dl, volg)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    t_fwd, t_adj = [], []
    for i in range(warmup + steps):
        flush.zero_()
        for g in call.grads.values():
            g.zero_()
        torch.cuda.synchronize()
        ev[0].record()
        call.run_forward()
        ev[1].record()
        call.run_adjoint()
        ev[2].record()
        torch.cuda.synchronize()
        if i >= warmup:
            t_fwd.append(ev[0].elapsed_time(ev[1]))
            t_adj.append(ev[1].elapsed_time(ev[2]))
    samples = int(call.term.sum().item())
    f, a = float(np.median(t_fwd)), float(np.median(t_adj))
    return {"workload": w.name, "volume_dtype": "f32", "gradients": sorted(call.grads),
            "tf_accumulation": ("delayed" if dl else "immediate") if tfg else None,
            "samples_per_step": samples, "forward_ms": f, "adjoint_ms": a,
            "samples_per_s": samples / ((f + a) * 1e-3), "kernels": [forward_kernel_name(sc), call.adjoint_name],
            "launch": {"forward": list(call.fwd_cfg), "adjoint": list(call.adj_cfg)}}


def time_tf_reconstruction(steps: int = 5, warmup: int = 3, w=None) -> dict:
    """The reference's CUDA forward + TF adjoint on the TF-reconstruction
    workload (256^3 FP32 volume of blobs + noise, 64-entry texture TF, 8 views
    at 256^2, step 0.25 voxel, Beer-Lambert): ``time_workload``."""
    from diffdvr_gb300 import scenes
    return time_workload(w or scenes.tf_reconstruction_256(), steps=steps, warmup=warmup)


if __name__ == "__main__":
    import json
    from diffdvr_gb300 import scenes
    print(json.dumps(time_tf_reconstruction(w=scenes.tf_reconstruction_256())), flush=True)
