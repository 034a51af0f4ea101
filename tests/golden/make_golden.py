"""Generates the golden fixtures of tests/golden/ from the REFERENCE's own code.

Run in a checkout where the reference sources are present:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

It builds the reference's CPU ray marcher (oracle/Makefile `ref` target:
renderer/renderer_kernels.cuh DvrKernelForwardHost / DvrKernelAdjointHost
compiled with a declaration-only AD shim), renders seeded small scenes for
every mode combination in FP32 and FP64 single-threaded (deterministic
atomics), and stores inputs and outputs as .npz.  It also converts the
reference's known-answer table unittests/NonConvexDensity.tsv (Gaussian TF +
Beer-Lambert along a density ramp, unittests/testNonConvexDensity.cpp:8-81).

The fixtures are data only; nothing at test time reads the reference.
"""
from __future__ import annotations

import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"  # deterministic atomics in the reference's adjoint

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from dvr_cases import all_mode_combos, make_case  # noqa: E402


def _case_arrays(prefix: str, case, out: dict) -> None:
    out[prefix + "volume"] = case.volume
    out[prefix + "tf"] = case.tf
    out[prefix + "modes"] = np.array([case.tf_mode, case.filter_mode, case.blend_mode, case.camera_mode,
                                      case.width, case.height], np.int32)
    out[prefix + "step"] = np.asarray(case.step, np.float32)
    out[prefix + "box"] = np.asarray([case.box_min, case.box_size], np.float32) if not isinstance(
        case.box_min, np.ndarray) else np.stack([case.box_min, case.box_size])
    out[prefix + "fov_y"] = np.float64(case.fov_y)
    if case.camera_mode == 0:
        out[prefix + "ray_start"] = case.ray_start
        out[prefix + "ray_dir"] = case.ray_dir
    else:
        out[prefix + "camera_matrix"] = case.camera_matrix


def main(ref_root: str) -> None:
    O.build(reference=True)
    if not O.reference_available():
        raise SystemExit("reference harness could not be built")
    out: dict = {}
    rng = np.random.default_rng(12345)
    for idx, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(1000 + idx, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam,
                         shape=(6, 7, 8), W=8, H=6, B=2)
        prefix = f"c{idx:02d}_"
        _case_arrays(prefix, case, out)
        sc = case.oracle_scene()
        c32, t32 = O.forward(sc, "reference", "f32")
        c64, t64 = O.forward(sc, "reference", "f64")
        adj = rng.normal(size=c32.shape).astype(np.float32)
        req = O.AdjointRequest(volume=True, tf=True, camera=(cam == 0), stepsize=True)
        g64 = O.adjoint(sc, c64, t64, adj, req, "reference", "f64")
        g32 = O.adjoint(sc, c32, t32, adj, req, "reference", "f32")
        out[prefix + "color_f32"], out[prefix + "term_f32"] = c32, t32
        out[prefix + "color_f64"], out[prefix + "term_f64"] = c64, t64
        out[prefix + "adj_color"] = adj
        for k, v in g64.items():
            out[prefix + k + "_f64"] = v
        for k, v in g32.items():
            out[prefix + k + "_f32"] = v
    np.savez_compressed(os.path.join(HERE, "modes.npz"), **out)

    # broadcasting: volume B=1 with TF B=2, per-pixel step sizes, box tensors,
    # broadcast step-size and camera gradients
    out = {}
    case = make_case(77, tf_mode=1, shape=(7, 8, 9), W=9, H=7, B=2)
    case.volume = case.volume[:1].copy()
    case.step = (0.4 / 8) * (1 + 0.25 * np.random.default_rng(5).uniform(size=(2, 7, 9))).astype(np.float32)
    case.box_min = np.array([[-0.5, -0.5, -0.5], [-0.45, -0.5, -0.55]], np.float32)
    case.box_size = np.array([[1.0, 1.0, 1.0], [0.9, 1.05, 1.1]], np.float32)
    sc = case.oracle_scene()
    _case_arrays("b_", case, out)
    out["b_step"] = case.step
    c32, t32 = O.forward(sc, "reference", "f32")
    c64, t64 = O.forward(sc, "reference", "f64")
    adj = np.random.default_rng(6).normal(size=c32.shape).astype(np.float32)
    req = O.AdjointRequest(volume=True, tf=True, camera=True, stepsize=True, stepsize_shape=(1, 1, 1),
                           camera_batch=1, volume_batch=1)
    g64 = O.adjoint(sc, c64, t64, adj, req, "reference", "f64")
    out["b_color_f32"], out["b_term_f32"], out["b_color_f64"], out["b_term_f64"] = c32, t32, c64, t64
    out["b_adj_color"] = adj
    for k, v in g64.items():
        out["b_" + k + "_f64"] = v
    np.savez_compressed(os.path.join(HERE, "broadcast.npz"), **out)

    # the reference's known-answer table
    tsv = os.path.join(ref_root, "unittests", "NonConvexDensity.tsv")
    rows = []
    with open(tsv) as f:
        header = f.readline()
        f.readline()
        for line in f:
            if line.strip():
                rows.append([float(v) for v in line.split()])
    gt = header.split("(red, alpha)=(")[1].split(")")[0].split(",")
    np.savez_compressed(os.path.join(HERE, "nonconvex_density.npz"), table=np.array(rows, np.float64),
                        ground_truth_red_alpha=np.array([float(gt[0]), float(gt[1])]),
                        columns=np.array(["d1", "red", "alpha", "loss", "grad"]))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    from oracle.oracle import REFERENCE_ROOT
    main(sys.argv[1] if len(sys.argv) > 1 else REFERENCE_ROOT)
