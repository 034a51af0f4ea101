"""The oracle (C restatement) pinned to the reference: golden fixtures made by
the reference's own CPU code, the reference's known-answer table, and (where
the reference sources exist) a direct comparison over all mode combinations."""
import numpy as np
import pytest

from dvr_cases import (all_mode_combos, edge_cases, golden, golden_case, golden_prefixes, make_case, rel_l2,
                       symmetric_error)


@pytest.fixture(scope="module")
def modes(oracle_built):
    return golden("modes.npz")


def test_port_forward_matches_reference_fixtures(oracle_built, modes):
    O = oracle_built
    for p in golden_prefixes(modes):
        case = golden_case(modes, p)
        sc = case.oracle_scene()
        c32, t32 = O.forward(sc, "port", "f32")
        c64, t64 = O.forward(sc, "port", "f64")
        assert np.array_equal(t32, modes[p + "term_f32"]), p
        assert np.array_equal(t64, modes[p + "term_f64"]), p
        assert symmetric_error(c32, modes[p + "color_f32"]) <= 2e-6, p
        assert symmetric_error(c64, modes[p + "color_f64"]) <= 1e-12, p


def test_port_adjoint_matches_reference_fixtures(oracle_built, modes):
    O = oracle_built
    for p in golden_prefixes(modes):
        case = golden_case(modes, p)
        sc = case.oracle_scene()
        req = O.AdjointRequest(volume=True, tf=True, camera=case.camera_mode == 0, stepsize=True)
        adj = modes[p + "adj_color"]
        g64 = O.adjoint(sc, modes[p + "color_f64"], modes[p + "term_f64"], adj, req, "port", "f64")
        g32 = O.adjoint(sc, modes[p + "color_f32"], modes[p + "term_f32"], adj, req, "port", "f32")
        for k in g64:
            assert symmetric_error(g64[k], modes[p + k + "_f64"]) <= 1e-11, (p, k)
            # multi-threaded atomics sum in a different order than the fixture
            # (TF gradients sum thousands of FP32 terms: up to ~2e-5 seen)
            assert symmetric_error(g32[k], modes[p + k + "_f32"]) <= 1e-4, (p, k)


def test_port_broadcasting_matches_reference_fixture(oracle_built):
    O = oracle_built
    g = golden("broadcast.npz")
    case = golden_case(g, "b_")
    sc = case.oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    assert np.array_equal(t64, g["b_term_f64"])
    assert symmetric_error(c64, g["b_color_f64"]) <= 1e-12
    req = O.AdjointRequest(volume=True, tf=True, camera=True, stepsize=True, stepsize_shape=(1, 1, 1),
                           camera_batch=1, volume_batch=1)
    gr = O.adjoint(sc, c64, t64, g["b_adj_color"], req, "port", "f64")
    for k in gr:
        assert symmetric_error(gr[k], g["b_" + k + "_f64"]) <= 1e-11, k


def nonconvex_scene(d1: float, O):
    """A 2x2x2 volume with density d0=-1 at x=0 and d1 at x=1, one ray along
    +x through the box [0,1]^3 with step 1/32: 33 samples on the density ramp
    (1-f)*d0 + f*d1 of unittests/testNonConvexDensity.cpp:25-42."""
    vol = np.zeros((1, 2, 2, 2))
    vol[0, 0], vol[0, 1] = -1.0, d1
    return O.Scene(width=1, height=1, volume=vol, tf=np.array([[[1, 0, 0, 1, 0, 0.5]]], float),
                   step_size=np.full((1, 1, 1), 1 / 32), box_min=np.zeros((1, 3)), box_size=np.ones((1, 3)),
                   filter_mode=1, camera_mode=0, tf_mode=3, blend_mode=0,
                   ray_start=np.array([[[[-1.0, 0.5, 0.5]]]]), ray_dir=np.array([[[[1.0, 0.0, 0.0]]]]))


def nonconvex_row(d1: float, gt, O, precision="f64"):
    sc = nonconvex_scene(d1, O)
    color, term = O.forward(sc, "port", precision)
    diff = color[0, 0, 0] - gt
    loss = float(np.linalg.norm(diff))
    # d|diff|/d(color); at the minimum (loss 0) the table lists a zero gradient
    adj_color = (diff / loss if loss > 0 else np.zeros_like(diff))[None, None, None, :]
    g = O.adjoint(sc, color, term, adj_color, O.AdjointRequest(volume=True), "port", precision)
    grad = float(g["adj_volume"][0, 1].sum())
    return color[0, 0, 0], int(term[0, 0, 0]), loss, grad


def test_oracle_reproduces_nonconvex_density_table(oracle_built):
    """The reference's known-answer table (unittests/NonConvexDensity.tsv):
    red, alpha, loss and d(loss)/d(d1), printed with 5 decimals."""
    O = oracle_built
    t = golden("nonconvex_density.npz")
    gt_color, _ = O.forward(nonconvex_scene(-1.0, O), "port", "f64")
    gt = gt_color[0, 0, 0]
    assert abs(gt[0] - t["ground_truth_red_alpha"][0]) <= 6e-4
    assert abs(gt[3] - t["ground_truth_red_alpha"][1]) <= 6e-4
    for d1, red, alpha, loss, grad in t["table"]:
        color, n, l, gr = nonconvex_row(d1, gt, O)
        assert n == 33
        assert abs(color[0] - red) <= 6e-6, d1
        assert abs(color[3] - alpha) <= 6e-6, d1
        assert abs(l - loss) <= 6e-6, d1
        assert abs(gr - grad) <= 6e-6 + 1e-4 * abs(grad), d1


@pytest.mark.parametrize("tf_mode", [0, 1, 2, 3])
def test_port_gradients_match_central_differences(oracle_built, tf_mode):
    """FP64 oracle adjoint against central finite differences of the FP64
    forward, for TF entries and voxels (the reference's checkAdjoint idea,
    unittests/check_adjoint.h:35-84, with central differences)."""
    O = oracle_built
    case = make_case(31 + tf_mode, tf_mode=tf_mode, shape=(5, 6, 7), W=6, H=5, B=1)
    sc = case.oracle_scene()
    sc.volume = sc.volume.astype(np.float64)
    sc.tf = sc.tf.astype(np.float64)
    rng = np.random.default_rng(tf_mode)
    color, term = O.forward(sc, "port", "f64")
    w = rng.normal(size=color.shape)
    g = O.adjoint(sc, color, term, w, O.AdjointRequest(volume=True, tf=True), "port", "f64")

    def loss(s):
        c, _ = O.forward(s, "port", "f64")
        return float((c * w).sum())

    flat_tf = [(r, c) for r in range(sc.tf.shape[1]) for c in range(sc.tf.shape[2])]
    for (r, c) in [flat_tf[i] for i in rng.choice(len(flat_tf), min(6, len(flat_tf)), replace=False)]:
        h = 1e-6 * max(1.0, abs(sc.tf[0, r, c]))
        tp, tm = sc.tf.copy(), sc.tf.copy()
        tp[0, r, c] += h
        tm[0, r, c] -= h
        sp, sm = O.Scene(**{**sc.__dict__, "tf": tp}), O.Scene(**{**sc.__dict__, "tf": tm})
        fd = (loss(sp) - loss(sm)) / (2 * h)
        assert abs(fd - g["adj_tf"][0, r, c]) <= 1e-5 * max(1.0, abs(fd)), (r, c)
    for _ in range(6):
        x, y, z = (int(rng.integers(0, n)) for n in sc.volume.shape[1:])
        h = 1e-6
        vp, vm = sc.volume.copy(), sc.volume.copy()
        vp[0, x, y, z] += h
        vm[0, x, y, z] -= h
        fd = (loss(O.Scene(**{**sc.__dict__, "volume": vp})) - loss(O.Scene(**{**sc.__dict__, "volume": vm}))) / (2 * h)
        assert abs(fd - g["adj_volume"][0, x, y, z]) <= 1e-5 * max(1.0, abs(fd)), (x, y, z)


def test_port_matches_reference_all_modes(oracle_built):
    """Direct restatement-vs-reference comparison (needs the reference sources)."""
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present: the golden fixtures pin the oracle instead")
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(500 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam)
        sc = case.oracle_scene()
        c1, t1 = O.forward(sc, "port", "f64")
        c2, t2 = O.forward(sc, "reference", "f64")
        assert np.array_equal(t1, t2)
        assert symmetric_error(c1, c2) <= 1e-12
        adj = np.random.default_rng(i).normal(size=c1.shape)
        req = O.AdjointRequest(volume=True, tf=True, camera=cam == 0, stepsize=True)
        g1 = O.adjoint(sc, c2, t2, adj, req, "port", "f64")
        g2 = O.adjoint(sc, c2, t2, adj, req, "reference", "f64")
        for k in g1:
            assert rel_l2(g1[k], g2[k]) <= 1e-12 or symmetric_error(g1[k], g2[k]) <= 1e-12, k


@pytest.mark.parametrize("camera_mode", [0, 1, 2])
def test_reference_parameter_block_images(oracle_built, camera_mode):
    """The GPU harness of the reference's CUDA kernels (oracle/ref_device.cu)
    has no accessor constructors: it writes each parameter block as a byte
    image (oracle/ref_image.h).  Here, on the CPU, the reference's own
    constructors build the same blocks from the same inputs, and every field
    of both, read through the accessors' getters, must agree: sizes, element
    strides, stride 0 for broadcast dimensions, pointers, scalars."""
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present")
    case = make_case(40 + camera_mode, tf_mode=1, camera_mode=camera_mode, B=2)
    sc = case.oracle_scene()
    for precision in ("f32", "f64"):
        req = O.AdjointRequest(volume=True, tf=True, camera=camera_mode == 0, stepsize=True)
        assert O.reference_image_check(sc, req, precision) == 0, precision
    # broadcast inputs and gradients: size-1 batch (and pixel) dimensions
    g = golden("broadcast.npz")
    bsc = golden_case(g, "b_").oracle_scene()
    req = O.AdjointRequest(volume=True, tf=True, camera=True, stepsize=True, stepsize_shape=(1, 1, 1),
                           camera_batch=1, volume_batch=1)
    assert O.reference_image_check(bsc, req, "f32") == 0
    assert O.reference_image_check(bsc, O.AdjointRequest(tf=True), "f32") == 0


def test_reference_cuda_kernel_names(oracle_built, tmp_path):
    """Every kernel oracle/ref_cuda.py launches is defined by
    oracle/ref_device.cu (read from its preprocessed source, not the cubin),
    and each adjoint kernel instantiates the reference's template with the
    derivative switches its name states."""
    import re
    import shutil
    import subprocess
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present")
    from oracle import ref_cuda as R
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path / "ref_device.ii"
    subprocess.run([nvcc, "-E", "-std=c++17", "-DUSE_DOUBLE_PRECISION=0", "-DNDEBUG", "-w", "-I", O.HERE,
                    "-I", f"{O.HERE}/ref_shim", "-I", O.REFERENCE_SOURCES, f"{O.HERE}/ref_device.cu", "-o", str(out)],
                   check=True)
    src = out.read_text()
    defined = set(re.findall(r"void (ref_\w+)\s*\(", src))
    want = {"ref_build_params"}
    for tfm, filt, blend, cam in all_mode_combos():
        sc = O.Scene(width=1, height=1, volume=None, tf=None, step_size=None, box_min=None, box_size=None,
                     filter_mode=filt, camera_mode=cam, tf_mode=tfm, blend_mode=blend)
        want.add(R.forward_kernel_name(sc))
        want.add(R.adjoint_kernel_name(sc, True, cam == 0, True, False, True))
    sc = O.Scene(width=1, height=1, volume=None, tf=None, step_size=None, box_min=None, box_size=None)
    want.add(R.adjoint_kernel_name(sc, False, False, True, False, False))
    want.update(R.timed_adjoint_name(*v) for v in R.TIMED_ADJOINTS.values())
    assert want == defined, (sorted(want - defined), sorted(defined - want))
    adj = list(re.finditer(r"void (ref_adj_\w+)\s*\(.*?DvrKernelAdjointImpl<[^>]*?,\s*(\d),\s*(\d),\s*(\d),"
                           r"\s*(\d),\s*(\d)\s*>", src, re.S))
    assert len(adj) == sum(n.startswith("ref_adj_") for n in want)
    for m in adj:
        assert m.group(1).endswith("_" + "".join(m.group(i) for i in range(2, 7))), m.group(1)


@pytest.mark.parametrize("filter_mode", [0, 1])
def test_port_matches_reference_edge_cases(oracle_built, filter_mode):
    """Degenerate inputs: the restatement against the reference's own CPU
    templates, FP64, forward and every gradient."""
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present")
    for name, case in edge_cases():
        case.filter_mode = filter_mode
        sc = case.oracle_scene()
        c1, t1 = O.forward(sc, "port", "f64")
        c2, t2 = O.forward(sc, "reference", "f64")
        assert np.array_equal(t1, t2), name
        assert c1.size == 0 or symmetric_error(c1, c2) <= 1e-12, name
        if name == "all rays miss the box":
            assert not t1.any() and not c1.any(), name
        if name == "one sample per ray":
            assert t1.max() <= 1, name
        adj = np.random.default_rng(3).normal(size=c1.shape)
        req = O.AdjointRequest(volume=True, tf=True, camera=True, stepsize=True)
        g1 = O.adjoint(sc, c2, t2, adj, req, "port", "f64")
        g2 = O.adjoint(sc, c2, t2, adj, req, "reference", "f64")
        for k in g1:
            assert g1[k].size == 0 or rel_l2(g1[k], g2[k]) <= 1e-12 or symmetric_error(g1[k], g2[k]) <= 1e-12, (
                name, k)


@pytest.mark.parametrize("tf_mode,R", [(0, 1), (1, 2), (1, 4), (1, 8), (2, 4)],
                         ids=["identity", "texture2", "texture4", "texture8", "linear4"])
def test_consistency_scene_port_matches_reference(oracle_built, tf_mode, R):
    """The scene of the reference's TF consistency test
    (unittests/testConsistencyTF.cpp:43-110): Marschner-Lobb 32^3 in the box
    [-0.5, 0.5]^3, 128 x 128 pixels, inverse view-projection camera at
    (-1, -0.5, 0) looking at the origin with up +z and 45 degrees, step
    0.5/64, trilinear, Beer-Lambert, TF entries U(0, 1).  Linear TF positions
    are 0, 1/3, 2/3, 1 (the reference's loop divides integers and so writes
    0, 0, 0, 1; the intended positions are used).  The restatement against
    the reference's CPU templates: FP64 exact to rounding, FP32 within the
    reference's symmetric metric 1e-5 on the image.  The FP32 TF gradient sums
    ~3 M terms into a few entries with atomics, so two runs of the reference
    itself differ by up to 2e-4 in that metric: both adjoints run on one
    thread here, where the restatement is bit-identical to the reference."""
    from diffdvr_gb300.camera import Camera
    from diffdvr_gb300.volume_io import marschner_lobb
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present")
    W = H = 128
    rng = np.random.default_rng(42)
    C = {0: 2, 1: 4, 2: 5}[tf_mode]
    tf = rng.uniform(0.0, 1.0, size=(1, R, C)).astype(np.float32)
    if tf_mode == 2:
        tf[0, :, 4] = np.arange(R) / (R - 1)
    mat = Camera.compute_matrix((-1.0, -0.5, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 45.0, W, H)[None]
    sc = O.Scene(width=W, height=H, volume=marschner_lobb(32), tf=tf,
                 step_size=np.full((1, 1, 1), 0.5 / 64, np.float32),
                 box_min=np.full((1, 3), -0.5, np.float32), box_size=np.ones((1, 3), np.float32),
                 filter_mode=1, camera_mode=1, tf_mode=tf_mode, blend_mode=0, camera_matrix=mat)
    req = O.AdjointRequest(tf=True)
    adj = rng.normal(size=(1, H, W, 4))
    grads = {}
    for precision, tol in (("f64", 1e-12), ("f32", 1e-5)):
        c1, t1 = O.forward(sc, "port", precision)
        c2, t2 = O.forward(sc, "reference", precision)
        assert t2.max() > 50  # rays cross the volume
        same = t1 == t2
        assert np.mean(~same) <= (0 if precision == "f64" else 0.001), precision
        assert symmetric_error(c1[same], c2[same]) <= tol, precision
        prev = O.set_threads(1)
        try:
            grads[precision] = (O.adjoint(sc, c2, t2, adj, req, "port", precision)["adj_tf"],
                                O.adjoint(sc, c2, t2, adj, req, "reference", precision)["adj_tf"])
        finally:
            O.set_threads(prev)
    port64, ref64 = grads["f64"]
    assert np.array_equal(port64, ref64)
    port32, ref32 = grads["f32"]
    assert np.array_equal(port32, ref32)


@pytest.mark.parametrize("tf_mode,R", [(0, 1), (1, 2), (1, 4), (1, 8), (2, 4)],
                         ids=["identity", "texture2", "texture4", "texture8", "linear4"])
def test_camera_consistency_scene_port_matches_reference(oracle_built, tf_mode, R):
    """The scene of the reference's camera consistency test
    (unittests/testConsistencyCamera.cpp:43-120): Marschner-Lobb 32^3 in the
    box [-0.5, 0.5]^3, 8 x 8 per-pixel rays of a camera at (-1, -0.5, 0)
    looking at the origin with up +z and 45 degrees, step 0.25, trilinear,
    Beer-Lambert, TF entries U(0, 1) (linear TF positions 0, 1/3, 2/3, 1).
    The ray start and direction gradients of the restatement against the
    reference's CPU templates: FP64 exact to rounding, FP32 within the
    reference's symmetric metric 1e-5 (per-pixel outputs, no atomics)."""
    from diffdvr_gb300 import scenes
    from diffdvr_gb300.volume_io import marschner_lobb
    O = oracle_built
    if not O.reference_available():
        pytest.skip("reference sources not present")
    W = H = 8
    rng = np.random.default_rng(43)
    C = {0: 2, 1: 4, 2: 5}[tf_mode]
    tf = rng.uniform(0.0, 1.0, size=(1, R, C)).astype(np.float32)
    if tf_mode == 2:
        tf[0, :, 4] = np.arange(R) / (R - 1)
    eye, up_in = np.array([-1.0, -0.5, 0.0]), np.array([0.0, 0.0, 1.0])
    front = -eye / np.linalg.norm(eye)
    right = np.cross(front, up_in)
    right /= np.linalg.norm(right)
    viewport = np.stack([eye, right, np.cross(right, front)])[None]
    rs, rd = scenes.generate_rays(viewport, np.radians(45.0), W, H)
    sc = O.Scene(width=W, height=H, volume=marschner_lobb(32), tf=tf, step_size=np.full((1, 1, 1), 0.25, np.float32),
                 box_min=np.full((1, 3), -0.5, np.float32), box_size=np.ones((1, 3), np.float32),
                 filter_mode=1, camera_mode=0, tf_mode=tf_mode, blend_mode=0, ray_start=rs, ray_dir=rd)
    req = O.AdjointRequest(camera=True)
    adj = rng.normal(size=(1, H, W, 4))
    for precision, tol in (("f64", 1e-12), ("f32", 1e-5)):
        c1, t1 = O.forward(sc, "port", precision)
        c2, t2 = O.forward(sc, "reference", precision)
        assert np.array_equal(t1, t2) and t2.max() >= 3, precision
        assert symmetric_error(c1, c2) <= tol, precision
        g1 = O.adjoint(sc, c2, t2, adj, req, "port", precision)
        g2 = O.adjoint(sc, c2, t2, adj, req, "reference", precision)
        for k in ("adj_ray_start", "adj_ray_dir"):
            assert np.abs(g2[k]).max() > 0, (precision, k)
            assert symmetric_error(g1[k], g2[k]) <= tol, (precision, k)
