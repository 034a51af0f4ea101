"""Forward-mode differentiation: renderForwardGradients and
forwardVariablesToGradients (renderer/renderer_kernels.cuh:131-240, :505-560).

The reference's forward mode is built on its dual-number library cudAD, which
is not part of the reference sources, so its kernels cannot be compiled
here.  The oracle restates the forward derivatives directly and is pinned by
the identity that ties the two gradient methods together: contracting the
forward variables with a colour adjoint must give the adjoint method's
gradients, and the adjoint method is pinned to the reference's own CPU
templates (tests/test_oracle.py).  Tolerance of that identity: relative L2
<= 1e-9 in FP64, except the Gaussian TF's sigma gradient, which the
reference's adjoint rounds through float (renderer/renderer_tf.cuh:591):
<= 1e-6.  The step-size derivative is checked against central finite
differences instead, because the reference's adjoint assigns rather than
accumulates the per-sample blend term of the step size
(renderer/renderer_blending.cuh:93, :158; the oracle's adjoint keeps this).

GPU parity: the CUDA forward variables against the FP64 oracle, on pixels
whose sample count agrees, relative L2 <= max(1e-3, 3 * r32) per variable
group with r32 the FP32 oracle's own error; colour and termination as the
forward tests check them.
"""
import copy

import numpy as np
import pytest

from dvr_cases import make_case, rel_l2, symmetric_error

MODES = [(tfm, filt, blend) for tfm in (0, 1, 2, 3) for filt in (0, 1) for blend in (0, 1)]


def _settings(O, case, camera=True, step=True, tf=True):
    D = 0
    kw = {}
    if camera:
        kw["d_ray_start"], kw["d_ray_dir"] = (0, 1, 2), (3, 4, 5)
        D = 6
    if step:
        kw["d_stepsize"] = D
        D += 1
    if tf:
        B, R, C = case.tf.shape
        kw["d_tf"] = np.arange(D, D + R * C, dtype=np.int32).reshape(1, R, C).repeat(B, 0)
        D += R * C
    return O.ForwardSettings(D=D, **kw)


# ------------------------------------------------------------------ oracle (CPU)
@pytest.mark.parametrize("tfm,filt,blend", MODES)
def test_oracle_forward_mode_values_match_forward(tfm, filt, blend, oracle_built):
    O = oracle_built
    for cam in (0, 2):
        case = make_case(11, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam, W=6, H=5, B=2)
        sc = case.oracle_scene()
        col, term, J = O.forward_gradients(sc, _settings(O, case))
        c0, t0 = O.forward(sc)
        assert np.array_equal(term, t0)
        assert np.array_equal(col, c0)
        assert np.all(np.isfinite(J))


@pytest.mark.parametrize("tfm,filt,blend", MODES)
@pytest.mark.parametrize("kind", ["port", "reference"])
def test_oracle_forward_mode_matches_adjoint(tfm, filt, blend, kind, oracle_built):
    """forward variables contracted with adj_color == the adjoint method."""
    O = oracle_built
    if kind == "reference" and not O.reference_available():
        pytest.skip("the reference's CPU templates are not built here")
    case = make_case(12, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=0, W=7, H=6, B=2)
    sc = case.oracle_scene()
    fs = _settings(O, case, step=False)
    col, term, J = O.forward_gradients(sc, fs)
    g = np.random.default_rng(3).standard_normal(col.shape)
    req = O.AdjointRequest(tf=True, camera=True)
    adj = O.adjoint(sc, col, term, g, req, kind=kind)
    fv = O.forward_variables_to_gradients(J, g, fs, O.AdjointRequest(tf=True, camera=True))
    for key in ("adj_ray_start", "adj_ray_dir"):
        assert rel_l2(fv[key], adj[key]) <= 1e-9, key
    if tfm == 3:
        assert rel_l2(fv["adj_tf"][..., :5], adj["adj_tf"][..., :5]) <= 1e-9
        assert rel_l2(fv["adj_tf"][..., 5], adj["adj_tf"][..., 5]) <= 1e-6
    else:
        assert rel_l2(fv["adj_tf"], adj["adj_tf"]) <= 1e-9


@pytest.mark.parametrize("tfm,filt,blend", MODES)
def test_oracle_forward_mode_stepsize_finite_differences(tfm, filt, blend, oracle_built):
    O = oracle_built
    case = make_case(13, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=0, W=6, H=5, B=1)
    sc = case.oracle_scene()
    for name in ("volume", "tf", "ray_start", "ray_dir", "box_min", "box_size"):
        setattr(sc, name, np.asarray(getattr(sc, name), np.float64))
    fs = O.ForwardSettings(D=1, d_stepsize=0)
    _, term, J = O.forward_gradients(sc, fs)
    st = float(np.asarray(sc.step_size).ravel()[0])
    h = st * 1e-6
    s1, s2 = copy.deepcopy(sc), copy.deepcopy(sc)
    s1.step_size = np.full((1, 1, 1), st + h)
    s2.step_size = np.full((1, 1, 1), st - h)
    c1, t1 = O.forward(s1)
    c2, t2 = O.forward(s2)
    ok = (t1 == term) & (t2 == term)
    assert ok.mean() > 0.9
    assert rel_l2(J[..., 0, :][ok], ((c1 - c2) / (2 * h))[ok]) <= 1e-6


def test_oracle_forward_mode_tf_finite_differences(oracle_built):
    """TF derivatives against central differences, every TF mode (FP64)."""
    O = oracle_built
    for tfm in (0, 1, 2, 3):
        case = make_case(14, tf_mode=tfm, filter_mode=1, blend_mode=0, camera_mode=0, W=5, H=4, B=1)
        sc = case.oracle_scene()
        for name in ("volume", "tf", "ray_start", "ray_dir", "box_min", "box_size"):
            setattr(sc, name, np.asarray(getattr(sc, name), np.float64))
        fs = _settings(O, case, camera=False, step=False)
        _, term, J = O.forward_gradients(sc, fs)
        R, C = sc.tf.shape[1:]
        for r in range(R):
            for c in range(C):
                h = 1e-7
                s1, s2 = copy.deepcopy(sc), copy.deepcopy(sc)
                s1.tf = sc.tf.copy()
                s1.tf[0, r, c] += h
                s2.tf = sc.tf.copy()
                s2.tf[0, r, c] -= h
                c1, t1 = O.forward(s1)
                c2, t2 = O.forward(s2)
                ok = (t1 == term) & (t2 == term)
                fd = ((c1 - c2) / (2 * h))[ok]
                an = J[..., r * C + c, :][ok]
                assert np.max(np.abs(an - fd)) <= 1e-5 * max(1.0, np.max(np.abs(fd))), (tfm, r, c)


# ------------------------------------------------------------------ GPU
def _gpu_forward_gradients(case, fs, volume_dtype=None):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    inp = case.inputs("cuda", volume_dtype)
    B = case.batch()
    color = torch.full((B, case.height, case.width, 4), float("nan"), device="cuda")
    term = torch.full((B, case.height, case.width), -7, dtype=torch.int32, device="cuda")
    grads = torch.full((B, case.height, case.width, fs.D, 4), float("nan"), device="cuda")
    s = pr.ForwardDifferencesSettings()
    s.D = fs.D
    s.d_stepsize = fs.d_stepsize
    s.d_rayStart = pr.int3(*fs.d_ray_start)
    s.d_rayDir = pr.int3(*fs.d_ray_dir)
    if fs.d_tf is not None:
        s.d_tf = torch.from_numpy(np.ascontiguousarray(fs.d_tf, np.int32)).cuda()
        s.has_tf_derivatives = True
    pr.Renderer.render_forward_gradients(inp, s, pr.RendererOutputs(color, term), grads)
    torch.cuda.synchronize()
    return s, color.cpu().numpy(), term.cpu().numpy(), grads.cpu().numpy()


def _groups(fs):
    g = {}
    if fs.d_ray_start[0] >= 0:
        g["camera"] = list(fs.d_ray_start) + list(fs.d_ray_dir)
    if fs.d_stepsize >= 0:
        g["step"] = [fs.d_stepsize]
    if fs.d_tf is not None:
        g["tf"] = sorted(set(int(i) for i in np.asarray(fs.d_tf).ravel() if i >= 0))
    return g


def _check_against_oracle(O, case, fs, color, term, J):
    sc = case.oracle_scene()
    c64, t64, J64 = O.forward_gradients(sc, fs, "f64")
    c32, t32, J32 = O.forward_gradients(sc, fs, "f32")
    same = (term == t64) & (t32 == t64)
    assert np.mean(term != t64) <= 0.02
    assert symmetric_error(color[same], c64[same]) <= 1e-4
    bad = []
    for name, idx in _groups(fs).items():
        ref = J64[same][:, idx]
        r32 = rel_l2(J32[same][:, idx], ref)
        err = rel_l2(J[same][:, idx], ref)
        tol = max(1e-3, 3 * r32)
        if not err <= tol:
            bad.append(f"{name}: rel L2 {err:.2e} > {tol:.1e}")
    return bad


@pytest.mark.gpu
def test_forward_gradients_all_modes(oracle_built, cuda_device):
    O = oracle_built
    failures = {}
    for i, (tfm, filt, blend) in enumerate(MODES):
        for cam in (0, 1, 2):
            case = make_case(300 + 3 * i + cam, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam,
                             W=12, H=10, B=2, pad_faces=True)
            fs = _settings(O, case)
            _, color, term, J = _gpu_forward_gradients(case, fs)
            bad = _check_against_oracle(O, case, fs, color, term, J)
            if bad:
                failures[(tfm, filt, blend, cam)] = bad
    assert not failures, failures


@pytest.mark.gpu
@pytest.mark.parametrize("vdt", ["float16", "bfloat16"])
def test_forward_gradients_half_volumes(vdt, oracle_built, cuda_device):
    import torch
    O = oracle_built
    dt = getattr(torch, vdt)
    case = make_case(341, tf_mode=1, filter_mode=1, blend_mode=0, camera_mode=0, W=12, H=10, B=2, pad_faces=True)
    # the oracle renders the rounded volume
    case.volume = torch.from_numpy(case.volume).to(dt).float().numpy()
    fs = _settings(O, case)
    _, color, term, J = _gpu_forward_gradients(case, fs, dt)
    bad = _check_against_oracle(O, case, fs, color, term, J)
    assert not bad, bad


@pytest.mark.gpu
def test_forward_gradients_several_passes_and_shared_indices(oracle_built, cuda_device):
    """D above one launch's range (1024 indices), indices shared between
    variables (derivatives add up) and untraced TF entries."""
    O = oracle_built
    case = make_case(342, tf_mode=1, filter_mode=1, blend_mode=0, camera_mode=0, W=9, H=7, B=1, R=300,
                     pad_faces=True)
    B, R, C = case.tf.shape
    d_tf = (7 + np.arange(R * C, dtype=np.int32)).reshape(B, R, C)
    d_tf[:, ::7, :] = -1          # not traced
    d_tf[:, 5, 3] = 2             # shares the index of ray_start.z
    d_tf[:, 6, :] = d_tf[:, 8, :]  # two entries on one index
    fs = O.ForwardSettings(D=7 + R * C, d_stepsize=6, d_ray_start=(0, 1, 2), d_ray_dir=(3, 4, 5), d_tf=d_tf)
    assert fs.D > 1024
    _, color, term, J = _gpu_forward_gradients(case, fs)
    bad = _check_against_oracle(O, case, fs, color, term, J)
    assert not bad, bad
    # untraced indices hold zeros
    unused = sorted(set(range(fs.D)) - set(int(i) for i in d_tf.ravel()) - set(range(7)))
    assert unused and np.all(J[..., unused, :] == 0)


@pytest.mark.gpu
def test_forward_variables_to_gradients_parity(oracle_built, cuda_device):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    O = oracle_built
    case = make_case(343, tf_mode=2, filter_mode=1, blend_mode=0, camera_mode=0, W=12, H=10, B=2, pad_faces=True)
    fs = _settings(O, case)
    s, color, term, J = _gpu_forward_gradients(case, fs)
    g = np.random.default_rng(5).standard_normal(color.shape).astype(np.float32)
    B, H, W = color.shape[:3]
    a = pr.AdjointOutputs()
    a.has_camera_derivatives = True
    a.adj_camera_ray_start = torch.zeros(B, H, W, 3, device="cuda")
    a.adj_camera_ray_dir = torch.zeros(B, H, W, 3, device="cuda")
    a.has_stepsize_derivatives = True
    a.adj_stepsize = torch.zeros(B, H, W, device="cuda")
    a.has_tf_derivatives = True
    a.adj_tf = torch.zeros(case.tf.shape, device="cuda")
    pr.Renderer.forward_variables_to_gradients(torch.from_numpy(J).cuda(), torch.from_numpy(g).cuda(), s, a)
    torch.cuda.synchronize()
    ref = O.forward_variables_to_gradients(J.astype(np.float64), g, fs,
                                           O.AdjointRequest(tf=True, camera=True, stepsize=True))
    assert rel_l2(a.adj_camera_ray_start.cpu().numpy(), ref["adj_ray_start"]) <= 1e-5
    assert rel_l2(a.adj_camera_ray_dir.cpu().numpy(), ref["adj_ray_dir"]) <= 1e-5
    assert rel_l2(a.adj_stepsize.cpu().numpy(), ref["adj_stepsize"]) <= 1e-5
    assert rel_l2(a.adj_tf.cpu().numpy(), ref["adj_tf"]) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("delayed", [False, True])
def test_autograd_forward_method_matches_adjoint_method(delayed, cuda_device):
    """diffdvr.Renderer(gradient_method="forward") gives the adjoint method's
    TF and camera (viewport) gradients."""
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from diffdvr_gb300.renderer import Renderer
    case = make_case(344, tf_mode=1, filter_mode=1, blend_mode=0, camera_mode=2, W=16, H=12, B=2, pad_faces=True)
    settings = case.inputs("cuda")
    viewport = torch.from_numpy(case.camera_matrix).cuda()
    grads = {}
    for method in ("adjoint", "forward"):
        r = Renderer(settings.clone(), optimize_camera=True, optimize_tf=True, gradient_method=method,
                     forward_delayed_gradients=delayed, fused_camera=False)
        tf = torch.from_numpy(case.tf).cuda().requires_grad_(True)
        cam = viewport.clone().requires_grad_(True)
        img = r(camera=cam, fov_y_radians=case.fov_y, tf=tf, volume=settings.volume)
        target = torch.linspace(0, 1, img.numel(), device="cuda").reshape(img.shape)
        ((img - target) ** 2).sum().backward()
        grads[method] = (tf.grad.cpu().numpy(), cam.grad.cpu().numpy(), img.detach().cpu().numpy())
    assert np.allclose(grads["adjoint"][2], grads["forward"][2], atol=1e-5)
    assert rel_l2(grads["forward"][0], grads["adjoint"][0]) <= 1e-3
    assert rel_l2(grads["forward"][1], grads["adjoint"][1]) <= 1e-3


@pytest.mark.gpu
def test_forward_gradients_validation(cuda_device):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from diffdvr_gb300._abi import DvrError
    case = make_case(345, tf_mode=1, W=6, H=5, B=1)
    inp = case.inputs("cuda")
    out = pr.RendererOutputs(torch.empty(1, 5, 6, 4, device="cuda"),
                             torch.empty(1, 5, 6, dtype=torch.int32, device="cuda"))

    def run(s, D=None, dtype=torch.float32):
        grads = torch.empty(1, 5, 6, s.D if D is None else D, 4, device="cuda", dtype=dtype)
        pr.Renderer.render_forward_gradients(inp, s, out, grads)

    s = pr.ForwardDifferencesSettings()
    with pytest.raises(DvrError, match="number of derivatives must be positive"):
        run(s, D=1)
    s.D = 3
    with pytest.raises(DvrError, match="at least one derivative must be activated"):
        run(s)
    s.d_stepsize = 3
    with pytest.raises(DvrError, match="d_stepsize"):
        run(s)
    s.d_stepsize = 0
    with pytest.raises(DvrError, match="gradientsOut"):
        run(s, D=2)
    with pytest.raises(DvrError, match="float32"):
        run(s, dtype=torch.float64)
    s.has_tf_derivatives = True
    with pytest.raises(DvrError, match="d_tf not defined"):
        run(s)
    s.d_tf = torch.zeros(case.tf.shape, dtype=torch.float32, device="cuda")
    with pytest.raises(DvrError, match="int32"):
        run(s)
    s.d_tf = torch.zeros((1, 2, 4), dtype=torch.int32, device="cuda")
    with pytest.raises(DvrError, match="d_tf"):
        run(s)
    s.d_tf = torch.full(case.tf.shape, -1, dtype=torch.int32, device="cuda")
    run(s)
    a = pr.AdjointOutputs()
    a.has_volume_derivatives = True
    a.adj_volume = torch.zeros(case.volume.shape, device="cuda")
    with pytest.raises(DvrError, match="volume derivatives are not supported"):
        pr.Renderer.forward_variables_to_gradients(torch.zeros(1, 5, 6, 3, 4, device="cuda"),
                                                   torch.zeros(1, 5, 6, 4, device="cuda"), s, a)
