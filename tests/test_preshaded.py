"""Pre-shaded volumes (VolumeFilterMode/TFMode Preshaded,
renderer/renderer_interpolation.cuh:393-579, renderer/renderer_tf.cuh:818-854)
and pre-shading (TFUtils::preshadeVolume, renderer/tf_utils_impl.cu:16-170).

Pinning: the oracle's pre-shaded forward and adjoint are compared with the
reference's own templates (oracle/_ref, where the reference sources are
present): bit-identical outputs, the adjoints run on one thread so that the
order of the volume-gradient atomics is fixed.  The reference's position adjoint for pre-shaded volumes
sums its z term with the y weights' selector
(renderer/renderer_interpolation.cuh:543-548, against the scalar filter's
:368-374); the plain kernel family keeps that, the optimized family
computes the exact derivative, which the oracle's exact variant gives and
central finite differences confirm on rays that start inside the box (their
entry distance is clamped to 0, so it does not move).

GPU tolerances as the density path: forward colour within max(1e-5, 3 e32)
of the FP64 oracle (symmetric metric, pixels whose sample count agrees),
gradients relative L2 <= max(1e-3, 3 r32).
"""
import copy

import numpy as np
import pytest

from dvr_cases import make_case, rel_l2, symmetric_error


def preshaded_case(seed, blend=0, cam=0, W=12, H=10, B=2, shape=(9, 10, 11), storage_round=None):
    case = make_case(seed, tf_mode=1, filter_mode=1, blend_mode=blend, camera_mode=cam, W=W, H=H, B=B, shape=shape)
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    # smooth colours and absorption, outer layers repeated (one-sided derivatives at the faces)
    g = np.stack(np.meshgrid(np.linspace(0, 1, X), np.linspace(0, 1, Y), np.linspace(0, 1, Z), indexing="ij"))
    vol = np.empty((4, X, Y, Z), np.float32)
    for c in range(4):
        w = rng.uniform(1, 4, 3)
        ph = rng.uniform(0, 6, 3)
        vol[c] = 0.5 + 0.45 * np.sin(w[0] * g[0] * 3 + ph[0]) * np.cos(w[1] * g[1] * 3 + ph[1]) * \
            np.sin(w[2] * g[2] * 3 + ph[2])
    vol[3] *= 6.0
    vol[:, 0], vol[:, -1] = vol[:, 1], vol[:, -2]
    vol[:, :, 0], vol[:, :, -1] = vol[:, :, 1], vol[:, :, -2]
    vol[:, :, :, 0], vol[:, :, :, -1] = vol[:, :, :, 1], vol[:, :, :, -2]
    if storage_round is not None:
        vol = storage_round(vol)
    case.volume = vol
    case.filter_mode = 3
    case.tf_mode = 5
    case.tf = np.zeros((1, 1, 1), np.float32)
    return case


# ------------------------------------------------------------------ oracle (CPU)
@pytest.mark.parametrize("blend", [0, 1])
@pytest.mark.parametrize("cam", [0, 1, 2])
def test_oracle_preshaded_matches_reference(blend, cam, oracle_built):
    O = oracle_built
    if not O.reference_available():
        pytest.skip("the reference's CPU templates are not built here")
    case = preshaded_case(21 + cam, blend, cam, W=7, H=6)
    sc = case.oracle_scene()
    g = np.random.default_rng(4).standard_normal((sc.batch(), sc.height, sc.width, 4))
    req = dict(volume=True, camera=cam == 0, stepsize=True)
    for prec in ("f64", "f32"):
        cp, tp = O.forward(sc, "port", prec)
        cr, tr = O.forward(sc, "reference", prec)
        assert np.array_equal(tp, tr) and np.array_equal(cp, cr)
        prev = O.set_threads(1)  # deterministic atomic sums: bit-identical then
        try:
            ap = O.adjoint(sc, cp, tp, g, O.AdjointRequest(**req), "port", prec)
            ar = O.adjoint(sc, cr, tr, g, O.AdjointRequest(**req), "reference", prec)
        finally:
            O.set_threads(prev)
        for k in ap:
            assert np.array_equal(ap[k], ar[k]), (prec, k)


def _inside_rays_case(seed, blend=0):
    """Rays that start inside the box: their entry distance is clamped to 0."""
    case = preshaded_case(seed, blend, 0, W=6, H=5, B=1)
    rng = np.random.default_rng(seed)
    n = case.width * case.height
    start = rng.uniform(-0.3, 0.3, (1, case.height, case.width, 3))
    d = rng.standard_normal((1, case.height, case.width, 3))
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    case.ray_start, case.ray_dir = start.astype(np.float32), d.astype(np.float32)
    assert n > 0
    return case


def test_oracle_preshaded_exact_position_adjoint_matches_finite_differences(oracle_built):
    O = oracle_built
    case = _inside_rays_case(31)
    sc = case.oracle_scene()
    for name in ("volume", "ray_start", "ray_dir", "box_min", "box_size", "step_size"):
        setattr(sc, name, np.asarray(getattr(sc, name), np.float64))
    col, term = O.forward(sc)
    g = np.random.default_rng(6).standard_normal(col.shape)
    exact = O.adjoint(sc, col, term, g, O.AdjointRequest(camera=True), exact_preshaded=True)
    ref = O.adjoint(sc, col, term, g, O.AdjointRequest(camera=True))
    h = 1e-7
    for arr, key in (("ray_start", "adj_ray_start"), ("ray_dir", "adj_ray_dir")):
        fd = np.zeros_like(exact[key])
        for c in range(3):
            s1, s2 = copy.deepcopy(sc), copy.deepcopy(sc)
            a1 = getattr(sc, arr).copy()
            a1[..., c] += h
            setattr(s1, arr, a1)
            a2 = getattr(sc, arr).copy()
            a2[..., c] -= h
            setattr(s2, arr, a2)
            c1, t1 = O.forward(s1)
            c2, t2 = O.forward(s2)
            assert np.array_equal(t1, term) and np.array_equal(t2, term)
            fd[..., c] = np.sum(g * (c1 - c2) / (2 * h), axis=-1)
        assert rel_l2(exact[key], fd) <= 1e-5, key
        # x and y terms agree with the reference's; its z term does not
        assert rel_l2(ref[key][..., :2], fd[..., :2]) <= 1e-5
        assert rel_l2(ref[key][..., 2], fd[..., 2]) > 1e-2


@pytest.mark.parametrize("tfm", [0, 1, 2, 3])
def test_oracle_preshade_volume_adjoint_matches_finite_differences(tfm, oracle_built):
    O = oracle_built
    case = make_case(41, tf_mode=tfm, W=4, H=4, B=1, shape=(5, 6, 7))
    # densities strictly inside (0, 1): the identity TF's clamp and the linear TF's end points are kinks
    density = 0.05 + 0.9 * case.volume[:1].astype(np.float64)
    tf = case.tf[:1].astype(np.float64)
    g = np.random.default_rng(8).standard_normal((4,) + density.shape[1:])
    adj = O.preshade_volume_adjoint(density, tf, tfm, g)
    h = 1e-7
    fd = np.sum(g * (O.preshade_volume(density + h, tf, tfm) - O.preshade_volume(density - h, tf, tfm)) / (2 * h),
                axis=0)[None]
    assert rel_l2(adj, fd) <= 1e-6


# ------------------------------------------------------------------ GPU
def _gpu_render(case, family, vdt=None):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    pr.set_kernel_family(family)
    inp = case.inputs("cuda", vdt)
    B = case.batch()
    out = pr.RendererOutputs(torch.full((B, case.height, case.width, 4), float("nan"), device="cuda"),
                             torch.full((B, case.height, case.width), -7, dtype=torch.int32, device="cuda"))
    pr.Renderer.render_forward(inp, out)
    torch.cuda.synchronize()
    return inp, out


def _forward_ok(O, case, color, term):
    sc = case.oracle_scene()
    c32, t32 = O.forward(sc, "port", "f32")
    c64, t64 = O.forward(sc, "port", "f64")
    agree = t32 == t64
    e32 = symmetric_error(c32[agree], c64[agree])
    tol = max(1e-5, 3 * e32)
    same = term == t64
    assert np.mean(~same) <= 0.02
    assert np.all(np.abs(term[~same] - t64[~same]) <= 1)
    assert symmetric_error(color[same], c64[same]) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["plain", "optimized"])
def test_preshaded_forward_all_modes(family, oracle_built, cuda_device):
    O = oracle_built
    for blend in (0, 1):
        for cam in (0, 1, 2):
            case = preshaded_case(50 + 3 * blend + cam, blend, cam)
            _, out = _gpu_render(case, family)
            _forward_ok(O, case, out.color.cpu().numpy(), out.terminationIndex.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("vdt", ["float16", "bfloat16"])
def test_preshaded_forward_half_storage(vdt, oracle_built, cuda_device):
    import torch
    dt = getattr(torch, vdt)
    case = preshaded_case(61, 0, 0, storage_round=lambda v: torch.from_numpy(v).to(dt).float().numpy())
    _, out = _gpu_render(case, "optimized", dt)
    _forward_ok(oracle_built, case, out.color.cpu().numpy(), out.terminationIndex.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["plain", "optimized"])
def test_preshaded_adjoint(family, oracle_built, cuda_device):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    O = oracle_built
    failures = []
    for blend in (0, 1):
        for cam in (0, 2):
            case = preshaded_case(70 + 2 * blend + cam, blend, cam)
            inp, out = _gpu_render(case, family)
            B, H, W = case.batch(), case.height, case.width
            g = np.random.default_rng(9).standard_normal((B, H, W, 4)).astype(np.float32) * 0.1
            a = pr.AdjointOutputs()
            a.has_volume_derivatives = True
            a.adj_volume = torch.zeros(case.volume.shape, device="cuda")
            if cam == 0:
                a.has_camera_derivatives = True
                a.adj_camera_ray_start = torch.zeros(B, H, W, 3, device="cuda")
                a.adj_camera_ray_dir = torch.zeros(B, H, W, 3, device="cuda")
            step = family == "plain"
            if step:
                a.has_stepsize_derivatives = True
                a.adj_stepsize = torch.zeros(B, H, W, device="cuda")
            pr.Renderer.render_adjoint(inp, out, torch.from_numpy(g).cuda(), a)
            torch.cuda.synchronize()
            got = {"adj_volume": a.adj_volume.cpu().numpy()}
            if cam == 0:
                got["adj_ray_start"] = a.adj_camera_ray_start.cpu().numpy()
                got["adj_ray_dir"] = a.adj_camera_ray_dir.cpu().numpy()
            if step:
                got["adj_stepsize"] = a.adj_stepsize.cpu().numpy()
            sc = case.oracle_scene()
            exact = family == "optimized"
            req = O.AdjointRequest(volume=True, camera=cam == 0, stepsize=step)
            c64, t64 = O.forward(sc, "port", "f64")
            c32, t32 = O.forward(sc, "port", "f32")
            r64 = O.adjoint(sc, c64, t64, g, req, "port", "f64", exact_preshaded=exact)
            r32 = O.adjoint(sc, c32, t32, g, req, "port", "f32", exact_preshaded=exact)
            for k, v in got.items():
                tol = max(1e-3, 3 * rel_l2(r32[k], r64[k]))
                err = rel_l2(v, r64[k])
                if not err <= tol:
                    failures.append((blend, cam, k, err, tol))
    assert not failures, failures


@pytest.mark.gpu
@pytest.mark.parametrize("tfm", [0, 1, 2, 3])
def test_preshade_volume_parity(tfm, oracle_built, cuda_device):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    O = oracle_built
    case = make_case(81 + tfm, tf_mode=tfm, W=4, H=4, B=1, shape=(17, 18, 19))
    density = torch.from_numpy(case.volume[:1].copy()).cuda().requires_grad_(True)
    tf = torch.from_numpy(case.tf[:1].copy()).cuda()
    color = pr.TFUtils.preshade_volume(density, tf, pr.TFMode(tfm))
    ref = O.preshade_volume(case.volume[:1], case.tf[:1], tfm)
    assert symmetric_error(color.detach().cpu().numpy(), ref) <= 1e-6
    g = torch.randn(color.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    (color * g).sum().backward()
    adj = O.preshade_volume_adjoint(case.volume[:1], case.tf[:1], tfm, g.cpu().numpy())
    assert rel_l2(density.grad.cpu().numpy(), adj) <= 1e-5


@pytest.mark.gpu
def test_preshade_then_render_autograd(oracle_built, cuda_device):
    """density -> preshade_volume -> pre-shaded rendering -> loss; the density
    gradient through both adjoints against the oracle's."""
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from diffdvr_gb300.renderer import Renderer
    O = oracle_built
    case = make_case(91, tf_mode=1, W=12, H=10, B=2, shape=(9, 10, 11), pad_faces=True)
    settings = case.inputs("cuda")
    settings.volume_filter_mode = pr.VolumeFilterMode.Preshaded
    settings.tf_mode = pr.TFMode.Preshaded
    tf = torch.from_numpy(case.tf[:1].copy()).cuda()
    density = torch.from_numpy(case.volume[:1].copy()).cuda().requires_grad_(True)
    r = Renderer(settings, optimize_volume=True)
    color = pr.TFUtils.preshade_volume(density, tf, pr.TFMode.Texture)
    img = r(volume=color, tf=torch.zeros(1, 1, 1, device="cuda"))
    g = torch.linspace(-1, 1, img.numel(), device="cuda").reshape(img.shape)
    (img * g).sum().backward()
    # oracle: the same chain with the exact adjoints
    rgba = O.preshade_volume(case.volume[:1], case.tf[:1], 1)
    pc = copy.deepcopy(case)
    pc.volume, pc.filter_mode, pc.tf_mode, pc.tf = rgba.astype(np.float32), 3, 5, np.zeros((1, 1, 1), np.float32)
    sc = pc.oracle_scene()
    sc.volume = rgba
    col, term = O.forward(sc)
    assert symmetric_error(img.detach().cpu().numpy(), col) <= 1e-4
    adj_rgba = O.adjoint(sc, col, term, g.cpu().numpy(), O.AdjointRequest(volume=True), exact_preshaded=True)
    ref = O.preshade_volume_adjoint(case.volume[:1], case.tf[:1], 1, adj_rgba["adj_volume"])
    assert rel_l2(density.grad.cpu().numpy(), ref) <= 1e-3


@pytest.mark.gpu
def test_preshaded_validation(cuda_device):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from diffdvr_gb300._abi import DvrError
    case = preshaded_case(95, W=6, H=5, B=1)
    inp = case.inputs("cuda")
    out = pr.RendererOutputs(torch.empty(1, 5, 6, 4, device="cuda"),
                             torch.empty(1, 5, 6, dtype=torch.int32, device="cuda"))
    pr.Renderer.render_forward(inp, out)
    bad = inp.clone()
    bad.tf_mode = pr.TFMode.Texture
    with pytest.raises(DvrError, match="both the filter mode and TF mode must be set to preshaded"):
        pr.Renderer.render_forward(bad, out)
    bad = inp.clone()
    bad.volume = inp.volume[:3]
    with pytest.raises(DvrError, match="It must be 4, but is 3"):
        pr.Renderer.render_forward(bad, out)
    with pytest.raises(DvrError, match="single-instance"):
        pr.Renderer.render_forward_batched([inp], [out])
    s = pr.ForwardDifferencesSettings()
    s.D, s.d_stepsize = 1, 0
    with pytest.raises(DvrError, match="pre-shaded"):
        pr.Renderer.render_forward_gradients(inp, s, out, torch.empty(1, 5, 6, 1, 4, device="cuda"))
    a = pr.AdjointOutputs()
    a.has_volume_derivatives = True
    a.adj_volume = torch.zeros(1, *case.volume.shape[1:], device="cuda")
    with pytest.raises(DvrError, match="adj_volume"):
        pr.Renderer.render_adjoint(inp, out, torch.zeros(1, 5, 6, 4, device="cuda"), a)
    # the no-allocation adjoint does not order rays in library scratch: it refuses pre-shaded volumes
    from test_zz_no_alloc import _adjoint_through_abi
    from diffdvr_gb300 import _abi
    with pytest.raises(DvrError, match="pre-shaded volumes take dvr_render_adjoint"):
        _adjoint_through_abi(_abi.load().dvr_render_adjoint_noalloc, case, inp, out,
                             torch.zeros(1, 5, 6, 4, device="cuda"))


@pytest.mark.gpu
@pytest.mark.parametrize("pool", ["full", 0.5])
def test_preshaded_adjoint_from_record(pool, oracle_built, cuda_device):
    """The optimized adjoint from the pre-shaded forward's sample record (one
    warp per ray; rays without room in the pool go through the per-lane
    kernel): volume and camera gradients against the oracle's exact variant,
    and all gradients, step size included, against the per-lane kernel
    without a record (relative L2 <= 1e-4: the record's opacities against
    the inverted blend)."""
    from dvr_cases import gpu_adjoint, gpu_forward
    O = oracle_built
    case = preshaded_case(97, 0, 0, W=40, H=36, B=2, shape=(20, 24, 28))
    inp, out = gpu_forward(case, record="full")
    if pool != "full":
        t = out.terminationIndex.cpu().numpy()
        inp, out = gpu_forward(case, record=int(pool * 4 * ((t + 1) // 2).sum()))
    off = out.sample_offset.cpu().numpy()
    term = out.terminationIndex.cpu().numpy()
    assert (off[term == 0] == -1).all()
    if pool == "full":
        assert (off[term > 0] >= 0).all()
    else:
        assert ((term > 0) & (off == -1)).any() and ((term > 0) & (off >= 0)).any()
    g = np.random.default_rng(12).standard_normal(out.color.shape).astype(np.float32) * 0.1
    got = gpu_adjoint(case, inp, out, g, volume=True, camera=True, stepsize=True)
    _, plain = gpu_forward(case)
    lane = gpu_adjoint(case, inp, plain, g, volume=True, camera=True, stepsize=True)
    for k in got:
        assert rel_l2(got[k], lane[k]) <= 1e-4, (k, rel_l2(got[k], lane[k]))
    sc = case.oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    c32, t32 = O.forward(sc, "port", "f32")
    req = O.AdjointRequest(volume=True, camera=True)
    r64 = O.adjoint(sc, c64, t64, g, req, "port", "f64", exact_preshaded=True)
    r32 = O.adjoint(sc, c32, t32, g, req, "port", "f32", exact_preshaded=True)
    for k in r64:
        tol = max(1e-3, 3 * rel_l2(r32[k], r64[k]))
        assert rel_l2(got[k], r64[k]) <= tol, (k, rel_l2(got[k], r64[k]), tol)
