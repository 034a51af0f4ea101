"""GPU parity: the CUDA kernels (through the C ABI) against the oracle and
the reference fixtures, for every mode combination and both kernel families.

Tolerances (stated per check):
* forward colour: the reference's symmetric metric |a-b|/max(1,|a|+|b|)
  against the FP64 oracle <= tol = max(1e-5, 3 * e32), where e32 is the
  same metric between the reference's own FP32 and FP64 computations of the
  case (the inverse-view-matrix camera is ill-conditioned in FP32: e32 reaches
  2e-5); against the FP32 oracle <= tol + e32.  Compared on pixels whose
  sample count agrees; the count may differ by one on rays whose last sample
  sits on the box exit or the early-out threshold up to rounding (<= 2% of
  pixels).  With nearest filtering a sample within rounding of a voxel
  boundary may pick the neighbouring voxel, so up to 2% of pixels may exceed
  tol there.
* gradients: relative L2 error against the FP64 oracle (forward + adjoint in
  FP64) <= max(1e-3, 3 * r32), r32 the reference FP32 build's own relative
  error, and at most 1% of entries off by more than 1e-3 of the largest
  reference entry.  Test volumes
  keep densities inside (0, 1) and repeat the outermost layers, so the
  derivatives of the identity TF and of the trilinear position are continuous
  at the box faces (rays entering through a face at the maximum coordinate
  have their first sample on the face, where the reference's derivative is
  one-sided).  Adjoint scenes keep rays short of opaque, where the reference's
  blend inversion (used by the plain family) is ill-conditioned in FP32; the
  checkpointed adjoint is checked on opaque rays separately.
"""
import numpy as np
import pytest
import torch

from dvr_cases import (all_mode_combos, golden, golden_case, golden_prefixes, gpu_adjoint, gpu_forward, make_case,
                       rel_l2, symmetric_error)

pytestmark = pytest.mark.gpu

FAMILIES = ["plain", "optimized"]


def _pixel_errors(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(1.0, np.abs(a) + np.abs(b)), axis=-1)


def _forward_errors(case, color, term, O, max_mismatch=0.02):
    """List of failed checks (empty when the forward output matches)."""
    sc = case.oracle_scene()
    c32, t32 = O.forward(sc, "port", "f32")
    c64, t64 = O.forward(sc, "port", "f64")
    agree = t32 == t64
    e32 = symmetric_error(c32[agree], c64[agree])
    tol64 = max(1e-5, 3 * e32)
    outliers = 0.02 if case.filter_mode == 0 else 0.0
    bad = []
    for prec, oc, ot, tol in (("f64", c64, t64, tol64), ("f32", c32, t32, tol64 + e32)):
        same = term == ot
        if np.mean(~same) > max_mismatch:
            bad.append(f"{prec}: termination mismatch on {np.mean(~same):.3f} of pixels")
        if not np.all(np.abs(term[~same] - ot[~same]) <= 1):
            bad.append(f"{prec}: termination index off by more than one")
        pe = _pixel_errors(color[same], oc[same])
        if pe.size and np.mean(pe > tol) > outliers:
            bad.append(f"{prec}: colour error {pe.max():.2e} > {tol:.1e} on {np.mean(pe > tol):.3f} of pixels")
    return bad


def _compare_forward(case, color, term, O):
    bad = _forward_errors(case, color, term, O)
    assert not bad, bad


@pytest.mark.parametrize("family", FAMILIES)
def test_forward_all_modes(family, oracle_built, cuda_device):
    O = oracle_built
    failures = {}
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(200 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam)
        _, out = gpu_forward(case, family)
        bad = _forward_errors(case, out.color.cpu().numpy(), out.terminationIndex.cpu().numpy(), O)
        if bad:
            failures[(tfm, filt, blend, cam)] = bad
    assert not failures, failures


@pytest.mark.parametrize("sort", [True, False], ids=["sorted-positions", "unsorted-positions"])
def test_linear_tf_interval_search(sort, oracle_built, cuda_device):
    """The optimized kernels search a piecewise-linear TF's control points
    by bisection when their positions are non-decreasing, and keep the
    reference's first-match scan when they are not
    (renderer/renderer_tf.cuh:294-300): 16 points, forward and adjoint
    (TF, volume and ray gradients) against the FP64 oracle, whose scan
    defines the interval either way."""
    O = oracle_built
    case = make_case(57, tf_mode=2, R=16, shape=(18, 20, 22), W=30, H=24, B=2, opacity=0.4, pad_faces=True)
    if not sort:
        rng = np.random.default_rng(3)
        for b in range(case.tf.shape[0]):
            case.tf[b, 1:-1, 4] = rng.permutation(case.tf[b, 1:-1, 4])
        assert np.any(np.diff(case.tf[..., 4], axis=1) < 0)
    inp, out = gpu_forward(case, "optimized", checkpoints=True)
    _compare_forward(case, out.color.cpu().numpy(), out.terminationIndex.cpu().numpy(), O)
    adj = np.random.default_rng(8).normal(size=out.color.shape)
    req = O.AdjointRequest(volume=True, tf=True, camera=True)
    ref, adj = reference_adjoint(case, O, out.terminationIndex.cpu().numpy(), adj, req)
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=True)
    bad = _grad_errors(got, ref)
    assert not bad, bad


@pytest.mark.parametrize("family", FAMILIES)
def test_forward_matches_reference_fixtures(family, oracle_built, cuda_device):
    """Against the reference's own FP64 and FP32 CPU renders (fixtures), with
    the tolerances of _forward_errors (e32 taken from the two fixtures)."""
    g = golden("modes.npz")
    failures = {}
    for p in golden_prefixes(g):
        case = golden_case(g, p)
        _, out = gpu_forward(case, family)
        color, term = out.color.cpu().numpy(), out.terminationIndex.cpu().numpy()
        agree = g[p + "term_f32"] == g[p + "term_f64"]
        e32 = symmetric_error(g[p + "color_f32"][agree], g[p + "color_f64"][agree])
        tol64 = max(1e-5, 3 * e32)
        outliers = 0.02 if case.filter_mode == 0 else 0.0
        for prec, tol in (("f64", tol64), ("f32", tol64 + e32)):
            same = term == g[p + "term_" + prec]
            pe = _pixel_errors(color[same], g[p + "color_" + prec][same])
            if np.mean(~same) > 0.05 or (pe.size and np.mean(pe > tol) > outliers):
                failures[(p, prec)] = (float(np.mean(~same)), float(pe.max()), tol)
    assert not failures, failures


def _grad_errors(got, ref, r32=None):
    bad = {}
    for k in got:
        r = rel_l2(got[k], ref[k])
        tol = max(1e-3, 3 * r32[k]) if r32 else 1e-3
        scale = max(float(np.max(np.abs(ref[k]))), 1e-30)
        pe = np.abs(np.asarray(got[k], np.float64) - ref[k]) / scale
        frac = float(np.mean(pe > 1e-3))
        if r > tol or frac > 0.01:
            bad[k] = (r, tol, frac)
    return bad


def reference_adjoint(case, O, gpu_term, adj, req, oracle_case=None):
    """FP64 oracle forward + adjoint of the same scene.  Pixels whose sample
    count differs from the GPU's get a zero output adjoint, in the returned
    adj as well, so both sides sum the same rays.  (Inverting the blend from
    the GPU's FP32 colour instead would amplify its rounding by 1/(1-alpha)
    on near-opaque rays.)"""
    sc = (oracle_case or case).oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    adj = np.where((gpu_term == t64)[..., None], adj, 0.0).astype(np.float32)
    return O.adjoint(sc, c64, t64, adj, req, "port", "f64"), adj


def _adjoint_case(case, family, O, checkpoints, stepsize, interval=16, record=None):
    cam = case.camera_mode == 0
    inp, out = gpu_forward(case, family, checkpoints=checkpoints, interval=interval, record=record)
    term = out.terminationIndex.cpu().numpy()
    adj = np.random.default_rng(7).normal(size=out.color.shape).astype(np.float32)
    req = O.AdjointRequest(volume=True, tf=True, camera=cam, stepsize=stepsize)
    ref, adj = reference_adjoint(case, O, term, adj, req)
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=cam, stepsize=stepsize, family=family)
    # the reference FP32 build's own error on the same rays, as a yardstick
    sc = case.oracle_scene()
    c32, t32 = O.forward(sc, "port", "f32")
    g32 = O.adjoint(sc, c32, t32, np.where((t32 == term)[..., None], adj, 0.0), req, "port", "f32")
    r32 = {k: rel_l2(g32[k], ref[k]) for k in g32}
    return got, ref, r32


@pytest.mark.parametrize("family,checkpoints,interval,record", [
    ("plain", False, 16, None), ("optimized", False, 16, None), ("optimized", True, 16, None),
    ("optimized", True, 5, None),
    # sample densities recorded by the forward: a pool for every ray, and one
    # for about half of them (the rest re-sample the volume)
    ("optimized", True, 16, "full"), ("optimized", True, 5, 0.15)])
def test_adjoint_all_modes(family, checkpoints, interval, record, oracle_built, cuda_device):
    O = oracle_built
    failures = {}
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        case = make_case(300 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam, opacity=0.25,
                         pad_faces=True)
        # the optimized family returns the full step-size derivative, the
        # reference (and the oracle) only the last blend term; checked by FD below
        got, ref, r32 = _adjoint_case(case, family, O, checkpoints, stepsize=(family == "plain"), interval=interval,
                                      record=record)
        bad = _grad_errors(got, ref, r32)
        if bad:
            failures[(tfm, filt, blend, cam)] = bad
    assert not failures, failures


@pytest.mark.parametrize("family", FAMILIES)
def test_broadcasting_matches_reference_fixture(family, oracle_built, cuda_device):
    """Volume B=1 with TF B=2, per-pixel step sizes, box tensors; gradients of
    broadcast inputs accumulate over the batch (atomics into stride-0 outputs)."""
    g = golden("broadcast.npz")
    case = golden_case(g, "b_")
    inp, out = gpu_forward(case, family, checkpoints=(family == "optimized"))
    term = out.terminationIndex.cpu().numpy()
    same = term == g["b_term_f64"]
    assert np.mean(~same) <= 0.02
    assert symmetric_error(out.color.cpu().numpy()[same], g["b_color_f64"][same]) <= 1e-5
    if np.all(same):
        # volume and TF gradients against the reference's FP64 adjoint; the
        # plain family inverts the blend in FP32, which loses accuracy on the
        # opaque rays of this scene, so it is held to 1e-2
        tol = 1e-3 if family == "optimized" else 1e-2
        got = gpu_adjoint(case, inp, out, g["b_adj_color"], volume=True, tf=True, family=family, volume_batch=1)
        for k in got:
            assert rel_l2(got[k], g["b_" + k + "_f64"]) <= tol, (k, rel_l2(got[k], g["b_" + k + "_f64"]))
    # broadcast camera / step-size gradients equal the per-batch gradients summed
    adj = g["b_adj_color"]
    full = gpu_adjoint(case, inp, out, adj, camera=True, stepsize=True, family=family)
    bc = gpu_adjoint(case, inp, out, adj, camera=True, stepsize=True, family=family, stepsize_shape=(1, 1, 1),
                     camera_batch=1)
    for k in ("adj_ray_start", "adj_ray_dir"):
        assert np.allclose(bc[k][0], full[k].sum(0), rtol=1e-5, atol=1e-6), k
    assert np.allclose(bc["adj_stepsize"].item(), full["adj_stepsize"].sum(), rtol=1e-5, atol=1e-6)


def test_plain_adjoint_immediate_and_delayed_tf_accumulation_agree(cuda_device, oracle_built):
    case = make_case(41, tf_mode=3, R=6)
    inp, out = gpu_forward(case, "plain")
    adj = np.random.default_rng(3).normal(size=(case.batch(), case.height, case.width, 4))
    a = gpu_adjoint(case, inp, out, adj, tf=True, family="plain", delayed=True)
    b = gpu_adjoint(case, inp, out, adj, tf=True, family="plain", delayed=False)
    assert rel_l2(a["adj_tf"], b["adj_tf"]) <= 1e-5


def _nonconvex_case(d1: float):
    from dvr_cases import Case
    vol = np.zeros((1, 2, 2, 2), np.float32)
    vol[0, 0], vol[0, 1] = -1.0, d1
    return Case(width=1, height=1, volume=vol, tf=np.array([[[1, 0, 0, 1, 0, 0.5]]], np.float32), tf_mode=3,
                filter_mode=1, blend_mode=0, camera_mode=0, step=1 / 32, box_min=(0.0, 0.0, 0.0),
                box_size=(1.0, 1.0, 1.0), ray_start=np.array([[[[-1.0, 0.5, 0.5]]]], np.float32),
                ray_dir=np.array([[[[1.0, 0.0, 0.0]]]], np.float32))


@pytest.mark.parametrize("family", FAMILIES)
def test_nonconvex_density_table_on_gpu(family, cuda_device):
    """The reference's known-answer table (unittests/NonConvexDensity.tsv)
    through the CUDA kernels: colour, loss and d(loss)/d(d1)."""
    t = golden("nonconvex_density.npz")
    _, o = gpu_forward(_nonconvex_case(-1.0), family)
    gt = o.color.cpu().numpy()[0, 0, 0].astype(np.float64)
    for d1, red, alpha, loss, grad in t["table"]:
        case = _nonconvex_case(d1)
        inp, out = gpu_forward(case, family, checkpoints=(family == "optimized"))
        c = out.color.cpu().numpy()[0, 0, 0].astype(np.float64)
        assert int(out.terminationIndex.item()) == 33
        diff = c - gt
        l = float(np.linalg.norm(diff))
        adj = (diff / l if l > 0 else np.zeros(4))[None, None, None, :]
        g = gpu_adjoint(case, inp, out, adj, volume=True, family=family)
        gr = float(g["adj_volume"][0, 1].sum())
        tol = 2e-5 if abs(d1) < 100 else 1e-4
        assert abs(c[0] - red) <= tol and abs(c[3] - alpha) <= tol, d1
        assert abs(l - loss) <= tol, d1
        assert abs(gr - grad) <= 3e-5 + 2e-3 * abs(grad), (d1, gr, grad)


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
def test_reduced_precision_storage(dtype, oracle_built, cuda_device):
    """Volume and TF stored in BF16/FP16, sampled and blended in FP32: against
    the FP64 oracle on the same rounded values (forward 1e-5, gradients 1e-3)."""
    O = oracle_built
    case = make_case(51, tf_mode=1, shape=(17, 19, 21), W=24, H=20, B=2, R=16, pad_faces=True)
    rounded = lambda a: torch.from_numpy(a).to(dtype).float().numpy()
    case_r = make_case(51, tf_mode=1, shape=(17, 19, 21), W=24, H=20, B=2, R=16, pad_faces=True)
    case_r.volume, case_r.tf = rounded(case.volume), rounded(case.tf)
    inp, out = gpu_forward(case, "optimized", volume_dtype=dtype, tf_dtype=dtype, checkpoints=True)
    color, term = out.color.cpu().numpy(), out.terminationIndex.cpu().numpy()
    _compare_forward(case_r, color, term, O)
    adj = np.random.default_rng(9).normal(size=color.shape)
    ref, adj = reference_adjoint(case, O, term, adj, O.AdjointRequest(volume=True, tf=True, camera=True),
                                 oracle_case=case_r)
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=True)
    bad = _grad_errors(got, ref)
    assert not bad, bad


@pytest.mark.parametrize("record", [None, "full", 0.4], ids=["checkpoints", "full-record", "partial-record"])
def test_batched_uneven_matches_single_instances(record, cuda_device):
    """Three instances of different sizes through the batched entry points
    against single-instance calls; with a sample record every ray owns a
    fixed run of its instance's pool (rays that do not fit in a pool of 40%
    get offset -1 and are re-marched from checkpoints)."""
    from diffdvr_gb300 import pyrenderer as pr
    cases = [make_case(61, tf_mode=3, shape=(9, 10, 11), W=20, H=12, B=1),
             make_case(62, tf_mode=3, shape=(17, 13, 15), W=33, H=17, B=2),
             make_case(63, tf_mode=3, shape=(5, 6, 7), W=8, H=8, B=1)]
    singles = [gpu_forward(c, "optimized", checkpoints=True) for c in cases]
    ins, outs = [], []
    for c in cases:
        inp = c.inputs("cuda")
        B = c.batch()
        ck = torch.empty(B, c.height, c.width, pr.Renderer.checkpoint_slots(inp), device="cuda")
        ins.append(inp)
        o = pr.RendererOutputs(torch.empty(B, c.height, c.width, 4, device="cuda"),
                               torch.empty(B, c.height, c.width, dtype=torch.int32, device="cuda"), ck, 32)
        if record is not None:
            full = pr.Renderer.sample_density_size(inp, B)
            n = full if record == "full" else max(4, int(full * record) // 4 * 4)
            o.sample_density = torch.full((n,), float("nan"), device="cuda")
            o.sample_offset = torch.full((B, c.height, c.width), -7, dtype=torch.int32, device="cuda")
        outs.append(o)
    pr.Renderer.render_forward_batched(ins, outs)
    if record is not None:
        for c, o in zip(cases, outs):
            off = o.sample_offset.cpu().numpy()
            rays = off.size
            cap = o.sample_density.numel() // 4 // rays
            want = np.arange(rays).reshape(off.shape) * cap
            hit = (o.terminationIndex.cpu().numpy() > 0) & (off >= 0)
            assert np.array_equal(off[off >= 0], want[off >= 0])
            assert (off >= -1).all() and (hit.any())
            if record == "full":
                assert (off[o.terminationIndex.cpu().numpy() > 0] >= 0).all()
    torch.cuda.synchronize()
    # the single-instance forward composites each warp's 32 samples with a scan,
    # the batched one sample by sample: equal up to rounding (a sample at the
    # early-termination threshold may go either way)
    for (si, so), o in zip(singles, outs):
        same = (so.terminationIndex == o.terminationIndex).cpu().numpy()
        assert same.mean() >= 0.98
        err = symmetric_error(so.color.cpu().numpy()[same], o.color.cpu().numpy()[same])
        assert err <= 1e-5, err
    adjs = [torch.randn_like(o.color) for o in outs]
    single_g, batch_g = [], []
    for c, (si, so), a in zip(cases, singles, adjs):
        single_g.append(gpu_adjoint(c, si, so, a.cpu().numpy(), volume=True, tf=True))
    aos = []
    for c in cases:
        ao = pr.AdjointOutputs()
        ao.has_volume_derivatives = True
        ao.adj_volume = torch.zeros(c.volume.shape, device="cuda")
        ao.has_tf_derivatives = True
        ao.adj_tf = torch.zeros(c.tf.shape, device="cuda")
        aos.append(ao)
    pr.Renderer.render_adjoint_batched(ins, outs, adjs, aos)
    torch.cuda.synchronize()
    for sg, ao in zip(single_g, aos):
        assert rel_l2(ao.adj_volume.cpu().numpy(), sg["adj_volume"]) <= 1e-4
        assert rel_l2(ao.adj_tf.cpu().numpy(), sg["adj_tf"]) <= 1e-4


def _batched_setup(cases):
    from diffdvr_gb300 import pyrenderer as pr
    ins, outs, aos, adjs = [], [], [], []
    g = torch.Generator(device="cuda").manual_seed(5)
    for c in cases:
        inp = c.inputs("cuda")
        B = c.batch()
        ck = torch.empty(B, c.height, c.width, pr.Renderer.checkpoint_slots(inp), device="cuda")
        ins.append(inp)
        outs.append(pr.RendererOutputs(torch.empty(B, c.height, c.width, 4, device="cuda"),
                                       torch.empty(B, c.height, c.width, dtype=torch.int32, device="cuda"), ck, 16))
        ao = pr.AdjointOutputs()
        ao.has_volume_derivatives = True
        ao.adj_volume = torch.zeros(c.volume.shape, device="cuda")
        ao.has_tf_derivatives = True
        ao.adj_tf = torch.zeros(c.tf.shape, device="cuda")
        aos.append(ao)
        adjs.append(torch.randn(B, c.height, c.width, 4, device="cuda", generator=g))
    return ins, outs, aos, adjs


def test_batched_calls_replay_in_a_cuda_graph(cuda_device):
    """Batched forward + adjoint captured into one CUDA graph and replayed
    twice give the eager batched results (the descriptors travel in the
    kernel parameters, so nothing goes stale between replays)."""
    from diffdvr_gb300 import pyrenderer as pr
    cases = [make_case(71, tf_mode=3, shape=(9, 10, 11), W=20, H=12, B=1),
             make_case(72, tf_mode=3, shape=(17, 13, 15), W=33, H=17, B=2)]
    ins, outs, aos, adjs = _batched_setup(cases)

    def step():
        pr.Renderer.render_forward_batched(ins, outs)
        for ao in aos:
            ao.adj_volume.zero_()
            ao.adj_tf.zero_()
        pr.Renderer.render_adjoint_batched(ins, outs, adjs, aos)

    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        step()
    torch.cuda.synchronize()
    ref = [(o.color.clone(), o.terminationIndex.clone(), a.adj_volume.clone(), a.adj_tf.clone())
           for o, a in zip(outs, aos)]
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            step()
    for _ in range(2):
        for o in outs:
            o.color.fill_(float("nan"))
            o.terminationIndex.fill_(-7)
        graph.replay()
        torch.cuda.synchronize()
        for (c, t, gv, gt), o, a in zip(ref, outs, aos):
            assert torch.equal(o.terminationIndex, t) and torch.equal(o.color, c)
            assert rel_l2(a.adj_volume.cpu().numpy(), gv.cpu().numpy()) <= 1e-5
            assert rel_l2(a.adj_tf.cpu().numpy(), gt.cpu().numpy()) <= 1e-5


def test_batched_more_instances_than_one_launch_holds(cuda_device):
    """26 instances (more than the 24 one launch carries) against single calls."""
    from diffdvr_gb300 import pyrenderer as pr
    cases = [make_case(200 + i, tf_mode=1, shape=(6 + i % 5, 7, 5 + i % 3), W=8 + i % 7, H=6 + i % 4, B=1 + i % 2)
             for i in range(26)]
    ins, outs, aos, adjs = _batched_setup(cases)
    pr.Renderer.render_forward_batched(ins, outs)
    pr.Renderer.render_adjoint_batched(ins, outs, adjs, aos)
    torch.cuda.synchronize()
    for c, o, a, adj in zip(cases, outs, aos, adjs):
        si, so = gpu_forward(c, "optimized", checkpoints=True)
        same = (so.terminationIndex == o.terminationIndex).cpu().numpy()
        assert same.mean() >= 0.98
        assert symmetric_error(so.color.cpu().numpy()[same], o.color.cpu().numpy()[same]) <= 1e-5
        g = gpu_adjoint(c, si, so, adj.cpu().numpy(), volume=True, tf=True)
        assert rel_l2(a.adj_volume.cpu().numpy(), g["adj_volume"]) <= 1e-4
        assert rel_l2(a.adj_tf.cpu().numpy(), g["adj_tf"]) <= 1e-4


def test_checkpointed_adjoint_is_exact_for_opaque_rays(oracle_built, cuda_device):
    """With high absorption the reference's blend inversion loses accuracy in
    FP32 (it divides by alpha - 1); the checkpointed adjoint does not."""
    O = oracle_built
    case = make_case(71, tf_mode=0, shape=(12, 12, 12), W=16, H=16, B=1)
    case.tf = np.array([[[60.0, 1.0]]], np.float32)
    inp, out = gpu_forward(case, "optimized", checkpoints=True)
    term = out.terminationIndex.cpu().numpy()
    assert np.mean(out.color[..., 3].cpu().numpy() > 0.999) > 0.2  # many rays are opaque
    adj = np.random.default_rng(2).normal(size=out.color.shape)
    ref, adj = reference_adjoint(case, O, term, adj, O.AdjointRequest(volume=True, tf=True))
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True)
    for k in got:
        assert rel_l2(got[k], ref[k]) <= 1e-3, (k, rel_l2(got[k], ref[k]))


def test_full_stepsize_gradient_matches_finite_differences(oracle_built, cuda_device):
    """The optimized family's step-size gradient against central differences
    of the FP64 forward (interior blobs, so no sample crosses the box exit)."""
    O = oracle_built
    case = make_case(81, tf_mode=2, shape=(16, 16, 16), W=12, H=12, B=1)
    g = np.zeros((1, 16, 16, 16), np.float32)
    g[0, 3:13, 3:13, 3:13] = case.volume[0, 3:13, 3:13, 3:13]
    case.volume = g
    case.tf[..., 3] *= 0.2
    inp, out = gpu_forward(case, "optimized", checkpoints=True)
    color = out.color.cpu().numpy()
    w = np.random.default_rng(4).normal(size=color.shape)
    got = gpu_adjoint(case, inp, out, w, stepsize=True, stepsize_shape=(1, 1, 1))
    sc = case.oracle_scene()
    s0 = float(case.step)
    h = 1e-4 * s0

    def loss(step):
        sc.step_size = np.full((1, 1, 1), step)
        c, _ = O.forward(sc, "port", "f64")
        return float((c * w).sum())

    fd = (loss(s0 + h) - loss(s0 - h)) / (2 * h)
    assert abs(got["adj_stepsize"].item() - fd) <= 1e-3 * max(1.0, abs(fd)), (got["adj_stepsize"].item(), fd)


def test_tf_gradient_finite_differences_16_entries(oracle_built, cuda_device):
    """TF-reconstruction setting at test size: texture TF R=64, Beer-Lambert,
    step 0.25 voxel; GPU TF gradient vs central FD in FP64 on 16 random entries."""
    from diffdvr_gb300 import scenes
    O = oracle_built
    rng = np.random.default_rng(11)
    vol = scenes.blob_volume(32, 8, rng, noise=0.02)
    tf = scenes.tf_texture(64, rng)
    lat, lon = scenes.fibonacci_sphere(2)
    vp = scenes.viewport_from_sphere(lat, lon, 3.0)
    rs, rd = scenes.generate_rays(vp, np.radians(45.0), 24, 24)
    from dvr_cases import Case
    case = Case(width=24, height=24, volume=vol, tf=tf, tf_mode=1, filter_mode=1, blend_mode=0, camera_mode=0,
                step=0.25 / 31, ray_start=rs, ray_dir=rd)
    inp, out = gpu_forward(case, "optimized", checkpoints=True)
    w = rng.normal(size=out.color.shape)
    got = gpu_adjoint(case, inp, out, w, tf=True)["adj_tf"]
    sc = case.oracle_scene()
    sc.tf = tf.astype(np.float64)
    sc.volume = vol.astype(np.float64)

    def loss(t):
        sc.tf = t
        c, _ = O.forward(sc, "port", "f64")
        return float((c * w).sum())

    base = tf.astype(np.float64)
    for e in rng.choice(64 * 4, 16, replace=False):
        r, c = divmod(int(e), 4)
        h = 1e-6
        tp, tm = base.copy(), base.copy()
        tp[0, r, c] += h
        tm[0, r, c] -= h
        fd = (loss(tp) - loss(tm)) / (2 * h)
        assert abs(got[0, r, c] - fd) <= 1e-3 * max(abs(fd), 1e-2), (r, c, got[0, r, c], fd)


def test_autograd_module_matches_direct_calls(cuda_device):
    from diffdvr_gb300 import Renderer, pyrenderer as pr
    case = make_case(91, tf_mode=1, B=2)
    inp = case.inputs("cuda")
    tf = inp.tf.clone().requires_grad_(True)
    vol = inp.volume.clone().requires_grad_(True)
    r = Renderer(inp, optimize_tf=True, optimize_volume=True)
    img = r(tf=tf, volume=vol)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    inp2, out2 = gpu_forward(case, "optimized", checkpoints=True)
    assert torch.allclose(img.detach(), out2.color)
    g = gpu_adjoint(case, inp2, out2, w.cpu().numpy(), volume=True, tf=True)
    assert rel_l2(tf.grad.cpu().numpy(), g["adj_tf"]) <= 1e-5
    assert rel_l2(vol.grad.cpu().numpy(), g["adj_volume"]) <= 1e-5


@pytest.mark.parametrize("sample_record", ["auto", 4096, False])
def test_autograd_module_sample_record(sample_record, cuda_device):
    """The module's TF gradient with the sample record (every ray, a 4 KB pool
    that holds a few rays, none) equals the direct adjoint without a record to
    rounding (relative L2 <= 1e-5)."""
    from diffdvr_gb300 import Renderer
    case = make_case(92, tf_mode=1, shape=(16, 18, 20), W=24, H=20, B=2, R=16, opacity=0.3, pad_faces=True)
    inp = case.inputs("cuda")
    tf = inp.tf.clone().requires_grad_(True)
    r = Renderer(inp, optimize_tf=True, sample_record=sample_record)
    img = r(tf=tf)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    inp2, out2 = gpu_forward(case, "optimized", checkpoints=True)
    assert symmetric_error(img.detach().cpu().numpy(), out2.color.cpu().numpy()) <= 1e-5
    g = gpu_adjoint(case, inp2, out2, w.cpu().numpy(), tf=True)
    assert rel_l2(tf.grad.cpu().numpy(), g["adj_tf"]) <= 1e-5


def test_camera_gradient_through_generate_rays(cuda_device):
    """optimize_camera: the module generates per-pixel rays from the viewport
    with differentiable torch ops and the adjoint returns ray gradients."""
    from diffdvr_gb300 import Renderer, pyrenderer as pr, scenes
    case = make_case(95, tf_mode=1, B=1)
    inp = case.inputs("cuda")
    vp = torch.from_numpy(scenes.viewport_from_sphere(0.3, 1.0, 2.0).astype(np.float32)).cuda().requires_grad_(True)
    r = Renderer(inp, optimize_camera=True)
    img = r(camera=vp, fov_y_radians=0.7)
    img.sum().backward()
    assert vp.grad is not None and torch.isfinite(vp.grad).all() and vp.grad.abs().sum() > 0


@pytest.mark.parametrize("views,viewports", [(1, 1), (3, 3), (2, 1)])
def test_fused_viewport_gradient_matches_generated_rays(views, viewports, cuda_device):
    """optimize_camera with the rays generated inside the kernel (the viewport
    gradient carried back through the ray generation per ray) against the
    per-pixel-ray path (rays from torch ops, the kernel's ray adjoint, autograd
    through the generation): relative L2 <= 1e-3 (the two generate the rays
    with different float rounding).  viewports == 1 with several views: one
    viewport broadcast over the views, its gradient summed."""
    from diffdvr_gb300 import Renderer, scenes
    case = make_case(96, tf_mode=1, B=views, shape=(16, 18, 20), W=24, H=20, opacity=0.4, pad_faces=True)
    inp = case.inputs("cuda")
    lat = np.array([0.3 + 0.2 * i for i in range(viewports)])
    lon = np.array([1.0 + 0.5 * i for i in range(viewports)])
    vps = torch.from_numpy(scenes.viewport_from_sphere(lat, lon, 2.0).astype(np.float32)).cuda()
    w = torch.randn(views, case.height, case.width, 4, device="cuda", generator=torch.Generator(device="cuda").manual_seed(4))
    grads = {}
    for fused in (True, False):
        vp = vps.clone().requires_grad_(True)
        r = Renderer(inp, optimize_camera=True, fused_camera=fused)
        img = r(camera=vp if viewports == views or fused else vp.expand(views, 3, 3), fov_y_radians=0.7)
        (img * w).sum().backward()
        grads[fused] = vp.grad.double().cpu().numpy()
    assert np.abs(grads[True]).max() > 0
    assert rel_l2(grads[True], grads[False]) <= 1e-3, rel_l2(grads[True], grads[False])


def test_cvol_volume_renders_in_file_order(tmp_path, cuda_device):
    """A Marschner-Lobb volume written to and read from a .cvol file keeps the
    file's x-fastest layout (strides 1, X, X*Y); rendering it gives exactly
    what its contiguous [x][y][z] copy gives, forward and TF gradient."""
    from diffdvr_gb300 import pyrenderer as pr, volume_io as vio
    path = str(tmp_path / "ml.cvol")
    vio.save_cvol(path, vio.marschner_lobb(41), dtype="float32")
    vol, world = vio.load_cvol(path)
    case = make_case(97, tf_mode=1, shape=(41, 41, 41), W=32, H=24, B=2, opacity=0.5)
    results = []
    for t in (torch.from_numpy(vol).cuda(), torch.from_numpy(np.ascontiguousarray(vol)).cuda()):
        assert t.is_contiguous() == (len(results) == 1)
        case.volume = vol
        inp = case.inputs("cuda")
        inp.volume = t
        B = case.batch()
        out = pr.RendererOutputs(torch.empty(B, case.height, case.width, 4, device="cuda"),
                                 torch.empty(B, case.height, case.width, dtype=torch.int32, device="cuda"),
                                 torch.empty(B, case.height, case.width, pr.Renderer.checkpoint_slots(inp), device="cuda"),
                                 16)
        pr.Renderer.render_forward(inp, out)
        a = pr.AdjointOutputs()
        a.has_tf_derivatives = True
        a.adj_tf = torch.zeros(case.tf.shape, device="cuda")
        pr.Renderer.render_adjoint(inp, out, torch.ones_like(out.color) * 1e-2, a)
        torch.cuda.synchronize()
        results.append((out.color.clone(), out.terminationIndex.clone(), a.adj_tf.clone()))
    (c0, t0, g0), (c1, t1, g1) = results
    assert torch.equal(t0, t1) and torch.equal(c0, c1)
    assert rel_l2(g0.cpu().numpy(), g1.cpu().numpy()) <= 1e-5


def test_invalid_inputs_raise(cuda_device):
    from diffdvr_gb300 import pyrenderer as pr
    case = make_case(99)
    inp, out = gpu_forward(case, "optimized")
    bad = inp.clone()
    bad.volume = inp.volume[0]
    with pytest.raises(RuntimeError, match="volume must be a tensor with 4 dimensions"):
        pr.Renderer.render_forward(bad, out)
    bad = inp.clone()
    bad.tf = inp.tf[:, :, :3]
    with pytest.raises(RuntimeError, match="tf must have 4 entries at dimension 2"):
        pr.Renderer.render_forward(bad, out)
    bad = inp.clone()
    bad.tf = inp.tf.cpu()
    with pytest.raises(RuntimeError, match="CPU tensor"):
        pr.Renderer.render_forward(bad, out)
    with pytest.raises(RuntimeError, match="At least one adjoint variable must be activated"):
        pr.Renderer.render_adjoint(inp, out, torch.zeros_like(out.color), pr.AdjointOutputs())
    wrong = pr.RendererOutputs(out.color[:, :, :-1], out.terminationIndex)
    with pytest.raises(RuntimeError, match="color must have"):
        pr.Renderer.render_forward(inp, wrong)


@pytest.mark.parametrize("fraction", ["full", 0.5])
def test_sample_density_record(fraction, cuda_device):
    """The forward's sample record: every ray with samples that got room holds
    n (density, incoming opacity) pairs in its own disjoint 4-aligned run of
    the pool: densities finite and inside the volume's range, opacities
    starting at 0, non-decreasing, below 1 and equal to the checkpoints a
    forward without record writes at multiples of the interval (recorded rays
    get no checkpoints); rays without samples or without room are -1;
    the adjoint from the record equals the re-sampling adjoint (relative L2
    <= 1e-5: the recorded opacities are the forward's, the re-march's agree
    to rounding)."""
    case = make_case(71, tf_mode=1, filter_mode=1, blend_mode=0, shape=(20, 24, 28), W=40, H=36, B=2, R=32,
                     opacity=0.3, pad_faces=True)
    inp, out = gpu_forward(case, checkpoints=True, record="full")
    if fraction != "full":
        # a pool for about half of the samples the rays actually recorded
        t = out.terminationIndex.cpu().numpy()
        inp, out = gpu_forward(case, checkpoints=True, record=int(fraction * 4 * ((t + 1) // 2).sum()))
    term = out.terminationIndex.cpu().numpy()
    off = out.sample_offset.cpu().numpy()
    pool = out.sample_density.cpu().numpy()
    assert ((off >= 0) | (off == -1)).all()
    assert (off[term == 0] == -1).all()
    hit = (term > 0) & (off >= 0)
    if fraction == "full":
        assert (off[term > 0] >= 0).all()
    else:
        assert ((term > 0) & (off == -1)).any() and hit.any()
    lo, hi = float(case.volume.min()), float(case.volume.max())
    ck_rec = out.checkpoints.cpu().numpy()
    assert np.isnan(ck_rec[hit]).all()  # recorded rays: checkpoints left untouched
    _, norec_out = gpu_forward(case, checkpoints=True)
    assert np.array_equal(norec_out.terminationIndex.cpu().numpy(), term)
    ck = norec_out.checkpoints.cpu().numpy()
    K = out.checkpoint_interval
    starts, ends = [], []
    for (bi, yi, xi), o, n in zip(np.argwhere(hit), off[hit], term[hit]):
        run = pool[4 * o: 4 * o + 2 * n].reshape(n, 2)
        d, a_in = run[:, 0], run[:, 1]
        assert np.isfinite(run).all() and d.min() >= lo - 1e-6 and d.max() <= hi + 1e-6
        assert a_in[0] == 0 and (np.diff(a_in) >= 0).all() and a_in.max() < 1
        js = np.arange(1, (n - 1) // K + 1)
        np.testing.assert_allclose(a_in[js * K], ck[bi, yi, xi, js - 1], rtol=0, atol=1e-6)
        starts.append(4 * o)
        ends.append(4 * o + 2 * n)
    order = np.argsort(starts)
    assert (np.asarray(starts)[order][1:] >= np.asarray(ends)[order][:-1]).all()
    assert max(ends) <= pool.size

    rng = np.random.default_rng(3)
    adj = rng.standard_normal(out.color.shape).astype(np.float32)
    got = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=True, stepsize=True)
    # re-sampling adjoint: the same forward outputs with the record-less forward's checkpoints
    plain_out = type(out)(out.color, out.terminationIndex, norec_out.checkpoints, out.checkpoint_interval)
    ref = gpu_adjoint(case, inp, plain_out, adj, volume=True, tf=True, camera=True, stepsize=True)
    for k in ref:
        assert rel_l2(got[k], ref[k]) <= 1e-5, (k, rel_l2(got[k], ref[k]))


@pytest.mark.parametrize("blend,per_batch,pool,interval", [(0, False, "full", 16), (1, False, "full", 16),
                                                           (0, True, "full", 16), (1, False, 0.5, 16),
                                                           (0, False, "full", 5), (1, True, "full", 64)])
def test_tf_only_adjoint_from_record(blend, per_batch, pool, interval, oracle_built, cuda_device):
    """TF gradient alone with checkpoints and a sample-density record (the
    texture-TF record kernel; rays without room in the pool go through the
    general kernel) against the FP64 oracle, tolerances as above; per_batch:
    a TF per batch entry and a TF gradient per batch entry; intervals that do
    not divide 32 make the kernel advance from a checkpoint to a step start."""
    O = oracle_built
    rng = np.random.default_rng(11 + blend)
    case = make_case(90 + blend, tf_mode=1, filter_mode=1, blend_mode=blend, shape=(20, 24, 28), W=40, H=36, B=2,
                     R=32, opacity=0.3, pad_faces=True)
    if not per_batch:
        case.tf = np.ascontiguousarray(case.tf[:1])  # one TF for both views, one TF gradient
    inp, out = gpu_forward(case, checkpoints=True, interval=interval, record="full")
    if pool != "full":
        t = out.terminationIndex.cpu().numpy()
        inp, out = gpu_forward(case, checkpoints=True, interval=interval,
                               record=int(pool * 4 * ((t + 1) // 2).sum()))
        t = out.terminationIndex.cpu().numpy()
        assert (out.sample_offset.cpu().numpy()[t > 0] == -1).any()
    term = out.terminationIndex.cpu().numpy()
    adj = rng.standard_normal(out.color.shape).astype(np.float32)
    ref, adj = reference_adjoint(case, O, term, adj, O.AdjointRequest(tf=True))
    got = gpu_adjoint(case, inp, out, adj, tf=True)
    assert got["adj_tf"].shape == case.tf.shape
    bad = _grad_errors(got, ref)
    assert not bad, bad
