"""The memory-lean TF-gradient adjoint: a texture TF's gradient from the
transmittance checkpoints alone, no sample record (pyrenderer path
"remarch").  One warp per ray re-marches the ray in chunks from their
checkpoints into shared memory and reverses each chunk with the record
adjoint's segment scan (renderer/renderer_kernels.cuh:367-444 for the
recursion, renderer/renderer_blending.cuh:63-98 for the blend adjoint).

Held against the FP64 oracle and against the record kernel (the same rays
read from the forward's sample record instead of re-marched) on rays longer
than one chunk, with even and odd intervals, both blend modes, both filters,
the direct and the texture corner gather, FP32 and BF16 storage; and with a
checkpoint buffer too short for the long rays, which go on to the general
kernel.
"""
import numpy as np
import pytest
import torch

from dvr_cases import gpu_adjoint, gpu_forward, make_case, rel_l2

pytestmark = pytest.mark.gpu

TEXTURE_TF = 1


def _case(seed, filt, blend, B=2):
    # 0.08-voxel steps through a 40-44 voxel box: rays up to about 750
    # samples, more than one 512-sample chunk
    c = make_case(seed, tf_mode=TEXTURE_TF, filter_mode=filt, blend_mode=blend, camera_mode=0,
                  shape=(40, 36, 44), W=24, H=20, B=B, step_voxels=0.08, opacity=0.05)
    return c


def _oracle(case, O, term, adj):
    sc = case.oracle_scene()
    c64, t64 = O.forward(sc, "port", "f64")
    adj = np.where((term == t64)[..., None], adj, 0.0).astype(np.float32)
    req = O.AdjointRequest(volume=False, tf=True, camera=False, stepsize=False)
    ref = O.adjoint(sc, c64, t64, adj, req, "port", "f64")
    c32, t32 = O.forward(sc, "port", "f32")
    g32 = O.adjoint(sc, c32, t32, np.where((t32 == term)[..., None], adj, 0.0), req, "port", "f32")
    return ref["adj_tf"], rel_l2(g32["adj_tf"], ref["adj_tf"]), adj


def _tf_grad(case, interval, dtype, gather, slots=None, record=None):
    from diffdvr_gb300 import pyrenderer as pr
    prev = pr.set_forward_gather(gather)
    try:
        if slots is None:
            inp, out = gpu_forward(case, "optimized", volume_dtype=dtype, checkpoints=True, interval=interval,
                                   record=record)
        else:
            # a checkpoint buffer of `slots` slots: rays beyond (slots + 1) * interval
            # samples are not covered
            pr.set_kernel_family("optimized")
            inp = case.inputs("cuda", dtype, None)
            B = case.batch()
            out = pr.RendererOutputs(torch.empty(B, case.height, case.width, 4, device="cuda"),
                                     torch.empty(B, case.height, case.width, dtype=torch.int32, device="cuda"),
                                     torch.empty(B, case.height, case.width, slots, device="cuda"), interval)
            pr.Renderer.render_forward(inp, out)
            torch.cuda.synchronize()
        term = out.terminationIndex.cpu().numpy()
        adj = np.random.default_rng(11).normal(size=out.color.shape).astype(np.float32)
        return inp, out, term, adj
    finally:
        pr.set_forward_gather(prev)


def _adjoint(case, inp, out, adj, gather):
    from diffdvr_gb300 import pyrenderer as pr
    prev = pr.set_forward_gather(gather)
    try:
        got = gpu_adjoint(case, inp, out, adj, tf=True)["adj_tf"]
        return got, pr.last_adjoint_path()
    finally:
        pr.set_forward_gather(prev)


@pytest.mark.parametrize("interval", [16, 7])
@pytest.mark.parametrize("filt,blend,gather,dtype", [
    (1, 0, "direct", torch.float32), (1, 1, "direct", torch.float32),
    (1, 0, "texture", torch.bfloat16), (1, 1, "texture", torch.float32),
    (0, 0, "direct", torch.bfloat16)],
    ids=["trilinear-beer-direct-f32", "trilinear-alpha-direct-f32", "trilinear-beer-texture-bf16",
         "trilinear-alpha-texture-f32", "nearest-beer-bf16"])
def test_remarch_adjoint_against_oracle_and_general_kernel(interval, filt, blend, gather, dtype, oracle_built,
                                                           cuda_device):
    O = oracle_built
    case = _case(900 + interval + 10 * blend + 20 * filt, filt, blend)
    if dtype != torch.float32:
        # the oracle sees the stored values
        case.volume = torch.from_numpy(case.volume).to(dtype).float().numpy()
    inp, out, term, adj = _tf_grad(case, interval, dtype, gather)
    assert int(term.max()) > 512, int(term.max())  # some rays span more than one chunk
    ref, r32, adj = _oracle(case, O, term, adj)
    got, path = _adjoint(case, inp, out, adj, gather)
    assert path == "remarch"
    assert rel_l2(got, ref) <= max(1e-3, 3 * r32), (rel_l2(got, ref), r32)
    # the record kernel over the same rays: the forward's (density, opacity)
    # record instead of the re-march from the checkpoints
    inp2, out2, term2, _ = _tf_grad(case, interval, dtype, gather, record="full")
    assert np.array_equal(term2, term)
    got2, path2 = _adjoint(case, inp2, out2, adj, gather)
    assert path2 == "record"
    assert rel_l2(got, got2) <= 2e-5, rel_l2(got, got2)


def test_remarch_adjoint_leaves_uncovered_rays_to_the_general_kernel(oracle_built, cuda_device):
    """Three checkpoint slots at interval 16 cover rays of up to 64 samples;
    the longer ones go to the general kernel, which inverts the blend."""
    O = oracle_built
    case = _case(931, 1, 0)
    inp, out, term, adj = _tf_grad(case, 16, torch.float32, "direct", slots=3)
    hit = term > 0
    assert np.any(term > 64) and np.any(hit & (term <= 64))
    ref, r32, adj = _oracle(case, O, term, adj)
    got, path = _adjoint(case, inp, out, adj, "direct")
    assert path == "remarch"
    assert rel_l2(got, ref) <= max(1e-3, 3 * r32), (rel_l2(got, ref), r32)


@pytest.mark.parametrize("gather", ["direct", "texture"])
def test_remarch_adjoint_with_a_broadcast_tf(gather, oracle_built, cuda_device):
    """One TF for both batch entries: the TF gradient sums the entries' rays
    through the per-warp slices, as the headline's eight views do."""
    O = oracle_built
    case = _case(941, 1, 0)
    case.tf = np.ascontiguousarray(case.tf[:1])
    inp, out, term, adj = _tf_grad(case, 16, torch.float32, gather)
    assert int(term.max()) > 512
    ref, r32, adj = _oracle(case, O, term, adj)
    got, path = _adjoint(case, inp, out, adj, gather)
    assert path == "remarch" and got.shape == case.tf.shape
    assert rel_l2(got, ref) <= max(1e-3, 3 * r32), (rel_l2(got, ref), r32)
    inp2, out2, term2, _ = _tf_grad(case, 16, torch.float32, gather, record="full")
    got2, path2 = _adjoint(case, inp2, out2, adj, gather)
    assert path2 == "record" and np.array_equal(term2, term)
    assert rel_l2(got, got2) <= 2e-5, rel_l2(got, got2)
