"""The forward's three ways of reading a trilinear sample's eight corners
(``pyrenderer.set_forward_gather``): eight loads from the volume ("direct"),
one cell-corner record per sample ("cells") and two ``tex2Dgather`` fetches
from the tiled, aproned slab texture ("texture").  All three read the same
clamped corners (renderer/renderer_interpolation.cuh:193-207) and share the
rest of the kernel, so the images, termination indices, checkpoints and
sample records must be bit-identical; the direct path is the one the parity
tests hold against the oracle.

The texture cases cover FP32 / FP16 / BF16 storage, per-entry and broadcast
volumes, every TF and blend mode, the three camera modes, ragged sizes, and a
slab count that needs several tiles per texture row with a partial last row.
"""
import numpy as np
import pytest
import torch

from dvr_cases import all_mode_combos, gpu_forward, make_case

MODES = ("direct", "cells", "texture")


def _render(case, mode, dtype, record=None):
    from diffdvr_gb300 import pyrenderer as pr
    prev = pr.set_forward_gather(mode)
    try:
        # a sample record needs the checkpoint buffer beside it (rays that
        # find the pool full checkpoint instead)
        _, out = gpu_forward(case, "optimized", volume_dtype=dtype, checkpoints=True, record=record)
    finally:
        pr.set_forward_gather(prev)
    res = {"color": out.color, "term": out.terminationIndex}
    if out.checkpoints is not None:
        res["checkpoints"] = out.checkpoints
    if record is not None:
        # rays claim their record runs in scheduling order: compare each
        # recorded ray's (density, opacity) pairs, not the pool's layout
        off = out.sample_offset.flatten().long()
        n = out.terminationIndex.flatten().long()
        pool = out.sample_density.view(-1, 2)
        k = torch.arange(int(n.max()) + 1, device=off.device)
        take = (off[:, None] >= 0) & (k[None, :] < n[:, None])
        idx = (2 * off[:, None] + k[None, :]).clamp(min=0)
        res["recorded"] = off >= 0
        res["record"] = torch.where(take[..., None], pool[idx.clamp(max=pool.shape[0] - 1)], 0.0)
    return {k: v.cpu() for k, v in res.items()}


def _assert_identical(a, b, what):
    for k in a:
        x, y = a[k], b[k]
        same = torch.equal(torch.nan_to_num(x, nan=-1e30), torch.nan_to_num(y, nan=-1e30)) if x.is_floating_point() \
            else torch.equal(x, y)
        assert same, (what, k, (x != y).sum().item() if x.shape == y.shape else (x.shape, y.shape))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.float32, torch.float16, torch.bfloat16], ids=["f32", "f16", "bf16"])
def test_gather_modes_are_bit_identical_in_every_mode(dtype, cuda_device):
    failures = []
    for i, (tfm, filt, blend, cam) in enumerate(all_mode_combos()):
        if filt != 1:
            continue  # nearest filtering reads one voxel directly in every mode
        case = make_case(700 + i, tf_mode=tfm, filter_mode=filt, blend_mode=blend, camera_mode=cam,
                         shape=(17, 19, 21), W=24, H=20, B=2)
        ref = _render(case, "direct", dtype)
        for mode in MODES[1:]:
            try:
                _assert_identical(ref, _render(case, mode, dtype), (tfm, blend, cam, mode))
            except AssertionError as e:
                failures.append(str(e))
    assert not failures, failures


@pytest.mark.gpu
@pytest.mark.parametrize("broadcast", [False, True], ids=["per-entry-volumes", "broadcast-volume"])
def test_gather_texture_with_many_slab_tiles(broadcast, cuda_device):
    """63 x-slabs of 600 x 9 voxels per entry, 3 entries: 189 slabs of 602
    texel rows exceed the gather texture's height in one column, so the slabs
    go four to a texture row, the last row holding one."""
    case = make_case(77, tf_mode=1, shape=(63, 600, 9), W=40, H=36, B=3, step_voxels=0.7)
    if broadcast:
        case.volume = case.volume[:1]
    ref = _render(case, "direct", torch.bfloat16)
    assert ref["color"][..., 3].max() > 0.05  # the scene is not empty
    _assert_identical(ref, _render(case, "texture", torch.bfloat16), "texture")


@pytest.mark.gpu
def test_gather_texture_with_sample_record(cuda_device):
    case = make_case(78, tf_mode=1, shape=(33, 20, 27), W=32, H=24, B=2)
    ref = _render(case, "direct", torch.bfloat16, record="full")
    _assert_identical(ref, _render(case, "texture", torch.bfloat16, record="full"), "texture+record")


@pytest.mark.gpu
def test_gather_texture_survives_shape_changes(cuda_device):
    """The library's texture is replaced when the volume's size changes and
    reused while it stays; renders in between stay identical."""
    cases = [make_case(80 + k, tf_mode=2, shape=s, W=20, H=16, B=1)
             for k, s in enumerate([(9, 10, 11), (30, 12, 7), (9, 10, 11)])]
    for c in cases:
        _assert_identical(_render(c, "direct", torch.float32), _render(c, "texture", torch.float32), c.volume.shape)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,broadcast,record", [(torch.float32, False, None), (torch.bfloat16, True, None),
                                                    (torch.float16, False, "full")],
                         ids=["f32", "bf16-broadcast-volume", "f16-record"])
def test_general_adjoint_reads_the_same_corners_from_the_texture(dtype, broadcast, record, cuda_device):
    """The general adjoint reads trilinear corners from the slab texture when
    it re-marches rays without a record or needs position derivatives: every
    gradient (volume, TF, per-pixel rays, step size) is the same as with
    corners loaded directly, up to the order of the atomic additions
    (relative L2 <= 1e-6)."""
    from diffdvr_gb300 import pyrenderer as pr
    from dvr_cases import gpu_adjoint, rel_l2
    case = make_case(79, tf_mode=2, filter_mode=1, blend_mode=0, camera_mode=0, shape=(21, 18, 25), W=30, H=22,
                     B=2, opacity=0.4)
    if broadcast:
        case.volume = case.volume[:1]
    inp, out = gpu_forward(case, "optimized", volume_dtype=dtype, checkpoints=True, record=record)
    adj = np.random.default_rng(3).normal(size=out.color.shape).astype(np.float32)
    grads = {}
    for mode in ("direct", "texture"):
        prev = pr.set_forward_gather(mode)
        try:
            grads[mode] = gpu_adjoint(case, inp, out, adj, volume=True, tf=True, camera=True, stepsize=True)
        finally:
            pr.set_forward_gather(prev)
    for k, ref in grads["direct"].items():
        assert np.abs(ref).max() > 0, k
        assert rel_l2(grads["texture"][k], ref) <= 1e-6, (k, rel_l2(grads["texture"][k], ref))


def test_forward_gather_switch(dvr_lib):
    from diffdvr_gb300 import pyrenderer as pr
    prev = pr.set_forward_gather("texture")
    try:
        assert pr.set_forward_gather("cells") == "texture"
        assert pr.set_forward_gather("direct") == "cells"
        with pytest.raises(RuntimeError):
            pr.set_forward_gather("bilinear")
        assert dvr_lib.dvr_set_forward_gather(7) < 0
        assert dvr_lib.dvr_get_forward_gather() == 1
    finally:
        pr.set_forward_gather(prev)
    assert pr.set_forward_gather(prev) == prev
