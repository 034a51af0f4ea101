"""The batched launches' tile-shape autotuner (diffdvr_gb300.autotune).

CPU: the size classes; the coordinate search over the classes' shapes with a
fake launch timer (it finds the per-class optimum of a separable cost, keeps
16x8 where no shape beats it by the noise margin); the JSON cache (a second
tuner on the same file and device reuses the choice without timing; another
device searches again).
GPU: tune() on a batch of instances of two size classes, and the batched
calls with tuned and with fixed shapes against the default 16x8 tiles (the
forward is computed per ray, so identical; gradients equal up to the order of
floating-point atomic additions, relative L2 <= 1e-5).
"""
import json

import numpy as np
import pytest

from diffdvr_gb300 import autotune as T


def test_size_class_rounds_sizes_and_keeps_modes():
    a = T.size_class((1, 96, 96, 96), 200, 100, 0.5, (1, 3, 0), "bf16", ("volume", "tf"))
    b = T.size_class((1, 128, 100, 70), 256, 256, 0.52, (1, 3, 0), "bf16", ("tf", "volume"))
    assert a == b == "vol128-img256-step0.5-f1t3b0-bf16-tf+volume"
    assert T.size_class((1, 32, 32, 32), 64, 64, 0.5, (1, 3, 0), "bf16", ("tf",)) != a
    assert T.size_class((1, 128, 128, 128), 256, 256, 0.25, (1, 3, 0), "bf16", ("tf", "volume")) != a
    assert T.size_class((1, 128, 128, 128), 256, 256, 0.5, (1, 1, 0), "bf16", ("tf", "volume")) != a


def _separable(costs):
    """A launch time that is the sum of each class's cost for its shape."""
    return lambda choice: sum(costs[c][s] for c, s in choice.items())


def test_search_finds_per_class_optimum_with_margin():
    costs = {"a": {0: 2.0, 1: 1.0, 2: 3.0},      # 32x4 clearly better
             "b": {0: 5.0, 1: 6.0, 2: 4.0},      # 8x16 clearly better
             "c": {0: 3.0, 1: 2.99, 2: 3.5}}     # within the margin: stays 16x8
    choice, best, base = T.search(["a", "b", "c"], _separable(costs))
    assert choice == {"a": 1, "b": 2, "c": 0}
    assert base == 10.0 and best == pytest.approx(8.0)


def test_choose_caches_per_device(tmp_path):
    path = str(tmp_path / "tiles.json")
    calls = []
    fwd = {"a": {0: 2.0, 1: 1.0, 2: 3.0}}
    adj = {"a": {0: 5.0, 1: 6.0, 2: 4.0}}

    def tf(choice):
        calls.append(("f", dict(choice)))
        return _separable(fwd)(choice)

    def ta(choice):
        calls.append(("a", dict(choice)))
        return _separable(adj)(choice)

    t = T.TileTuner(cache_path=path, device="GPU A")
    assert t.choose(["a"], tf, ta) == ({"a": 1}, {"a": 2})
    assert t.timed and len(calls) == 6
    saved = json.load(open(path))
    assert saved["GPU A"]["a"] == {"forward": 1, "adjoint": 2}
    calls.clear()
    t2 = T.TileTuner(cache_path=path, device="GPU A")
    assert t2.choose(["a"], tf, ta) == ({"a": 1}, {"a": 2})
    assert calls == [] and not t2.timed
    t3 = T.TileTuner(cache_path=path, device="GPU B")
    fwd["a"][0] = 0.5
    assert t3.choose(["a"], tf, ta) == ({"a": 0}, {"a": 2})
    assert len(calls) == 6
    assert set(json.load(open(path))) == {"GPU A", "GPU B"}


def test_unreadable_cache_is_ignored(tmp_path):
    path = tmp_path / "tiles.json"
    path.write_text("not json")
    t = T.TileTuner(cache_path=str(path), device="GPU A")
    assert t.cache == {}
    assert t.choose(["c"], lambda ch: float(ch["c"] + 1), lambda ch: float(3 - ch["c"])) == ({"c": 0}, {"c": 2})
    assert json.load(open(path))["GPU A"]["c"]["adjoint"] == 2


@pytest.mark.gpu
@pytest.mark.parametrize("record", [False, True])
def test_tuned_batched_calls_match_default_tiles(cuda_device, tmp_path, record):
    import torch
    from diffdvr_gb300 import pyrenderer as pr
    from dvr_cases import make_case, rel_l2
    cases = [make_case(81, tf_mode=3, shape=(20, 16, 24), W=40, H=20, B=1),
             make_case(82, tf_mode=3, shape=(9, 10, 11), W=70, H=9, B=1),
             make_case(83, tf_mode=3, shape=(20, 16, 24), W=36, H=24, B=1)]
    ins, outs, adjs, aos = [], [], [], []
    rng = np.random.default_rng(4)
    for c in cases:
        inp = c.inputs("cuda")
        ck = torch.empty(1, c.height, c.width, pr.Renderer.checkpoint_slots(inp), device="cuda")
        ins.append(inp)
        outs.append(pr.RendererOutputs(torch.empty(1, c.height, c.width, 4, device="cuda"),
                                       torch.empty(1, c.height, c.width, dtype=torch.int32, device="cuda"), ck, 16))
        if record:  # the forward's sample record: the adjoint reads it instead of re-marching
            outs[-1].sample_density = torch.empty(pr.Renderer.sample_density_size(inp, 1), device="cuda")
            outs[-1].sample_offset = torch.empty(1, c.height, c.width, dtype=torch.int32, device="cuda")
        adjs.append(torch.from_numpy(rng.normal(size=(1, c.height, c.width, 4)).astype(np.float32)).cuda())
        a = pr.AdjointOutputs()
        a.has_tf_derivatives = True
        a.adj_tf = torch.zeros(c.tf.shape, device="cuda")
        a.has_volume_derivatives = True
        a.adj_volume = torch.zeros(c.volume.shape, device="cuda")
        aos.append(a)
    pr.Renderer.render_forward_batched(ins, outs)
    kept = [o.sample_offset.clone() for o in outs] if record else []
    tuner = T.TileTuner(cache_path=str(tmp_path / "tiles.json"), warmup=1, repeats=3)
    fs, as_ = tuner.tune(ins, outs, adjs, aos, storage="f32")
    # the tuner ran on scratch outputs (with a record of their own) and left the caller's record alone
    assert all(torch.equal(k, o.sample_offset) for k, o in zip(kept, outs))
    assert tuner.timed and len(fs) == len(as_) == 3 and all(s in T.SHAPES for s in fs + as_)
    assert fs[0] == fs[2] and as_[0] == as_[2]  # one size class
    # the tuner's runs did not touch the caller's gradients
    assert all(float(a.adj_tf.abs().sum()) == 0 and float(a.adj_volume.abs().sum()) == 0 for a in aos)

    def run(fshapes, ashapes):
        res = []
        for a in aos:
            a.adj_tf.zero_()
            a.adj_volume.zero_()
        pr.Renderer.render_forward_batched(ins, outs, fshapes)
        pr.Renderer.render_adjoint_batched(ins, outs, adjs, aos, ashapes)
        torch.cuda.synchronize()
        for o, a in zip(outs, aos):
            res.append((o.color.cpu().numpy(), o.terminationIndex.cpu().numpy(), a.adj_tf.cpu().numpy(),
                        a.adj_volume.cpu().numpy()))
        return res

    base = run(None, None)
    for fsh, ash in (([1, 1, 1], [1, 1, 1]), ([2, 2, 2], [2, 2, 2]), (fs, as_)):
        got = run(fsh, ash)
        for (c0, t0, g0, v0), (c1, t1, g1, v1) in zip(base, got):
            assert np.array_equal(t0, t1) and np.array_equal(c0, c1)
            assert rel_l2(g1, g0) <= 1e-5 and rel_l2(v1, v0) <= 1e-5
