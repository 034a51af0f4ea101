"""Per-component adjoint checks of the oracle (FP64), after the reference's
unit tests: each step function of the march (blending, TF evaluation, volume
sampling, ray stepping) against central finite differences of its own
forward, with the reference's input shapes, draw counts and tolerances
(unittests/testAdjointBlending.cpp:10-77, testAdjointTF.cpp:10-232,
testAdjointInterpolation.cpp:23-108, testAdjointCamera.cpp:10-81).  The
reference draws with std::default_random_engine(42); numpy's generator with
seed 42 stands in (same distributions, other values).

A gradient g matches a difference quotient f as Catch's
Approx(f).epsilon(rel).margin(abs) would: |g - f| <= abs or
|g - f| <= rel * max(|g|, |f|).  The reference's harness takes one-sided
differences (unittests/check_adjoint.h:35-84); these are central, so they
meet the same tolerances with room to spare.
"""
import numpy as np
import pytest

H = 1e-5  # the reference's finite-difference step


def _close(g, f, rel, abs_):
    g, f = np.asarray(g, np.float64), np.asarray(f, np.float64)
    d = np.abs(g - f)
    return np.all((d <= abs_) | (d <= rel * np.maximum(np.abs(g), np.abs(f))))


def _central(fn, x, i, h=H):
    xp, xm = np.array(x, np.float64), np.array(x, np.float64)
    xp.flat[i] += h
    xm.flat[i] -= h
    return (np.asarray(fn(xp), np.float64) - np.asarray(fn(xm), np.float64)) / (2 * h)


@pytest.mark.parametrize("mode", [0, 1], ids=["beer_lambert", "alpha"])
def test_blend_adjoint(oracle_built, mode):
    """20 draws of U(0.01, 0.99) for the accumulator, the sample and the step;
    the adjoint inverts the blend (recovers the accumulator in front of the
    sample) and matches the differences of the blended accumulator with
    respect to all nine inputs (eps 1e-5, rel 1e-5, abs 1e-6)."""
    O = oracle_built
    rng = np.random.default_rng(42)
    for _ in range(20):
        x = rng.uniform(0.01, 0.99, size=9)  # acc[4], cur[4], step
        adj_out = rng.normal(size=4)
        f = lambda v: O.blend_step(mode, v[:4], v[4:8], v[8])
        acc_out = f(x)
        acc_in, adj_acc, adj_cur, adj_step = O.blend_step_adjoint(mode, acc_out, x[4:8], x[8], adj_out)
        assert np.allclose(acc_in, x[:4], rtol=1e-9, atol=1e-12)
        got = np.concatenate([adj_acc, adj_cur, [adj_step]])
        fd = np.array([_central(f, x, i) @ adj_out for i in range(9)])
        assert _close(got, fd, 1e-5, 1e-6), (got, fd)


def _tf(rng, mode, R):
    if mode == 0:
        return rng.uniform(0.01, 0.99, size=(1, 1, 2))
    if mode == 1:
        return rng.uniform(0.0, 1.0, size=(1, R, 4))
    if mode == 2:
        tf = np.zeros((1, R, 5))
        tf[0, :, :4] = rng.uniform(0.0, 1.0, size=(R, 4))
        tf[0, :, 4] = np.sort(rng.uniform(0.0, 1.0, size=R))
        tf[0, 0, 4], tf[0, -1, 4] = 0.0, 1.0
        return tf
    tf = np.zeros((1, R, 6))
    tf[0, :, :4] = rng.uniform(0.0, 1.0, size=(R, 4))
    tf[0, :, 4] = rng.uniform(0.0, 1.0, size=R)    # mu
    tf[0, :, 5] = rng.uniform(0.05, 0.5, size=R)   # sigma
    return tf


@pytest.mark.parametrize("mode,R,tol", [
    (0, 1, (1e-4, 1e-6)), (1, 8, (1e-4, 1e-6)), (2, 5, (1e-4, 1e-6)), (3, 4, (1e-3, 1e-4))],
    ids=["identity", "texture", "linear", "gaussian"])
def test_tf_adjoint(oracle_built, mode, R, tol):
    """10 TFs x 10 densities in (0.01, 0.99): the density derivative and the
    TF gradient of adj . tf(density) against differences (eps 1e-5; rel 1e-4,
    abs 1e-6; Gaussian rel 1e-3, abs 1e-4).  Densities within 10 eps of a
    texel centre or control point, where the TF has a kink, are skipped."""
    O = oracle_built
    rng = np.random.default_rng(42)
    rel, abs_ = tol
    checked = 0
    for _ in range(10):
        tf = _tf(rng, mode, R)
        kinks = (np.arange(R) + 0.5) / R if mode == 1 else tf[0, :, 4] if mode == 2 else np.array([])
        for _ in range(10):
            d = float(rng.uniform(0.01, 0.99))
            if kinks.size and np.min(np.abs(kinks - d)) < 10 * H:
                continue
            adj = rng.normal(size=4)
            adj_d, adj_tf = O.tf_step_adjoint(tf, mode, d, adj)
            fd_d = (O.tf_step(tf, mode, d + H) - O.tf_step(tf, mode, d - H)) @ adj / (2 * H)
            assert _close(adj_d, fd_d, rel, abs_), (d, adj_d, fd_d)
            fd_tf = np.array([_central(lambda t: O.tf_step(t, mode, d), tf, i) @ adj for i in range(tf.size)])
            assert _close(adj_tf.reshape(-1), fd_tf, rel, abs_), (d, adj_tf.reshape(-1), fd_tf)
            checked += 1
    assert checked >= 90


@pytest.mark.parametrize("filter_mode", [1, 0], ids=["trilinear", "nearest"])
def test_sample_adjoint(oracle_built, filter_mode):
    """A 2 x 3 x 4 volume: the position derivative and the volume gradient of
    adj * sample(pos) against differences (eps 1e-5, rel 1e-5, abs 1e-6), at
    20 positions inside the volume away from cell faces.  Nearest sampling is
    piecewise constant: no position derivative, a one-voxel volume gradient."""
    O = oracle_built
    rng = np.random.default_rng(42)
    vol = rng.uniform(0.0, 1.0, size=(1, 2, 3, 4))
    hi = np.array(vol.shape[1:]) - 1.0
    for _ in range(20):
        while True:
            pos = rng.uniform(0.0, 1.0, size=3) * hi
            if np.min(np.abs(pos - np.round(pos))) > 1e-3:
                break
        adj = float(rng.normal())
        adj_pos, adj_vol = O.sample_step_adjoint(vol, filter_mode, pos, adj)
        fd_pos = np.array([_central(lambda p: O.sample_step(vol, filter_mode, p), pos, i) * adj for i in range(3)])
        assert _close(adj_pos, fd_pos, 1e-5, 1e-6), (pos, adj_pos, fd_pos)
        fd_vol = np.array([_central(lambda v: O.sample_step(v, filter_mode, pos), vol, i) * adj
                           for i in range(vol.size)])
        assert _close(adj_vol.reshape(-1), fd_vol, 1e-5, 1e-6), pos
        if filter_mode == 0:
            assert np.count_nonzero(adj_vol) == 1 and not adj_pos.any()


def test_ray_step_adjoint(oracle_built):
    """10 steps of one ray, box minimum (-0.2, -0.3, -0.4), voxel size
    (0.1, 0.05, 0.07), 20 draws of U(0.01, 0.99) for the ray start, direction
    and step: the derivatives of the sample positions with respect to the
    seven ray parameters against differences (eps 1e-5, rel 1e-5, abs 1e-6)."""
    O = oracle_built
    rng = np.random.default_rng(42)
    box_min, voxel, n = [-0.2, -0.3, -0.4], [0.1, 0.05, 0.07], 10
    for _ in range(20):
        x = rng.uniform(0.01, 0.99, size=7)
        adj_pos = rng.normal(size=(n, 3))
        f = lambda v: O.ray_steps(v[:3], v[3:6], box_min, voxel, 0.0, v[6], n).reshape(-1)
        a_start, a_dir, a_step = O.ray_steps_adjoint(x[:3], x[3:6], box_min, voxel, 0.0, x[6], adj_pos)
        got = np.concatenate([a_start, a_dir, [a_step]])
        fd = np.array([_central(f, x, i) @ adj_pos.reshape(-1) for i in range(7)])
        assert _close(got, fd, 1e-5, 1e-6), (got, fd)
