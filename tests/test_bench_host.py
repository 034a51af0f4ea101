"""bench.py's host-side logic on the CPU: the algorithmic bytes behind
`roofline.achieved`, the clock record's parsing, the peak fallback, the
batched workload's instances and its CPU arm, and the workload options."""
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_algorithmic_bytes_of_the_recorded_tf_reconstruction_step():
    """Forward: V*s_v volume + P*(16 colour + 4 termination + 4 record
    offset) + c*4 checkpoints + S*8 record.  Record adjoint: P*(4 termination
    + 16 adj_color + 4 offset) + S*8 record + the TF gradient read and
    written.  At 256^3 BF16, 8 views of 256^2, 90 M samples, every ray
    recorded (no checkpoints): about 766 MB and 730 MB."""
    w = SimpleNamespace(grads=("tf",))
    V, s_v, P, S, R_C = 256 ** 3, 2, 8 * 256 * 256, 90_000_000, 64 * 4
    fwd, adj = bench.algorithmic_bytes(w, s_v, V, P, S, ck_written=0, recorded=True, record_kernel=True,
                                       tf_numel=R_C)
    assert fwd == V * s_v + P * 24 + S * 8
    assert adj == P * 24 + S * 8 + R_C * 8
    assert fwd == pytest.approx(766e6, rel=0.01)
    assert adj == pytest.approx(730e6, rel=0.01)


def test_algorithmic_bytes_of_the_general_adjoint():
    """Without a record the adjoint re-reads the volume and the checkpoints
    and read-modify-writes each requested gradient once (volume V*4*2,
    camera P*24*2, TF R*C*4*2)."""
    V, s_v, P, c, R_C = 128 ** 3, 4, 64 * 256 * 256, 12345, 2
    w = SimpleNamespace(grads=("volume",))
    fwd, adj = bench.algorithmic_bytes(w, s_v, V, P, 0, ck_written=c, recorded=False, record_kernel=False,
                                       tf_numel=R_C)
    assert fwd == V * s_v + P * 20 + c * 4
    assert adj == V * s_v + P * 20 + c * 4 + V * 8
    w = SimpleNamespace(grads=("tf", "volume", "camera"))
    _, adj = bench.algorithmic_bytes(w, s_v, V, P, 0, ck_written=c, recorded=False, record_kernel=False,
                                     tf_numel=R_C)
    assert adj == V * s_v + P * 20 + c * 4 + R_C * 8 + V * 8 + P * 48


def test_compulsory_bytes_of_the_measurement_plan():
    """The roofline's primary bytes: volume once per launch, colour +
    termination written by the forward and read back with the output adjoint
    by the adjoint, checkpoints (4 B) written and read, gradients
    read-modify-written once; no sample record.  At the TF-reconstruction
    workload with every ray recorded (no checkpoints) the forward moves
    33.6 MB + 10.5 MB."""
    V, s_v, P, R_C = 256 ** 3, 2, 8 * 256 * 256, 64 * 4
    w = SimpleNamespace(grads=("tf",))
    fwd, adj = bench.compulsory_bytes(w, s_v, V, P, ck_written=0, tf_numel=R_C)
    assert fwd == V * s_v + P * 20
    assert fwd == pytest.approx(44.0e6, rel=0.01)
    assert adj == V * s_v + P * 36 + R_C * 8
    c = 1000
    w = SimpleNamespace(grads=("tf", "volume", "camera"))
    fwd, adj = bench.compulsory_bytes(w, s_v, V, P, ck_written=c, tf_numel=R_C)
    assert fwd == V * s_v + P * 20 + c * 4
    assert adj == V * s_v + P * 36 + c * 4 + R_C * 8 + V * 8 + P * 48
    # the forward method: forward variables written once and read once by the contraction
    w = SimpleNamespace(grads=("tf",))
    fwd, adj = bench.compulsory_bytes(w, s_v, V, P, ck_written=0, tf_numel=R_C, D=R_C)
    assert fwd == V * s_v + P * 20 + P * R_C * 16
    assert adj == P * R_C * 16 + P * 16 + R_C * 8


def test_issue_bound_from_the_committed_profile(monkeypatch, tmp_path):
    """Warp instructions per sample x samples / time against 152 SMs x 4
    issue slots x the maximum clock."""
    d = bench.issue_bound("tf_reconstruction_256", "forward", 90_000_000, 0.8)
    assert d is not None and d["unit"] == "T warp-instr/s"
    per = d["warp_instructions_per_sample"]
    assert d["achieved"] == pytest.approx(per * 90e6 / 0.8e-3 / 1e12)
    assert d["peak"] == pytest.approx(152 * 4 * 2070e6 / 1e12)
    assert 0 < d["frac"] < 1.2
    # every kernel the bench line asks for has its committed figure: the
    # record arm's forward and adjoint, the memory-lean arm's re-march adjoint
    for kernel in ("forward", "adjoint", "adjoint_remarch"):
        assert bench.issue_bound("tf_reconstruction_256", kernel, 90_000_000, 1.0) is not None, kernel
    assert bench.issue_bound("no_such_workload", "forward", 1, 1.0) is None
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.issue_bound("tf_reconstruction_256", "forward", 1, 1.0) is None


def test_clock_record_summary():
    """Median SM clock under load, the maximum clock, and every throttle
    reason seen active in any sample of the timed region."""
    cs = bench.ClockSampler(0)
    cs.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = cs.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    cs.lines = ["0, 1500, 2070, 700, 0x48, Active, Active, Not Active, Not Active"]
    assert cs.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]
    cs.lines = []
    assert cs.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_peak_falls_back_without_measured_peaks(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"hbm_gbs": 6786.2}')
    assert bench.measured_peaks() == (6786.2, "measured")


def test_batched_uneven_instances():
    """The batched workload's instances: volume edges and image sizes from
    their sets, a 4-Gaussian TF with widths in [0.02, 0.2], step 0.5 voxel,
    per-pixel rays of one view, TF and volume gradients."""
    from diffdvr_gb300 import scenes
    ws = scenes.batched_uneven(seed=3, n=6, n_blobs=2)
    assert len(ws) == 6
    for w in ws:
        res = w.volume.shape[1]
        assert w.volume.shape == (1, res, res, res) and res in (32, 64, 96, 128, 192, 256)
        assert w.width == w.height and w.width in (64, 128, 256, 512)
        assert w.ray_start.shape == w.ray_dir.shape == (1, w.height, w.width, 3)
        assert w.tf.shape == (1, 4, 6) and np.all((w.tf[0, :, 5] >= 0.02) & (w.tf[0, :, 5] <= 0.2))
        assert w.step_size == pytest.approx(0.5 / (res - 1))
        assert (w.tf_mode, w.filter_mode, w.blend_mode) == (3, 1, 0) and set(w.grads) == {"tf", "volume"}


def test_batched_reference_arm_times_every_instance(monkeypatch):
    """The CPU arm of the batched workload times each instance with an equal
    share of the budget and reports the mean rate."""
    from diffdvr_gb300 import scenes
    ws = scenes.batched_uneven(seed=3, n=2, n_blobs=2)
    seen = []

    def fake_time_cpu(w, volume, budget, kind):
        seen.append((w, budget))
        return 10.0 * len(seen), ""

    monkeypatch.setattr(bench, "time_cpu", fake_time_cpu)
    rate, desc = bench.time_cpu_instances(ws, 1.0, "port")
    assert [w for w, _ in seen] == ws and all(b == pytest.approx(0.5) for _, b in seen)
    assert rate == pytest.approx(15.0) and "2 instances" in desc


def test_workload_options_parse(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "batched_uneven_32"])
    a = bench.parse()
    assert (a.res, a.views, a.image) == (256, 1, 512) and bench.WORKLOADS[a.workload]["instances"] == 32
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    assert bench.parse().workload == "tf_reconstruction_256"


def test_crop_keeps_the_sampling_grid(oracle_built):
    """A crop's box is the sub-volume's extent on the same voxel grid: a
    world point samples the same density in the crop as in the full volume
    (the oracle's trilinear sample), and the chosen views' rays are kept."""
    from diffdvr_gb300 import scenes
    O = oracle_built
    w = scenes.plain_cpu_64(seed=0)
    w.ray_start = np.concatenate([w.ray_start, w.ray_start])  # a second view looking the other way
    w.ray_dir = np.concatenate([w.ray_dir, -w.ray_dir])
    w.viewport = np.concatenate([w.viewport, w.viewport])
    c = scenes.crop(w, (10, 20, 30), 16, views=[1])
    assert c.volume.shape == (1, 16, 16, 16) and c.ray_dir.shape == (1, 128, 128, 3)
    assert np.array_equal(c.ray_dir[0], w.ray_dir[1])
    voxel = np.asarray(w.box_size) / 63
    assert np.allclose(np.asarray(c.box_size) / 15, voxel)
    assert np.allclose(c.box_min, np.asarray(w.box_min) + np.array([10, 20, 30]) * voxel)
    rng = np.random.default_rng(0)
    for _ in range(20):
        p = np.array([10, 20, 30]) + rng.uniform(0.0, 15.0, 3)  # voxel coordinates of the full volume
        assert O.sample_step(c.volume, 1, p - [10, 20, 30]) == pytest.approx(O.sample_step(w.volume, 1, p), abs=1e-6)
    with pytest.raises(ValueError):
        scenes.crop(w, (60, 0, 0), 16)


def _orbit_checks(w, views, image, fov_deg=45.0, radius=3.0):
    assert w.ray_start.shape == w.ray_dir.shape == (views, image, image, 3)
    eyes = w.ray_start[:, 0, 0]
    assert np.allclose(np.linalg.norm(eyes, axis=1), radius, rtol=1e-5)  # orbit camera around the origin
    assert np.allclose(np.linalg.norm(w.ray_dir, axis=-1), 1.0, atol=1e-5)
    assert w.fov_y == pytest.approx(np.radians(fov_deg))
    assert tuple(w.box_min) == (-0.5, -0.5, -0.5) and tuple(w.box_size) == (1.0, 1.0, 1.0)


def test_workloads_follow_their_configurations():
    """The seeded synthetic workloads have the shapes and distributions of
    the configurations they stand for (at reduced sizes where the generator
    takes them): blob or ellipsoid volumes in [0, 1], the TF type and size,
    orbit views at radius 3 and 45 degrees, the step in voxels, the
    gradients."""
    from diffdvr_gb300 import scenes
    w = scenes.tf_reconstruction_256(seed=1, res=32, views=8, image=16)
    _orbit_checks(w, 8, 16)
    assert w.volume.shape == (1, 32, 32, 32) and 0 <= w.volume.min() and w.volume.max() <= 1
    assert w.tf.shape == (1, 64, 4) and (w.tf_mode, w.filter_mode, w.blend_mode) == (1, 1, 0)
    assert w.step_size == pytest.approx(0.25 / 31) and w.grads == ("tf",)
    lat, _ = scenes.fibonacci_sphere(8)
    assert len(np.unique(np.round(lat, 6))) == 8  # distinct Fibonacci views

    w = scenes.absorption_recon_128(seed=2, views=4, image=8)
    _orbit_checks(w, 4, 8)
    assert w.volume.shape == (1, 128, 128, 128) and w.volume.min() == 0.0
    inside = w.volume[w.volume > 0]
    assert inside.min() >= 0.2 and inside.max() <= 1.0  # ellipsoid densities U(0.2, 1) on a zero background
    assert np.array_equal(w.tf, [[[20.0, 1.0]]]) and w.tf_mode == 0 and w.grads == ("volume",)
    assert w.step_size == pytest.approx(0.5 / 127)

    w = scenes.large_mixed_512(seed=4, res=32, views=2, image=8)
    _orbit_checks(w, 2, 8)
    assert w.tf.shape == (1, 16, 5) and w.tf_mode == 2 and w.tf[0, 0, 4] == 0 and w.tf[0, -1, 4] == 1
    assert np.all(np.diff(w.tf[0, :, 4]) >= 0) and w.tf[0, :, 3].max() > 1  # sorted positions, absorption x10
    assert set(w.grads) == {"camera", "volume", "tf"} and w.step_size == pytest.approx(0.5 / 31)

    w = scenes.plain_cpu_64(seed=0)
    _orbit_checks(w, 1, 128)
    assert w.volume.shape == (1, 64, 64, 64) and w.tf.shape == (1, 8, 5) and set(w.grads) == {"tf", "volume"}

    p = scenes.preshaded_256(seed=1, res=16, views=2, image=8)
    assert p.volume.shape == (4, 16, 16, 16) and (p.tf_mode, p.filter_mode) == (5, 3)


def test_ray_gradient_report_leaves_out_rounding_decided_rays():
    """oracle.check's ray-gradient report: rays whose first sample lies on
    the box face at the upper end of an axis (the cell there is decided by
    rounding) are left out of the unambiguous-ray figure and counted; a ray
    entering through a lower face is kept; the raw figure keeps them all."""
    from oracle import check, oracle as O
    starts = np.array([[2.0, 0.01, 0.02], [-2.0, 0.01, 0.02], [0.03, 2.0, -0.01], [0.02, 0.01, -2.0]])
    dirs = np.array([[-1.0, 0, 0], [1.0, 0, 0], [0, -1.0, 0], [0, 0, 1.0]])
    sc = O.Scene(width=4, height=1, volume=np.zeros((1, 9, 9, 9), np.float32), tf=np.zeros((1, 2, 2), np.float32),
                 step_size=np.full((1, 1, 1), 0.3, np.float32), box_min=np.array([[-0.5, -0.5, -0.5]], np.float32),
                 box_size=np.ones((1, 3), np.float32), filter_mode=1, tf_mode=0, blend_mode=0, camera_mode=0)
    sc.ray_start = starts.reshape(1, 1, 4, 3).astype(np.float32)
    sc.ray_dir = dirs.reshape(1, 1, 4, 3).astype(np.float32)
    decided = check.rounding_decided_rays(sc)
    assert decided.tolist() == [[[True, False, True, False]]]
    rng = np.random.default_rng(4)
    g64 = rng.normal(size=(1, 1, 4, 3))
    g32 = g64 * (1 + 1e-6 * rng.normal(size=g64.shape))
    got = g64.copy()
    got[0, 0, 0] += 5.0  # a whole sample's derivative apart on a decided ray
    r = check._well_conditioned(got, g32, g64, decided)
    assert r["rays"] == 4 and r["rays_left_out"] == 2
    assert r["rel_l2_unambiguous_rays"] == 0.0 and r["rel_l2_f32_unambiguous_rays"] < 1e-5
    assert check.rel_l2(got, g64) > 1e-1


def test_gather_model_against_the_l2_peak():
    """The gather model's bytes per second and its fraction of the measured
    L2 copy bandwidth."""
    g = bench.gather_model(1e9, 1.0, {"GBps": 2000.0, "how": "test"})
    assert g["achieved_GBps"] == pytest.approx(1000.0) and g["frac"] == pytest.approx(0.5)
    assert g["bytes_per_step"] == 10**9 and g["l2_peak_GBps"] == 2000.0
