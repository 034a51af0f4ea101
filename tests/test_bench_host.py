"""bench.py's host-side arithmetic on the CPU: the algorithmic bytes behind
`roofline.achieved`, the clock record's parsing and the peak fallback."""
import os
import sys
from types import SimpleNamespace

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
