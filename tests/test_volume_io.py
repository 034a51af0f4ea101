"""The .cvol format and the Marschner-Lobb volume (diffdvr_gb300.volume_io):
round trips, the header layout, x-fastest file order, the reference's own
C60Large.cvol where the reference sources are present, and known values of
the Marschner-Lobb function."""
import os

import numpy as np
import pytest

from diffdvr_gb300 import volume_io as vio
from oracle.oracle import REFERENCE_ROOT

REF_CVOL = os.path.join(REFERENCE_ROOT, "pytests", "volumes", "C60Large.cvol")


@pytest.mark.parametrize("dtype,tol", [("float32", 0.0), ("uint8", 0.5 / 255), ("uint16", 0.5 / 65535)])
def test_cvol_round_trip(tmp_path, dtype, tol):
    rng = np.random.default_rng(0)
    vol = rng.uniform(0, 1, (1, 5, 7, 9)).astype(np.float32)
    path = str(tmp_path / "v.cvol")
    vio.save_cvol(path, vol, world_size=(2.0, 3.0, 4.0), dtype=dtype)
    size = os.path.getsize(path)
    assert size == 64 + 5 * 7 * 9 * {"float32": 4, "uint8": 1, "uint16": 2}[dtype]
    hdr = vio.read_cvol_header(path)
    assert hdr["size"] == (5, 7, 9) and not hdr["compressed"]
    np.testing.assert_allclose(hdr["world_size"], (2.0, 3.0, 4.0), rtol=1e-12)
    got, world = vio.load_cvol(path)
    assert got.shape == (1, 5, 7, 9) and got.dtype == np.float32
    np.testing.assert_allclose(got, vol, rtol=0, atol=tol + 1e-7)
    # file order is x fastest: the first X values are vol[0, :, 0, 0]
    with open(path, "rb") as f:
        f.seek(64)
        first = np.frombuffer(f.read(5 * np.dtype(dtype).itemsize), dtype=dtype)
    scale = {"float32": 1.0, "uint8": 1 / 255, "uint16": 1 / 65535}[dtype]
    np.testing.assert_allclose(first.astype(np.float64) * scale, got[0, :, 0, 0], rtol=0, atol=1e-6)
    # the returned view keeps the file's memory order: strides 1, X, X*Y elements
    assert got[0].strides == (4, 4 * 5, 4 * 5 * 7)


def test_cvol_rejects_bad_files(tmp_path):
    p = str(tmp_path / "bad.cvol")
    with open(p, "wb") as f:
        f.write(b"xvol" + bytes(60))
    with pytest.raises(ValueError, match="magic"):
        vio.load_cvol(p)
    vol = np.zeros((2, 2, 2), np.float32)
    vio.save_cvol(p, vol)
    with open(p, "r+b") as f:  # mark compressed
        f.seek(56)
        f.write(b"\x01")
    with pytest.raises(NotImplementedError, match="LZ4"):
        vio.load_cvol(p)


@pytest.mark.skipif(not os.path.exists(REF_CVOL), reason="the reference's dataset is not present")
def test_reference_c60_volume():
    hdr = vio.read_cvol_header(REF_CVOL)
    assert hdr["size"] == (128, 128, 128) and hdr["dtype"] == 0 and not hdr["compressed"]
    vol, world = vio.load_cvol(REF_CVOL)
    assert vol.shape == (1, 128, 128, 128) and 0.0 <= vol.min() and vol.max() <= 1.0
    with open(REF_CVOL, "rb") as f:
        f.seek(64 + 128 * 128 * 64)  # slice z = 64
        raw = np.frombuffer(f.read(128 * 128), np.uint8).reshape(128, 128)  # [y][x]
    # bit-identical to the reference loader's src[i] / 255.0f (renderer/volume.cpp:244)
    assert np.array_equal(vol[0, :, :, 64], raw.T.astype(np.float32) / np.float32(255.0))


@pytest.mark.parametrize("dtype,mx", [("uint8", 255), ("uint16", 65535)])
def test_cvol_integer_values_divide_like_the_reference(tmp_path, dtype, mx):
    """Every integer value v loads as float32(v) / float32(max), bit for bit,
    as the reference's loader computes it (renderer/volume.cpp:244, :251);
    multiplying by the reciprocal differs in the last bit for some values."""
    n = mx + 1
    path = str(tmp_path / "all.cvol")
    vio.save_cvol(path, (np.arange(n, dtype=np.float64) / mx).reshape(n, 1, 1), dtype=dtype)
    got, _ = vio.load_cvol(path)
    want = np.arange(n, dtype=np.float32) / np.float32(mx)
    assert np.array_equal(got[0, :, 0, 0], want)


def test_marschner_lobb_values():
    R = 65  # the grid holds 0 and +-1 exactly
    v = vio.marschner_lobb(R)
    assert v.shape == (1, R, R, R) and v.dtype == np.float32
    c = R // 2
    assert abs(v[0, c, c, c] - 0.6) < 1e-7          # r = 0, z = 0: (1 + 0.25 * 2) / 2.5
    assert abs(v[0, c, c, R - 1] - 0.2) < 1e-7      # z = 1: (0 + 0.5) / 2.5
    assert abs(v[0, c, c, 0] - 1.0) < 1e-7          # z = -1: (2 + 0.5) / 2.5
    assert 0.0 <= v.min() and v.max() <= 1.0 + 1e-6
    # a generic point against the formula
    g = -1.0 + np.arange(R, dtype=np.float32) * np.float32(2.0 / (R - 1))
    x, y, z = float(g[10]), float(g[40]), float(g[23])
    r = np.hypot(x, y)
    ref = ((1 - np.sin(np.pi * z / 2)) + 0.25 * (1 + np.cos(12 * np.pi * np.cos(np.pi * r / 2)))) / 2.5
    assert abs(v[0, 10, 40, 23] - ref) < 1e-6
