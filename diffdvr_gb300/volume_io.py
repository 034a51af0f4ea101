"""Volume inputs of the ray marcher: the ``.cvol`` file format and the
Marschner-Lobb test volume.

``.cvol`` (renderer/volume.cpp:62-270): a 64-byte header

    bytes 0-3    magic "cvol"
    bytes 4-27   size X, Y, Z            (3 x uint64, little endian)
    bytes 28-51  voxel size X, Y, Z      (3 x float64; world size = voxel size x size)
    bytes 52-55  data type               (int32: 0 uint8, 1 uint16, 2 float32)
    byte  56     compression flag        (0: raw, else LZ4 chunks)
    bytes 57-63  padding

followed by the X*Y*Z values with x fastest (slice by slice in z).  Integer
data are scaled to [0, 1] (value / 255 or / 65535).  The renderer's volume
layout is [b][x][y][z]; ``load_cvol`` returns a view with exactly the file's
memory order (strides 1, X, X*Y in elements along x, y, z), which the
renderer accepts as it is.  LZ4-compressed files are written in chunks
whose framing the reference's LZ4 wrapper defines (renderer/volume.cpp:127-137);
loading one raises NotImplementedError.

Marschner-Lobb (renderer/volume_implicit.cpp:28-42, sampled as
renderer/volume.cpp:369-387): on [-1, 1]^3 sampled at ``resolution`` points
per axis,

    rho(x, y, z) = ((1 - sin(pi z / 2)) + alpha (1 + cos(2 pi fM cos(pi r / 2))))
                   / (2 (1 + alpha)),   r = sqrt(x^2 + y^2),

with fM = 6 and alpha = 0.25 by default (Marschner and Lobb, "An evaluation
of reconstruction filters for volume rendering", 1994).  The grid
coordinates are computed in float32 and the function in float64, as the
reference does.
"""
from __future__ import annotations

import struct
from typing import Tuple

import numpy as np

MAGIC = b"cvol"
HEADER_BYTES = 64
_TYPES = {0: np.uint8, 1: np.uint16, 2: np.float32}
# integer data are divided by the type's maximum in float32, as the
# reference's loader does (renderer/volume.cpp:244, :251)
_DIVISOR = {0: np.float32(255.0), 1: np.float32(65535.0), 2: None}


def read_cvol_header(path: str) -> dict:
    """The header fields of a .cvol file."""
    with open(path, "rb") as f:
        h = f.read(HEADER_BYTES)
    if len(h) < HEADER_BYTES or h[:4] != MAGIC:
        raise ValueError(f"{path}: not a .cvol file (illegal magic number)")
    sx, sy, sz = struct.unpack_from("<3Q", h, 4)
    vx, vy, vz = struct.unpack_from("<3d", h, 28)
    dtype, = struct.unpack_from("<i", h, 52)
    compressed = h[56] != 0
    if dtype not in _TYPES:
        raise ValueError(f"{path}: unknown data type {dtype}")
    return {"size": (int(sx), int(sy), int(sz)), "voxel_size": (vx, vy, vz), "dtype": dtype,
            "compressed": compressed,
            "world_size": (vx * sx, vy * sy, vz * sz)}


def load_cvol(path: str) -> Tuple[np.ndarray, Tuple[float, float, float]]:
    """Loads a .cvol file; returns (volume, world_size) with volume a float32
    array of shape 1*X*Y*Z in the file's x-fastest memory order."""
    hdr = read_cvol_header(path)
    if hdr["compressed"]:
        raise NotImplementedError(f"{path}: LZ4-compressed .cvol files are not supported "
                                  "(their chunk framing is that of the reference's LZ4 wrapper)")
    X, Y, Z = hdr["size"]
    n = X * Y * Z
    if n > np.iinfo(np.int32).max:
        raise ValueError(f"{path}: the volume must have fewer than 2^31 voxels")
    t = _TYPES[hdr["dtype"]]
    raw = np.fromfile(path, dtype=np.dtype(t).newbyteorder("<"), count=n, offset=HEADER_BYTES)
    if raw.size != n:
        raise ValueError(f"{path}: truncated data ({raw.size} of {n} values)")
    div = _DIVISOR[hdr["dtype"]]
    data = raw.astype(np.float32) / div if div is not None else raw.astype(np.float32)
    # file order: x fastest -> [z][y][x] in C order -> view as [x][y][z]
    vol = data.reshape(Z, Y, X).transpose(2, 1, 0)[None]
    return vol, hdr["world_size"]


def save_cvol(path: str, volume, world_size=(1.0, 1.0, 1.0), dtype: str = "float32") -> None:
    """Writes a volume (X*Y*Z or 1*X*Y*Z, any layout) as an uncompressed
    .cvol file with float32, uint8 or uint16 data (integers: round(v * max),
    values clamped to [0, 1])."""
    v = np.asarray(volume, dtype=np.float64)
    if v.ndim == 4:
        if v.shape[0] != 1:
            raise ValueError("save_cvol writes one volume (batch size 1)")
        v = v[0]
    if v.ndim != 3:
        raise ValueError("the volume must have 3 dimensions (X, Y, Z)")
    X, Y, Z = v.shape
    code = {"uint8": 0, "uint16": 1, "float32": 2}[dtype]
    if code == 2:
        body = v.astype(np.float32)
    else:
        mx = 255.0 if code == 0 else 65535.0
        body = np.rint(np.clip(v, 0.0, 1.0) * mx).astype(_TYPES[code])
    header = bytearray(HEADER_BYTES)
    header[0:4] = MAGIC
    struct.pack_into("<3Q", header, 4, X, Y, Z)
    struct.pack_into("<3d", header, 28, *(float(world_size[i]) / v.shape[i] for i in range(3)))
    struct.pack_into("<i", header, 52, code)
    with open(path, "wb") as f:
        f.write(bytes(header))
        f.write(np.ascontiguousarray(body.transpose(2, 1, 0)).astype(body.dtype.newbyteorder("<")).tobytes())


def marschner_lobb(resolution: int, fM: float = 6.0, alpha: float = 0.25) -> np.ndarray:
    """The Marschner-Lobb test volume at resolution^3 on [-1, 1]^3, float32,
    shape 1*R*R*R ([b][x][y][z], z fastest)."""
    R = int(resolution)
    if R < 2:
        raise ValueError("resolution must be at least 2")
    scale = np.float32(2.0) / np.float32(R - 1)
    c = (np.float32(-1.0) + np.arange(R, dtype=np.float32) * scale).astype(np.float32).astype(np.float64)
    x, y, z = c[:, None, None], c[None, :, None], c[None, None, :]
    r = np.sqrt(x * x + y * y)
    pr = np.cos(2 * np.pi * fM * np.cos(np.pi * r / 2))
    num = (1 - np.sin(np.pi * z / 2)) + alpha * (1 + pr)
    return (num / (2 * (1 + alpha))).astype(np.float32)[None]
