"""The shared-memory run of the re-march adjoint (dvr_record.cuh), checked on
the CPU for every checkpoint interval the entry points accept (1 to 64).

The kernel stores chunk sample i at i + pad * floor(i / L), L = ceil(len / 32)
and pad = 1 when L is even, computing floor(i / L) as a truncated FP32
product (i + 1/2) * (1 / L); lane j of the reverse pass reads its segment
[j L, j L + L) at k + j * pad.  This file restates that arithmetic in FP32
and checks, for the chunk cap and run size read from the kernel source:
the FP32 floor is exact, entries are distinct and inside the run, the
writer's and the reader's index agree, the 64-bit reads of a half-warp fall
in distinct bank pairs, and every chunk starts at a checkpoint.
"""
import os
import re

import numpy as np
import pytest

SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "diffdvr_gb300", "csrc", "dvr_record.cuh")


def _source_constants():
    text = open(SRC).read()
    cap = int(re.search(r"constexpr int kRemarchCap = (\d+);", text).group(1))
    extra = int(re.search(r"remarch_run_entries\(int chunk\) \{ return chunk \+ (\d+); \}", text).group(1))
    return cap, extra


def _chunk(K, cap):
    unit = K if K % 2 == 0 else 2 * K
    return unit * (cap // unit) if unit <= cap else 0


def _fp32_floor(i, L):
    inv = np.float32(1.0) / np.float32(L)
    return (((i.astype(np.float32) + np.float32(0.5)).astype(np.float32) * inv).astype(np.float32)).astype(np.int64)


@pytest.mark.parametrize("K", list(range(1, 65)))
def test_run_layout_for_every_interval(K):
    cap, extra = _source_constants()
    chunk = _chunk(K, cap)
    assert chunk > 0 and chunk % K == 0 and chunk % 2 == 0 and chunk <= cap
    entries = chunk + extra
    for length in range(1, chunk + 1):
        L = (length + 31) >> 5
        pad = (L & 1) ^ 1
        i = np.arange(length, dtype=np.int64)
        q = i // L
        assert np.array_equal(_fp32_floor(i, L), q), (K, length)
        phys = i + pad * q
        assert phys.max() < entries and np.unique(phys).size == length
        # the reader: lane j walks k in [min(len, j L), min(len, j L + L)) at k + j pad
        for j in range(32):
            s0 = min(length, j * L)
            s1 = min(length, s0 + L)
            k = np.arange(s0, s1)
            assert np.array_equal(k + j * pad, phys[s0:s1])
        # 64-bit reads: the lanes of each half-warp in distinct bank pairs
        stride = L + pad
        for t in range(L):
            for half in (0, 16):
                lanes = [j for j in range(half, half + 16) if j * L + t < length]
                banks = [((j * stride + t) * 2) % 32 for j in lanes]
                assert len(set(banks)) == len(banks), (K, length, t)
