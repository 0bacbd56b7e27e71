"""The mixed force kernel accumulates fixed-point force sums without
float->int64 conversion instructions: each term v is split exactly as
v = rint(v/2^23) * 2^23 + l and both parts are rounded by the magic-number
method (kernels_force.cu, FixAcc).  This emulates that arithmetic bit for bit
with IEEE float32 on the CPU and checks it equals rint(v) summed in int64,
for every term magnitude the split handles (|v| <= 2^44)."""
from __future__ import annotations

import numpy as np

M = np.float32(12582912.0)            # 1.5 * 2^23
MB = np.uint32(0x4B400000)
FOLD = 256


def split_sum(values: np.ndarray) -> int:
    """Terms of one lane (at most 256; longer lists take the exact path)."""
    assert len(values) <= FOLD
    hi = np.uint32(0)
    lo = np.uint32(0)
    n = 0
    for v in values.astype(np.float32):
        assert abs(float(v)) <= 2.0 ** 44   # larger terms are re-accumulated exactly
        t = np.float32(v * np.float32(2.0 ** -23))
        a = np.float32(t + M)
        h = np.float32(a - M)
        l = np.float32(np.float64(h) * -8388608.0 + np.float64(v))   # fmaf: one rounding
        b = np.float32(l + M)
        hi = np.uint32((int(hi) + int(a.view(np.uint32))) & 0xFFFFFFFF)
        lo = np.uint32((int(lo) + int(b.view(np.uint32))) & 0xFFFFFFFF)
        n += 1
    hh = np.uint32((int(hi) - n * int(MB)) & 0xFFFFFFFF).view(np.int32)
    ll = np.uint32((int(lo) - n * int(MB)) & 0xFFFFFFFF).view(np.int32)
    return (int(hh) << 23) + int(ll)


def exact_sum(values: np.ndarray) -> int:
    return int(sum(int(np.rint(np.float64(v))) for v in values.astype(np.float32)))


def test_split_exact_random_magnitudes():
    rng = np.random.default_rng(0)
    for scale_exp in (0, 10, 22, 23, 30, 40, 42):
        v = (rng.standard_normal(256) * 2.0 ** scale_exp).astype(np.float32)
        assert split_sum(v) == exact_sum(v), scale_exp


def test_split_exact_ties_and_edges():
    edges = [0.5, 1.5, 2.5, -0.5, -1.5, 2.0 ** 22, -2.0 ** 22, 2.0 ** 23 + 2.0 ** 22, 1.5 * 2 ** 23,
             2.0 ** 44, -2.0 ** 44, 2.0 ** 44 * 0.9999999, 3.0 * 2 ** 22, 1e-30, -1e-30, 0.0, 7.5,
             (2 ** 23 - 1) * 2.0 ** 21, 0.49999997, 8388607.5, 8388608.5, -8388607.5]
    v = np.array(edges, dtype=np.float32)
    assert split_sum(v) == exact_sum(v)
    for e in edges:
        one = np.array([e], dtype=np.float32)
        assert split_sum(one) == exact_sum(one), e


def test_split_exact_full_lane():
    """A lane's maximum of 256 terms, all near the top of the exact range."""
    rng = np.random.default_rng(1)
    v = np.clip(rng.standard_normal(256) * 2.0 ** 43, -2.0 ** 44, 2.0 ** 44).astype(np.float32)
    assert split_sum(v) == exact_sum(v)
    same = np.full(256, 2.0 ** 44, dtype=np.float32)
    assert split_sum(same) == exact_sum(same)
    assert split_sum(-same) == exact_sum(-same)
