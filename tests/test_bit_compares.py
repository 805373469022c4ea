"""The integer comparisons on bit patterns that the kernels use in place of FP comparisons
(csrc/gom_device.cuh: is_zero, pos_finite_or_inf, gt_nonneg, lt_of_nonneg, nan_bits), restated
here on numpy's int64 / int32 views and checked against the FP comparisons over every pair of a
table of special and ordinary values (signed zeros, subnormals, infinities, NaNs of both signs),
each helper where its precondition holds.  The device runs the same check
(gom_selftest_compares, tests/test_gpu_measure.py)."""
import numpy as np
import pytest


def _table(dtype):
    f = np.finfo(dtype)
    base = [0.0, float(f.smallest_subnormal), float(f.tiny) * (1 - f.eps), float(f.tiny), 1e-30, 1e-5, 0.25, 0.5,
            1.0, 1.0 + float(f.eps), 2.0, 50.0, 3.14159, 0.1, float(f.max), np.inf, np.nan]
    v = np.array(base, dtype=dtype)
    return np.concatenate([v, -v])   # -0, negatives, -inf, a NaN with its sign bit set


@pytest.mark.parametrize("dtype,itype,inf_bits", [(np.float64, np.int64, 0x7ff0000000000000),
                                                 (np.float32, np.int32, 0x7f800000)])
def test_bit_pattern_comparisons(dtype, itype, inf_bits):
    v = _table(dtype)
    b = v.view(itype).astype(np.int64)
    is_nan = np.isnan(v)
    with np.errstate(invalid="ignore"):
        # is_zero: the pattern shifted left by one is zero
        shifted = (b.astype(np.uint64) << np.uint64(1)) & np.uint64(2 ** (8 * np.dtype(itype).itemsize) - 1)
        assert np.array_equal(shifted == 0, v == 0)
        # pos_finite_or_inf: 0 < bits <= inf
        assert np.array_equal((b > 0) & (b <= inf_bits), v > 0)
        # nan_bits: magnitude above inf
        assert np.array_equal((b & (2 ** (8 * np.dtype(itype).itemsize - 1) - 1)) > inf_bits, is_nan)
        checked = 0
        for i, x in enumerate(v):
            for j, y in enumerate(v):
                xb, yb = b[i], b[j]
                if yb >= 0 or is_nan[j]:   # gt_nonneg: y >= +0 or NaN
                    got = yb >= 0 and yb <= inf_bits and xb > yb and xb <= inf_bits
                    assert got == (x > y), (x, y)
                    checked += 1
                if xb >= 0:                # lt_of_nonneg: x with its sign bit clear
                    got = yb <= inf_bits and xb < yb
                    assert got == (x < y), (x, y)
                    checked += 1
    assert checked > 500
