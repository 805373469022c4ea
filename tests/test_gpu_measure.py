"""The device measurements and self-tests of the library: the FP64 warp-issue rate with all and
with one active lane per warp (gom_measure_fp64_issue), and the integer comparisons on bit
patterns that the kernels use in place of FP64 comparisons, each against the FP comparison it
stands for on special values (gom_selftest_compares)."""
import pytest

from gom_release_gb300.core import GomError, measure_fp64_issue, measure_fp64_peak, selftest_compares

pytestmark = pytest.mark.gpu


def test_bit_pattern_comparisons_equal_fp_comparisons(gpu_lib):
    checked, bad = selftest_compares(gpu_lib)
    assert checked > 2000
    assert bad == 0


def test_fp64_issue_rate_measured(gpu_lib):
    full = measure_fp64_issue(gpu_lib, 32)
    one = measure_fp64_issue(gpu_lib, 1)
    assert full > 0.0 and one > 0.0
    # thread rate / 32 and the warp rate of the same chains agree
    assert abs(measure_fp64_peak(gpu_lib) * 1e9 / 2.0 / 32.0 - full) < 0.1 * full   # GFLOP/s: 2 flops an FMA
    with pytest.raises(GomError):
        measure_fp64_issue(gpu_lib, 0)
