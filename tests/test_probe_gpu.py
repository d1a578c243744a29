"""The device probe that sets the FP64 path's roofline denominator."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_plausible(pkg):
    tf = pkg.measure_fp64_peak(0)
    assert 0.3 < tf < 5.0

