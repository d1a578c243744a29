"""Device probes that set the roofline denominators and tile shapes."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_plausible(pkg):
    tf = pkg.measure_fp64_peak(0)
    assert 0.3 < tf < 5.0


def test_mma_cycles_grow_with_width(pkg):
    cyc = {n: pkg.measure_mma_cycles(0, n) for n in (32, 64, 128, 256)}
    assert all(8.0 < v < 1000.0 for v in cyc.values()), cyc
    assert cyc[256] > cyc[32], cyc
