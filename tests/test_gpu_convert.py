"""The mixed form's float <-> double conversions on the integer pipes give the hardware
conversion's bits (IEEE round to nearest, ties to even) on seeded bit patterns: random ones
over the whole double range, exact halfway cases, the ends of the float range, signed zeros
and ordinary magnitudes."""
import pytest

from cfd3d_gb300 import native

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_conversions_match_hardware(seed):
    d2f, f2d = native.convert_selftest(1 << 24, seed)
    assert (d2f, f2d) == (0, 0)


def test_convert_selftest_rejects_bad_arguments():
    with pytest.raises(native.Cfd3dError):
        native.convert_selftest(0)


def test_convert_rate_measures():
    r = native.convert_rate()
    assert set(r) == {"d2f_hw", "d2f_int", "f2d_hw", "f2d_int"}
    assert all(v > 0.0 for v in r.values())
