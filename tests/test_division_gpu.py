"""The engine's division by a constant divisor (j2d5pt's /118, j3d27pt's
/159, and any divisor a caller passes) is bit-identical to IEEE division."""
import numpy as np
import pytest

from gbstencil import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [118.0, 159.0, 3.0, 0.1, 7.25, -118.0, 1e-6, 3e5, 0.3])
def test_float_checked_division_every_input(d):
    assert capi.check_division(np.float32, d, 0, checked=True) == 0


@pytest.mark.parametrize("d", [118.0, 159.0])
def test_float_unchecked_division_proven_for_artifact_divisors(d):
    """The engine skips the remainder test only for these divisors."""
    assert capi.check_division(np.float32, d, 0, checked=False) == 0


@pytest.mark.parametrize("d", [118.0, 159.0, 3.0, 0.1, -7.25, 1e-20, 0.3])
def test_double_division_sampled(d):
    assert capi.check_division(np.float64, d, 1 << 26, checked=True) == 0
