"""The integer-pipe float<->double conversions of the mixed path against the hardware conversions.

Every FP32 value that meets an FP64 one in the mixed kernels goes through f2d / d2f (dyn_common.cuh);
the mixed path's parity rests on their being bit-identical to plain casts. Widening is checked over all
2^32 binary32 encodings, narrowing over the widened values and 2^32 hashed binary64 encodings (raw bit
patterns, binary32's exponent range, exact rounding ties and their neighbours)."""
import pytest

pytestmark = pytest.mark.gpu


def test_conversions_bit_identical_to_hardware():
    from atsat_gb300 import dyn
    widen, narrow = dyn.conv_selftest(1 << 32)
    assert (widen, narrow) == (0, 0)
