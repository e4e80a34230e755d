"""The device's compact compensation codec (srs_comp.h) against the oracle.

The FP32 engines store each Euler compensation term c as the IEEE half of
c * 2^24, rounded to nearest even and saturated to +-65504 (a NaN stays a
NaN).  srs_comp_round_trip runs that round trip on the device, through the
forward engines' form and through the plain adjoint's packed form; the
oracle restates it with the compiler's _Float16.  Inputs: every finite half
value and every rounding tie between neighbouring halves (both signs),
values across the whole FP32 range, zeros of both signs, infinities, NaN.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs():
    h = np.arange(0, 0x7C00, dtype=np.uint16).view(np.float16).astype(np.float32)
    mid = (h[:-1] + h[1:]) / np.float32(2.0)
    scaled = np.concatenate([h, -h, mid, -mid]) * np.float32(2.0 ** -24)
    rng = np.random.default_rng(9)
    wide = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-40, 38, 20000)).astype(np.float32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 65504 * 2.0 ** -24, 65520 * 2.0 ** -24,
                        -65520 * 2.0 ** -24, 2.0 ** -49, 3 * 2.0 ** -50], np.float32)
    return np.concatenate([scaled, wide, special])


@pytest.mark.parametrize("packed", [False, True])
def test_device_codec_equals_oracle(srs, oracle, packed):
    x = _inputs()
    got = srs.comp_round_trip(x, packed=packed)
    want = np.array([oracle.lib.or_comp_round_trip(float(v)) for v in x], np.float32)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    # bit for bit, zeros' signs included
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))
