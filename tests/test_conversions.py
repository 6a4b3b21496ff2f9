"""The integer-pipe conversions of the mixed stage against the hardware
conversions, over magnitudes from the conserved volume integrals' range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_integer_conversions_match_hardware():
    from knc import abi
    rng = np.random.default_rng(5)
    x = np.concatenate([
        rng.standard_normal(200000) * np.exp(rng.uniform(-80, 80, 200000)),   # |x| in ~[1e-35, 1e35]
        np.array([0.0, -0.0, 1.0, -1.0, 0.5, 3.0e38, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24,
                  1.0 + 2.0 ** -24 + 2.0 ** -40, np.nextafter(1.0, 2.0)]),
    ]).astype(np.float64)
    out = np.empty((len(x), 4))
    st = abi.load().knc_test_conversions(abi.dptr(x), len(x), abi.dptr(out))
    assert st == 0
    normal = np.abs(x) >= 1.1754943508222875e-38
    assert np.array_equal(out[normal, 0], out[normal, 1])          # d2f: round to nearest even
    assert np.array_equal(out[:, 2], out[:, 1])                    # f2d exact
    assert np.array_equal(out[:, 3], x * 0.5)                      # exact halving
