"""Order properties of the closing, checked on the oracle (CPU): the
closing and its dilation contain the input (extensive), and a smaller input
never gives a larger closing (monotone), in both modes and for both
structuring elements.  The reference pairs a dilation by r + 1 with an
erosion by r - 1, so the closing is not idempotent and that is not asked."""
import numpy as np
import pytest

from broxy_gb300 import synth
from oracle import oracle as O


@pytest.mark.parametrize("res", [16, 32])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("se", [0, 1])
def test_closing_extensive_and_monotone(res, mode, se):
    rng = np.random.default_rng(1000 * res + 10 * mode + se)
    for seed in range(2):
        X2 = synth.random_grid(res, 300 + seed)
        X1 = X2 & rng.integers(0, 256, size=X2.shape, dtype=np.uint8)
        for r in (2, 4):
            R = O.scale_grid(res, uniform=r)
            D2, _, C2 = O.close(X2, res, [res] * 3, R, mode, se)
            _, _, C1 = O.close(X1, res, [res] * 3, R, mode, se)
            assert np.array_equal(D2 & X2, X2)
            assert np.array_equal(C2 & X2, X2)
            assert np.array_equal(C1 & C2, C1)
