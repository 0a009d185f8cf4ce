"""The comparison helpers the parity tests share: a NaN or an infinity on either side must fail a
bar, never pass it (Python's max(worst, nan) keeps worst, so a NaN result would slip through a
running maximum)."""
import numpy as np

from conftest import relmax


def test_relmax_values():
    b = np.array([1.0, -2.0, 4.0])
    assert relmax(b, b) == 0.0
    assert abs(relmax(b + np.array([0.0, 0.0, 1e-12]), b) - 1e-12 / 4.0) <= 1e-16
    assert relmax(np.zeros(3), np.zeros(3)) == 0.0


def test_relmax_non_finite_fails_every_bar():
    b = np.array([1.0, 2.0, 3.0])
    for bad in (np.nan, np.inf, -np.inf):
        a = b.copy()
        a[1] = bad
        assert not relmax(a, b) <= 1e300
        assert not relmax(b, a) <= 1e300
        # the same through a running maximum, as the step loops accumulate it
        worst = 0.0
        for x, y in ((b, b), (a, b), (b, b)):
            worst = max(worst, relmax(x, y))
        assert not worst <= 1e300


def test_running_maximum_keeps_nan():
    worst = 0.0
    for e in (1e-14, float("nan"), 1e-15):
        worst = float(np.maximum(worst, e))
    assert np.isnan(worst) and not worst <= 1.0
