"""The CPU reference of the proposal MLP's backward formulas against finite
differences.  The bf16 rounding of the activations makes the loss piecewise
constant at the scale of a finite-difference step, so the check runs on the
smooth surrogate (activations unrounded); the biases are not quantised, so
their gradients are exact derivatives of that surrogate."""
import numpy as np

from mlp_reference import F, H, forward_backward


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.integers(0, 40, size=(64, F)).astype(np.uint8)
    y = rng.normal(1.0, 0.5, size=64)
    w1 = rng.normal(0, 0.2, size=(H, F))
    b1 = rng.normal(0, 0.1, size=H)
    w2 = rng.normal(0, 0.2, size=H)
    b2 = 0.3
    fb = lambda *a: forward_backward(*a, round_h=False)  # noqa: E731
    loss, gw1, gb1, gw2, gb2 = fb(w1, b1, w2, b2, x, y)
    eps = 1e-4
    # biases are not quantised: exact finite differences up to bf16 rounding of h
    for k in (0, 7, 63):
        d = np.zeros(H)
        d[k] = eps
        num = (fb(w1, b1 + d, w2, b2, x, y)[0] - fb(w1, b1 - d, w2, b2, x, y)[0]) / (2 * eps)
        assert abs(num - gb1[k]) < 1e-3 * max(1e-3, abs(gb1[k])) + 1e-6
    num = (fb(w1, b1, w2, b2 + eps, x, y)[0] - fb(w1, b1, w2, b2 - eps, x, y)[0]) / (2 * eps)
    assert abs(num - gb2) < 1e-3 * max(1.0, abs(gb2))
    assert gw1.shape == (H, F) and gw2.shape == (H,) and np.isfinite(loss)
