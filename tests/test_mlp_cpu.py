"""The CPU reference of the learned-guess MLP: its backward pass agrees with
finite differences of its own loss (so it can check the device gradients)."""
import numpy as np

import knc_oracle
from knc import abi, learned


def _setup(n=16, seed=3):
    rng = np.random.default_rng(seed)
    w = learned.init_weights(seed)
    x = rng.normal(size=(n, 3)).astype(np.float32)
    y = rng.normal(size=n).astype(np.float32)
    w[abi.KNC_MLP_OFF_XMEAN:abi.KNC_MLP_OFF_XMEAN + 3] = 0.1
    w[abi.KNC_MLP_OFF_XSCALE:abi.KNC_MLP_OFF_XSCALE + 3] = 0.9
    w[abi.KNC_MLP_OFF_B1:abi.KNC_MLP_OFF_B1 + 64] = rng.normal(size=64) * 0.1
    return w, x, y


def test_oracle_gradient_matches_finite_differences(oracle_lib):
    w, x, y = _setup()
    _, loss, grad = knc_oracle.mlp_forward_backward(w, x, y, round_bf16=False)
    assert np.isfinite(loss) and loss > 0
    # every parameter group, without the bf16 rounding (a staircase in the
    # parameters that finite differences cannot see through)
    rng = np.random.default_rng(0)
    idx = [abi.KNC_MLP_OFF_B3]
    for off, size in [(abi.KNC_MLP_OFF_W1, 192), (abi.KNC_MLP_OFF_B1, 64), (abi.KNC_MLP_OFF_W2, 4096),
                      (abi.KNC_MLP_OFF_B2, 64), (abi.KNC_MLP_OFF_W3, 64)]:
        idx += list(off + rng.choice(size, 5, replace=False))
    for k in idx:
        h = 1e-3
        wp = w.copy(); wp[k] += h
        wm = w.copy(); wm[k] -= h
        lp = knc_oracle.mlp_forward_backward(wp, x, y, round_bf16=False)[1]
        lm = knc_oracle.mlp_forward_backward(wm, x, y, round_bf16=False)[1]
        fd = (lp - lm) / (float(wp[k]) - float(wm[k]))
        assert abs(fd - grad[k]) <= 1e-3 * max(1e-3, abs(grad[k])) + 1e-6, (k, fd, grad[k])


def test_features_match_formula():
    pairs = np.array([[2.0, 0.3, 0.4, 0.7, 1.0, 0.1, 0.1, 0.2]])
    x, y = learned.features(pairs)
    d, s, tau = 2.0, 0.5, 0.7
    a = tau * (tau + 2 * d) - s * s
    assert np.allclose(x[0], [np.log(tau / d), -np.log(1 - s / (d + tau)), np.log(a / d ** 2)], rtol=1e-5)
    assert np.allclose(y[0], np.log(0.1), rtol=1e-6)


def test_features_scale_invariant():
    pairs = np.array([[2.0, 0.3, 0.4, 0.7, 1.0, 0.1, 0.1, 0.2]])
    scaled = pairs.copy()
    scaled[:, :4] *= 1e5
    scaled[:, [4, 7]] *= 1e5
    x0, y0 = learned.features(pairs)
    x1, y1 = learned.features(scaled)
    assert np.allclose(x0, x1, rtol=1e-5, atol=1e-5) and np.allclose(y0, y1, rtol=1e-6)
