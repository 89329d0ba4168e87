"""The CPU checker of the learned predictor: its analytic gradients agree
with central finite differences when the bfloat16 roundings are switched
off (a check of the checker itself)."""
import numpy as np

import oracle.mlp_ref as R


def test_reference_gradients_match_finite_differences(monkeypatch):
    monkeypatch.setattr(R, "bf16", lambda a: np.asarray(a, dtype=np.float64))
    rng = np.random.default_rng(0)
    params = [rng.normal(0, 0.3, s) for s in [(R.HID, R.IN), (R.HID,), (R.HID, R.HID), (R.HID,),
                                              (R.OUT_PAD, R.HID), (R.OUT_PAD,)]]
    X = rng.normal(size=(5, R.IN))
    T = rng.normal(size=(5, R.OUT_PAD))
    loss, grads = R.loss_and_grads(params, X, T)
    eps = 1e-6
    for t, (p, g) in enumerate(zip(params, grads)):
        for _ in range(6):
            idx = tuple(rng.integers(0, d) for d in p.shape)
            if t in (4, 5) and idx[0] >= R.OUT:
                continue
            old = p[idx]
            p[idx] = old + eps
            lp, _ = R.loss_and_grads(params, X, T)
            p[idx] = old - eps
            lm, _ = R.loss_and_grads(params, X, T)
            p[idx] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(fd), (t, idx, fd, g[idx])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0], dtype=np.float32)
    got = R.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -6 and got[3] == -2.5
