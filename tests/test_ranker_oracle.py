"""The ranker's CPU oracle (oracle/ranker_oracle.py) pinned by itself: its
analytic gradient equals central finite differences of its loss (without the
bf16 rounding, which makes the loss piecewise constant in the weights), and
its bf16 rounding is round-to-nearest-even. No GPU needed."""

import numpy as np

import ranker_oracle as R


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    n = 64
    x = rng.normal(size=(n, R.FEAT))
    y = (rng.random(n) < 0.3).astype(np.float64)
    w = rng.uniform(0.5, 3.0, n)
    p = R.init_params(3).astype(np.float64)
    _, g, _ = R.loss_and_grad(p, x, y, w, round_bf16=False)
    h = 1e-4
    idx = list(range(0, R.B1, 37)) + list(range(R.B1, R.W2, 7)) + list(range(R.W2, R.B2, 5)) + [R.B2]
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _, _ = R.loss_and_grad(pp.astype(np.float32), x, y, w, round_bf16=False)
        lm, _, _ = R.loss_and_grad(pm.astype(np.float32), x, y, w, round_bf16=False)
        # float32 params: use the actually representable step
        step = float(np.float32(p[i] + h)) - float(np.float32(p[i] - h))
        fd = (lp - lm) / step
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_round_to_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.01171875, 1.0078125, -2.5, 3.140625, 1e-20], np.float32)
    r = R.bf16_round(vals)
    assert r[0] == 1.0
    assert r[1] == 1.0            # halfway (1 + 2^-8): ties to even -> 1.0
    assert r[2] == 1.015625       # halfway above an odd mantissa: rounds up to even
    assert r[3] == 1.0078125      # exactly representable
    assert r[4] == -2.5
    assert (r.view(np.uint32) & 0xFFFF == 0).all()
