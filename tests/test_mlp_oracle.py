"""The surrogate network's CPU oracle, pinned by float64 finite differences
(its gradient formulas), plus its bf16 rounding rule."""
import numpy as np

from oracle import mlp_oracle as mo


def _tiny(seed, sizes=(3, 8, 8, 2)):
    rng = np.random.default_rng(seed)
    return [(rng.normal(size=(k, n)) / np.sqrt(k), 0.1 * rng.normal(size=n)) for k, n in zip(sizes[:-1], sizes[1:])]


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0], dtype=np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 and r[4] == -2.5
    assert np.all(np.abs(mo.bf16(np.linspace(-3, 3, 1001, dtype=np.float32)) -
                         np.linspace(-3, 3, 1001, dtype=np.float32)) <= 2 ** -8 * 3)


def test_gradients_match_finite_differences():
    params = _tiny(0)
    rng = np.random.default_rng(1)
    X = rng.normal(size=(5, 3))
    T = rng.normal(size=(5, 2))
    w = np.array([1.0, 0.5])

    def loss(ps):
        Y, _ = mo.forward(ps, X, rounding=False, dtype=np.float64)
        return mo.loss_grad(Y, T, w, dtype=np.float64)[0]

    Y, cache = mo.forward(params, X, rounding=False, dtype=np.float64)
    _, dY = mo.loss_grad(Y, T, w, dtype=np.float64)
    grads = mo.backward(params, cache, dY, rounding=False, dtype=np.float64)
    h = 1e-6
    for li, (W, b) in enumerate(params):
        for arr, g in ((W, grads[li][0]), (b, grads[li][1])):
            for idx in list(np.ndindex(arr.shape))[:6]:
                old = arr[idx]
                arr[idx] = old + h
                lp = loss(params)
                arr[idx] = old - h
                lm = loss(params)
                arr[idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - g[idx]) <= 1e-7 * max(1.0, abs(fd)), (li, idx, fd, g[idx])


def test_adam_step_matches_formula():
    params = [(np.ones((2, 2), np.float32), np.zeros(2, np.float32))]
    grads = [(np.full((2, 2), 0.5, np.float32), np.ones(2, np.float32))]
    st = mo.adam_state(params)
    out = mo.adam(params, grads, st, 1, 1e-3)
    # first step: m_hat = g, v_hat = g^2 -> update lr * sign(g)
    assert np.allclose(out[0][0], 1.0 - 1e-3, atol=1e-7)
    assert np.allclose(out[0][1], -1e-3, atol=1e-7)
