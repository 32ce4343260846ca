"""Host side of the surrogate (no GPU): the Chebyshev encoding of eigenvector
fields is exact at full length, the features are finite and scaled, and the
target encoding inverts."""
import numpy as np

from stab_gb300 import surrogate as su


def test_chebyshev_round_trip_is_exact():
    rng = np.random.default_rng(0)
    ny = 32
    v = rng.normal(size=5 * ny) + 1j * rng.normal(size=5 * ny)
    c = su.chebyshev_coefficients(v, ny, ncheb=ny)
    back = su.chebyshev_eval(c, ny)
    p = int(np.argmax(np.abs(v)))
    assert np.max(np.abs(back - v / v[p])) < 1e-12


def test_truncated_expansion_of_smooth_fields():
    ny = 32
    eta = np.cos(np.pi * np.arange(ny) / (ny - 1))
    f = np.stack([np.exp(eta), np.sin(2 * eta), eta ** 3, np.cos(eta), 1 + 0 * eta], axis=1)
    v = (f * (1 + 0.5j)).reshape(-1)
    back = su.chebyshev_eval(su.chebyshev_coefficients(v, ny), ny)
    p = int(np.argmax(np.abs(v)))
    assert np.max(np.abs(back - v / v[p])) < 1e-10


def test_features_and_targets():
    P = su.sample_params(1000, 3)
    X = su.features(P["M"], P["Re"], P["alpha"], P["beta"], P["width"])
    assert X.shape == (1000, 6) and np.all(np.isfinite(X)) and np.max(np.abs(X)) < 2.0
    w = P["alpha"] * (0.9 - 0.001j)
    coef = np.ones((1000, 5, su.NCHEB)) * (0.5 - 0.25j)
    t = su.Surrogate.raw_targets(w, P["alpha"], coef)
    assert np.allclose(t[:, 0], 0.9) and np.allclose(t[:, 1], -0.1)
    s = su.Surrogate.__new__(su.Surrogate)
    s.mean, s.std = t.mean(0), np.maximum(t.std(0), 1e-6)
    w2, c2 = s.decode(((t - s.mean) / s.std).astype(np.float32), P["alpha"])
    assert np.allclose(w2, w, rtol=1e-6) and np.allclose(c2, coef, atol=1e-6)
