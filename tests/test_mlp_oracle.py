"""The FP64 network oracle's backpropagation against central finite differences."""
import numpy as np

from oracle import mlp_oracle as mo


def _params(rng, i, h1, h2, o):
    return [rng.standard_normal((h1, i)) / np.sqrt(i), 0.1 * rng.standard_normal(h1),
            rng.standard_normal((h2, h1)) / np.sqrt(h1), 0.1 * rng.standard_normal(h2),
            rng.standard_normal((o, h2)) / np.sqrt(h2), 0.1 * rng.standard_normal(o)]


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng, 6, 5, 4, 7)
    x = rng.standard_normal((3, 6))
    t = rng.standard_normal((3, 7))
    valid = 5
    _, g = mo.loss_and_gradients(p, x, t, valid, emulate_bf16=False)
    h = 1e-6
    for k in range(6):
        flat = p[k].reshape(-1)
        for idx in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp = mo.loss_only(p, x, t, valid)
            flat[idx] = old - h
            lm = mo.loss_only(p, x, t, valid)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            an = g[k].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-7 + 1e-5 * abs(fd), (k, idx, fd, an)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38])
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0           # tie -> even
    assert r[2] == 1.0 + 2 ** -7                  # representable
    assert r[3] == 1.0 + 2 ** -6                  # tie -> even (upwards)
    assert r[4] == -2.5
    assert np.isfinite(r[5])


def test_gelu_derivative():
    z = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    assert np.abs(fd - mo.gelu_deriv(z)).max() < 1e-8
