"""The CPU oracle of the learned preconditioner's network (oracle/unet_ref.py)
checked on its own: parameter gradients against central finite differences,
and the transposes it uses (pool, nearest up-sampling, trilinear
prolongation) against their forward maps by dot-product identities."""
import numpy as np

import unet_ref as U


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    n = 8
    x = rng.standard_normal((n, n, n, 2))
    p = U.init_params(1) + 0.01 * rng.standard_normal(U.n_params())
    w = rng.standard_normal((n, n, n))
    y, cache = U.forward(p, x)
    g = U.backward(p, cache, w)
    off, _ = U.param_offsets()
    idx = []
    for name, ci, co in U.LAYERS:  # a few weights and the first bias of every layer
        w0, b0, _, _ = off[name]
        idx += list(rng.choice(np.arange(w0, b0), 3, replace=False)) + [b0]
    h = 1e-6
    for k in idx:
        e = np.zeros_like(p)
        e[k] = h
        fd = (np.sum(w * U.forward(p + e, x)[0]) - np.sum(w * U.forward(p - e, x)[0])) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_transposes():
    rng = np.random.default_rng(4)
    a = rng.standard_normal((8, 8, 8, 3))
    b = rng.standard_normal((4, 4, 4, 3))
    assert np.isclose(np.sum(U.pool(a) * b), np.sum(a * U.pool_backward(b)))
    assert np.isclose(np.sum(U.up(b) * a), np.sum(b * U.up_backward(a)))
    f = rng.standard_normal((8, 8, 8))
    c = rng.standard_normal((4, 4, 4))
    assert np.isclose(np.sum(U.prolong(c) * f), np.sum(c * U.prolong_adjoint(f)))
    # prolongation reproduces constants
    assert np.allclose(U.prolong(np.full((4, 4, 4), 2.5)), 2.5)
