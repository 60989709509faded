"""The CPU restatement of the surrogate network (oracle/mlp_oracle.py), pinned by finite
differences of its own loss: the network has no reference counterpart."""
import os
import sys

import numpy as np

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "oracle"))
import mlp_oracle as M  # noqa: E402


def test_bf16_rounds_to_nearest_even():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -8 + 2 ** -20, -2.5, 3.0e-39], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # halfway, ties to even
    assert r[2] == np.float32(1 + 2 ** -6)  # halfway, ties to even (upwards)
    assert r[3] == np.float32(1 + 2 ** -7)  # above halfway
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-39) < 2 ** -133 * 2 ** 8


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    n_in, width, n_out, m = 8, 16, 5, 7
    n = sum(a[0] * a[1] + b[0] for a, b in M.shapes(n_in, width, n_out))
    p = rng.normal(0, 0.4, n)
    x = rng.normal(0, 1, (m, n_in))
    t = rng.normal(0, 1, (m, n_out))
    loss, g = M.loss_and_grads(p, x, t, n_in, width, n_out, emulate=False)
    h = 1e-6
    for i in rng.choice(n, 60, replace=False):
        e = np.zeros(n)
        e[i] = h
        lp, _ = M.loss_and_grads(p + e, x, t, n_in, width, n_out, emulate=False)
        lm, _ = M.loss_and_grads(p - e, x, t, n_in, width, n_out, emulate=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    y = M.forward(p, x, n_in, width, n_out, emulate=False)
    assert abs(np.mean((y - t) ** 2) - loss) < 1e-12


def test_emulated_rounding_stays_close_to_exact():
    rng = np.random.default_rng(5)
    n_in, width, n_out, m = 64, 256, 132, 64
    n = sum(a[0] * a[1] + b[0] for a, b in M.shapes(n_in, width, n_out))
    p = rng.uniform(-1, 1, n) * 0.1
    x = rng.normal(0, 1, (m, n_in))
    t = rng.normal(0, 1, (m, n_out))
    l0, g0 = M.loss_and_grads(p, x, t, n_in, width, n_out, emulate=False)
    l1, g1 = M.loss_and_grads(p, x, t, n_in, width, n_out, emulate=True)
    assert abs(l1 - l0) < 1e-2 * l0
    assert np.linalg.norm(g1 - g0) < 5e-2 * np.linalg.norm(g0)
