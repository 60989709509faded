"""The statistics helpers behind the surrogate-against-exact comparison in bench.py: block
standard errors over the last three quarters of a run, the extended-energy drift fit, and the
comparison in units of combined standard errors (CPU only)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_series_stats_mean_block_error_and_drift():
    rng = np.random.default_rng(3)
    n = 4000
    temps = 1.0 + 0.01 * rng.standard_normal(n)
    pots = 50.0 + rng.standard_normal(n // 2)
    # extended energy rising by 0.25 per bead per 10^4 steps, sampled every 40 steps
    n_beads, e_every = 100, 40
    steps = e_every * (np.arange(n // 2) + 1)
    ext = n_beads * (7.0 + 0.25e-4 * steps)
    st = bench._series_stats(temps, pots, ext, 20, e_every, n_beads)
    tail = temps[n // 4:]
    assert st["T_mean"] == pytest.approx(tail.mean())
    # 8 block means of independent samples: their standard error is close to sd / sqrt(len)
    assert st["T_se"] == pytest.approx(tail.std() / np.sqrt(len(tail)), rel=0.6)
    assert st["potential_mean"] == pytest.approx(pots[len(pots) // 4:].mean())
    assert st["drift_per_bead_per_1e4_steps"] == pytest.approx(0.25, rel=1e-9)
    assert st["samples"] == n


def test_compare_stats_z_scores():
    a = {"4": {"T_mean": 1.0, "T_se": 0.003, "potential_mean": 10.0, "potential_se": 0.4,
               "drift_per_bead_per_1e4_steps": -0.002, "drift_se": 0.0003}}
    b = {"4": {"T_mean": 1.004, "T_se": 0.004, "potential_mean": 10.0, "potential_se": 0.3,
               "drift_per_bead_per_1e4_steps": -0.001, "drift_se": 0.0004}}
    c = bench._compare_stats(a, b)
    assert c["4"]["T_z"] == pytest.approx(0.8)
    assert c["4"]["potential_z"] == pytest.approx(0.0)
    assert c["4"]["drift_z"] == pytest.approx(2.0)
    assert c["max_abs_z"] == pytest.approx(2.0)
    assert c["beyond_2se"] == 0 and c["compared"] == 3
