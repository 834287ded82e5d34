"""Synthetic film generator: exact unit axes (the parallel-branch condition of find_neighbors)."""
from __future__ import annotations

import numpy as np

from cnt_film_monte_carlo_gb300 import film as F


def test_unit_axes_are_exact_and_close_to_the_requested_direction():
    rng = np.random.default_rng(5)
    phi = rng.uniform(0, np.pi, 50000)
    tilt = rng.uniform(-np.pi / 2, np.pi / 2, 50000)
    # directions almost along y (a0, a2 tiny) are the hard case for the rounded sum
    phi[:2000] = np.pi / 2 + rng.uniform(-0.02, 0.02, 2000)
    tilt[:2000] = rng.uniform(-0.01, 0.01, 2000)
    a = F.unit_axes(phi, tilt)
    assert (F._dot3(a) == 1.0).all()
    want = np.stack([np.cos(phi) * np.cos(tilt), np.sin(phi) * np.cos(tilt), np.sin(tilt)], axis=1)
    assert np.abs(a - want).max() < 1e-11


def test_large_lognormal_film_generates():
    f = F.lognormal_tubes(2000, 500.0, 0.4, (1500.0, 1500.0, 50.0), seed=7)
    assert (F._dot3(f.orient) == 1.0).all()
    assert f.n_sites == int(f.tube_offsets[-1])
