"""Diffusion-coefficient fit (host) and its batch bookkeeping (CPU)."""
import numpy as np

from cnt_film_monte_carlo_gb300 import diffusion
from cnt_film_monte_carlo_gb300 import tables
from helpers import synthetic_film
from oracle import oracle as O


def test_fit_recovers_known_slope_and_ci_covers():
    rng = np.random.default_rng(0)
    B, n_steps, n_exc = 32, 200, 32 * 32 * 10
    counts = diffusion.batch_counts(n_exc, B)
    assert counts.sum() == n_exc and np.all(counts == n_exc // B)
    t = np.arange(1, n_steps + 1) * 1e-12
    D = np.array([3e-4, 1e-4, 2e-6])
    hits = 0
    for trial in range(40):
        slopes = D[None, :] * (1 + 0.05 * rng.standard_normal((B, 3)))
        msd = (2 * slopes[None, :, :] * t[:, None, None] + 1e-24 * rng.standard_normal((n_steps, B, 3)))
        msd *= counts[None, :, None]
        d, ci = diffusion.fit(msd, n_exc, t)
        assert np.all(np.abs(d - D) < 5 * ci + 1e-12)
        hits += np.all(np.abs(d - D) <= ci)
    assert hits >= 30  # ~95% coverage per axis


def test_oracle_batch_sums_add_up():
    f = synthetic_film(20, 40.0, (80, 80, 6), seed=2)
    tab = tables.forster_2d(1e15)
    a = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, 2e5)
    a.create_excitons(1, 0, 1000, 3)
    mb = a.step_batches(1e-13, 5, 8)
    b = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, 2e5)
    b.create_excitons(1, 0, 1000, 3)
    m = b.step(1e-13, 5)
    np.testing.assert_allclose(mb.sum(axis=1), m, rtol=1e-13)
    d = a.excitons()["delta"]
    for k in range(8):
        sel = (np.arange(1000) // 32) % 8 == k
        np.testing.assert_allclose(mb[-1, k], (d[sel] ** 2).sum(axis=0), rtol=1e-13)
