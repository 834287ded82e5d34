"""Diffusion coefficient with a confidence interval from batch MSD curves.

The reference only plots MSD/t (visualization/monte_carlo_results.py:478-500).  Here, per
exciton batch and axis, D_b = slope/2 of the least-squares line through <dx^2>(t) over the last
``fit_fraction`` of the steps; D = mean over batches, 95% CI = t(0.975, B-1) sd / sqrt(B)
(the library's kmc_fit_diffusion, host only).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def batch_counts(n_excitons: int, batches: int) -> np.ndarray:
    """Excitons per batch: exciton i belongs to batch (i // 32) % batches."""
    idx = np.arange(n_excitons)
    return np.bincount((idx // 32) % batches, minlength=batches).astype(np.int64)


def fit(msd_batches: np.ndarray, n_excitons: int, times: np.ndarray, fit_fraction: float = 0.8):
    """msd_batches: [n_steps][batches][3] sums of one film; returns (D[3], ci95[3]) in m^2/s."""
    m = np.ascontiguousarray(msd_batches, dtype=np.float64)
    return fit_counts(m, batch_counts(n_excitons, m.shape[1]), times, fit_fraction)


def fit_counts(msd_batches: np.ndarray, counts: np.ndarray, times: np.ndarray, fit_fraction: float = 0.8):
    """As fit, with the excitons of every batch given (e.g. batches gathered from replicas)."""
    m = np.ascontiguousarray(msd_batches, dtype=np.float64)
    n_steps, batches = m.shape[0], m.shape[1]
    counts = np.ascontiguousarray(counts, dtype=np.int64)
    if counts.shape != (batches,):
        raise ValueError("one exciton count per batch")
    t = np.ascontiguousarray(times, dtype=np.float64)
    D = np.zeros(3)
    ci = np.zeros(3)
    rc = L.load().kmc_fit_diffusion(L.ptr(m, C.c_double), L.ptr(counts, C.c_int64), L.ptr(t, C.c_double), n_steps,
                                    batches, fit_fraction, L.ptr(D, C.c_double), L.ptr(ci, C.c_double))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, "kmc_fit_diffusion failed")
    return D, ci
