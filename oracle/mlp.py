"""CPU oracle for the learned rate surrogate -- TEST INFRASTRUCTURE ONLY.

Only the tests, the entry point's smoke check and the benchmark's CPU leg use this module, and
only to check the CUDA path; the product never calls it.

What it restates:

* ``species_rates``: the chirality-resolved Förster-form labeller that stands in for the
  reference's exciton_transfer rates (src/exciton_transfer/exciton_transfer.cpp:380-441, not
  built here).  It generalises the Förster formula of create_forster_scatt_table
  (src/monte_carlo/monte_carlo.cpp:174-187) taken at zero axis shifts,
  gamma_0 cos^2(theta) (1 nm / d)^6, with a donor/acceptor factor, an angle floor and a near-field
  length.  With neutral species (equal energies and diameters), floor 0 and near-field 0 it is
  that formula bit for bit -- the pin against the reference.  Against exciton_transfer itself
  parity is unpinned: that model is not built.
* ``features``, ``forward``, ``loss_and_grad``, ``adam``: the 4 -> 64 -> 64 -> 1 GELU network
  with BF16 weight matrices (FP32 biases and pair embedding, FP32 master weights), in float64
  arithmetic on the BF16-rounded weights, so that the GPU's FP32 accumulation is checked against
  a more exact sum.
"""
from __future__ import annotations

import math

import numpy as np

H = 64          # hidden width
IN = 4          # inputs: log-distance, angle, 2-wide chirality-pair embedding
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
OFF_E = 4548    # OFF_B3 + 1 rounded up to a multiple of 4
GELU_K0 = math.sqrt(2.0 / math.pi)
GELU_K1 = 0.044715


def n_params(n_species: int) -> int:
    return OFF_E + 2 * n_species * n_species


def species_rates(model: dict, dist, theta, donor, acceptor) -> np.ndarray:
    """rate = gamma_0 s_ab (cos^2 theta + floor) (1 nm / sqrt(d^2 + l^2))^6 with
    s_ab = (D_a D_b / D_ref^2) exp(-dE^2 / (2 w^2)) min(1, exp(-dE / kT)), dE = E_b - E_a."""
    dist = np.asarray(dist, np.float64)
    theta = np.asarray(theta, np.float64)
    a = np.asarray(donor)
    b = np.asarray(acceptor)
    e = np.asarray(model["energy"], np.float64)
    dia = np.asarray(model["diameter"], np.float64)
    de = e[b] - e[a]
    s = (dia[a] * dia[b]) / (model["diameter_ref"] * model["diameter_ref"])
    s = s * np.exp(-(de * de) / (2 * model["width"] * model["width"]))
    s = s * np.where(de > 0, np.exp(-de / model["kT"]), 1.0)
    c = np.cos(theta)
    ell = model["near_field"]
    r = np.sqrt(dist * dist + ell * ell)
    return model["gamma_0"] * s * (c * c + model["floor"]) * (1.e-9 / r) ** 6


def species_table(model: dict, dist, theta) -> np.ndarray:
    """[n_species][n_species][n_dist][n_theta] table of species_rates."""
    ns = len(model["energy"])
    dist = np.asarray(dist, np.float64)
    theta = np.asarray(theta, np.float64)
    a, b, i, k = np.meshgrid(np.arange(ns), np.arange(ns), np.arange(len(dist)), np.arange(len(theta)),
                             indexing="ij")
    return species_rates(model, dist[i], theta[k], a, b)


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 value, ties to even (finite inputs)."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def features(dist, theta, d_min, d_max) -> np.ndarray:
    """[n][2] float32: ln(d / d_min) 2 / ln(d_max / d_min) - 1 and theta 4 / pi - 1."""
    dist = np.asarray(dist, np.float64)
    theta = np.asarray(theta, np.float64)
    x0 = np.log(dist / d_min) * (2.0 / math.log(d_max / d_min)) - 1.0
    x1 = theta * (4.0 / math.pi) - 1.0
    return np.stack([x0, x1], 1).astype(np.float32)


def unpack(params, n_species, quantize=True):
    """The three weight matrices rounded to BF16, biases and the pair embedding read as FP32.  With
    quantize=False every parameter is taken as given in float64 (finite-difference checks)."""
    if quantize:
        p = np.asarray(params, np.float32).astype(np.float64)
        q = bf16(params).astype(np.float64)
    else:
        p = q = np.asarray(params, np.float64)
    npair = n_species * n_species
    return {
        "W1": q[OFF_W1:OFF_B1].reshape(H, IN), "b1": p[OFF_B1:OFF_W2],
        "W2": q[OFF_W2:OFF_B2].reshape(H, H), "b2": p[OFF_B2:OFF_W3],
        "W3": q[OFF_W3:OFF_B3], "b3": p[OFF_B3],
        "E": p[OFF_E:OFF_E + 2 * npair].reshape(npair, 2),
    }


def gelu(z):
    t = np.tanh(GELU_K0 * (z + GELU_K1 * z ** 3))
    return 0.5 * z * (1 + t), t


def gelu_grad(z, t):
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * GELU_K0 * (1 + 3 * GELU_K1 * z * z)


def forward(params, n_species, feat, pair, quantize=True):
    """Network output y (normalised log-rate) and the activations backward needs."""
    w = unpack(params, n_species, quantize)
    x = np.concatenate([np.asarray(feat, np.float64), w["E"][np.asarray(pair)]], 1)
    z1 = x @ w["W1"].T + w["b1"]
    a1, t1 = gelu(z1)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2, t2 = gelu(z2)
    y = a2 @ w["W3"] + w["b3"]
    return y, (w, x, z1, t1, a1, z2, t2, a2)


def loss_and_grad(params, n_species, feat, pair, target, quantize=True):
    """Mean squared error of y against target and its gradient with respect to every parameter
    (the gradient of the BF16 weights, applied to the FP32 master copy)."""
    y, (w, x, z1, t1, a1, z2, t2, a2) = forward(params, n_species, feat, pair, quantize)
    n = len(y)
    r = y - np.asarray(target, np.float64)
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    g = np.zeros(n_params(n_species))
    g[OFF_W3:OFF_B3] = a2.T @ dy
    g[OFF_B3] = dy.sum()
    d2 = dy[:, None] * w["W3"][None, :] * gelu_grad(z2, t2)
    g[OFF_W2:OFF_B2] = (d2.T @ a1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    d1 = (d2 @ w["W2"]) * gelu_grad(z1, t1)
    g[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    dx = d1 @ w["W1"]
    dE = np.zeros((n_species * n_species, 2))
    np.add.at(dE, np.asarray(pair), dx[:, 2:])
    g[OFF_E:] = dE.ravel()
    return loss, g


def adam(params, m, v, g, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (bias-corrected) of the FP32 master weights; step counts from 1."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    p = np.asarray(params, np.float64) - lr * mh / (np.sqrt(vh) + eps)
    return p.astype(np.float32), m, v


def targets(log_rate, log_mean, log_scale) -> np.ndarray:
    """Normalised labels as the device stores them (float32)."""
    return ((np.asarray(log_rate, np.float64) - log_mean) / log_scale).astype(np.float32)
