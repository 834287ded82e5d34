"""Learned pair-rate surrogate for mixed-chirality films.

The reference fills one rate table per film from exciton_transfer
(src/exciton_transfer/exciton_transfer.cpp:380-441), for one chirality pair.  A film of several
chiralities needs a table per (donor, acceptor) pair.  This module trains the engine's
4 -> 64 -> 64 -> 1 network (the kmc_mlp_* calls: forward, backward and Adam kernels on the GPU)
on labelled (distance, angle, pair) samples and turns it into a KMC_TABLE_2D_SPECIES table that
the neighbour build reads per site pair.

Labels come from the reference's exciton-transfer model on the GPU
(``exciton.PairLabeller``: exciton_transfer::first_order between tubes of the film's
chiralities); its own tables stay the fallback and the yardstick of the network's error
(``rate_errors``, and the diffusion coefficient of a film run with each table).  A closed-form
chirality-resolved Förster labeller (kmc_species_rates, a model dict from ``species_model``)
serves the unit tests of the network's kernels, which need cheap labels of a known form.
"""
from __future__ import annotations

import math

import numpy as np

from . import engine as E

A_LATTICE = 0.246e-9  # graphene lattice constant, m
CHIRALITIES = ((6, 5), (7, 5), (8, 3), (8, 4))
E11_EV = (1.27, 1.21, 1.30, 1.12)  # approximate E11 exciton energies of those tubes, eV
D_RANGE = (0.5e-9, 10e-9)          # centre distances of the tables, m
BATCH = 152 * 128                  # one 128-sample chunk per SM per step


def tube_diameter(n: int, m: int) -> float:
    """Diameter of an (n, m) tube: a sqrt(n^2 + n m + m^2) / pi."""
    return A_LATTICE * math.sqrt(n * n + n * m + m * m) / math.pi


def species_model(chiralities=CHIRALITIES, energies_ev=E11_EV, gamma_0=1e15, width_ev=0.1, kT_ev=0.02585,
                  floor=0.05, near_field=0.3e-9, reference=(7, 5)) -> dict:
    """Parameters of the labeller for a set of chiralities (diameters relative to ``reference``)."""
    return {
        "chiralities": tuple(chiralities),
        "gamma_0": float(gamma_0),
        "energy": np.asarray(energies_ev, np.float64),
        "diameter": np.asarray([tube_diameter(*c) for c in chiralities]),
        "diameter_ref": tube_diameter(*reference),
        "width": float(width_ev),
        "kT": float(kT_ev),
        "floor": float(floor),
        "near_field": float(near_field),
    }


def neutral_model(n_species: int = 1, gamma_0: float = 1e15) -> dict:
    """Equal chiralities, no angle floor, no near-field length: the plain Förster form."""
    return {"chiralities": ((7, 5),) * n_species, "gamma_0": float(gamma_0), "energy": np.zeros(n_species),
            "diameter": np.ones(n_species), "diameter_ref": 1.0, "width": 1.0, "kT": 1.0, "floor": 0.0,
            "near_field": 0.0}


def n_species(labeller) -> int:
    """Chiralities of a labeller: an exciton.PairLabeller or a closed-form model dict."""
    return labeller.n_species if hasattr(labeller, "n_species") else len(labeller["energy"])


def label(labeller, dist, theta, donor, acceptor) -> np.ndarray:
    """Pair rates (1/s) from an exciton.PairLabeller or a closed-form model dict."""
    if hasattr(labeller, "rates"):
        return labeller.rates(dist, theta, donor, acceptor)
    return E.species_rates(labeller, dist, theta, donor, acceptor)


def contact_distance(labeller, donor, acceptor) -> np.ndarray:
    """Closest centre distance of two tubes (m) per pair, below which the labeller's rate is flat;
    0 for a labeller without one (the closed-form model)."""
    donor, acceptor = np.asarray(donor), np.asarray(acceptor)
    if not hasattr(labeller, "contact"):
        return np.zeros(np.broadcast(donor, acceptor).shape)
    S = n_species(labeller)
    c = np.array([[labeller.contact(a, b) for b in range(S)] for a in range(S)])
    return c[donor, acceptor]


def draw_samples(labeller, n: int, seed: int = 0, d_range=D_RANGE, log_distance: bool = False) -> dict:
    """n labelled samples: distance uniform (or, with log_distance, uniform in ln d, which puts
    more samples where rates are large and change fastest), folded angle uniform, donor and
    acceptor uniform."""
    rng = np.random.default_rng(seed)
    S = n_species(labeller)
    u = rng.uniform(0.0, 1.0, n)
    theta = rng.uniform(0.0, math.pi / 2, n)
    donor = rng.integers(0, S, n).astype(np.int32)
    acceptor = rng.integers(0, S, n).astype(np.int32)
    # a labeller with a contact distance (exciton.PairLabeller) is flat below it: samples start there
    lo = np.maximum(d_range[0], contact_distance(labeller, donor, acceptor))
    if log_distance:
        dist = np.exp(np.log(lo) + u * (math.log(d_range[1]) - np.log(lo)))
    else:
        dist = lo + u * (d_range[1] - lo)
    rate = label(labeller, dist, theta, donor, acceptor)
    return {"dist": dist, "theta": theta, "donor": donor, "acceptor": acceptor,
            "pair": (donor * S + acceptor).astype(np.int32), "log_rate": np.log(rate)}


def grids(n_dist: int = 96, n_theta: int = 91, d_range=D_RANGE):
    """Distance grid (m) and folded-angle grid (rad) of the tables."""
    return np.linspace(d_range[0], d_range[1], n_dist), np.linspace(0.0, math.pi / 2, n_theta)


def labeller_table(labeller, dist, theta) -> dict:
    """The labeller's own KMC_TABLE_2D_SPECIES table (the fallback the network replaces)."""
    S = n_species(labeller)
    dist = np.asarray(dist, np.float64)
    theta = np.asarray(theta, np.float64)
    a, b, i, k = np.meshgrid(np.arange(S), np.arange(S), np.arange(len(dist)), np.arange(len(theta)), indexing="ij")
    rate = label(labeller, dist[i.ravel()], theta[k.ravel()], a.ravel(), b.ravel())
    return {"kind": 3, "grids": [dist, theta], "rate": rate.reshape(S, S, len(dist), len(theta))}


def single_table(labeller, dist, theta, species: int = 1) -> dict:
    """One chirality's table used for every pair: a film modelled without the surrogate."""
    dist = np.asarray(dist, np.float64)
    theta = np.asarray(theta, np.float64)
    i, k = np.meshgrid(np.arange(len(dist)), np.arange(len(theta)), indexing="ij")
    s = np.full(i.size, species)
    rate = label(labeller, dist[i.ravel()], theta[k.ravel()], s, s)
    return {"kind": 2, "grids": [dist, theta], "rate": rate.reshape(len(dist), len(theta))}


class RateSurrogate:
    """The network of one engine context, trained on labelled samples."""

    def __init__(self, engine: E.Engine, labeller, d_range=D_RANGE):
        self.e = engine
        self.labeller = labeller
        self.S = n_species(labeller)
        self.d_range = d_range

    def fit(self, samples: dict, epochs: int = 200, batch: int = BATCH, lr: float = 3e-3, lr_final: float = 3e-5,
            seed: int = 1) -> dict:
        """Initialise (output scaled to the labels' mean and spread) and train with Adam.  On a
        GB300, 200 epochs over 2M samples take 1.5 s and reach a median rate error of 0.2 %."""
        lr_ = samples["log_rate"]
        self.e.mlp_init(self.S, self.d_range[0], self.d_range[1], float(lr_.mean()), float(lr_.std()), seed)
        self.e.mlp_set_samples(samples["dist"], samples["theta"], samples["pair"], lr_)
        return self.e.mlp_train(epochs, batch, lr, lr_final)

    def _clamp(self, dist, pair):
        pair = np.asarray(pair)
        return np.maximum(np.asarray(dist, np.float64), contact_distance(self.labeller, pair // self.S, pair % self.S))

    def predict(self, dist, theta, pair) -> np.ndarray:
        """ln(rate) of the network; below a pair's contact distance, its value at contact (the
        labeller's rates are flat there and the network is trained from contact outwards)."""
        return self.e.mlp_predict(self._clamp(dist, pair), theta, pair)

    def table(self, dist, theta) -> dict:
        dist, theta = np.asarray(dist, np.float64), np.asarray(theta, np.float64)
        rate = self.e.mlp_rate_table(dist, theta)
        if hasattr(self.labeller, "contact"):  # rows below contact take the contact-distance rate
            for a in range(self.S):
                for b in range(self.S):
                    dc = self.labeller.contact(a, b)
                    rows = np.nonzero(dist < dc)[0]
                    if len(rows):
                        at = np.exp(self.e.mlp_predict(np.full(len(theta), dc), theta,
                                                       np.full(len(theta), a * self.S + b, np.int32)))
                        rate[a, b, rows, :] = at[None, :]
        return {"kind": 3, "grids": [dist, theta], "rate": rate}

    def rate_errors(self, samples: dict) -> dict:
        """Relative rate error |rate_net / rate_label - 1| over held-out samples."""
        pred = self.predict(samples["dist"], samples["theta"], samples["pair"])
        rel = np.abs(np.expm1(pred - samples["log_rate"]))
        return {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max())}


def film_diffusion(film, species, n_species_: int, table: dict, n_excitons: int, n_steps: int, dt: float,
                   velocity: float, seed: int, r_max: float = 10e-9, batches: int = 32, device: int = 0):
    """Diffusion coefficient (D[3], 95% CI[3], m^2/s) of a mixed film run with a rate table:
    uniform injection, mixed-precision hops, MSD in ``batches`` exciton batches."""
    from . import _lib as L
    from . import diffusion

    e = E.Engine(device)
    try:
        e.load_films(film)
        e.set_species(species, n_species_)
        e.set_table(table)
        e.build(r_max)
        e.set_msd_batches(batches)
        e.init_excitons(n_excitons, seed, L.KMC_INJECT_UNIFORM)
        e.run(n_steps, dt, velocity, L.KMC_PREC_MIXED)
        msd = e.msd_batches(0, n_steps)[0]
    finally:
        e.close()
    t = np.arange(1, n_steps + 1) * dt
    return diffusion.fit(msd, n_excitons, t)


def site_species(film, tube_species) -> np.ndarray:
    """Per-site chirality index from one index per tube of a Film."""
    lens = np.diff(film.tube_offsets)
    return np.repeat(np.asarray(tube_species, np.int32), lens)
