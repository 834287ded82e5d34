"""Synthetic CNT films and the reference's mesh format.

A film is a set of straight carbon-nanotube (CNT) segments ("sites").  Each tube is cut
into segments of equal length; each site has a position (segment centre), a unit
orientation (the tube axis) and links to its left/right neighbour on the same tube
(-1 at a tube end).  This is the data the reference reads in
``monte_carlo::create_scatterers`` (src/monte_carlo/monte_carlo.h:199-271):

* six text matrices ``single_cnt.{pos,orient}.{x,y,z}.dat``, one row per tube and one
  column per point, positions in nm (scaled by 1e-9 on load, :211,225,239);
* site ``n = i * n_cols + j`` for tube ``i``, point ``j``; ``left = n - 1`` if ``j > 0``,
  ``right = n + 1`` if ``j + 1 < n_cols`` (:249-262).

The reference's real meshes came from a separate project and are not available; films
here are generated with a seeded numpy Generator.  Ragged films (tubes of different
lengths) cannot be written as one matrix; they are held in memory as site arrays with
tube offsets and passed to the engine directly.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

MESH_FILES = (
    "single_cnt.pos.x.dat",
    "single_cnt.pos.y.dat",
    "single_cnt.pos.z.dat",
    "single_cnt.orient.x.dat",
    "single_cnt.orient.y.dat",
    "single_cnt.orient.z.dat",
)


@dataclasses.dataclass
class Film:
    """Sites of one film.  ``pos_nm`` and ``orient`` are (n, 3) float64; ``left``/``right``
    are (n,) int32 site indices or -1; ``tube_offsets`` is (n_tubes + 1,) int64."""

    pos_nm: np.ndarray
    orient: np.ndarray
    left: np.ndarray
    right: np.ndarray
    tube_offsets: np.ndarray

    @property
    def n_sites(self) -> int:
        return int(self.pos_nm.shape[0])

    @property
    def n_tubes(self) -> int:
        return int(self.tube_offsets.shape[0] - 1)

    def pos_m(self) -> np.ndarray:
        """Positions in metres, scaled exactly as the reference scales its mesh (x * 1e-9)."""
        return self.pos_nm * 1.0e-9

    def is_rectangular(self) -> bool:
        lens = np.diff(self.tube_offsets)
        return bool(lens.size > 0 and np.all(lens == lens[0]))


def _dot3(a: np.ndarray) -> np.ndarray:
    """dot(a, a) per row in the engine's order: ((0 + a0 a0) + a2 a2) + (0 + a1 a1)."""
    return (a[:, 0] * a[:, 0] + a[:, 2] * a[:, 2]) + a[:, 1] * a[:, 1]


def unit_axes(phi: np.ndarray, tilt: np.ndarray) -> np.ndarray:
    """Unit tube axes from azimuth and tilt, nudged so that dot(a, a) == 1.0 exactly.

    Same-tube pairs take the reference's parallel branch only when dot(a1, a2) == 1
    exactly (src/monte_carlo/scatterer.cpp:46); an axis whose rounded self dot product is
    not exactly 1 would send same-tube pairs down the general branch with sin^2 ~ 1e-16.
    """
    phi = np.asarray(phi, dtype=np.float64)
    tilt = np.asarray(tilt, dtype=np.float64)
    a = np.stack([np.cos(phi) * np.cos(tilt), np.sin(phi) * np.cos(tilt), np.sin(tilt)], axis=1)
    for _ in range(4):
        bad = _dot3(a) != 1.0
        if not bad.any():
            break
        a[bad] = a[bad] / np.sqrt(_dot3(a[bad]))[:, None]
    todo = np.nonzero(_dot3(a) != 1.0)[0]
    # The rest: a1 enters the rounded sum last, so keep a2, move a0 by a few ulps and solve
    # a1 = +-sqrt(1 - fl(a0^2 + a2^2)), trying the nearby doubles.  Directions that admit no
    # such a1 are turned by up to 1e-12 rad (a fixed pseudo-random turn per attempt) and tried
    # again.
    for attempt in range(128):
        if todo.size == 0:
            break
        jit = np.random.default_rng(attempt).uniform(-1.0, 1.0, (2, todo.size)) * (1e-12 if attempt else 0.0)
        p = phi[todo] + jit[0]
        t = tilt[todo] + jit[1]
        v = np.stack([np.cos(p) * np.cos(t), np.sin(p) * np.cos(t), np.sin(t)], axis=1)
        v /= np.sqrt(_dot3(v))[:, None]
        sgn = np.where(v[:, 1] < 0, -1.0, 1.0)
        left = np.ones(len(todo), dtype=bool)
        for k0 in sorted(range(-4, 5), key=abs):
            for k1 in sorted(range(-4, 5), key=abs):
                idx = np.nonzero(left)[0]
                if idx.size == 0:
                    break
                w = v[idx].copy()
                w[:, 0] += k0 * np.spacing(np.abs(w[:, 0]))
                s02 = w[:, 0] * w[:, 0] + w[:, 2] * w[:, 2]
                a1 = np.sqrt(np.maximum(1.0 - s02, 0.0))
                w[:, 1] = sgn[idx] * (a1 + k1 * np.spacing(a1))
                ok = (_dot3(w) == 1.0) & (s02 <= 1.0)
                a[todo[idx[ok]]] = w[ok]
                left[idx[ok]] = False
        todo = todo[left]
    if todo.size:
        raise RuntimeError("could not make a unit axis with dot(a, a) == 1")
    return a


def straight_tubes(
    n_tubes: int,
    lengths_nm,
    box_nm=(500.0, 500.0, 10.0),
    max_tilt_deg: float = 5.0,
    segment_nm: float = 1.0,
    seed: int = 0,
) -> Film:
    """Straight tubes with uniform centres in ``box_nm``, azimuth U[0, pi) and tilt
    U[-max_tilt, max_tilt] out of the x-y plane, cut into ``segment_nm`` segments.
    ``lengths_nm`` is a scalar (all tubes alike) or one length per tube."""
    rng = np.random.default_rng(seed)
    lengths = np.broadcast_to(np.asarray(lengths_nm, dtype=np.float64), (n_tubes,)).copy()
    n_pts = np.maximum(1, np.rint(lengths / segment_nm).astype(np.int64))
    centres = rng.uniform(0.0, 1.0, size=(n_tubes, 3)) * np.asarray(box_nm, dtype=np.float64)
    phi = rng.uniform(0.0, np.pi, size=n_tubes)
    tilt = np.deg2rad(rng.uniform(-max_tilt_deg, max_tilt_deg, size=n_tubes))
    axes = unit_axes(phi, tilt)
    offsets = np.zeros(n_tubes + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(n_pts)
    n = int(offsets[-1])
    tube = np.repeat(np.arange(n_tubes), n_pts)
    j = np.arange(n) - offsets[tube]
    s = (j.astype(np.float64) + 0.5 - n_pts[tube] / 2.0) * segment_nm
    pos = centres[tube] + s[:, None] * axes[tube]
    orient = axes[tube].copy()
    left = np.where(j > 0, np.arange(n) - 1, -1).astype(np.int32)
    right = np.where(j + 1 < n_pts[tube], np.arange(n) + 1, -1).astype(np.int32)
    return Film(pos, orient, left, right, offsets)


def lognormal_tubes(n_tubes, median_nm, sigma, box_nm, seed=0, max_tilt_deg=5.0, segment_nm=1.0,
                    max_len_nm=None) -> Film:
    """Tubes with lognormal lengths (median, sigma), otherwise as ``straight_tubes``."""
    rng = np.random.default_rng(seed + 0x5EED)
    lengths = median_nm * np.exp(sigma * rng.standard_normal(n_tubes))
    if max_len_nm is not None:
        lengths = np.minimum(lengths, max_len_nm)
    lengths = np.maximum(lengths, segment_nm)
    return straight_tubes(n_tubes, lengths, box_nm, max_tilt_deg, segment_nm, seed)


def write_mesh(film: Film, directory: str) -> None:
    """Write the six matrices of ``create_scatterers`` (positions in nm, full precision)."""
    if not film.is_rectangular():
        raise ValueError("the reference mesh format needs the same number of points on every tube")
    os.makedirs(directory, exist_ok=True)
    rows, cols = film.n_tubes, int(film.tube_offsets[1] - film.tube_offsets[0])
    mats = [film.pos_nm[:, c].reshape(rows, cols) for c in range(3)]
    mats += [film.orient[:, c].reshape(rows, cols) for c in range(3)]
    for name, m in zip(MESH_FILES, mats):
        np.savetxt(os.path.join(directory, name), m, fmt="%.17g")


def read_mesh(directory: str) -> Film:
    """Read a mesh directory the way ``create_scatterers`` does."""
    mats = []
    for name in MESH_FILES:
        m = np.loadtxt(os.path.join(directory, name), dtype=np.float64, ndmin=2)
        mats.append(m)
    rows, cols = mats[0].shape
    for m in mats:
        if m.shape != (rows, cols):
            raise ValueError("mesh matrices differ in shape")
    pos = np.stack([m.reshape(-1) for m in mats[:3]], axis=1)
    orient = np.stack([m.reshape(-1) for m in mats[3:]], axis=1)
    n = rows * cols
    j = np.arange(n) % cols
    left = np.where(j > 0, np.arange(n) - 1, -1).astype(np.int32)
    right = np.where(j + 1 < cols, np.arange(n) + 1, -1).astype(np.int32)
    offsets = np.arange(rows + 1, dtype=np.int64) * cols
    return Film(pos, orient, left, right, offsets)
