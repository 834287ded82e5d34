"""Output files of the contacts (steady-state flux) mode in the reference's formats.

* ``scatterer_statistics.dat``: get_scatterer_statistics (src/monte_carlo/monte_carlo.h:691-719),
  written once by init.
* ``population_profile.dat``: save_population_profile (:525-581), one row per step with the
  exciton density count / (area dy) of every y slab.
* ``region_current.dat``: save_currents (:584-643), one row per step with the current
  count / (interface area dt) through every slab interface.
* ``particle_path.<n>.dat``: track_particle (:786-818), the position after every step of one
  exciton walked from contact 1 to the last slab.

The reference writes them with iostreams in std::scientific (precision 6), all but the first also
with std::showpos, which prints a sign on every signed value -- also on the interface numbers of the
current-file header ("interface+0"), but not on the unsigned section numbers ("section0").
Densities and currents are formed from integer counts here exactly as there (one FP64 division
by one FP64 product), so the files agree character for character.
"""
from __future__ import annotations

import math

import numpy as np


def _div(a: float, b: float) -> float:
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


def _e(x: float, plus: bool) -> str:
    """iostream std::scientific (with std::showpos when plus) of a double."""
    if math.isnan(x):
        s = "nan"
        return ("-" if math.copysign(1.0, x) < 0 else ("+" if plus else "")) + s
    return f"{x:+e}" if plus else f"{x:e}"


def slab_positions(ymin: float, dy: float, n: int) -> np.ndarray:
    """Slab centres ymin + (i + 0.5) dy (monte_carlo.h:553, 708)."""
    return np.array([ymin + (float(i) + 0.5) * dy for i in range(n)])


def interface_positions(ymin: float, dy: float, n: int) -> np.ndarray:
    """Interfaces ymin + dy i, i = 1..n-1 (save_currents :595-597)."""
    return np.array([ymin + dy * float(i) for i in range(1, n)])


def interface_areas(area) -> np.ndarray:
    """(area[i-1] + area[i]) / 2 (save_currents :597)."""
    a = np.asarray(area, dtype=np.float64)
    return np.array([(a[i - 1] + a[i]) / 2 for i in range(1, len(a))])


def scatterer_statistics_text(ymin: float, dy: float, stat_pop, n_sites: int, area) -> str:
    out = ["position,distribution,population,density\n"]
    pos = slab_positions(ymin, dy, len(stat_pop))
    for i, p in enumerate(stat_pop):
        p = int(p)
        out.append(f"{_e(pos[i], False)},{_e(_div(float(p), float(n_sites)), False)},{p},"
                   f"{_e(_div(float(p), float(area[i]) * dy), False)}\n")
    return "".join(out)


def population_header(area, ymin: float, dy: float) -> str:
    n = len(area)
    pos = slab_positions(ymin, dy, n)
    return ("area" + "".join("," + _e(float(a), True) for a in area) + "\n\n"
            + "dy" + ("," + _e(dy, True)) * n + "\n\n"
            + "section pos" + "".join("," + _e(float(p), True) for p in pos) + "\n\n"
            + "time" + "".join(f",section{i}" for i in range(n)) + "\n")


def population_row(time: float, counts, area, dy: float) -> str:
    return _e(time, True) + "".join("," + _e(_div(float(c), float(a) * dy), True) for c, a in zip(counts, area)) + "\n"


def current_header(area, ymin: float, dy: float) -> str:
    n = len(area)
    aif = interface_areas(area)
    y = interface_positions(ymin, dy, n)
    return ("interface area" + "".join("," + _e(float(a), True) for a in aif) + "\n\n"
            + "interface pos" + "".join("," + _e(float(v), True) for v in y) + "\n\n"
            + "time" + "".join(f",interface{i:+d}" for i in range(n - 1)) + "\n")


def current_row(time: float, counts, area, dt: float) -> str:
    aif = interface_areas(area)
    return _e(time, True) + "".join("," + _e(_div(float(c), float(a) * dt), True) for c, a in zip(counts, aif)) + "\n"


def track_text(path) -> str:
    """particle_path.<n>.dat: "   x y z" per step (scientific, showpos), then an empty line."""
    return "".join(f"   {_e(float(x), True)} {_e(float(y), True)} {_e(float(z), True)}\n" for x, y, z in path) + "\n"


# ---------------------------------------------------------------- flux-gradient diffusion coefficient
def _csv_rows(text: str):
    return [line.split(",") for line in text.splitlines()]


def read_population(text: str) -> dict:
    """population_profile.dat as the reference's get_population reads it
    (visualization/monte_carlo_results.py:70-109, without its low-pass filter, which only the
    plots use): area, dy and section positions from the header rows, the densities per step,
    and their average over the steps."""
    rows = _csv_rows(text)
    area = np.array([float(v) for v in rows[0][1:]])
    dy = np.array([float(v) for v in rows[2][1:]])
    pos = np.array([float(v) for v in rows[4][1:]])
    data = np.array([[float(v) for v in r] for r in rows[7:] if r and r[0]])
    pop = data[:, 1:]
    return {"time": data[:, 0], "pop": pop, "area": area, "dy": dy, "pos": pos, "avg_pop": pop.mean(axis=0)}


def read_current(text: str) -> dict:
    """region_current.dat as the reference's get_current reads it (monte_carlo_results.py:31-68,
    without the filter): interface areas and positions, the current per step and its average over
    the steps (the steady current)."""
    rows = _csv_rows(text)
    area = np.array([float(v) for v in rows[0][1:]])
    pos = np.array([float(v) for v in rows[2][1:]])
    data = np.array([[float(v) for v in r] for r in rows[5:] if r and r[0]])
    cur = data[:, 1:]
    return {"time": data[:, 0], "current": cur, "area": area, "pos": pos, "steady": cur.mean(axis=0)}


def flux_gradient_diffusion(population: dict, current: dict) -> np.ndarray:
    """The contacts mode's diffusion coefficient at every slab interface, as the reference's
    post-processing forms it (monte_carlo_results.py:428-442): the steady current over the
    gradient of the average density, D_k = steady_k / ((avg_pop[k+1] - avg_pop[k]) / dy[k]).
    A current down the gradient gives a negative value, as there."""
    dp_dy = np.diff(population["avg_pop"]) / population["dy"][:-1]
    with np.errstate(divide="ignore", invalid="ignore"):
        return current["steady"] / dp_dy


def flux_gradient_diffusion_from_counts(population_counts, current_counts, area, dy: float, dt: float) -> np.ndarray:
    """The same coefficient from the engine's counts ([steps][n_segments] excitons per slab,
    [steps][n_segments - 1] net crossings per interface) instead of the files' rounded values."""
    pc = np.asarray(population_counts, dtype=np.float64)
    cc = np.asarray(current_counts, dtype=np.float64)
    area = np.asarray(area, dtype=np.float64)
    avg_pop = (pc / (area * dy)).mean(axis=0)
    steady = (cc / (interface_areas(area) * dt)).mean(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        return steady / (np.diff(avg_pop) / dy)
