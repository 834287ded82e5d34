"""Rate tables for the engine (the reference's scattering_struct, src/monte_carlo/scattering_struct.h).

* ``forster_4d``: the reference's own Förster table on its 4-D (theta, z_shift,
  axis_shift_1, axis_shift_2) grid, built by the library exactly as
  ``create_forster_scatt_table`` (monte_carlo.cpp:156-200) builds it.
* ``forster_2d``: a 2-D (centre distance, folded angle) table -- the table shape of the
  benchmark films -- filled with the same Förster formula evaluated at zero axis shifts,
  where it reduces to gamma_0 cos^2(theta) (1 nm / d)^6.  It stands in for tables labelled
  by the reference's exciton_transfer model, which this package does not compute.
* ``read_reference_table``: a table saved by ``scattering_struct::save`` (:56-94).
"""
from __future__ import annotations

import os

import numpy as np

REF_PI = 3.141592  # src/helper/constants.h:10; the reference scales theta grids with it

FORSTER_GAMMA = 1.0e15  # "forster" rate type, monte_carlo.cpp:51-53
WONG_GAMMA = 1.0e13     # "wong" rate type, monte_carlo.cpp:55-57


def linspace(start: float, end: float, num: int) -> np.ndarray:
    """arma::linspace as the engine defines it: start + i (end - start)/(num - 1), last = end."""
    num = int(num)
    if num == 1:
        return np.array([float(end)])
    out = np.empty(num)
    delta = (float(end) - float(start)) / float(num - 1)
    for i in range(num - 1):
        out[i] = float(start) + float(i) * delta
    out[num - 1] = float(end)
    return out


def forster_4d(gamma_0, theta_deg, zshift, ash1, ash2) -> dict:
    from .engine import forster_table

    return forster_table(gamma_0, theta_deg, zshift, ash1, ash2)


def forster_2d(gamma_0: float = FORSTER_GAMMA, distance_m=(0.5e-9, 10e-9, 96), theta_deg=(0.0, 90.0, 91)) -> dict:
    """Built by the library (kmc_forster2d_table), so that the C++ and Python drivers use the
    same table bit for bit."""
    from .engine import forster2d_table

    return forster2d_table(gamma_0, distance_m, theta_deg)


def read_reference_table(directory: str) -> dict:
    """Load scat_table.{theta,z_shift,axis_shift_1,axis_shift_2,rates}.dat."""
    base = os.path.join(directory, "scat_table")
    g = [np.loadtxt(base + f".{n}.dat", ndmin=1) for n in ("theta", "z_shift", "axis_shift_1", "axis_shift_2")]
    with open(base + ".rates.dat") as f:
        lines = [ln.strip() for ln in f]
    vals = [float(v) for v in lines[4:] if v]
    rate = np.asarray(vals).reshape([len(x) for x in g])
    return {"kind": 4, "grids": g, "rate": rate}
