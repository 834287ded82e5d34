"""GB300-native exciton-hopping kinetic Monte Carlo for carbon-nanotube films.

A drop-in engine for the Green-Kubo hot path of amirhosseindavoody/cnt_film_monte_carlo:
excitons hop over the segments ("sites") of a CNT film with dwell times drawn from each
site's total transfer rate, the next site chosen by a cumulative-rate search over its
neighbour list, free flight along the tube between hops, and the time-binned mean squared
displacement reduced to a diffusion coefficient.  Mixed-chirality films read one rate table
per (donor, acceptor) chirality pair, which a small network trained on the GPU can build
(``surrogate``).  All compute runs in hand-written CUDA kernels for sm_103a behind the C ABI of
include/cntkmc.h.
"""
from .film import Film, lognormal_tubes, read_mesh as read_mesh_files, straight_tubes, write_mesh  # noqa: F401

__all__ = ["Film", "straight_tubes", "lognormal_tubes", "write_mesh", "read_mesh_files", "Engine", "monte_carlo",
           "RateSurrogate"]


def __getattr__(name):
    if name == "Engine":
        from .engine import Engine

        return Engine
    if name == "monte_carlo":
        from .monte_carlo import monte_carlo

        return monte_carlo
    if name == "RateSurrogate":
        from .surrogate import RateSurrogate

        return RateSurrogate
    raise AttributeError(name)
