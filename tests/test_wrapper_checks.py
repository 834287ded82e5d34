"""The Python wrappers refuse numpy buffers shorter than the counts the C ABI reads (CPU).

The C entry points take plain pointers and read as many elements as their counts say, so a
short or mismatched array would be read past its end.  The wrappers compare every buffer with
its count first and raise KmcError(KMC_ERR_ARG) without calling the library.  The Engine checks
run before any device call; they are exercised here on an Engine made without a device.
"""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import surrogate as SG


class _NoLib:
    """Stands in for the library: any call means a check let a bad buffer through."""

    def __getattr__(self, name):
        raise AssertionError(f"{name} called with a buffer the wrapper should have refused")


def bare_engine(**attrs):
    e = object.__new__(E.Engine)
    e.lib, e.h = _NoLib(), None
    e.__dict__.update(attrs)
    return e


def refused(fn, *args, **kw):
    with pytest.raises(L.KmcError) as ei:
        fn(*args, **kw)
    assert ei.value.code == L.KMC_ERR_ARG
    return str(ei.value)


def test_load_arrays_needs_one_row_per_site():
    f = F.straight_tubes(2, 5.0, box_nm=(20, 20, 2), seed=1)
    e = bare_engine()
    n = f.n_sites
    off = np.array([0, n], np.int64)
    p, o = f.pos_m(), f.orient
    refused(e.load_arrays, off, p[:-1], o, f.left, f.right)
    refused(e.load_arrays, off, p, o[:-1], f.left, f.right)
    refused(e.load_arrays, off, p, o, f.left[:-1], f.right)
    refused(e.load_arrays, off, p, o, f.left, f.right[:-1])
    refused(e.load_arrays, np.array([0, n + 1], np.int64), p, o, f.left, f.right)
    refused(e.load_arrays, np.array([n], np.int64), p, o, f.left, f.right)


def test_set_table_needs_rates_for_every_grid_point():
    e = bare_engine()
    g4 = [np.linspace(0, 1, k) for k in (3, 4, 2, 2)]
    refused(e.set_table, {"kind": 4, "grids": g4, "rate": np.zeros(3 * 4 * 2 * 2 - 1)})
    refused(e.set_table, {"kind": 4, "grids": g4[:2], "rate": np.zeros(12)})
    g2 = [np.linspace(0, 1, 5), np.linspace(0, 1, 6)]
    refused(e.set_table, {"kind": 2, "grids": g2, "rate": np.zeros((5, 5))})
    refused(e.set_table, {"kind": 3, "grids": g2, "rate": np.zeros((2, 3, 5, 6))})
    refused(e.set_table, {"kind": 3, "grids": g2, "rate": np.zeros((2, 2, 5, 5))})


def test_species_neighbors_and_samples_are_sized():
    e = bare_engine(offsets=np.array([0, 10], np.int64))
    refused(e.set_species, np.zeros(9, np.int32), 2)
    refused(bare_engine().set_species, np.zeros(10, np.int32), 2)  # nothing loaded yet
    refused(bare_engine().neighbors, 10, 100)                      # nothing built yet
    e = bare_engine(_nbr={"n_sites": 10, "nnz": 100})
    refused(e.neighbors, 10, 99)
    refused(e.neighbors, 11, 100)
    e = bare_engine(mlp_species=2)
    d = np.ones(5)
    refused(e.mlp_set_samples, d, d[:4], np.zeros(5, np.int32), d)
    refused(e.mlp_set_samples, d, d, np.zeros(4, np.int32), d)
    refused(e.mlp_set_samples, d, d, np.zeros(5, np.int32), d[:3])
    refused(e.mlp_predict, d, d[:4], np.zeros(5, np.int32))
    refused(e.mlp_predict, d, d, np.zeros(6, np.int32))


def test_host_functions_check_their_buffers():
    f = F.straight_tubes(2, 5.0, box_nm=(20, 20, 2), seed=1)
    p, o = f.pos_m(), f.orient
    lim = [-1, 1, -1, 1, -1, 1]
    refused(E.trim_sites, p[:-1], o, f.left, f.right, lim)
    refused(E.trim_sites, p, o, f.left, f.right[:-1], lim)
    refused(E.trim_sites, p, o, f.left, f.right, lim[:5])
    model = SG.species_model()
    d = np.full(4, 2e-9)
    z = np.zeros(4, np.int32)
    refused(E.species_rates, model, d, d[:3], z, z)
    refused(E.species_rates, model, d, d, z[:3], z)
    bad = dict(model)
    bad["diameter"] = np.asarray(model["diameter"])[:-1]
    refused(E.species_rates, bad, d, d, z, z)
    # the unchanged call still works
    assert np.all(E.species_rates(model, d, d * 0, z, z) > 0)


def test_exciton_wrappers_check_geometry_and_grids():
    from cnt_film_monte_carlo_gb300 import exciton as X

    e = bare_engine()
    refused(X.coulomb_j, e, None, None, [[0, 0]], [1e-9, 0.0, 0.0])
    refused(X.davoody_table, e, None, None, theta_deg=(0, 180, 0))
    refused(X.davoody_table, e, None, None, zshift=(1e-9, 2e-9, float("nan")))
    big = (0.0, 1.0, 2**31 - 1)
    refused(X.davoody_table, e, None, None, theta_deg=big, zshift=big, ash1=big, ash2=big)


def test_rate_counts_are_exact_for_huge_grids():
    # the rate count of a table is the exact product of its grid lengths (np.prod would wrap in
    # int64 for grids whose product passes 2^63): 2^16 points per grid is 2^64 rates, refused
    e = bare_engine()
    g = np.zeros(1 << 16)
    refused(e.set_table, {"kind": 4, "grids": [g, g, g, g], "rate": np.zeros(1)})
