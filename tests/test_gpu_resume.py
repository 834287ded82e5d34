"""Checkpoint/resume through kmc_get_excitons / kmc_set_excitons on the GPU.

n steps in one context against k steps, a saved state, and n - k steps in a fresh context
restored from it: every exciton's site, position, displacement, dwell clock, heading, Philox
counter and hop count equal bit for bit, in both precisions, with region injection (excitons
removed and reinjected, region_mode) and uniform injection, two films with their own seeds.  The
resumed run's MSD bins are the uninterrupted run's bins k.. (sums of device atomics: 1e-12
relative).  Bad states are refused before anything is written.
"""
import ctypes as C

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables

pytestmark = pytest.mark.gpu

V, BIN = 2e5, 1e-12
KEYS = ("site", "pos", "delta", "ff", "heading", "draws", "hops")


def films():
    return [F.straight_tubes(60, 150.0, box_nm=(300.0, 300.0, 10.0), max_tilt_deg=5.0, seed=11),
            F.lognormal_tubes(80, 120.0, 0.5, (250.0, 250.0, 12.0), seed=12)]


def engine(fs, tab, mode, n_exc=(1500, 900), seeds=(5, 77)):
    e = E.Engine(0)
    e.load_films(fs)
    e.set_table(tab)
    e.build(10e-9)
    e.init_excitons(list(n_exc), list(seeds), mode, 5)
    return e


@pytest.fixture(scope="module")
def setup():
    return films(), tables.forster_2d(1e15)


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
@pytest.mark.parametrize("mode", [L.KMC_INJECT_REGION, L.KMC_INJECT_UNIFORM])
def test_resume_is_bit_exact(setup, precision, mode):
    fs, tab = setup
    n, k = 60, 23
    e = engine(fs, tab, mode)
    e.run(n, BIN, V, precision)
    full, msd_full = e.excitons(), e.msd(0, n)
    assert e.stats()["hops"] > 0
    e.close()

    e = engine(fs, tab, mode)
    e.run(k, BIN, V, precision)
    saved = e.excitons()
    e.close()

    e = engine(fs, tab, mode)
    e.set_excitons(saved)
    back = e.excitons()
    for key in KEYS:  # the restored state reads back unchanged
        assert np.array_equal(back[key], saved[key]), key
    e.run(n - k, BIN, V, precision)
    res = e.excitons()
    for key in KEYS:
        assert np.array_equal(res[key], full[key]), key
    np.testing.assert_allclose(e.msd(0, n - k), msd_full[:, k:], rtol=1e-12, atol=0)
    e.close()


def test_resume_across_precisions(setup):
    # a state saved by the mixed kernel continues in the FP64 kernel
    fs, tab = setup
    e = engine(fs, tab, L.KMC_INJECT_REGION)
    e.run(40, BIN, V, L.KMC_PREC_FP64)
    full = e.excitons()
    e.close()
    e = engine(fs, tab, L.KMC_INJECT_REGION)
    e.run(17, BIN, V, L.KMC_PREC_MIXED)
    saved = e.excitons()
    e.close()
    e = engine(fs, tab, L.KMC_INJECT_REGION)
    e.set_excitons(saved)
    e.run(23, BIN, V, L.KMC_PREC_FP64)
    res = e.excitons()
    e.close()
    for key in KEYS:
        assert np.array_equal(res[key], full[key]), key


def test_bad_states_are_refused(setup):
    fs, tab = setup
    e = E.Engine(0)
    e.load_films(fs)
    e.set_table(tab)
    e.build(10e-9)
    i32, f64, u64, i64 = np.zeros(1, np.int32), np.zeros(3), np.zeros(1, np.uint64), np.zeros(1, np.int64)
    rc = e.lib.kmc_set_excitons(e.h, L.ptr(i32, C.c_int32), L.ptr(f64, C.c_double), L.ptr(f64, C.c_double),
                                L.ptr(f64, C.c_double), L.ptr(i32, C.c_int32), L.ptr(u64, C.c_uint64),
                                L.ptr(i64, C.c_int64))
    assert rc == L.KMC_ERR_STATE  # no exciton set laid out yet
    e.init_excitons([10, 10], [1, 2], L.KMC_INJECT_UNIFORM)
    e.run(3, BIN, V)
    good = e.excitons()
    n_sites = [f.n_sites for f in fs]
    bad = []
    for key, idx, val in (("site", 3, -1), ("site", 12, n_sites[1]), ("heading", 0, 2), ("hops", 5, -1),
                          ("ff", 1, np.nan), ("ff", 2, -1.0), ("pos", (4, 1), np.inf), ("delta", (0, 2), np.nan)):
        s = {k: v.copy() for k, v in good.items()}
        s[key][idx] = val
        bad.append(s)
    for s in bad:
        with pytest.raises(L.KmcError) as ei:
            e.set_excitons(s)
        assert ei.value.code == L.KMC_ERR_ARG
        after = e.excitons()
        for key in KEYS:  # nothing written
            assert np.array_equal(after[key], good[key]), key
    with pytest.raises(ValueError):
        e.set_excitons({k: v[:-1] for k, v in good.items()})
    e.close()
