"""The benchmark configurations at their stated size and duration, on the GPU.

Short runs are bit-exact elsewhere; these runs are long enough for the rare events of the mixed
form (an FP64 re-resolve every ~4e4 hops, link crossings, step ends) to happen millions of times.

* cfg 1: 100 straight tubes x 200 nm (500 x 500 x 10 nm box), 10^4 excitons, Philox seed 1234,
  10 ns in 1 ps bins (10,000 MSD bins, ~2e11 hops).  Mixed = plain FP64 for every exciton over
  the whole run (site, position, displacement, dwell clock, heading, draw and hop counters); the
  first 128 excitons equal an oracle run of just them; the MSD sums agree to 1e-12; D from 32
  exciton batches lies inside the 95 % interval of the oracle's 128-exciton sub-ensemble.
* cfg 2 film: 10^5 excitons (seed 1) for 1 ns: mixed = plain FP64 for every exciton.
* cfg 3: all 256 films (seeds 0-255, 27.7 M excitons) for one 1 ps bin in one persistent launch:
  spatial work order = slot order = plain FP64, every exciton and every film's MSD sums.

The plain FP64 kernel runs with 32-thread blocks, so that a few thousand excitons reach every SM,
and the mixed run, the FP64 run and the oracle run side by side (each engine owns its stream; the
library's calls release the interpreter lock).
"""
import threading

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import diffusion
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu

V, BIN = 2e5, 1e-12
KEYS = ("site", "pos", "delta", "ff", "heading", "draws", "hops")
MSD_RTOL = 1e-12


def bench_film():
    return F.straight_tubes(100, 200.0, box_nm=(500.0, 500.0, 10.0), max_tilt_deg=5.0, seed=1234)


def gpu_run(films, tab, n_exc, seeds, steps, precision, order=L.KMC_ORDER_AUTO, batches=1, block=None):
    e = E.Engine(0)
    e.load_films(films)
    e.set_table(tab)
    e.build(10e-9)
    e.set_work_order(order)
    e.set_graph(False)
    if block is not None:
        e.set_launch_config(block, 32)
    e.set_msd_batches(batches)
    e.init_excitons(n_exc, seeds, L.KMC_INJECT_UNIFORM)
    used = e.work_order()
    e.run(steps, BIN, V, precision)
    out = {"x": e.excitons(), "msd": e.msd(0, steps), "stats": e.stats(), "order": used}
    if batches > 1:
        out["batches"] = e.msd_batches(0, steps)
    e.close()
    return out


def in_threads(**jobs):
    """Run the named callables side by side; return their results (re-raise the first error)."""
    res, err = {}, []

    def wrap(name, fn):
        try:
            res[name] = fn()
        except BaseException as ex:  # noqa: BLE001 - re-raised in the test's thread
            err.append(ex)

    ts = [threading.Thread(target=wrap, args=(k, f)) for k, f in jobs.items()]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if err:
        raise err[0]
    return res


def assert_same(a, b):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k


def test_cfg1_ten_nanoseconds():
    f = bench_film()
    tab = tables.forster_2d(1e15)
    n_exc, seed, steps, B, n_o = 10_000, 1234, 10_000, 32, 128

    def oracle():
        sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, V, n_threads=16)
        sim.create_excitons(1, 0, n_o, seed)
        ob = sim.step_batches(BIN, steps, 4)  # 4 batches of 32 excitons
        return sim.excitons(), ob

    r = in_threads(mixed=lambda: gpu_run([f], tab, n_exc, seed, steps, L.KMC_PREC_MIXED, batches=B),
                   fp64=lambda: gpu_run([f], tab, n_exc, seed, steps, L.KMC_PREC_FP64, batches=B, block=32),
                   oracle=oracle)
    gm, gf = r["mixed"], r["fp64"]
    assert_same(gm["x"], gf["x"])
    assert gm["stats"]["hops"] == gf["stats"]["hops"] > 1e11
    np.testing.assert_allclose(gm["msd"], gf["msd"], rtol=MSD_RTOL)
    np.testing.assert_allclose(gm["batches"], gf["batches"], rtol=MSD_RTOL)
    ox, ob = r["oracle"]
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert np.array_equal(gm["x"][k][:n_o], ox[k]), k
    t = np.arange(1, steps + 1) * BIN
    d_gpu, ci_gpu = diffusion.fit(gm["batches"][0], n_exc, t)
    d_o, ci_o = diffusion.fit(ob, n_o, t)
    assert np.all(np.isfinite(d_gpu)) and np.all(ci_gpu > 0)
    assert np.all(np.abs(d_gpu - d_o) <= ci_o), (d_gpu, ci_gpu, d_o, ci_o)


def test_cfg2_film_one_nanosecond():
    f = bench_film()
    tab = tables.forster_2d(1e15)
    n_exc, seed, steps = 100_000, 1, 1000
    r = in_threads(mixed=lambda: gpu_run([f], tab, n_exc, seed, steps, L.KMC_PREC_MIXED),
                   fp64=lambda: gpu_run([f], tab, n_exc, seed, steps, L.KMC_PREC_FP64))
    gm, gf = r["mixed"], r["fp64"]
    assert_same(gm["x"], gf["x"])
    assert gm["stats"]["hops"] == gf["stats"]["hops"] > 2e11
    assert gm["stats"]["exact_resolves"] > 1_000_000  # the rare path ran millions of times
    np.testing.assert_allclose(gm["msd"], gf["msd"], rtol=MSD_RTOL)


def test_cfg3_all_films_one_bin():
    films, n_exc = [], []
    for i in range(256):
        rng = np.random.default_rng(i)
        n_t = int(rng.integers(50, 2001))
        films.append(F.lognormal_tubes(n_t, 300.0, 0.5, (1000.0, 1000.0, 20.0), seed=i))
        n_exc.append(100 * n_t)
    tab = tables.forster_2d(1e15)
    seeds = list(range(256))
    gs = gpu_run(films, tab, n_exc, seeds, 1, L.KMC_PREC_MIXED, L.KMC_ORDER_SPATIAL)
    assert gs["order"] == L.KMC_ORDER_SPATIAL
    assert gs["stats"]["hops"] > 5e10
    for precision, order in ((L.KMC_PREC_MIXED, L.KMC_ORDER_SLOTS), (L.KMC_PREC_FP64, L.KMC_ORDER_AUTO)):
        g = gpu_run(films, tab, n_exc, seeds, 1, precision, order)
        assert_same(gs["x"], g["x"])
        assert g["stats"]["hops"] == gs["stats"]["hops"]
        np.testing.assert_allclose(g["msd"], gs["msd"], rtol=MSD_RTOL)  # [film][step][3], every film
        del g
